// `plothisto plothisto_settings.nml path/to/samples.csv`: the reference's
// re-binning program (src/plot_histogram.f90:7-42).
#include "driver.hpp"

int main(int argc, char** argv) { return rgdriver::plothisto_main(argc, argv); }
