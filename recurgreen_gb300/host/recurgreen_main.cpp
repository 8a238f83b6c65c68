// `recurgreen settings.nml [more.nml ...] [--outdir DIR]`: the reference's
// program (src/main.f90:7-33) for the tdistrib task, on the GPU library.
#include "driver.hpp"

int main(int argc, char** argv) { return rgdriver::recurgreen_main(argc, argv); }
