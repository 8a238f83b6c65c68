// `waveguide_test`: the reference's test program src/waveguide.test.f90
// (parameters, unitarity of v1 and v2, v1 against v2), on the GPU library.
#include "driver.hpp"

int main(int argc, char** argv) { return rgdriver::waveguide_test_main(argc, argv); }
