// Host side of the `recurgreen` and `plothisto` programs: the settings
// files, the tasks (tdistrib, wavefunction, tprofile, tprofile_group,
// tpattern) and the re-binning of saved samples, as the reference's drivers
// do them (src/main.f90:7-877, src/plot_histogram.f90),
// on top of the C++ interface of include/recurgreen.hpp.
#pragma once

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace rgdriver {

// Console tags of src/base_utils.f90:48-50 (colour codes only on a terminal).
std::string tag_info();
std::string tag_warn();
std::string tag_error();
std::string tag_test();

// A stop of the reference's driver: the message goes to stderr, then
// "RecurGreen: Invalid arguments, aborting..." and a non-zero exit status.
struct Stop : std::runtime_error {
  explicit Stop(const std::string& msg) : std::runtime_error(msg) {}
};

// One value of a namelist entry: the raw text of each comma-separated item.
struct NmlValue {
  std::vector<std::string> items;
  std::string line;  // the source line of the entry, for error messages
};
using NmlGroup = std::map<std::string, NmlValue>;  // keys in lower case

// Reads group `&name ... /` of a namelist file, as Fortran's namelist read
// finds it: the first group of that name (case-insensitive), `!` comments
// outside quotes, `key = v1, v2, ...` entries.  Throws Stop with the
// reference's "Invalid entry in namelist" message on a malformed entry or on
// a key outside `allowed`; a missing group is an error too.
NmlGroup read_namelist(const std::string& text, const std::string& name, const std::vector<std::string>& allowed);

// Typed accessors (default when the key is absent; Stop on a bad value).
std::string nml_string(const NmlGroup& g, const std::string& key, const std::string& def);
long nml_int(const NmlGroup& g, const std::string& key, long def);
double nml_real(const NmlGroup& g, const std::string& key, double def);
bool nml_logical(const NmlGroup& g, const std::string& key, bool def);
// An array entry (`tm = 0.1, 0.4, ...`): exactly n reals, or `def` when absent.
std::vector<double> nml_reals(const NmlGroup& g, const std::string& key, size_t n, const std::vector<double>& def);

// Fortran G0.d output as gfortran writes it (F form with d significant
// digits for 0.1 <= |x| < 10^d, else 0.ddddE+-e).
std::string format_g0(double x, int d = 16);

// Bin edges: Chebyshev nodes (src/main.f90:233, src/plot_histogram.f90:84)
// or linear (src/plot_histogram.f90:82), nbins + 1 values on [xmin, xmax].
std::vector<double> chebyshev_bins(int nbins, double xmin = 0.0, double xmax = 1.0);
std::vector<double> linear_bins(int nbins, double xmin = 0.0, double xmax = 1.0);

// histogram (GPU) + eps/10 + normalize_histogram + moving_average
// (src/base_utils.f90:491-570): rows (bin centre, density).
struct Density {
  std::vector<double> centre, rho;
  double missing = 0.0;
};
Density density(const std::vector<double>& samples, const std::vector<double>& bins);

// read_real_array (src/base_utils.f90:663-697): the first list-directed real
// of every line; lines without one are skipped.
std::vector<double> read_real_array(const std::string& path);

// unique_filename (src/base_utils.f90:825-840): base<i>ext, first free i >= 1.
std::string unique_filename(const std::string& base, const std::string& ext);
// create_directory (src/base_utils.f90:846-849): mkdir -p.
void create_directory(const std::string& dir);

// `recurgreen settings.nml ...`, `plothisto settings.nml samples.csv` and
// `waveguide_test` (the reference's src/waveguide.test.f90).
int recurgreen_main(int argc, char** argv);
int plothisto_main(int argc, char** argv);
int waveguide_test_main(int argc, char** argv);

}  // namespace rgdriver
