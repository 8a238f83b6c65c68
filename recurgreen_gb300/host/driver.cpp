// The `recurgreen` and `plothisto` drivers (see driver.hpp).
#include "driver.hpp"

#include <sys/stat.h>
#include <unistd.h>

#include <cctype>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <limits>
#include <sstream>

#include "recurgreen.hpp"

namespace rgdriver {

namespace {

const char* kProgram = "RecurGreen-GB300 (recursive Green sweep on GB300)";
const char* kStopMessage = "RecurGreen: Invalid arguments, aborting...";

std::string lower(std::string s) {
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

std::string strip(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

bool is_ident_start(char c) { return std::isalpha((unsigned char)c) || c == '_'; }
bool is_ident(char c) { return std::isalnum((unsigned char)c) || c == '_'; }

// A namelist body with the source line of every character.
struct Body {
  std::string text;
  std::vector<int> line;  // index into `lines`
};

[[noreturn]] void invalid_entry(const std::string& line) {
  throw Stop("Invalid entry in namelist: " + strip(line) + "...");
}

// Fortran real (list-directed): [sign] digits [. digits] [(e|d) [sign] digits],
// or nan / inf / infinity.
bool parse_real(const std::string& tok, double* out) {
  std::string t = lower(strip(tok));
  if (t.empty()) return false;
  std::string u = (t[0] == '+' || t[0] == '-') ? t.substr(1) : t;
  const double sign = (t[0] == '-') ? -1.0 : 1.0;
  if (u == "nan") {
    *out = std::numeric_limits<double>::quiet_NaN();
    return true;
  }
  if (u == "inf" || u == "infinity") {
    *out = sign * std::numeric_limits<double>::infinity();
    return true;
  }
  size_t i = 0, nd = 0;
  while (i < u.size() && std::isdigit((unsigned char)u[i])) ++i, ++nd;
  if (i < u.size() && u[i] == '.') {
    ++i;
    while (i < u.size() && std::isdigit((unsigned char)u[i])) ++i, ++nd;
  }
  if (nd == 0) return false;
  std::string num = u.substr(0, i);
  if (i < u.size()) {
    if (u[i] != 'e' && u[i] != 'd') return false;
    size_t j = i + 1;
    if (j < u.size() && (u[j] == '+' || u[j] == '-')) ++j;
    const size_t k0 = j;
    while (j < u.size() && std::isdigit((unsigned char)u[j])) ++j;
    if (j == k0 || j != u.size()) return false;
    num += "e" + u.substr(i + 1);
  }
  char* end = nullptr;
  const double v = std::strtod(num.c_str(), &end);
  if (!end || *end != '\0') return false;
  *out = sign * v;
  return true;
}

bool parse_int(const std::string& tok, long* out) {
  const std::string t = strip(tok);
  size_t i = (!t.empty() && (t[0] == '+' || t[0] == '-')) ? 1 : 0;
  if (i >= t.size()) return false;
  for (size_t j = i; j < t.size(); ++j)
    if (!std::isdigit((unsigned char)t[j])) return false;
  errno = 0;
  const long v = std::strtol(t.c_str(), nullptr, 10);
  if (errno) return false;
  *out = v;
  return true;
}

const NmlValue* find(const NmlGroup& g, const std::string& key) {
  auto it = g.find(key);
  return it == g.end() ? nullptr : &it->second;
}

std::string timestamp() {
  std::time_t now = std::time(nullptr);
  std::tm lt{};
  localtime_r(&now, &lt);
  char buf[64];
  std::strftime(buf, sizeof buf, "%Y-%m-%d at %H:%M:%S %z", &lt);
  return buf;
}

std::string fmt_int(long v) { return std::to_string(v); }

// Fortran F0.d, including the F0.0 form "3." (a decimal point always).
std::string f0(double x, int d) {
  std::string s = recurgreen::format_f0(x, d);
  if (d == 0) s += ".";
  return s;
}

void write_rows(std::FILE* fp, const Density& d) {
  for (size_t j = 0; j < d.rho.size(); ++j)
    std::fprintf(fp, "%s, %s\n", format_g0(d.centre[j]).c_str(), format_g0(d.rho[j]).c_str());
}

std::string read_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  std::ostringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

bool file_exists(const std::string& path) {
  struct stat st;
  return ::stat(path.c_str(), &st) == 0;
}

}  // namespace

std::string tag_info() { return "[INFO] "; }
std::string tag_warn() {
  return isatty(STDOUT_FILENO) ? "[\033[1m\033[93mWARN\033[0m] " : "[WARN] ";
}
std::string tag_error() {
  return isatty(STDERR_FILENO) ? "[\033[1m\033[31mERROR\033[0m] " : "[ERROR] ";
}
std::string tag_test() {
  return isatty(STDOUT_FILENO) ? "[\033[1m\033[36mTEST\033[0m] " : "[TEST] ";
}

NmlGroup read_namelist(const std::string& text, const std::string& name, const std::vector<std::string>& allowed) {
  // Lines without comments (`!` outside quotes).
  std::vector<std::string> lines;
  {
    std::istringstream in(text);
    std::string raw;
    while (std::getline(in, raw)) {
      if (!raw.empty() && raw.back() == '\r') raw.pop_back();
      std::string out;
      char q = 0;
      for (char c : raw) {
        if (q) {
          out += c;
          if (c == q) q = 0;
        } else if (c == '\'' || c == '"') {
          q = c;
          out += c;
        } else if (c == '!') {
          break;
        } else {
          out += c;
        }
      }
      lines.push_back(out);
    }
  }
  const std::string want = "&" + lower(name);
  size_t start = lines.size();
  size_t col = 0;
  for (size_t k = 0; k < lines.size(); ++k) {
    const std::string s = lines[k];
    size_t a = 0;
    while (a < s.size() && std::isspace((unsigned char)s[a])) ++a;
    if (lower(s.substr(a, want.size())) == want &&
        (a + want.size() == s.size() || !is_ident(s[a + want.size()]))) {
      start = k;
      col = a + want.size();
      break;
    }
  }
  if (start == lines.size())
    throw Stop("Invalid entry in namelist: group &" + name + " not found...\n" + tag_warn() +
               "Try checking the spelling of the namelist groups...");
  // Body up to the terminating `/` outside quotes.
  Body body;
  bool closed = false;
  for (size_t k = start; k < lines.size() && !closed; ++k) {
    const std::string& s = lines[k];
    char q = 0;
    for (size_t c = (k == start ? col : 0); c < s.size(); ++c) {
      const char ch = s[c];
      if (q) {
        if (ch == q) q = 0;
      } else if (ch == '\'' || ch == '"') {
        q = ch;
      } else if (ch == '/') {
        closed = true;
        break;
      }
      body.text += ch;
      body.line.push_back((int)k);
    }
    body.text += '\n';
    body.line.push_back((int)k);
  }
  if (!closed) invalid_entry(lines.back());
  // Entries.
  NmlGroup g;
  const std::string& t = body.text;
  size_t i = 0;
  auto skip_sep = [&](size_t p) {
    while (p < t.size() && (std::isspace((unsigned char)t[p]) || t[p] == ',')) ++p;
    return p;
  };
  auto starts_entry = [&](size_t p) {  // identifier, spaces, '='
    if (p >= t.size() || !is_ident_start(t[p])) return false;
    while (p < t.size() && is_ident(t[p])) ++p;
    while (p < t.size() && std::isspace((unsigned char)t[p])) ++p;
    return p < t.size() && t[p] == '=';
  };
  for (i = skip_sep(i); i < t.size(); i = skip_sep(i)) {
    const std::string& src = lines[body.line[i]];
    if (!is_ident_start(t[i])) invalid_entry(src);
    size_t j = i;
    while (j < t.size() && is_ident(t[j])) ++j;
    const std::string key = lower(t.substr(i, j - i));
    while (j < t.size() && std::isspace((unsigned char)t[j])) ++j;
    if (j >= t.size() || t[j] != '=') invalid_entry(src);
    bool ok = false;
    for (const auto& a : allowed) ok = ok || a == key;
    if (!ok) invalid_entry(src);
    NmlValue v;
    v.line = src;
    i = j + 1;
    for (;;) {
      while (i < t.size() && std::isspace((unsigned char)t[i])) ++i;
      if (i >= t.size()) break;
      if (t[i] == ',') {
        ++i;
        continue;
      }
      if (starts_entry(i)) break;
      std::string item;
      if (t[i] == '\'' || t[i] == '"') {
        const char q = t[i++];
        while (i < t.size()) {
          if (t[i] == q) {
            if (i + 1 < t.size() && t[i + 1] == q) {  // doubled quote
              item += q;
              i += 2;
              continue;
            }
            ++i;
            break;
          }
          item += t[i++];
        }
        item = "\x01" + item;  // marks a quoted string
      } else {
        while (i < t.size() && !std::isspace((unsigned char)t[i]) && t[i] != ',') item += t[i++];
      }
      v.items.push_back(item);
    }
    if (v.items.empty()) invalid_entry(src);
    g[key] = v;
  }
  return g;
}

std::string nml_string(const NmlGroup& g, const std::string& key, const std::string& def) {
  const NmlValue* v = find(g, key);
  if (!v) return def;
  std::string s = v->items[0];
  if (!s.empty() && s[0] == '\x01') s = s.substr(1);
  // Fortran character variables compare without trailing blanks.
  while (!s.empty() && s.back() == ' ') s.pop_back();
  return s;
}

long nml_int(const NmlGroup& g, const std::string& key, long def) {
  const NmlValue* v = find(g, key);
  if (!v) return def;
  long x = 0;
  if (v->items.size() != 1 || !parse_int(v->items[0], &x)) invalid_entry(v->line);
  return x;
}

double nml_real(const NmlGroup& g, const std::string& key, double def) {
  const NmlValue* v = find(g, key);
  if (!v) return def;
  double x = 0.0;
  if (v->items.size() != 1 || !parse_real(v->items[0], &x)) invalid_entry(v->line);
  return x;
}

bool nml_logical(const NmlGroup& g, const std::string& key, bool def) {
  const NmlValue* v = find(g, key);
  if (!v) return def;
  std::string s = lower(strip(v->items[0]));
  if (v->items.size() != 1 || s.empty()) invalid_entry(v->line);
  if (s[0] == '.') s = s.substr(1);
  if (!s.empty() && s[0] == 't') return true;
  if (!s.empty() && s[0] == 'f') return false;
  invalid_entry(v->line);
}

std::vector<double> nml_reals(const NmlGroup& g, const std::string& key, size_t n, const std::vector<double>& def) {
  const NmlValue* v = find(g, key);
  if (!v) return def;
  std::vector<double> out;
  for (const std::string& it : v->items) {
    double x = 0.0;
    if (!parse_real(it, &x)) invalid_entry(v->line);
    out.push_back(x);
  }
  if (out.size() != n) invalid_entry(v->line);
  return out;
}

std::string format_g0(double x, int d) {
  if (std::isnan(x)) return "NaN";
  if (std::isinf(x)) return x > 0 ? "Infinity" : "-Infinity";
  const std::string sign = std::signbit(x) ? "-" : "";
  const double ax = std::fabs(x);
  if (ax == 0.0) return sign + "0." + std::string(d - 1, '0');
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.*e", d - 1, ax);  // D.DDDDe+XX
  const std::string s = buf;
  const size_t epos = s.find('e');
  std::string digits = s.substr(0, 1) + s.substr(2, epos - 2);
  const int e10 = std::atoi(s.c_str() + epos + 1) + 1;  // ax = 0.DDDD * 10^e10
  if (0 <= e10 && e10 <= d) {
    if (e10 == 0) return sign + "0." + digits;
    return sign + digits.substr(0, e10) + "." + digits.substr(e10);
  }
  return sign + "0." + digits + "E" + (e10 < 0 ? "-" : "+") + std::to_string(std::abs(e10));
}

std::vector<double> chebyshev_bins(int nbins, double xmin, double xmax) {
  const double pi = std::acos(-1.0);
  std::vector<double> b(nbins + 1);
  for (int i = 1; i <= nbins + 1; ++i) b[i - 1] = xmin + (xmax - xmin) * (1.0 - std::cos(pi * (i - 1) / nbins)) / 2;
  return b;
}

std::vector<double> linear_bins(int nbins, double xmin, double xmax) {
  std::vector<double> b(nbins + 1);
  for (int i = 1; i <= nbins + 1; ++i) b[i - 1] = xmin + (xmax - xmin) * (i - 1) / nbins;
  return b;
}

Density density(const std::vector<double>& samples, const std::vector<double>& bins) {
  Density d;
  std::vector<double> h = recurgreen::histogram(samples, bins, &d.missing);
  const double eps10 = std::numeric_limits<double>::epsilon() / 10.0;
  for (double& v : h) v += eps10;
  double npoints = 0.0;
  for (double v : h) npoints += v;  // sum(histo), in order
  d.rho.resize(h.size());
  d.centre.resize(h.size());
  for (size_t j = 0; j < h.size(); ++j) {
    d.rho[j] = h[j] / (npoints * (bins[j + 1] - bins[j]));
    d.centre[j] = ((0.0 + bins[j]) + bins[j + 1]) / 2;
  }
  return d;
}

std::vector<double> read_real_array(const std::string& path) {
  std::vector<double> out;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    size_t a = 0;
    while (a < line.size() && std::isspace((unsigned char)line[a])) ++a;
    size_t b = a;
    while (b < line.size() && !std::isspace((unsigned char)line[b]) && line[b] != ',' && line[b] != '/') ++b;
    double v;
    if (b > a && parse_real(line.substr(a, b - a), &v)) out.push_back(v);
  }
  return out;
}

std::string unique_filename(const std::string& base, const std::string& ext) {
  for (long i = 1; i < 1000000000L; ++i) {
    const std::string f = base + std::to_string(i) + ext;
    if (!file_exists(f)) return f;
  }
  throw Stop("Too many files (nmax=1000000000), no valid filename !");
}

void create_directory(const std::string& dir) {
  std::string cur;
  for (size_t i = 0; i < dir.size(); ++i) {
    cur += dir[i];
    if (dir[i] == '/' || i + 1 == dir.size()) {
      if (!cur.empty() && cur != "/" && ::mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST)
        throw Stop("Cannot create directory: " + cur);
    }
  }
}

// ---------------------------------------------------------------------------
// recurgreen: task tdistrib (src/main.f90:73-123)
// ---------------------------------------------------------------------------
namespace {

void write_preamble(std::FILE* fp, const recurgreen::Waveguide& w, long nseed, long nbins, long nthreads,
                    double tsec, long seed0 = 1) {
  // a run that starts at seed0 != 1 names its seed range, so files of
  // disjoint ranges stay apart
  if (seed0 != 1) std::fprintf(fp, "%%%% Seeds %ld..%ld\n", seed0, seed0 + nseed - 1);
  std::fprintf(fp, "%%%% Computed on %s by %s\n", timestamp().c_str(), kProgram);
  w.print_parameters(fp, "%%");
  const double speed = nseed / tsec;
  std::fprintf(fp, "%%%% Nseed=%ld, Nbins=%ld, Nthreads=%ld, Time=%s s, Speed=%s seed/s\n", nseed, nbins, nthreads,
               format_g0(tsec, 6).c_str(), format_g0(speed, 6).c_str());
}

// The &waveguide group (src/main.f90:83), plus the optional ny.
recurgreen::Parameters waveguide_parameters(const std::string& text) {
  const NmlGroup wg = read_namelist(text, "waveguide",
                                    {"boundtype", "wol", "exfac", "dscat", "dabso", "aratio", "nxdiso", "nxfree",
                                     "napera", "naperb", "ny"});
  recurgreen::Parameters p;
  p.boundtype = nml_string(wg, "boundtype", "dirichlet");
  p.wol = nml_real(wg, "wol", 0.0);
  p.exfac = nml_real(wg, "exfac", 1.0);
  p.dscat = nml_real(wg, "dscat", 0.0);
  p.dabso = nml_real(wg, "dabso", 0.0);
  p.aratio = nml_real(wg, "aratio", 1.0);
  p.nxdiso = (int)nml_int(wg, "nxdiso", 0);
  p.nxfree = (int)nml_int(wg, "nxfree", 0);
  p.napera = nml_real(wg, "napera", 1.0);
  p.naperb = nml_real(wg, "naperb", 1.0);
  p.ny = (int)nml_int(wg, "ny", 0);
  return p;
}

void task_tdistrib(const std::string& text, const std::string& root) {
  const recurgreen::Parameters p = waveguide_parameters(text);
  // seed0 (optional, default 1): the first seed, so that runs over disjoint
  // seed ranges add up to one run over their union.
  const NmlGroup td = read_namelist(text, "tdistrib", {"nseed", "nbins", "nthreads", "save_eigvals", "seed0"});
  const long nseed = nml_int(td, "nseed", 0);
  const long seed0 = nml_int(td, "seed0", 1);
  const long nbins = nml_int(td, "nbins", 0);
  const long nthreads = nml_int(td, "nthreads", 1);
  const bool save_eigvals = nml_logical(td, "save_eigvals", false);

  recurgreen::Waveguide w(p);
  const std::string info = strip(tag_info());
  w.print_parameters(stdout, info);
  std::printf("%sNseed=%ld, Nbins=%ld, Nthreads=%ld\n", tag_info().c_str(), nseed, nbins, nthreads);
  if (nthreads < 1)
    throw Stop("Invalid number of threads, received " + fmt_int(nthreads) + " expected >0, aborting...");
  if (nseed < 0) throw Stop("Invalid number of seeds, received " + fmt_int(nseed) + " expected >=0, aborting...");
  if (nbins < 1) throw Stop("Invalid number of bins, received " + fmt_int(nbins) + " expected >0, aborting...");
  if (seed0 < 1) throw Stop("Invalid first seed, received seed0=" + fmt_int(seed0) + ", expected >0, aborting...");
  if (seed0 + nseed - 1 > 2147483647L)
    throw Stop("Invalid seed range, seed0+nseed-1=" + fmt_int(seed0 + nseed - 1) + " exceeds 2147483647, aborting...");

  // The seed loop (src/main.f90:134-179) as one batched GPU launch.
  std::vector<int32_t> seeds(nseed);
  for (long k = 0; k < nseed; ++k) seeds[k] = (int32_t)(seed0 + k);
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<double> tallvals = nseed > 0 ? w.tdistrib_batch(seeds) : std::vector<double>();
  const double tsec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::printf("\n%sDone, computation time is %s s.\n", tag_info().c_str(), f0(tsec, 2).c_str());

  // prepare_distrib (src/main.f90:223-251).
  const std::vector<double> bins = chebyshev_bins((int)nbins);
  const Density d = density(tallvals, bins);
  if (d.missing != 0.0) {
    std::printf("%sSome transmission eigenvalues are out of the bounds [%s, %s].\n%sThere are %s missing "
                "eigenvalues in the histogram, continuing anyway...\n",
                tag_warn().c_str(), f0(bins.front(), 6).c_str(), f0(bins.back(), 6).c_str(), tag_warn().c_str(),
                f0(d.missing, 1).c_str());
  }

  // save_distrib / save_raw_eigvals (src/main.f90:257-328).
  const std::string dir = w.generate_directory(root) + "distrib/";
  create_directory(dir);
  const std::string fname = unique_filename(dir + "result_", ".distrib.csv");
  std::FILE* fp = std::fopen(fname.c_str(), "w");
  if (!fp) throw Stop("Cannot open file: " + fname);
  write_preamble(fp, w, nseed, nbins, nthreads, tsec, seed0);
  std::fprintf(fp, "tm, rho\n");
  write_rows(fp, d);
  std::fclose(fp);
  std::printf("%sResult written in file: %s\n", tag_info().c_str(), fname.c_str());
  if (save_eigvals) {
    const std::string ename = unique_filename(dir + "result_", ".eigvals.csv");
    std::FILE* fe = std::fopen(ename.c_str(), "w");
    if (!fe) throw Stop("Cannot open file: " + ename);
    write_preamble(fe, w, nseed, nbins, nthreads, tsec, seed0);
    std::fprintf(fe, "%%%% Transmission eigenvalues (%zu values)\n", tallvals.size());
    for (double v : tallvals) std::fprintf(fe, "%s\n", format_g0(v).c_str());
    std::fclose(fe);
    std::printf("%sEigenvalues saved in file: %s\n", tag_info().c_str(), ename.c_str());
  }
}

// print_timestamp + print_parameters (src/base_utils.f90:722-739,
// src/waveguide.f90:1003-1018).
void write_header(std::FILE* fp, const recurgreen::Waveguide& w) {
  std::fprintf(fp, "%%%% Computed on %s by %s\n", timestamp().c_str(), kProgram);
  w.print_parameters(fp, "%%");
}

// save_real_matrix (src/base_utils.f90:639-657) with 'g0.16' and ', ': the
// nrow x ncol matrix a(i, j) = at(i, j), one row per line.
template <class F>
void write_matrix(std::FILE* fp, size_t nrow, size_t ncol, F at) {
  for (size_t i = 0; i < nrow; ++i) {
    for (size_t j = 0; j < ncol; ++j)
      std::fprintf(fp, "%s%s", format_g0(at(i, j)).c_str(), j + 1 < ncol ? ", " : "\n");
  }
}

std::FILE* open_output(const std::string& fname) {
  std::FILE* fp = std::fopen(fname.c_str(), "w");
  if (!fp) throw Stop("Cannot open file: " + fname);
  return fp;
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

std::vector<int32_t> seeds_1_to(long nseed) {
  std::vector<int32_t> seeds(nseed);
  for (long k = 0; k < nseed; ++k) seeds[k] = (int32_t)(k + 1);
  return seeds;
}

// task_wavefunction and save_wavefunction (src/main.f90:335-398).
void task_wavefunction(const std::string& text, const std::string& root) {
  const recurgreen::Parameters p = waveguide_parameters(text);
  const NmlGroup wf = read_namelist(text, "wavefunction", {"iseed", "ipos", "imode"});
  const long iseed = nml_int(wf, "iseed", 1), ipos = nml_int(wf, "ipos", 1), imode = nml_int(wf, "imode", 1);
  recurgreen::Waveguide w(p);
  w.print_parameters(stdout, strip(tag_info()));
  std::printf("%sWavefunction parameters: iseed=%ld, ipos=%ld, imode=%ld\n", tag_info().c_str(), iseed, ipos, imode);
  std::vector<double> data;
  w.compute_wavefunction((int)iseed, (int)ipos, (int)imode, data);
  std::printf("%sSaving the wavefunction to a CSV file...\n", tag_info().c_str());
  const std::string dir = w.generate_directory(root) + "wavefun/";
  create_directory(dir);
  const std::string fname = unique_filename(dir + "result_", ".wavefun.csv");
  std::FILE* fp = open_output(fname);
  write_header(fp, w);
  std::fprintf(fp, "%%%% Wavefunction parameters: iseed=%ld, ipos=%ld, imode=%ld\n", iseed, ipos, imode);
  std::fprintf(fp, "x, y, repsi, impsi, upot\n");
  const size_t rows = data.size() / 5;
  write_matrix(fp, rows, 5, [&](size_t i, size_t j) { return data[j * rows + i]; });
  std::fclose(fp);
  std::printf("%sResult written in file: %s\n", tag_info().c_str(), fname.c_str());
}

// task_tprofile and save_tprofile (src/main.f90:405-565).
void task_tprofile(const std::string& text, const std::string& root) {
  const recurgreen::Parameters p = waveguide_parameters(text);
  const NmlGroup tp = read_namelist(text, "tprofile", {"tmin", "tmax", "nseed", "nthreads"});
  const double tmin = nml_real(tp, "tmin", 0.0), tmax = nml_real(tp, "tmax", 1.0);
  const long nseed = nml_int(tp, "nseed", 0);
  recurgreen::Waveguide w(p);
  w.print_parameters(stdout, strip(tag_info()));
  if (nseed <= 0)
    throw Stop("Invalid number of disorder realizations (received " + fmt_int(nseed) + "), aborting...");
  const int nx = w.get_nx();
  std::vector<double> prof, tavg;
  std::vector<int32_t> nt;
  const auto t0 = std::chrono::steady_clock::now();
  w.tprofile_batch(seeds_1_to(nseed), RG_PROFILE_TPROFILE, {tmin}, {tmax}, prof, nt, tavg);
  const double tsec = seconds_since(t0);
  long nsample = 0;
  for (long k = 0; k < nseed; ++k) nsample += nt[k] != 0;
  if (nsample == 0)
    std::printf("%sFound no transmission eigenfunction (nsample=%ld), results will be undetermined...\n",
                tag_warn().c_str(), nsample);
  else
    std::printf("%sFound %ld/%ld transmission eigenfunctions, now averaging...\n", tag_info().c_str(), nsample,
                nseed);
  std::vector<double> avg(nx, 0.0);
  for (long k = 0; k < nseed; ++k)
    if (nt[k] != 0)
      for (int ix = 0; ix < nx; ++ix) avg[ix] = avg[ix] + prof[(size_t)k * nx + ix];
  for (int ix = 0; ix < nx; ++ix) avg[ix] = avg[ix] / (double)nsample;
  const std::string dir = w.generate_directory(root) + "tprofile/";
  create_directory(dir);
  char params[512];
  std::snprintf(params, sizeof params,
                "%%%% Transmission profile parameters: Found nsample=%ld / nseed=%ld, nx=%d, tmin=%s, tmax=%s, "
                "time=%s s.\n",
                nsample, nseed, nx, format_g0(tmin, 6).c_str(), format_g0(tmax, 6).c_str(), f0(tsec, 3).c_str());
  const std::string raw = unique_filename(dir + "result_", ".raw.csv");
  std::FILE* fp = open_output(raw);
  write_header(fp, w);
  std::fputs(params, fp);
  std::fprintf(fp, "%%%% Here follows, on each line, the function |psi_T(x)|^2 for a given realization of the "
                   "disorder.\n");
  write_matrix(fp, nseed, nx, [&](size_t k, size_t ix) { return prof[k * nx + ix]; });
  std::fclose(fp);
  std::printf("%sRaw profile data written in file: %s\n", tag_info().c_str(), raw.c_str());
  const std::string avgf = unique_filename(dir + "result_", ".avg.csv");
  const std::vector<double> x = w.get_xmesh();
  fp = open_output(avgf);
  write_header(fp, w);
  std::fputs(params, fp);
  std::fprintf(fp, "x, tprofile\n");
  for (int ix = 0; ix < nx; ++ix) std::fprintf(fp, "%s, %s\n", format_g0(x[ix]).c_str(), format_g0(avg[ix]).c_str());
  std::fclose(fp);
  std::printf("%sAverage profile written in file: %s\n", tag_info().c_str(), avgf.c_str());
}

// task_tprofile_group and save_tprofile_group (src/main.f90:572-728).
void task_tprofile_group(const std::string& text, const std::string& root) {
  constexpr int nprofile = 4;
  const recurgreen::Parameters p = waveguide_parameters(text);
  const NmlGroup tg = read_namelist(text, "tprofile_group", {"tm", "dt", "nseed", "nthreads"});
  const std::vector<double> tm = nml_reals(tg, "tm", nprofile, std::vector<double>(nprofile, 0.0));
  const std::vector<double> dt = nml_reals(tg, "dt", nprofile, std::vector<double>(nprofile, 0.0));
  const long nseed = nml_int(tg, "nseed", 0);
  recurgreen::Waveguide w(p);
  w.print_parameters(stdout, strip(tag_info()));
  if (nseed <= 0)
    throw Stop("Invalid number of disorder realizations (received " + fmt_int(nseed) + "), aborting...");
  const int nx = w.get_nx();
  std::vector<double> prof, tavgdata;
  std::vector<int32_t> nt;
  const auto t0 = std::chrono::steady_clock::now();
  w.tprofile_batch(seeds_1_to(nseed), RG_PROFILE_GROUP, tm, dt, prof, nt, tavgdata);
  const double tsec = seconds_since(t0);
  std::vector<double> avg((size_t)nx * nprofile, 0.0);
  long nsample[nprofile] = {0, 0, 0, 0};
  for (int ip = 0; ip < nprofile; ++ip) {
    for (long k = 0; k < nseed; ++k) {
      if (nt[(size_t)k * nprofile + ip] == 0) continue;
      for (int ix = 0; ix < nx; ++ix)
        avg[(size_t)ip * nx + ix] = avg[(size_t)ip * nx + ix] + prof[((size_t)k * nprofile + ip) * nx + ix];
      ++nsample[ip];
    }
    if (nsample[ip] != 0) {
      std::printf("%sProfile %d/%d : Found %ld/%ld transmission eigenfunctions, now averaging...\n",
                  tag_info().c_str(), ip + 1, nprofile, nsample[ip], nseed);
      for (int ix = 0; ix < nx; ++ix) avg[(size_t)ip * nx + ix] = avg[(size_t)ip * nx + ix] / (double)nsample[ip];
    } else {
      std::printf("%sProfile %d/%d : Found no transmission eigenstate (nsample=%ld), results will be "
                  "undetermined...\n", tag_warn().c_str(), ip + 1, nprofile, nsample[ip]);
    }
  }
  double tsum = 0.0;
  for (double v : tavgdata) tsum += v;
  const double tavg = tsum / nseed;
  double var = 0.0;
  for (double v : tavgdata) var += (v - tavg) * (v - tavg);
  const double uctavg = std::sqrt(var) / nseed;
  const std::string dir = w.generate_directory(root) + "tprofile_group/";
  create_directory(dir);
  const std::string fname = unique_filename(dir + "result_", ".csv");
  const std::vector<double> x = w.get_xmesh();
  std::FILE* fp = open_output(fname);
  write_header(fp, w);
  auto join6 = [](const std::vector<double>& v) {
    std::string s;
    for (size_t i = 0; i < v.size(); ++i) s += (i ? ", " : "") + format_g0(v[i], 6);
    return s;
  };
  std::fprintf(fp, "%%%% Transmission profile parameters: nx=%d, tm=[%s], dt=[%s].\n", nx, join6(tm).c_str(),
               join6(dt).c_str());
  std::fprintf(fp, "%%%% Results: Found nsample=[%ld, %ld, %ld, %ld] over nseed=%ld, tavg=%s+-%s, time=%s s.\n",
               nsample[0], nsample[1], nsample[2], nsample[3], nseed, format_g0(tavg, 6).c_str(),
               format_g0(uctavg, 6).c_str(), f0(tsec, 3).c_str());
  std::fprintf(fp, "x");
  for (int ip = 0; ip < nprofile; ++ip) std::fprintf(fp, ", tprofile%s", f0(tm[ip], 4).c_str());
  std::fprintf(fp, "\n");
  write_matrix(fp, nx, nprofile + 1,
               [&](size_t ix, size_t j) { return j == 0 ? x[ix] : avg[(j - 1) * nx + ix]; });
  std::fclose(fp);
  std::printf("%sAverage profiles written in file: %s\n", tag_info().c_str(), fname.c_str());
}

// task_tpattern (src/main.f90:735-877): the mean over seeds of |t_{b,imu}|^2
// and |r_{b,imu}|^2 ('incident'), of their column sums ('total'), or of
// |d_{b,imu}|^2 for the deposition matrix d at the middle of the medium from
// the first slice ('deposition', rprob zero).
void task_tpattern(const std::string& text, const std::string& root) {
  const NmlGroup tp = read_namelist(text, "tpattern", {"nseed", "imode", "nthreads", "probatype"});
  const long nseed = nml_int(tp, "nseed", 0);
  const long imode = nml_int(tp, "imode", 1);
  const std::string probatype = nml_string(tp, "probatype", "incident");
  if (nseed <= 0)
    throw Stop("Invalid number of disorder realizations (received " + fmt_int(nseed) + "), aborting...");
  if (probatype != "incident" && probatype != "total" && probatype != "deposition")
    throw Stop("Invalid probatype, received '" + probatype + "', expected incident/total/deposition, aborting...");
  recurgreen::Waveguide w(waveguide_parameters(text));
  const int M = w.get_nmu();
  const recurgreen::Parameters wp = w.get_parameters();
  const long imu = wp.boundtype == "periodic" ? (imode + M / 2 - 1) % M + 1 : imode;
  if (imu < 1 || imu > M)
    throw Stop("Invalid incident mode imode=" + fmt_int(imode) + ", expected in [1, " + fmt_int(M) + "], aborting...");
  const int fpos = wp.nxfree + wp.nxdiso / 2 + 1;  // src/main.f90:769-770
  std::vector<double> tsum(M, 0.0), rsum(M, 0.0);
  const auto t0 = std::chrono::steady_clock::now();
  const long chunk = 256;
  std::vector<std::complex<double>> t, r;
  auto prob = [](std::complex<double> z) {  // abs(z)**2, as the reference writes it
    const double a = std::abs(z);
    return a * a;
  };
  for (long s0 = 1; s0 <= nseed; s0 += chunk) {
    std::vector<int32_t> seeds;
    for (long sd = s0; sd < s0 + chunk && sd <= nseed; ++sd) seeds.push_back((int32_t)sd);
    const size_t mm = (size_t)M * M;
    if (probatype == "deposition") {
      w.deposition_batch(seeds, fpos, 1, (int)imu, t);
      for (size_t k = 0; k < seeds.size(); ++k)
        for (int b = 0; b < M; ++b) tsum[b] += prob(t[k * M + b]);
      continue;
    }
    w.refl_trans_v1_batch(seeds, &r, t);
    for (size_t k = 0; k < seeds.size(); ++k) {  // seed order, as the Fortran sum over dim=2
      const std::complex<double>* tk = t.data() + k * mm;
      const std::complex<double>* rk = r.data() + k * mm;
      for (int b = 0; b < M; ++b) {
        double tpb = 0.0, rpb = 0.0;
        if (probatype == "incident") {
          tpb = prob(tk[(size_t)(imu - 1) * M + b]);
          rpb = prob(rk[(size_t)(imu - 1) * M + b]);
        } else {  // column b summed over its rows
          for (int i = 0; i < M; ++i) {
            tpb += prob(tk[(size_t)b * M + i]);
            rpb += prob(rk[(size_t)b * M + i]);
          }
        }
        tsum[b] += tpb;
        rsum[b] += rpb;
      }
    }
  }
  const double tsec = seconds_since(t0);
  const std::string dir = w.generate_directory(root) + "tpattern/";
  create_directory(dir);
  const std::string fname = unique_filename(dir + "result_", ".csv");
  std::FILE* fp = open_output(fname);
  write_header(fp, w);
  std::fprintf(fp, "%%%% Radiation pattern parameters: probatype='%s', nseed=%ld, imode=%ld, time=%s s.\n",
               probatype.c_str(), nseed, imode, f0(tsec, 3).c_str());
  std::fprintf(fp, "imu, tprob, rprob\n");
  for (int b = 0; b < M; ++b)
    std::fprintf(fp, "%d, %s, %s\n", b + 1, format_g0(tsum[b] / nseed).c_str(), format_g0(rsum[b] / nseed).c_str());
  std::fclose(fp);
  std::printf("%sAverage profiles written in file: %s\n", tag_info().c_str(), fname.c_str());
}

// execute_file (src/main.f90:41-65).
void execute_file(const std::string& text, const std::string& root) {
  const NmlGroup s = read_namelist(text, "settings", {"task"});
  const std::string task = nml_string(s, "task", "");
  if (task == "tdistrib") {
    task_tdistrib(text, root);
  } else if (task == "wavefunction") {
    task_wavefunction(text, root);
  } else if (task == "tprofile") {
    task_tprofile(text, root);
  } else if (task == "tprofile_group") {
    task_tprofile_group(text, root);
  } else if (task == "tpattern") {
    task_tpattern(text, root);
  } else {
    throw Stop("Unknown task '" + task + "', aborting...");
  }
}

int stop_exit(const std::string& msg) {
  std::fprintf(stderr, "%s%s\n", tag_error().c_str(), msg.c_str());
  std::fprintf(stderr, "STOP %s\n", kStopMessage);
  return 1;
}

}  // namespace

int recurgreen_main(int argc, char** argv) {
  std::printf("====== This is %s ======\n", kProgram);
  std::fflush(stdout);
  std::string root = "out";
  std::vector<std::string> files;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--outdir" && i + 1 < argc) {
      root = argv[++i];
    } else {
      files.push_back(a);
    }
  }
  if (files.empty()) std::fprintf(stderr, "%sNo settings file provided, doing nothing...\n", tag_error().c_str());
  int rc = 0;
  for (const std::string& f : files) {
    if (!file_exists(f)) {
      std::fprintf(stderr, "%sFile not found: %s\n", tag_error().c_str(), f.c_str());
      rc = 1;
      continue;
    }
    std::ifstream probe(f);
    if (!probe) {
      std::fprintf(stderr, "%sCannot open file: %s\n", tag_error().c_str(), f.c_str());
      rc = 1;
      continue;
    }
    std::printf("%sReading file: %s\n", tag_info().c_str(), f.c_str());
    std::fflush(stdout);
    try {
      execute_file(read_file(f), root);
    } catch (const Stop& e) {
      std::fflush(stdout);
      return stop_exit(e.what());
    } catch (const recurgreen::Error& e) {
      std::fflush(stdout);
      return stop_exit(e.what());
    }
  }
  return rc;
}

// ---------------------------------------------------------------------------
// plothisto (src/plot_histogram.f90)
// ---------------------------------------------------------------------------
int plothisto_main(int argc, char** argv) {
  std::printf("====== This is PlotHisto (from %s) ======\n", kProgram);
  std::fflush(stdout);
  try {
    if (argc != 3) {
      std::printf("%sUsage: $ ./plothisto plothisto_settings.nml path/to/samples.csv\n", tag_info().c_str());
      throw Stop("Two files expected, doing nothing...");
    }
    const std::string cfg = argv[1], data = argv[2];
    if (!file_exists(cfg)) throw Stop("File not found: " + cfg);
    if (!file_exists(data)) throw Stop("File not found: " + data);
    const NmlGroup s = read_namelist(read_file(cfg), "settings", {"bintype", "nbins", "xmin", "xmax"});
    const std::string bintype = nml_string(s, "bintype", "chebyshev");
    const long nbins = nml_int(s, "nbins", 0);
    const double xmin = nml_real(s, "xmin", 0.0), xmax = nml_real(s, "xmax", 1.0);
    const std::vector<double> samples = read_real_array(data);
    std::printf("%sFound %zu samples in the data file...\n", tag_info().c_str(), samples.size());
    if (nbins < 1)
      throw Stop("Invalid number of bins (nbins=" + fmt_int(nbins) + " must be positive), aborting...");
    if (!(xmax > xmin)) throw Stop("Invalid binning range, aborting...");
    std::vector<double> bins;
    if (bintype == "linear") {
      bins = linear_bins((int)nbins, xmin, xmax);
    } else if (bintype == "chebyshev") {
      bins = chebyshev_bins((int)nbins, xmin, xmax);
    } else {
      throw Stop("Unknown binning type '" + bintype + "', aborting...");
    }
    const Density d = density(samples, bins);
    if (d.missing != 0.0) {
      std::printf("%sSome samples are out of the bounds [%s, %s].\n%sThere are %s missing samples in the histogram "
                  "(%s%%), continuing anyway...\n",
                  tag_warn().c_str(), f0(bins.front(), 6).c_str(), f0(bins.back(), 6).c_str(), tag_warn().c_str(),
                  f0(d.missing, 0).c_str(), f0(100.0 * d.missing / samples.size(), 2).c_str());
    }
    // save_histo: replot_<i>.distrib.csv beside the data file, with its preamble.
    const size_t slash = data.rfind('/');
    const std::string dir = slash == std::string::npos ? "" : data.substr(0, slash + 1);
    const std::string out = unique_filename(dir + "replot_", ".distrib.csv");
    std::FILE* fp = std::fopen(out.c_str(), "w");
    if (!fp) throw Stop("Cannot open file: " + out);
    std::ifstream in(data);
    std::string line;
    while (std::getline(in, line)) {  // copy_preamble (src/base_utils.f90:856-872)
      if (line.empty() || (line[0] != '%' && line[0] != '#')) break;
      if (line.size() > 300) line.resize(300);
      while (!line.empty() && (line.back() == ' ' || line.back() == '\r')) line.pop_back();
      std::fprintf(fp, "%s\n", line.c_str());
    }
    std::fprintf(fp, "tm, rho\n");
    write_rows(fp, d);
    std::fclose(fp);
    std::printf("%sReplot written in file: %s\n", tag_info().c_str(), out.c_str());
  } catch (const Stop& e) {
    std::fflush(stdout);
    return stop_exit(e.what());
  } catch (const recurgreen::Error& e) {
    std::fflush(stdout);
    return stop_exit(e.what());
  }
  return 0;
}

// ---------------------------------------------------------------------------
// waveguide_test (src/waveguide.test.f90): the reference's physics checks,
// printed the same way: the parameters of the test guide, the unitarity
// defect ||t^H t + r^H r - 1|| of versions 1 and 2 (test_unitarity,
// src/waveguide.f90:561-590) and ||r_v1 - r_v2||, ||t_v1 - t_v2||
// (test_green_v1_v2, src/waveguide.f90:598-623), for seeds 1..5.
// ---------------------------------------------------------------------------
namespace {

using cvec = std::vector<std::complex<double>>;

// norm2_complex (src/base_utils.f90:208-229): the Frobenius norm.
double norm2(const cvec& a) {
  double s = 0.0;
  for (const auto& z : a) s += std::norm(z);
  return std::sqrt(s);
}

// ||t^H t + r^H r - 1|| for nmu x nmu column-major t and r.
double unitarity_defect(const cvec& t, const cvec& r, int n) {
  cvec d((size_t)n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      std::complex<double> s = (i == j) ? -1.0 : 0.0;
      for (int k = 0; k < n; ++k)
        s += std::conj(t[(size_t)i * n + k]) * t[(size_t)j * n + k] + std::conj(r[(size_t)i * n + k]) * r[(size_t)j * n + k];
      d[(size_t)j * n + i] = s;
    }
  return norm2(d);
}

cvec difference(const cvec& a, const cvec& b) {
  cvec d(a.size());
  for (size_t e = 0; e < a.size(); ++e) d[e] = a[e] - b[e];
  return d;
}

std::string seed_field(int iseed) {  // '(i5)'
  char buf[16];
  std::snprintf(buf, sizeof buf, "%5d", iseed);
  return buf;
}

recurgreen::Parameters test_guide(int nxdiso, int nxfree) {  // src/waveguide.test.f90:25-39,62-73
  recurgreen::Parameters p;
  p.boundtype = "dirichlet";
  p.wol = 4.30;
  p.aratio = 1.0;
  p.exfac = 1.2;
  p.dscat = 0.2;
  p.dabso = 0.0;
  p.napera = 1.0;
  p.naperb = 1.0;
  p.nxdiso = nxdiso;
  p.nxfree = nxfree;
  return p;
}

}  // namespace

int waveguide_test_main(int, char**) {
  try {
    std::printf("====== TEST INIT_WAVEGUIDE ======\n");
    {
      recurgreen::Waveguide w(test_guide(10, 2));
      w.print_parameters(stdout, "|");
    }
    const int nseed = 5;
    recurgreen::Waveguide w(test_guide(100, 20));
    const int n = w.get_nmu();
    cvec r1, t1, r2, t2;
    for (int version = 1; version <= 2; ++version) {
      std::printf("====== TEST UNITARITY V%d ======\n", version);
      if (version == 1) w.print_parameters(stdout, "|");
      for (int iseed = 1; iseed <= nseed; ++iseed) {
        if (version == 1) w.compute_refl_trans_v1(iseed, r1, t1);
        else w.compute_refl_trans_v2(iseed, r1, t1);
        std::printf("%s#%s | norm(t'*t + r'*r - 1) = %s (expected 0).\n", tag_test().c_str(),
                    seed_field(iseed).c_str(), format_g0(unitarity_defect(t1, r1, n), 6).c_str());
      }
    }
    std::printf("====== TEST GREEN V1/V2 ======\n");
    w.print_parameters(stdout, "|");
    for (int iseed = 1; iseed <= nseed; ++iseed) {
      w.compute_refl_trans_v1(iseed, r1, t1);
      w.compute_refl_trans_v2(iseed, r2, t2);
      std::printf("%s#%s | norm(r_v1 - r_v2) = %s (expected 0).\n", tag_test().c_str(), seed_field(iseed).c_str(),
                  format_g0(norm2(difference(r1, r2)), 6).c_str());
      std::printf("%s#%s | norm(t_v1 - t_v2) = %s (expected 0).\n", tag_test().c_str(), seed_field(iseed).c_str(),
                  format_g0(norm2(difference(t1, t2)), 6).c_str());
    }
  } catch (const recurgreen::Error& e) {
    std::fflush(stdout);
    return stop_exit(e.what());
  }
  return 0;
}

}  // namespace rgdriver
