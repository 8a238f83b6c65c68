/*
 * recurgreen.hpp -- C++ host interface over the C ABI of recurgreen.h.
 *
 * recurgreen::Waveguide mirrors the reference's `type(waveguide_t)`
 * (src/waveguide.f90:13-73): the constructor is `init`, the copy constructor
 * `init_copy`, the destructor `del`, and the type-bound procedures keep their
 * names (get_nmu, get_neigv, get_nx, get_xmesh, get_parameters,
 * compute_tdistrib, compute_refl_trans_v1, compute_refl_trans_v2, compute_wavefunction,
 * compute_deposition, compute_itx_profile, compute_tprofile,
 * compute_tprofile_group, print_parameters, generate_directory).  Where the reference prints a message and stops
 * (src/base_utils.f90:56-57), these methods throw recurgreen::Error carrying
 * the library's status code and message.  Header-only; link against
 * librecurgreen_gb300.so.
 */
#ifndef RECURGREEN_HPP
#define RECURGREEN_HPP

#include <complex>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "recurgreen.h"

namespace recurgreen {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc) {
  if (rc != RG_OK) throw Error(rc, rg_last_error());
}

// The `&waveguide` namelist (src/main.f90:83) plus the transverse grid size ny
// (0: the reference's ny = nmu).
struct Parameters {
  std::string boundtype = "dirichlet";
  int nxdiso = 0, nxfree = 0;
  double wol = 0, exfac = 1, aratio = 1, dscat = 0, dabso = 0, napera = 1, naperb = 1;
  int ny = 0;
};

// Fortran F0.d as gfortran writes it: no field width, so a value below one
// in magnitude has no leading zero (0.2 -> ".200000", -0.5 -> "-.500000").
inline std::string format_f0(double x, int d = 6) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.*f", d, x);
  std::string s = buf;
  if (s.rfind("0.", 0) == 0) return s.substr(1);
  if (s.rfind("-0.", 0) == 0) return "-" + s.substr(2);
  return s;
}

class Waveguide {
 public:
  // init (src/waveguide.f90:81-85): validates the parameters with the
  // reference's messages and builds the waveguide on the current CUDA device.
  explicit Waveguide(const Parameters& p) {
    rg_params c{};
    if (p.boundtype == "dirichlet") {
      c.boundtype = RG_BOUND_DIRICHLET;
    } else if (p.boundtype == "periodic") {
      c.boundtype = RG_BOUND_PERIODIC;
    } else {
      c.boundtype = -1;  // rejected by rg_init with the reference's message
    }
    c.nxdiso = p.nxdiso;
    c.nxfree = p.nxfree;
    c.wol = p.wol;
    c.exfac = p.exfac;
    c.aratio = p.aratio;
    c.dscat = p.dscat;
    c.dabso = p.dabso;
    c.napera = p.napera;
    c.naperb = p.naperb;
    c.ny = p.ny;
    check(rg_init(&c, &h_));
  }
  // init_copy (src/waveguide.f90:262-270).
  Waveguide(const Waveguide& o) { check(rg_init_copy(o.h_, &h_)); }
  Waveguide& operator=(const Waveguide& o) {
    if (this != &o) {
      rg_waveguide* n = nullptr;
      check(rg_init_copy(o.h_, &n));
      rg_del(h_);
      h_ = n;
    }
    return *this;
  }
  Waveguide(Waveguide&& o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  Waveguide& operator=(Waveguide&& o) noexcept {
    if (this != &o) {
      rg_del(h_);
      h_ = o.h_;
      o.h_ = nullptr;
    }
    return *this;
  }
  // del (src/waveguide.f90:275-286).
  ~Waveguide() { rg_del(h_); }

  rg_waveguide* handle() const { return h_; }

  // Getters (src/waveguide.f90:291-350) and the derived sizes.
  int get_nmu() const { return rg_get_nmu(h_); }
  int get_neigv() const { return rg_get_neigv(h_); }
  int get_nx() const { return rg_get_nx(h_); }
  int get_ny() const { return rg_get_ny(h_); }
  int get_nprop() const { return rg_get_nprop(h_); }
  void get_window(int* imin, int* imax, int* jmin, int* jmax) const {
    check(rg_get_window(h_, imin, imax, jmin, jmax));
  }
  std::vector<double> get_xmesh() const {
    std::vector<double> x(get_nx());
    check(rg_get_xmesh(h_, x.data(), (int64_t)x.size()));
    return x;
  }
  Parameters get_parameters() const {
    rg_params c{};
    check(rg_get_parameters(h_, &c));
    Parameters p;
    p.boundtype = c.boundtype == RG_BOUND_PERIODIC ? "periodic" : "dirichlet";
    p.nxdiso = c.nxdiso;
    p.nxfree = c.nxfree;
    p.wol = c.wol;
    p.exfac = c.exfac;
    p.aratio = c.aratio;
    p.dscat = c.dscat;
    p.dabso = c.dabso;
    p.napera = c.napera;
    p.naperb = c.naperb;
    p.ny = c.ny;
    return p;
  }

  // compute_tdistrib (src/waveguide.f90:392-462): chunk iseed of tallvals.
  void compute_tdistrib(int iseed, std::vector<double>& tallvals) {
    check(rg_compute_tdistrib(h_, iseed, tallvals.data(), (int64_t)tallvals.size()));
  }
  // compute_refl_trans_v1 (src/waveguide.f90:469-519): nmu x nmu, column-major.
  void compute_refl_trans_v1(int iseed, std::vector<std::complex<double>>& rmat,
                             std::vector<std::complex<double>>& tmat) {
    const size_t n = (size_t)get_nmu() * get_nmu();
    rmat.resize(n);
    tmat.resize(n);
    check(rg_compute_refl_trans_v1(h_, iseed, reinterpret_cast<double*>(rmat.data()),
                                   reinterpret_cast<double*>(tmat.data())));
  }
  // The seed loop of src/main.f90:134-179 as one batched launch: neigv
  // eigenvalues per seed, in seed order.  Throws on the first bad status
  // unless `status` is given (then every realization's status is returned).
  std::vector<double> tdistrib_batch(const std::vector<int32_t>& seeds, std::vector<int32_t>* status = nullptr) {
    std::vector<double> out(seeds.size() * (size_t)get_neigv());
    std::vector<int32_t> st(seeds.size());
    const int rc = rg_tdistrib_batch(h_, seeds.data(), (int)seeds.size(), out.data(), st.data());
    if (status) {
      *status = st;
      if (rc != RG_OK && rc != RG_ERR_SINGULAR && rc != RG_ERR_NOCONV) check(rc);
    } else {
      check(rc);
    }
    return out;
  }

  // compute_refl_trans_v1 for many seeds (the tpattern loop,
  // src/main.f90:796-830): t and r of seeds[k] at offset k*nmu*nmu of tmat
  // and rmat (each matrix column-major); rmat may be null.
  void refl_trans_v1_batch(const std::vector<int32_t>& seeds, std::vector<std::complex<double>>* rmat,
                           std::vector<std::complex<double>>& tmat) {
    const size_t n = seeds.size() * (size_t)get_nmu() * get_nmu();
    tmat.resize(n);
    if (rmat) rmat->resize(n);
    check(rg_refl_trans_v1_batch(h_, seeds.data(), (int)seeds.size(),
                                 rmat ? reinterpret_cast<double*>(rmat->data()) : nullptr,
                                 reinterpret_cast<double*>(tmat.data()), nullptr));
  }

  // compute_tprofile (src/waveguide.f90:843-907): |psi_T(x)|^2 averaged over
  // the transmission eigenstates with tmin <= T <= tmax; returns nt.
  int compute_tprofile(int iseed, double tmin, double tmax, std::vector<double>& tprofile) {
    tprofile.resize(get_nx());
    int nt = 0;
    check(rg_compute_tprofile(h_, iseed, tmin, tmax, tprofile.data(), (int64_t)tprofile.size(), &nt));
    return nt;
  }
  // compute_itx_profile (src/waveguide.f90:764-825).
  void compute_itx_profile(int iseed, double tmin, double tmax, std::vector<double>& itx) {
    itx.resize(get_nx());
    check(rg_compute_itx_profile(h_, iseed, tmin, tmax, itx.data(), (int64_t)itx.size()));
  }
  // compute_tprofile_group (src/waveguide.f90:924-997): tprofile is nx x
  // nprofile, column-major (profile ip at ip*nx); returns Tavg.
  double compute_tprofile_group(int iseed, const std::vector<double>& tm, const std::vector<double>& dt,
                                std::vector<double>& tprofile, std::vector<int32_t>& nt) {
    tprofile.resize((size_t)get_nx() * tm.size());
    nt.resize(tm.size());
    double tavg = 0.0;
    if (tm.size() != dt.size()) throw Error(RG_ERR_INVALID_ARG, "tm and dt differ in length");
    check(rg_compute_tprofile_group(h_, iseed, (int)tm.size(), tm.data(), dt.data(), tprofile.data(),
                                    (int64_t)tprofile.size(), nt.data(), &tavg));
    return tavg;
  }
  // The profiles of many seeds (kind RG_PROFILE_*): profiles[(k*nprofile + w)*nx + ix],
  // nt[k*nprofile + w], tavg[k].
  void tprofile_batch(const std::vector<int32_t>& seeds, int kind, const std::vector<double>& a,
                      const std::vector<double>& b, std::vector<double>& profiles, std::vector<int32_t>& nt,
                      std::vector<double>& tavg) {
    if (a.size() != b.size()) throw Error(RG_ERR_INVALID_ARG, "window bounds differ in length");
    profiles.resize(seeds.size() * a.size() * (size_t)get_nx());
    nt.resize(seeds.size() * a.size());
    tavg.resize(seeds.size());
    check(rg_tprofile_batch(h_, seeds.data(), (int)seeds.size(), kind, (int)a.size(), a.data(), b.data(),
                            profiles.data(), nt.data(), tavg.data(), nullptr));
  }
  // compute_deposition (src/waveguide.f90:710-745): nmu x nmu, column-major.
  void compute_deposition(int iseed, int fpos, int ipos, std::vector<std::complex<double>>& depmat) {
    depmat.resize((size_t)get_nmu() * get_nmu());
    check(rg_compute_deposition(h_, iseed, fpos, ipos, reinterpret_cast<double*>(depmat.data())));
  }
  // Column col (1-based; 0: all) of the deposition matrix of many seeds.
  void deposition_batch(const std::vector<int32_t>& seeds, int fpos, int ipos, int col,
                        std::vector<std::complex<double>>& out) {
    out.resize(seeds.size() * (size_t)get_nmu() * (col > 0 ? 1 : get_nmu()));
    check(rg_deposition_batch(h_, seeds.data(), (int)seeds.size(), fpos, ipos, col,
                              reinterpret_cast<double*>(out.data()), nullptr));
  }
  // compute_refl_trans_v2 (src/waveguide.f90:526-553): nmu x nmu, column-major.
  void compute_refl_trans_v2(int iseed, std::vector<std::complex<double>>& rmat,
                             std::vector<std::complex<double>>& tmat) {
    const size_t n = (size_t)get_nmu() * get_nmu();
    rmat.resize(n);
    tmat.resize(n);
    check(rg_compute_refl_trans_v2(h_, iseed, reinterpret_cast<double*>(rmat.data()),
                                   reinterpret_cast<double*>(tmat.data())));
  }
  // compute_wavefunction (src/waveguide.f90:636-698): (nx*ny) x 5, column-major
  // (columns x, y, Re psi, Im psi, upot).
  void compute_wavefunction(int iseed, int ipos, int imode, std::vector<double>& wfundata) {
    const int64_t rows = (int64_t)get_nx() * get_ny();
    wfundata.resize(5 * (size_t)rows);
    check(rg_compute_wavefunction(h_, iseed, ipos, imode, wfundata.data(), rows));
  }

  // print_parameters (src/waveguide.f90:1003-1018): three lines, each
  // starting with `prefix`.
  void print_parameters(std::FILE* fp, const std::string& prefix) const {
    const Parameters p = get_parameters();
    int imin, imax, jmin, jmax;
    get_window(&imin, &imax, &jmin, &jmax);
    std::fprintf(fp, "%s Waveguide 2D with boundtype='%s', W/lambda=%s, exfac=%s, Nmode=%d, Nprop=%d\n",
                 prefix.c_str(), p.boundtype.c_str(), format_f0(p.wol).c_str(), format_f0(p.exfac).c_str(),
                 get_nmu(), get_nprop());
    std::fprintf(fp, "%s Filtering: NAper_a=%s (Nmode_a=%d), NAper_b=%s (Nmode_b=%d), Neigv=%d\n", prefix.c_str(),
                 format_f0(p.napera).c_str(), jmax - jmin + 1, format_f0(p.naperb).c_str(), imax - imin + 1,
                 get_neigv());
    std::fprintf(fp, "%s Medium: L/lscat=%s, L/labso=%s, Nx_diso=%d, Nx_free=%d, aratio=L/W=%s\n",
                 prefix.c_str(), format_f0(p.dscat).c_str(), format_f0(p.dabso).c_str(), p.nxdiso, p.nxfree,
                 format_f0(p.aratio).c_str());
  }

  // generate_directory (src/waveguide.f90:1046-1067): root/dscat_X/dabso_Y/wol_Z/boundtype/
  // with X, Y, Z written as F0.6 and trailing zeros removed.
  std::string generate_directory(const std::string& root = "out") const {
    const Parameters p = get_parameters();
    auto folder = [](const char* stem, double v) {
      std::string s = std::string(stem) + (v < 1.0 ? "0" : "") + format_f0(v);
      while (!s.empty() && (s.back() == '0' || s.back() == ' ')) s.pop_back();
      return s;
    };
    return root + "/" + folder("dscat_", p.dscat) + "/" + folder("dabso_", p.dabso) + "/" + folder("wol_", p.wol) +
           "/" + p.boundtype + "/";
  }

 private:
  rg_waveguide* h_ = nullptr;
};

// histogram (src/base_utils.f90:491-516) on the GPU: counts of samples in
// the nbins = bins.size() - 1 intervals, and the number of missing samples.
inline std::vector<double> histogram(const std::vector<double>& samples, const std::vector<double>& bins,
                                     double* missing) {
  std::vector<double> h(bins.size() > 0 ? bins.size() - 1 : 0);
  check(rg_histogram(samples.data(), (int64_t)samples.size(), bins.data(), (int)h.size(), h.data(), missing));
  return h;
}

// diagonalize_ahca (src/base_utils.f90:394-444) on the GPU: T (n values,
// descending) and U (n x n, column-major) with A^H A = U diag(T) U^H for the
// m x n column-major matrix a.
inline void diagonalize_ahca(const std::vector<std::complex<double>>& a, int m, int n, std::vector<double>& T,
                             std::vector<std::complex<double>>& U) {
  if ((int64_t)a.size() != (int64_t)m * n) throw Error(RG_ERR_INVALID_ARG, "diagonalize_ahca: a is not m x n");
  T.resize(n);
  U.resize((size_t)n * n);
  check(rg_diagonalize_ahca(reinterpret_cast<const double*>(a.data()), m, n, T.data(),
                            reinterpret_cast<double*>(U.data())));
}

}  // namespace recurgreen

#endif  // RECURGREEN_HPP
