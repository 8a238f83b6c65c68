// Host side of the full Green-function entry points (kernels in
// rg_green.cu): the reference's argument checks and messages
// (src/waveguide.f90:636-997), device buffers sized per call, realizations
// chunked by device memory, and the launch sequence
//   forward sweep keeping (S_n, Z_n) of every slice (symmetric kernel for
//     Dirichlet guides of up to 64 modes, pivoted blocked kernel otherwise
//     and for the items the symmetric one flags)
//   -> eigenvectors of t^H t and their selection (profiles)
//   -> back-substitution on the source vectors
//   -> window sums (profiles) or wavefunction pixels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rg_internal.h"

using rg::cplx;
using rg::DeviceGuard;
using rg::status_text;
using rg::GreenView;

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

// gfortran's G0.d edit descriptor (d significant digits), used in the
// reference's messages ('(a,g0.3,a)').
std::string g0(double x, int d) {
  if (std::isnan(x)) return "NaN";
  if (std::isinf(x)) return x > 0 ? "Infinity" : "-Infinity";
  const std::string sign = std::signbit(x) ? "-" : "";
  const double ax = std::fabs(x);
  if (ax == 0.0) return sign + "0." + std::string(d - 1, '0');
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.*e", d - 1, ax);
  const std::string s = buf;
  const size_t epos = s.find('e');
  const std::string digits = s.substr(0, 1) + s.substr(2, epos - 2);
  const int e10 = std::atoi(s.c_str() + epos + 1) + 1;
  if (0 <= e10 && e10 <= d) {
    if (e10 == 0) return sign + "0." + digits;
    return sign + digits.substr(0, e10) + "." + digits.substr(e10);
  }
  return sign + "0." + digits + "E" + (e10 < 0 ? "-" : "+") + std::to_string(std::abs(e10));
}

// One device allocation carved into 256-byte aligned pieces.
class Arena {
 public:
  ~Arena() { cudaFree(base_); }
  size_t add(size_t bytes) {
    const size_t off = size_;
    size_ += (bytes + 255) & ~(size_t)255;
    return off;
  }
  int alloc() {
    if (size_ == 0) size_ = 256;
    const cudaError_t e = cudaMalloc(&base_, size_);
    if (e != cudaSuccess) {
      cudaGetLastError();
      base_ = nullptr;
      return rg::fail(RG_ERR_NOMEM, "device allocation of " + std::to_string(size_) + " bytes failed");
    }
    return RG_OK;
  }
  template <class T>
  T* at(size_t off) const {
    return reinterpret_cast<T*>(static_cast<char*>(base_) + off);
  }

 private:
  void* base_ = nullptr;
  size_t size_ = 0;
};

// Realizations per launch: what fits in half the free device memory (at most
// 96 GiB), rounded down to whole waves of two CTAs per SM when larger.
// RG_GREEN_CHUNK=k caps it at k (tests use it to run several chunks).
int chunk_size(const GreenView& v, int n, size_t per_item) {
  const char* cap = std::getenv("RG_GREEN_CHUNK");
  const long cap_n = (cap && *cap) ? std::strtol(cap, nullptr, 10) : 0;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    free_b = (size_t)8 << 30;
  }
  const size_t budget = std::min(free_b / 2, (size_t)96 << 30);
  int64_t c = (int64_t)(budget / std::max<size_t>(per_item, 1));
  c = std::max<int64_t>(1, std::min<int64_t>(c, n));
  const int wave = 2 * v.sm_count;
  if (c > wave && c < n) c -= c % wave;
  if (cap_n > 0 && c > cap_n) c = cap_n;
  return (int)c;
}

// The forward sweep of nk realizations with the state of every slice kept,
// Fisher-Lee t (sqrt(real(mu)), full nmu x nmu) to d_t when given, source at
// slice `source` (0-based).  Dirichlet guides run a symmetric kernel (12 M^3
// per slice): the shared-memory one up to 64 modes, the blocked one above;
// the items it flags, and periodic guides, run the pivoted blocked kernel
// (16 M^3), which also keeps the states.  Planned before the arena is allocated: plan_sweep
// reserves the workspace and the flag list, launch_dump_sweep fills in the
// pointers and launches.
struct DumpSweep {
  rg::SweepArgs sym{};    // symmetric kernel (used when use_sym)
  rg::SweepArgs piv{};    // pivoted blocked kernel: every item, or the flagged ones
  bool use_sym = false, sym_blocked = false;
  int grid_sym = 0, grid_piv = 0;
  size_t off_work = 0, off_flags = 0;
};

int plan_sweep(const GreenView& v, int nk, int source, Arena& ar, DumpSweep* ds, int mode = rg::kModeTmat) {
  rg::SweepArgs a{};
  a.mode = mode;
  a.nreal = nk;
  a.wgs = v.d_desc;
  a.work_counter = v.d_counter;
  a.max_M = v.nmu;
  a.max_ny = v.ny;
  a.inject_at = source;
  ds->use_sym = v.symmetric != 0;
  ds->sym_blocked = v.nmu > rg::kMaxModesSmem;
  int64_t stride = 0, stride_sym = 0;
  int rc;
  ds->piv = a;
  ds->piv.force_large = 1;
  if ((rc = rg::sweep_large_plan(ds->piv, v.sm_count, &ds->grid_piv, &stride))) return rc;
  size_t work = sizeof(double2) * (size_t)stride * (ds->grid_piv / (ds->piv.cluster > 0 ? ds->piv.cluster : 1));
  ds->piv.work_stride = stride;
  if (ds->use_sym) {
    ds->sym = a;
    ds->sym.symmetric = 1;
    ds->sym.sym_tau = v.sym_tau;
    ds->sym.tensor_r = v.tensor_r;
    ds->sym.split_inverse = v.split_inverse;
    rc = ds->sym_blocked ? rg::sweep_large_sym_plan(ds->sym, v.sm_count, &ds->grid_sym, &stride_sym)
                         : rg::sweep_sym_plan(ds->sym, v.sm_count, &ds->grid_sym, &stride_sym);
    if (rc) return rc;
    ds->sym.work_stride = stride_sym;
    const int slots_sym = ds->grid_sym / (ds->sym.cluster > 0 ? ds->sym.cluster : 1);
    work = std::max(work, sizeof(double2) * (size_t)stride_sym * slots_sym);
    // The re-run takes the flagged items: queue length in counter 1, its
    // own position in counter 2.
    ds->piv.count_ptr = v.d_counter + 1;
    ds->piv.work_counter = v.d_counter + 2;
    ds->off_flags = ar.add(sizeof(int32_t) * (size_t)nk);
  }
  ds->off_work = ar.add(work);
  return RG_OK;
}

int launch_dump_sweep(const GreenView& v, DumpSweep& ds, const Arena& ar, int nk, const int32_t* d_seeds,
                      const double* d_upot, double2* d_dump, double2* d_t, int32_t* d_status,
                      double* d_teig = nullptr, cudaStream_t stream = nullptr) {
  cudaStream_t st = stream ? stream : v.stream;
  for (rg::SweepArgs* a : {&ds.sym, &ds.piv}) {
    a->nreal = nk;
    a->work = ar.at<double2>(ds.off_work);
    a->seeds = d_seeds;
    if (d_upot) {
      a->upot = d_upot;
      a->pot_rstride = (int64_t)v.nxdiso * v.ny;
      a->pot_xstride = v.ny;
      a->pot_ystride = 1;
    }
    a->state_dump = d_dump;
    a->tout = d_t;
    a->teig = d_teig;
    a->status = d_status;
  }
  RG_CUDA(cudaMemsetAsync(v.d_counter, 0, sizeof(int) * rg::kQueueCounters, st));
  int rc;
  if (ds.use_sym) {
    ds.sym.flag_list = ar.at<int32_t>(ds.off_flags);
    ds.piv.item_idx = ds.sym.flag_list;
    rc = ds.sym_blocked ? rg::launch_sweep_large_sym(ds.sym, st, ds.grid_sym)
                        : rg::launch_sweep_sym(ds.sym, st, ds.grid_sym);
    if (rc) return rc;
  }
  return rg::launch_sweep_large(ds.piv, st, ds.grid_piv);
}

int check_window_args(const GreenView& v, int kind, int nprof, const double* a, const double* b) {
  if (kind == RG_PROFILE_TPROFILE || kind == RG_PROFILE_ITX) {
    // src/waveguide.f90:775-781,853-859
    for (int w = 0; w < nprof; ++w) {
      const double tmin = a[w], tmax = b[w];
      if (tmin < 0.0 || tmin > 1.0)
        return rg::fail(RG_ERR_INVALID_ARG, "Invalid Tmin, received Tmin=" + g0(tmin, 3) + ", expected in [0, 1], aborting...");
      if (tmax < 0.0 || tmax > 1.0)
        return rg::fail(RG_ERR_INVALID_ARG, "Invalid Tmax, received Tmax=" + g0(tmax, 3) + ", expected in [0, 1], aborting...");
      if (tmin >= tmax) return rg::fail(RG_ERR_INVALID_ARG, "Invalid range (Tmin >= Tmax), aborting...");
    }
    return RG_OK;
  }
  if (kind == RG_PROFILE_GROUP) {
    // src/waveguide.f90:937-946 and the size check of diagonalize_ahca, src/base_utils.f90:413-414
    for (int w = 0; w < nprof; ++w)
      if (a[w] < 0.0 || a[w] > 1.0)
        return rg::fail(RG_ERR_INVALID_ARG, "Invalid transmission value, expected in [0, 1], aborting...");
    for (int w = 0; w < nprof; ++w)
      if (b[w] <= 0.0 || b[w] > 0.5)
        return rg::fail(RG_ERR_INVALID_ARG, "Invalid transmission half-width, expected 0 < dt <= 1/2, aborting...");
    if (v.neigv != v.jmax - v.jmin + 1)
      return rg::fail(RG_ERR_INVALID_ARG, "RecurGreen v1.0: zgesvd: Invalid number of singular values, aborting...");
    return RG_OK;
  }
  return rg::fail(RG_ERR_INVALID_ARG, "rg_tprofile_batch: unknown profile kind " + std::to_string(kind));
}

int check_position(const GreenView& v, int pos, const char* which, const char* name) {
  if (pos < 1 || v.nx < pos)
    return rg::fail(RG_ERR_INVALID_ARG, std::string("Invalid ") + which + " position index, received " + name + "=" +
                                            std::to_string(pos) + ", expected in 1.." + std::to_string(v.nx) +
                                            ", aborting...");
  return RG_OK;
}

}  // namespace

extern "C" {

int rg_tprofile_batch(rg_waveguide* w, const int32_t* seeds, int n, int kind, int nprof, const double* a,
                      const double* b, double* profiles, int32_t* nt, double* tavg, int32_t* status) {
  rg::NvtxRange nvtx_range("rg_tprofile_batch");
  GreenView v{};
  int rc = rg::green_view(w, &v);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!seeds || !profiles)) || nprof < 1 || nprof > 32 || !a || !b)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_tprofile_batch: invalid argument");
  if ((rc = check_window_args(v, kind, nprof, a, b))) return rc;
  if (n == 0) return RG_OK;
  DeviceGuard g(v.device);
  const int M = v.nmu, nx = v.nx;
  const bool group = kind == RG_PROFILE_GROUP;
  const int row0 = group ? v.imin - 1 : 0, nr = group ? v.imax - v.imin + 1 : M;
  const int col0 = group ? v.jmin - 1 : 0, nc = group ? v.jmax - v.jmin + 1 : M;
  const size_t mm = (size_t)M * M;
  const int64_t estride = rg::eigvec_work_stride(nr, nc);
  const size_t per_item = sizeof(double2) * (2 * nx * mm + mm + (size_t)estride + (size_t)nc * M) +
                          sizeof(double) * ((size_t)nc * nx + (size_t)nprof * nx + nc + 1) +
                          sizeof(int32_t) * (4 + 2 * (size_t)nc + nprof);
  const int chunk = chunk_size(v, n, per_item);

  Arena ar;
  const size_t o_seed = ar.add(sizeof(int32_t) * chunk), o_st = ar.add(sizeof(int32_t) * 2 * chunk);
  const size_t o_dump = ar.add(sizeof(double2) * 2 * nx * mm * chunk), o_t = ar.add(sizeof(double2) * mm * chunk);
  const size_t o_ew = ar.add(sizeof(double2) * (size_t)estride * chunk);
  const size_t o_tv = ar.add(sizeof(double) * (size_t)nc * chunk);
  const size_t o_ws = ar.add(sizeof(double2) * (size_t)nc * M * chunk);
  const size_t o_mb = ar.add(sizeof(uint32_t) * (size_t)nc * chunk), o_ks = ar.add(sizeof(int32_t) * chunk);
  const size_t o_nt = ar.add(sizeof(int32_t) * (size_t)nprof * chunk), o_ta = ar.add(sizeof(double) * chunk);
  const size_t o_pr = ar.add(sizeof(double) * (size_t)nc * nx * chunk);
  const size_t o_out = ar.add(sizeof(double) * (size_t)nprof * nx * chunk);
  const size_t o_ab = ar.add(sizeof(double) * 2 * nprof);
  DumpSweep ds;
  if ((rc = plan_sweep(v, chunk, 0, ar, &ds))) return rc;
  if ((rc = ar.alloc())) return rc;
  cudaStream_t s = v.stream;
  double* d_ab = ar.at<double>(o_ab);
  RG_CUDA(cudaMemcpyAsync(d_ab, a, sizeof(double) * nprof, cudaMemcpyHostToDevice, s));
  RG_CUDA(cudaMemcpyAsync(d_ab + nprof, b, sizeof(double) * nprof, cudaMemcpyHostToDevice, s));
  std::vector<int32_t> st(2 * (size_t)chunk);
  int bad = RG_OK;
  for (int k0 = 0; k0 < n; k0 += chunk) {
    const int nk = std::min(chunk, n - k0);
    int32_t* d_st = ar.at<int32_t>(o_st);
    RG_CUDA(cudaMemcpyAsync(ar.at<int32_t>(o_seed), seeds + k0, sizeof(int32_t) * nk, cudaMemcpyHostToDevice, s));
    if ((rc = launch_dump_sweep(v, ds, ar, nk, ar.at<int32_t>(o_seed), nullptr, ar.at<double2>(o_dump),
                                ar.at<double2>(o_t), d_st)))
      return rc;
    rg::EigvecArgs e{};
    e.nreal = nk;
    e.a = ar.at<double2>(o_t);
    e.astride = (int64_t)mm;
    e.lda = M;
    e.row0 = row0;
    e.nr = nr;
    e.col0 = col0;
    e.nc = nc;
    e.work = ar.at<double2>(o_ew);
    e.work_stride = estride;
    e.tvals = ar.at<double>(o_tv);
    e.nprof = nprof;
    e.centered = group ? 1 : 0;
    e.wa = d_ab;
    e.wb = d_ab + nprof;
    e.M = M;
    e.sqmu = v.desc.sqmu_r;
    e.wsel = ar.at<double2>(o_ws);
    e.member = ar.at<uint32_t>(o_mb);
    e.ksel = ar.at<int32_t>(o_ks);
    e.nt = ar.at<int32_t>(o_nt);
    e.tavg = ar.at<double>(o_ta);
    e.status = d_st + chunk;
    if ((rc = rg::launch_eigvec(e, s))) return rc;
    rg::BackArgs bk{};
    bk.nreal = nk;
    bk.M = M;
    bk.nx = nx;
    bk.dump = ar.at<double2>(o_dump);
    bk.bmat = v.desc.bmat;
    bk.src = e.wsel;
    bk.src_stride = (int64_t)nc * M;
    bk.kmax = nc;
    bk.kcount = e.ksel;
    bk.i_lo = 0;
    bk.out_mode = rg::kBackProfile;
    bk.prof = ar.at<double>(o_pr);
    if ((rc = rg::launch_back(bk, s))) return rc;
    rg::WindowArgs wa{};
    wa.nreal = nk;
    wa.nx = nx;
    wa.kmax = nc;
    wa.nprof = nprof;
    wa.kind = kind;
    wa.wol = v.wol;
    wa.wa = d_ab;
    wa.wb = d_ab + nprof;
    wa.ksel = e.ksel;
    wa.member = e.member;
    wa.nt = e.nt;
    wa.prof = bk.prof;
    wa.out = ar.at<double>(o_out);
    if ((rc = rg::launch_windows(wa, s))) return rc;
    RG_CUDA(cudaMemcpyAsync(profiles + (size_t)k0 * nprof * nx, wa.out, sizeof(double) * (size_t)nk * nprof * nx,
                            cudaMemcpyDeviceToHost, s));
    if (nt)
      RG_CUDA(cudaMemcpyAsync(nt + (size_t)k0 * nprof, e.nt, sizeof(int32_t) * (size_t)nk * nprof,
                              cudaMemcpyDeviceToHost, s));
    if (tavg) RG_CUDA(cudaMemcpyAsync(tavg + k0, e.tavg, sizeof(double) * nk, cudaMemcpyDeviceToHost, s));
    RG_CUDA(cudaMemcpyAsync(st.data(), d_st, sizeof(int32_t) * 2 * chunk, cudaMemcpyDeviceToHost, s));
    RG_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < nk; ++k) {
      const int sk = st[k] != RG_OK ? st[k] : st[(size_t)chunk + k];
      if (status) status[k0 + k] = sk;
      if (!bad && sk != RG_OK) bad = sk;
    }
  }
  if (bad) return rg::fail(bad, status_text(bad));
  return RG_OK;
}

int rg_compute_tprofile(rg_waveguide* w, int iseed, double tmin, double tmax, double* tprofile, int64_t len,
                        int* nt) {
  GreenView v{};
  int rc = rg::green_view(w, &v);
  if (rc) return rc;
  if (!tprofile) return rg::fail(RG_ERR_INVALID_ARG, "rg_compute_tprofile: NULL argument");
  if ((rc = check_window_args(v, RG_PROFILE_TPROFILE, 1, &tmin, &tmax))) return rc;
  if (len != v.nx)  // src/waveguide.f90:860-863
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid size for tprofile, received " + std::to_string(len) + ", expected " +
                                            std::to_string(v.nx) + ", aborting...");
  const int32_t s = iseed;
  int32_t n1 = 0;
  rc = rg_tprofile_batch(w, &s, 1, RG_PROFILE_TPROFILE, 1, &tmin, &tmax, tprofile, &n1, nullptr, nullptr);
  if (nt) *nt = n1;
  return rc;
}

int rg_compute_itx_profile(rg_waveguide* w, int iseed, double tmin, double tmax, double* itx, int64_t len) {
  GreenView v{};
  int rc = rg::green_view(w, &v);
  if (rc) return rc;
  if (!itx) return rg::fail(RG_ERR_INVALID_ARG, "rg_compute_itx_profile: NULL argument");
  if ((rc = check_window_args(v, RG_PROFILE_ITX, 1, &tmin, &tmax))) return rc;
  if (len != v.nx)  // src/waveguide.f90:782-785
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid size for itx, received " + std::to_string(len) + ", expected " +
                                            std::to_string(v.nx) + ", aborting...");
  const int32_t s = iseed;
  return rg_tprofile_batch(w, &s, 1, RG_PROFILE_ITX, 1, &tmin, &tmax, itx, nullptr, nullptr, nullptr);
}

int rg_compute_tprofile_group(rg_waveguide* w, int iseed, int nprof, const double* tm, const double* dt,
                              double* tprofile, int64_t len, int32_t* nt, double* tavg) {
  GreenView v{};
  int rc = rg::green_view(w, &v);
  if (rc) return rc;
  if (!tprofile || !tm || !dt || nprof < 1 || nprof > 32)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_compute_tprofile_group: invalid argument");
  for (int k = 0; k < nprof; ++k)  // src/waveguide.f90:937-946
    if (tm[k] < 0.0 || tm[k] > 1.0)
      return rg::fail(RG_ERR_INVALID_ARG, "Invalid transmission value, expected in [0, 1], aborting...");
  for (int k = 0; k < nprof; ++k)
    if (dt[k] <= 0.0 || dt[k] > 0.5)
      return rg::fail(RG_ERR_INVALID_ARG, "Invalid transmission half-width, expected 0 < dt <= 1/2, aborting...");
  if (len != (int64_t)v.nx * nprof)
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid size for tprofile, received " + std::to_string(len) +
                                            " values, expected (" + std::to_string(v.nx) + ", " +
                                            std::to_string(nprof) + "), aborting...");
  const int32_t s = iseed;
  return rg_tprofile_batch(w, &s, 1, RG_PROFILE_GROUP, nprof, tm, dt, tprofile, nt, tavg, nullptr);
}

int rg_deposition_batch(rg_waveguide* w, const int32_t* seeds, int n, int fpos, int ipos, int col, double* out,
                        int32_t* status) {
  rg::NvtxRange nvtx_range("rg_deposition_batch");
  GreenView v{};
  int rc = rg::green_view(w, &v);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!seeds || !out))) return rg::fail(RG_ERR_INVALID_ARG, "rg_deposition_batch: invalid argument");
  // src/waveguide.f90:718-726
  if ((rc = check_position(v, fpos, "final", "fpos"))) return rc;
  if ((rc = check_position(v, ipos, "initial", "ipos"))) return rc;
  const int M = v.nmu, nx = v.nx;
  if (col < 0 || col > M)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_deposition_batch: column " + std::to_string(col) + " not in 0.." +
                                            std::to_string(M));
  if (n == 0) return RG_OK;
  DeviceGuard g(v.device);
  const int k = col > 0 ? 1 : M;
  const size_t mm = (size_t)M * M;
  const size_t per_item = sizeof(double2) * (2 * nx * mm + (size_t)k * M) + sizeof(int32_t) * 4;
  const int chunk = chunk_size(v, n, per_item);
  Arena ar;
  const size_t o_seed = ar.add(sizeof(int32_t) * chunk), o_st = ar.add(sizeof(int32_t) * chunk);
  const size_t o_dump = ar.add(sizeof(double2) * 2 * nx * mm * chunk);
  const size_t o_w = ar.add(sizeof(double2) * (size_t)k * M);
  const size_t o_out = ar.add(sizeof(double2) * (size_t)k * M * chunk);
  DumpSweep ds;
  if ((rc = plan_sweep(v, chunk, ipos - 1, ar, &ds))) return rc;
  if ((rc = ar.alloc())) return rc;
  cudaStream_t s = v.stream;
  // Source vectors sqrt(real(mu_c)) e_c: the right factor of 2i sqmu G sqmu.
  std::vector<cplx> wsrc((size_t)k * M, cplx(0.0, 0.0));
  for (int q = 0; q < k; ++q) {
    const int c = col > 0 ? col - 1 : q;
    wsrc[(size_t)q * M + c] = v.sqmu_r[c];
  }
  RG_CUDA(cudaMemcpyAsync(ar.at<double2>(o_w), wsrc.data(), sizeof(double2) * wsrc.size(), cudaMemcpyHostToDevice, s));
  std::vector<int32_t> st(chunk);
  int bad = RG_OK;
  for (int k0 = 0; k0 < n; k0 += chunk) {
    const int nk = std::min(chunk, n - k0);
    RG_CUDA(cudaMemcpyAsync(ar.at<int32_t>(o_seed), seeds + k0, sizeof(int32_t) * nk, cudaMemcpyHostToDevice, s));
    if ((rc = launch_dump_sweep(v, ds, ar, nk, ar.at<int32_t>(o_seed), nullptr, ar.at<double2>(o_dump), nullptr,
                                ar.at<int32_t>(o_st))))
      return rc;
    rg::BackArgs bk{};
    bk.nreal = nk;
    bk.M = M;
    bk.nx = nx;
    bk.dump = ar.at<double2>(o_dump);
    bk.bmat = v.desc.bmat;
    bk.src = ar.at<double2>(o_w);
    bk.src_stride = 0;
    bk.kmax = k;
    bk.i_lo = fpos - 1;
    bk.out_mode = rg::kBackColumns;
    bk.only_lo = 1;
    bk.left = v.desc.sqmu_r;
    bk.cols = ar.at<double2>(o_out);
    if ((rc = rg::launch_back(bk, s))) return rc;
    RG_CUDA(cudaMemcpyAsync(out + 2 * (size_t)k0 * k * M, bk.cols, sizeof(double2) * (size_t)nk * k * M,
                            cudaMemcpyDeviceToHost, s));
    RG_CUDA(cudaMemcpyAsync(st.data(), ar.at<int32_t>(o_st), sizeof(int32_t) * nk, cudaMemcpyDeviceToHost, s));
    RG_CUDA(cudaStreamSynchronize(s));
    for (int q = 0; q < nk; ++q) {
      if (status) status[k0 + q] = st[q];
      if (!bad && st[q] != RG_OK) bad = st[q];
    }
  }
  if (bad) return rg::fail(bad, status_text(bad));
  return RG_OK;
}

int rg_compute_deposition(rg_waveguide* w, int iseed, int fpos, int ipos, double* depmat) {
  if (!depmat) return rg::fail(RG_ERR_INVALID_ARG, "rg_compute_deposition: NULL argument");
  const int32_t s = iseed;
  return rg_deposition_batch(w, &s, 1, fpos, ipos, 0, depmat, nullptr);
}

int rg_compute_refl_trans_v2(rg_waveguide* w, int iseed, double* rmat, double* tmat) {
  rg::NvtxRange nvtx_range("rg_compute_refl_trans_v2");
  GreenView v{};
  int rc = rg::green_view(w, &v);
  if (rc) return rc;
  if (!tmat) return rg::fail(RG_ERR_INVALID_ARG, "rg_compute_refl_trans_v2: NULL argument");
  // src/waveguide.f90:526-553: the full solve with the identity source at
  // slice 1; t = 2i sqmu X_nx sqmu, r = -1 + 2i sqmu X_1 sqmu.
  if ((rc = rg_compute_deposition(w, iseed, v.nx, 1, tmat))) return rc;
  if (rmat) {
    if ((rc = rg_compute_deposition(w, iseed, 1, 1, rmat))) return rc;
    for (int i = 0; i < v.nmu; ++i) rmat[2 * ((size_t)i * v.nmu + i)] -= 1.0;
  }
  return RG_OK;
}

int rg_compute_wavefunction(rg_waveguide* w, int iseed, int ipos, int imode, double* wfundata, int64_t rows) {
  rg::NvtxRange nvtx_range("rg_compute_wavefunction");
  GreenView v{};
  int rc = rg::green_view(w, &v);
  if (rc) return rc;
  if (!wfundata) return rg::fail(RG_ERR_INVALID_ARG, "rg_compute_wavefunction: NULL argument");
  const int M = v.nmu, nx = v.nx, ny = v.ny;
  // src/waveguide.f90:646-654
  if (imode < 1 || M < imode)
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid initial mode index, received imode=" + std::to_string(imode) +
                                            ", expected in 1.." + std::to_string(M) + ", aborting...");
  if ((rc = check_position(v, ipos, "initial", "ipos"))) return rc;
  if (rows != (int64_t)nx * ny)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_compute_wavefunction: rows must be nx*ny = " +
                                            std::to_string((int64_t)nx * ny));
  // src/waveguide.f90:657-661: imode 1 is the ground state of a periodic guide.
  const int imu = v.periodic ? (imode + M / 2 - 1) % M + 1 : imode;
  DeviceGuard g(v.device);
  const size_t mm = (size_t)M * M;
  Arena ar;
  const size_t o_seed = ar.add(sizeof(int32_t)), o_st = ar.add(sizeof(int32_t));
  const size_t o_pot = ar.add(sizeof(double) * (size_t)v.nxdiso * ny);
  const size_t o_dump = ar.add(sizeof(double2) * 2 * nx * mm);
  const size_t o_w = ar.add(sizeof(double2) * M), o_y = ar.add(sizeof(double2) * (size_t)nx * M);
  const size_t o_modal = ar.add(sizeof(double2) * (size_t)ny * M);
  const size_t o_x = ar.add(sizeof(double) * nx), o_ym = ar.add(sizeof(double) * ny);
  const size_t o_out = ar.add(sizeof(double) * 5 * (size_t)nx * ny);
  DumpSweep ds;
  if ((rc = plan_sweep(v, 1, ipos - 1, ar, &ds))) return rc;
  if ((rc = ar.alloc())) return rc;
  cudaStream_t s = v.stream;
  // The modal matrix modal(iy, imu) = chi_imu(y_iy) of src/waveguide.f90:179-185
  // (periodic) and :221-227 (Dirichlet), stored [iy][imu].
  std::vector<cplx> modal((size_t)ny * M);
  for (int n = 0; n < M; ++n)
    for (int i = 0; i < ny; ++i) {
      const double arg = 2 * kPi * v.wol * v.kpmesh[n] * v.ymesh[i];
      modal[(size_t)i * M + n] = v.periodic ? std::exp(cplx(0.0, arg)) / std::sqrt((double)ny)
                                            : cplx(std::sqrt(2.0 / ny) * std::sin(arg), 0.0);
    }
  std::vector<cplx> wsrc(M, cplx(0.0, 0.0));
  wsrc[imu - 1] = cplx(1.0, 0.0);
  const int32_t seed = iseed;
  RG_CUDA(cudaMemcpyAsync(ar.at<int32_t>(o_seed), &seed, sizeof seed, cudaMemcpyHostToDevice, s));
  RG_CUDA(cudaMemcpyAsync(ar.at<double2>(o_modal), modal.data(), sizeof(double2) * modal.size(), cudaMemcpyHostToDevice, s));
  RG_CUDA(cudaMemcpyAsync(ar.at<double2>(o_w), wsrc.data(), sizeof(double2) * M, cudaMemcpyHostToDevice, s));
  RG_CUDA(cudaMemcpyAsync(ar.at<double>(o_x), v.xmesh, sizeof(double) * nx, cudaMemcpyHostToDevice, s));
  RG_CUDA(cudaMemcpyAsync(ar.at<double>(o_ym), v.ymesh, sizeof(double) * ny, cudaMemcpyHostToDevice, s));
  rg::PotArgs pa{};
  pa.nxdiso = v.nxdiso;
  pa.ny = ny;
  pa.nreal = 1;
  pa.stdu = v.stdu;
  pa.seeds = ar.at<int32_t>(o_seed);
  pa.jumppoly = v.desc.jumppoly;
  pa.upot = ar.at<double>(o_pot);
  if ((rc = rg::launch_potential(pa, s))) return rc;
  if ((rc = launch_dump_sweep(v, ds, ar, 1, nullptr, pa.upot, ar.at<double2>(o_dump), nullptr, ar.at<int32_t>(o_st))))
    return rc;
  rg::BackArgs bk{};
  bk.nreal = 1;
  bk.M = M;
  bk.nx = nx;
  bk.dump = ar.at<double2>(o_dump);
  bk.bmat = v.desc.bmat;
  bk.src = ar.at<double2>(o_w);
  bk.kmax = 1;
  bk.i_lo = 0;
  bk.out_mode = rg::kBackColumns;
  bk.cols = ar.at<double2>(o_y);
  if ((rc = rg::launch_back(bk, s))) return rc;
  rg::WavefunArgs wf{};
  wf.nx = nx;
  wf.ny = ny;
  wf.M = M;
  wf.nxfree = v.nxfree;
  wf.nxdiso = v.nxdiso;
  wf.y = bk.cols;
  wf.modal = ar.at<double2>(o_modal);
  wf.xmesh = ar.at<double>(o_x);
  wf.ymesh = ar.at<double>(o_ym);
  wf.upot = pa.upot;
  wf.out = ar.at<double>(o_out);
  if ((rc = rg::launch_wavefun(wf, s))) return rc;
  int32_t st = 0;
  RG_CUDA(cudaMemcpyAsync(wfundata, wf.out, sizeof(double) * 5 * (size_t)nx * ny, cudaMemcpyDeviceToHost, s));
  RG_CUDA(cudaMemcpyAsync(&st, ar.at<int32_t>(o_st), sizeof st, cudaMemcpyDeviceToHost, s));
  RG_CUDA(cudaStreamSynchronize(s));
  if (st != RG_OK) return rg::fail(st, status_text(st));
  return RG_OK;
}

int rg_sweep_states(rg_waveguide* w, const double* d_upot, int n, double* d_states, double* d_tfilt, double* d_teig,
                    int32_t* d_status, void* stream) {
  rg::NvtxRange nvtx_range("rg_sweep_states");
  GreenView v{};
  int rc = rg::green_view(w, &v);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!d_upot || !d_teig || !d_status)))
    return rg::fail(RG_ERR_INVALID_ARG, "rg_sweep_states: invalid argument");
  if (n == 0) return RG_OK;
  DeviceGuard g(v.device);
  cudaStream_t s = (cudaStream_t)stream;  // taken literally: 0 is CUDA's default stream
  Arena ar;
  DumpSweep ds;
  if ((rc = plan_sweep(v, n, 0, ar, &ds, rg::kModeEig))) return rc;
  if ((rc = ar.alloc())) return rc;
  rc = launch_dump_sweep(v, ds, ar, n, nullptr, d_upot, (double2*)d_states, (double2*)d_tfilt, d_status, d_teig,
                         s ? s : cudaStreamLegacy);
  if (rc) return rc;
  // The workspace is freed when this call returns: wait for the sweep.
  RG_CUDA(cudaStreamSynchronize(s ? s : cudaStreamLegacy));
  return RG_OK;
}

int rg_diagonalize_ahca(const double* a, int m, int n, double* T, double* U) {
  rg::NvtxRange nvtx_range("rg_diagonalize_ahca");
  if (!a || !T || !U || m < 1 || n < 1) return rg::fail(RG_ERR_INVALID_ARG, "rg_diagonalize_ahca: invalid argument");
  Arena ar;
  const int64_t es = rg::eigvec_work_stride(m, n);
  const size_t o_a = ar.add(sizeof(double2) * (size_t)m * n), o_w = ar.add(sizeof(double2) * (size_t)es);
  const size_t o_t = ar.add(sizeof(double) * n), o_u = ar.add(sizeof(double2) * (size_t)n * n);
  const size_t o_st = ar.add(sizeof(int32_t));
  int rc = ar.alloc();
  if (rc) return rc;
  cudaStream_t s = 0;
  RG_CUDA(cudaMemcpyAsync(ar.at<double2>(o_a), a, sizeof(double2) * (size_t)m * n, cudaMemcpyHostToDevice, s));
  rg::EigvecArgs e{};
  e.nreal = 1;
  e.a = ar.at<double2>(o_a);
  e.lda = m;
  e.nr = m;
  e.nc = n;
  e.work = ar.at<double2>(o_w);
  e.work_stride = es;
  e.tvals = ar.at<double>(o_t);
  e.u = ar.at<double2>(o_u);
  e.status = ar.at<int32_t>(o_st);
  if ((rc = rg::launch_eigvec(e, s))) return rc;
  int32_t st = 0;
  RG_CUDA(cudaMemcpyAsync(T, e.tvals, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  RG_CUDA(cudaMemcpyAsync(U, e.u, sizeof(double2) * (size_t)n * n, cudaMemcpyDeviceToHost, s));
  RG_CUDA(cudaMemcpyAsync(&st, e.status, sizeof st, cudaMemcpyDeviceToHost, s));
  RG_CUDA(cudaStreamSynchronize(s));
  if (st != RG_OK) return rg::fail(st, status_text(st));
  return RG_OK;
}

}  // extern "C"
