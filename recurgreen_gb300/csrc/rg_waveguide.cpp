// Host side of the C ABI: the waveguide object (init_waveguide and friends,
// src/waveguide.f90:81-350), device tables, batching and error handling.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <new>
#include <string>
#include <vector>

#include "rg_internal.h"

using rg::cplx;
using rg::DeviceGuard;
using rg::status_text;

namespace rg {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(RG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------
// xoshiro256 jump-ahead.  The state update of xoshiro256 is linear over
// GF(2); its characteristic polynomial p(x) (degree 256) is recovered with
// Berlekamp-Massey from one state bit, and advancing the state by d steps is
// multiplication by x^d mod p(x), evaluated on the state by Horner's rule.
// ---------------------------------------------------------------------------
namespace {

struct State {
  uint64_t s[4];
};

inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

inline void step(State& st) {
  uint64_t* s = st.s;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl(s[3], 45);
}

struct CharPoly {
  uint64_t w[5];  // bit i = coefficient of x^i, degree 256
};

CharPoly compute_charpoly() {
  const int N = 512;
  State st{{0x9e3779b97f4a7c15ULL, 0xbf58476d1ce4e5b9ULL, 0x94d049bb133111ebULL, 0x2545f4914f6cdd1dULL}};
  std::vector<int> seq(N);
  for (int i = 0; i < N; ++i) {
    seq[i] = (int)(st.s[0] & 1ULL);
    step(st);
  }
  // Berlekamp-Massey over GF(2).
  std::vector<int> C(N + 1, 0), B(N + 1, 0), T;
  C[0] = B[0] = 1;
  int L = 0, m = 1;
  for (int n = 0; n < N; ++n) {
    int d = seq[n];
    for (int i = 1; i <= L; ++i) d ^= C[i] & seq[n - i];
    if (!d) {
      ++m;
    } else if (2 * L <= n) {
      T = C;
      for (int i = 0; i + m <= N; ++i) C[i + m] ^= B[i];
      L = n + 1 - L;
      B = T;
      m = 1;
    } else {
      for (int i = 0; i + m <= N; ++i) C[i + m] ^= B[i];
      ++m;
    }
  }
  CharPoly p{};
  // p(x) = x^L C(1/x)
  for (int i = 0; i <= L; ++i)
    if (C[L - i]) p.w[i >> 6] |= 1ULL << (i & 63);
  if (L != 256) p.w[4] = 0;  // flagged by the self-check below
  return p;
}

const CharPoly& charpoly() {
  static const CharPoly p = compute_charpoly();
  return p;
}

// a * b mod p for polynomials of degree < 256.
void mulmod(const uint64_t a[4], const uint64_t b[4], uint64_t out[4]) {
  const CharPoly& p = charpoly();
  uint64_t prod[9] = {0};
  for (int i = 0; i < 256; ++i) {
    if (!((a[i >> 6] >> (i & 63)) & 1ULL)) continue;
    const int ws = i >> 6, bs = i & 63;
    for (int w = 0; w < 4; ++w) {
      prod[w + ws] ^= b[w] << bs;
      if (bs) prod[w + ws + 1] ^= b[w] >> (64 - bs);
    }
  }
  for (int deg = 511; deg >= 256; --deg) {
    if (!((prod[deg >> 6] >> (deg & 63)) & 1ULL)) continue;
    const int sh = deg - 256, ws = sh >> 6, bs = sh & 63;
    for (int w = 0; w < 5; ++w) {
      prod[w + ws] ^= p.w[w] << bs;
      if (bs && w + ws + 1 < 9) prod[w + ws + 1] ^= p.w[w] >> (64 - bs);
    }
  }
  for (int w = 0; w < 4; ++w) out[w] = prod[w];
}

void apply_jump(State& st, const uint64_t poly[4]) {
  State acc{{0, 0, 0, 0}};
  for (int i = 0; i < 256; ++i) {
    if ((poly[i >> 6] >> (i & 63)) & 1ULL)
      for (int k = 0; k < 4; ++k) acc.s[k] ^= st.s[k];
    step(st);
  }
  st = acc;
}

// One-time check that jump(d) equals d single steps.
int rng_selfcheck() {
  static int result = -1;
  static std::once_flag once;
  std::call_once(once, [] {
    if (charpoly().w[4] != 1ULL) {
      result = 1;
      return;
    }
    State a{{0x0123456789abcdefULL, 0xfedcba9876543210ULL, 0x0f1e2d3c4b5a6978ULL, 0x8796a5b4c3d2e1f0ULL}};
    State b = a;
    uint64_t poly[4];
    jump_polynomial(12345, poly);
    apply_jump(a, poly);
    for (int i = 0; i < 12345; ++i) step(b);
    result = std::memcmp(a.s, b.s, sizeof a.s) != 0;
  });
  return result;
}

}  // namespace

void jump_polynomial(uint64_t distance, uint64_t out[4]) {
  uint64_t result[4] = {1, 0, 0, 0};  // x^0
  uint64_t base[4] = {2, 0, 0, 0};    // x^1
  while (distance) {
    if (distance & 1ULL) mulmod(result, base, result);
    mulmod(base, base, base);
    distance >>= 1;
  }
  std::memcpy(out, result, sizeof result);
}

}  // namespace rg

// ---------------------------------------------------------------------------
// The waveguide handle.
// ---------------------------------------------------------------------------
// Entries of the argument set a cached batch graph was captured with.
constexpr int kGraphKey = 15;

struct rg_waveguide {
  rg_params p{};
  int nmu = 0, ny = 0, nx = 0, imin = 0, imax = 0, jmin = 0, jmax = 0, neigv = 0, nprop = 0;
  double kl = 0, kdx = 0, dos = 0, stdu = 0;
  std::vector<double> xmesh, ymesh, kpmesh;
  std::vector<cplx> mumesh, bmat, aedge, abulk, sqmu_c, sqmu_r;
  std::vector<double> costab;    // [ny][2*nmu+1], Dirichlet
  std::vector<cplx> expfac;      // [ny][nmu], periodic
  std::vector<uint64_t> jump;    // [ny][4]

  int device = 0, sm_count = 0;
  cudaStream_t stream = nullptr;
  double2 *d_bmat = nullptr, *d_aedge = nullptr, *d_abulk = nullptr, *d_sqmu_c = nullptr, *d_sqmu_r = nullptr;
  double* d_costab = nullptr;
  double2* d_expfac = nullptr;
  uint64_t* d_jump = nullptr;
  int* d_counter = nullptr;
  rg::WgDesc h_desc{};           // the kernels' view of this waveguide (device pointers)
  rg::WgDesc* d_desc = nullptr;  // its device copy
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  cudaEvent_t ev_sweep0 = nullptr, ev_sweep1 = nullptr;  // around the last batch's sweep launches
  bool sweep_timed = false;
  rg_batch_info last_batch{};  // launch configuration of the last batch (rerun read on demand)
  // The last batch launch, captured as a CUDA graph and replayed while its
  // arguments (sizes, buffers, workspace, kernel choice) stay the same.
  cudaGraphExec_t graph = nullptr;
  int64_t graph_key[kGraphKey] = {0};
  // rg_tdistrib_multi with this handle first: its device buffers (kept for
  // the next call), one stream per kernel class, and the class launches
  // captured as one CUDA graph (parallel branches), replayed while the
  // launch plans and buffers stay the same.
  static constexpr int kMultiClasses = 4;
  void* d_multi = nullptr;
  size_t multi_bytes = 0;
  cudaStream_t multi_streams[kMultiClasses] = {};
  cudaEvent_t multi_fork = nullptr, multi_join[kMultiClasses] = {};
  cudaGraphExec_t multi_graph = nullptr;
  std::vector<int64_t> multi_key;
  int multi_replays = 0;
};

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

template <class T>
int upload(T** dst, const void* src, size_t bytes) {
  if (bytes == 0) {
    *dst = nullptr;
    return RG_OK;
  }
  RG_CUDA(cudaMalloc((void**)dst, bytes));
  RG_CUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
  return RG_OK;
}

void free_device(rg_waveguide* w) {
  cudaFree(w->d_bmat);
  cudaFree(w->d_aedge);
  cudaFree(w->d_abulk);
  cudaFree(w->d_sqmu_c);
  cudaFree(w->d_sqmu_r);
  cudaFree(w->d_costab);
  cudaFree(w->d_expfac);
  cudaFree(w->d_jump);
  cudaFree(w->d_counter);
  cudaFree(w->d_desc);
  cudaFree(w->d_scratch);
  if (w->graph) cudaGraphExecDestroy(w->graph);
  w->graph = nullptr;
  if (w->multi_graph) cudaGraphExecDestroy(w->multi_graph);
  w->multi_graph = nullptr;
  w->multi_key.clear();
  cudaFree(w->d_multi);
  w->d_multi = nullptr;
  w->multi_bytes = 0;
  for (int c = 0; c < rg_waveguide::kMultiClasses; ++c) {
    if (w->multi_streams[c]) cudaStreamDestroy(w->multi_streams[c]);
    if (w->multi_join[c]) cudaEventDestroy(w->multi_join[c]);
    w->multi_streams[c] = nullptr;
    w->multi_join[c] = nullptr;
  }
  if (w->multi_fork) cudaEventDestroy(w->multi_fork);
  w->multi_fork = nullptr;
  if (w->ev_sweep0) cudaEventDestroy(w->ev_sweep0);
  if (w->ev_sweep1) cudaEventDestroy(w->ev_sweep1);
  w->ev_sweep0 = w->ev_sweep1 = nullptr;
  w->sweep_timed = false;
  if (w->stream) cudaStreamDestroy(w->stream);
  w->d_bmat = w->d_aedge = w->d_abulk = w->d_sqmu_c = w->d_sqmu_r = nullptr;
  w->d_costab = nullptr;
  w->d_expfac = nullptr;
  w->d_jump = nullptr;
  w->d_counter = nullptr;
  w->d_desc = nullptr;
  w->d_scratch = nullptr;
  w->scratch_bytes = 0;
  w->stream = nullptr;
}

// Host tables of init_waveguide, src/waveguide.f90:81-255.
int build_tables(rg_waveguide* w, const rg_params& p) {
  const double eps = 2.220446049250313e-16;
  if (p.wol < eps) return rg::fail(RG_ERR_INVALID_ARG, "Invalid width-to-wavelength ratio.");
  if (p.aratio < eps) return rg::fail(RG_ERR_INVALID_ARG, "Invalid aspect ratio.");
  if (p.exfac < 1.0 || p.exfac > 1e4)
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid modal basis extension factor. It must be in [1, 10000].");
  if (p.nxfree < 0) return rg::fail(RG_ERR_INVALID_ARG, "Invalid number of x points, cannot be negative.");
  if (p.nxdiso < 1 || p.nxdiso + 2 * p.nxfree < 2)
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid number of x points, need nxdiso >= 1 and nx >= 2.");
  if (p.dscat < 0.0 || p.dabso < 0.0) return rg::fail(RG_ERR_INVALID_ARG, "Invalid optical depth, cannot be negative.");
  if (!(p.napera > 0.0 && p.napera <= 1.0))
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid filtering parameter napera (expected in ]0, 1]).");
  if (!(p.naperb > 0.0 && p.naperb <= 1.0))
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid filtering parameter naperb (expected in ]0, 1]).");
  if (p.ny < 0) return rg::fail(RG_ERR_INVALID_ARG, "Invalid ny, cannot be negative.");

  w->p = p;
  w->kl = 2.0 * kPi * p.wol * p.aratio;
  w->nx = p.nxdiso + 2 * p.nxfree;
  w->kdx = w->kl / p.nxdiso;
  w->xmesh.resize(w->nx);
  for (int i = 1; i <= w->nx; ++i) w->xmesh[i - 1] = p.aratio * (i - 0.5 - p.nxfree) / p.nxdiso;

  if (p.boundtype == RG_BOUND_PERIODIC) {
    if (std::fmod(p.wol, 1.0) == 0.0)
      return rg::fail(RG_ERR_INVALID_ARG, "Invalid width wol, cannot be an integer for 'periodic' boundary conditions.");
    w->nmu = 2 * (int)std::floor(p.exfac * p.wol) + 1;
    w->imin = w->nmu / 2 + 1 - (int)std::floor(p.naperb * p.wol);
    w->imax = w->nmu / 2 + 1 + (int)std::floor(p.naperb * p.wol);
    w->jmin = w->nmu / 2 + 1 - (int)std::floor(p.napera * p.wol);
    w->jmax = w->nmu / 2 + 1 + (int)std::floor(p.napera * p.wol);
    w->neigv = 2 * (int)std::floor(std::min(p.napera, p.naperb) * p.wol) + 1;
    w->nprop = 2 * (int)std::floor(p.wol) + 1;
  } else if (p.boundtype == RG_BOUND_DIRICHLET) {
    if (std::fmod(p.wol, 0.5) == 0.0)
      return rg::fail(RG_ERR_INVALID_ARG,
                      "Invalid width wol, cannot be a half integer for 'dirichlet' boundary conditions.");
    w->nmu = (int)std::floor(2 * p.exfac * p.wol);
    w->imin = 1;
    w->imax = (int)std::floor(2 * p.naperb * p.wol);
    w->jmin = 1;
    w->jmax = (int)std::floor(2 * p.napera * p.wol);
    w->neigv = (int)std::floor(2 * std::min(p.napera, p.naperb) * p.wol);
    w->nprop = (int)std::floor(2 * p.wol);
  } else {
    return rg::fail(RG_ERR_INVALID_ARG, "Unknown boundary condition type.");
  }
  const int M = w->nmu;
  if (M < 1 || w->neigv < 1) return rg::fail(RG_ERR_INVALID_ARG, "Waveguide has no modes (wol too small).");
  w->ny = p.ny > 0 ? p.ny : M;
  const int ny = w->ny;
  w->ymesh.resize(ny);
  for (int i = 1; i <= ny; ++i) w->ymesh[i - 1] = (i - 0.5) / ny;
  w->kpmesh.resize(M);
  if (p.boundtype == RG_BOUND_PERIODIC)
    for (int n = 1; n <= M; ++n) w->kpmesh[n - 1] = (n - M / 2 - 1) / p.wol;
  else
    for (int n = 1; n <= M; ++n) w->kpmesh[n - 1] = 0.5 * n / p.wol;

  // mumesh, dos, bmat and the A diagonals: src/waveguide.f90:240-248,357-363.
  w->mumesh.resize(M);
  w->bmat.resize(M);
  w->aedge.resize(M);
  w->abulk.resize(M);
  w->sqmu_c.resize(M);
  w->sqmu_r.resize(M);
  double dos = 0.0;
  for (int n = 0; n < M; ++n) {
    const double kp = w->kpmesh[n];
    w->mumesh[n] = std::sqrt(cplx(1.0 - kp * kp, p.dabso / w->kl));
    dos += std::real(1.0 / std::sqrt(cplx(1.0 - kp * kp, 0.0)));
  }
  w->dos = dos / (p.wol * (2.0 * kPi) * (2.0 * kPi));
  const cplx iu(0.0, 1.0);
  for (int n = 0; n < M; ++n) {
    const cplx mu = w->mumesh[n];
    w->bmat[n] = mu / std::sin(mu * w->kdx);
    const cplx cot = mu / std::tan(mu * w->kdx);
    w->aedge[n] = iu * mu - cot;
    w->abulk[n] = -2.0 * cot;
    w->sqmu_c[n] = std::sqrt(mu);                              // src/waveguide.f90:443
    w->sqmu_r[n] = cplx(std::sqrt(std::real(mu)), 0.0);       // src/waveguide.f90:510
  }
  w->stdu = std::sqrt(p.dscat * ny / (2.0 * kPi * kPi * w->dos * p.wol * p.nxdiso));  // src/waveguide.f90:370

  // Projection tables.  Dirichlet modes chi_m(y) = sqrt(2/ny) sin(pi m y)
  // give (modal^T diag(U) modal)[a][c] = cc[|a-c|] - cc[a+c+2] with
  // cc[d] = sum_j U_j cos(pi d y_j) / ny; periodic modes exp(2 pi i k y)/sqrt(ny)
  // give the Hermitian Toeplitz f[c-a] with f[d] = sum_j U_j exp(2 pi i d y_j) / ny.
  if (p.boundtype == RG_BOUND_DIRICHLET) {
    const int nd = 2 * M + 1;
    w->costab.resize((size_t)ny * nd);
    for (int j = 0; j < ny; ++j)
      for (int d = 0; d < nd; ++d) w->costab[(size_t)j * nd + d] = std::cos(kPi * d * w->ymesh[j]) / ny;
  } else {
    w->expfac.resize((size_t)ny * M);
    for (int j = 0; j < ny; ++j)
      for (int d = 0; d < M; ++d)
        w->expfac[(size_t)j * M + d] = cplx(std::cos(2 * kPi * d * w->ymesh[j]), std::sin(2 * kPi * d * w->ymesh[j])) / (double)ny;
  }
  // Jump polynomials: column iy of the potential starts 2*nxdiso*iy draws in.
  w->jump.assign((size_t)ny * 4, 0);
  uint64_t step_poly[4], cur[4] = {1, 0, 0, 0};
  rg::jump_polynomial(2ULL * (uint64_t)p.nxdiso, step_poly);
  for (int iy = 0; iy < ny; ++iy) {
    std::memcpy(&w->jump[(size_t)iy * 4], cur, sizeof cur);
    rg::mulmod(cur, step_poly, cur);
  }
  return RG_OK;
}

int upload_tables(rg_waveguide* w) {
  RG_CUDA(cudaGetDevice(&w->device));
  RG_CUDA(cudaDeviceGetAttribute(&w->sm_count, cudaDevAttrMultiProcessorCount, w->device));
  RG_CUDA(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
  const size_t cb = sizeof(double2) * w->nmu;
  int rc;
  if ((rc = upload(&w->d_bmat, w->bmat.data(), cb))) return rc;
  if ((rc = upload(&w->d_aedge, w->aedge.data(), cb))) return rc;
  if ((rc = upload(&w->d_abulk, w->abulk.data(), cb))) return rc;
  if ((rc = upload(&w->d_sqmu_c, w->sqmu_c.data(), cb))) return rc;
  if ((rc = upload(&w->d_sqmu_r, w->sqmu_r.data(), cb))) return rc;
  if ((rc = upload(&w->d_costab, w->costab.data(), sizeof(double) * w->costab.size()))) return rc;
  if ((rc = upload(&w->d_expfac, w->expfac.data(), sizeof(double2) * w->expfac.size()))) return rc;
  if ((rc = upload(&w->d_jump, w->jump.data(), sizeof(uint64_t) * w->jump.size()))) return rc;
  RG_CUDA(cudaMalloc((void**)&w->d_counter, sizeof(int) * rg::kQueueCounters));
  rg::WgDesc d{};
  d.M = w->nmu;
  d.ny = w->ny;
  d.nx = w->nx;
  d.nxdiso = w->p.nxdiso;
  d.nxfree = w->p.nxfree;
  d.row0 = w->imin - 1;
  d.nrow = w->imax - w->imin + 1;
  d.col0 = w->jmin - 1;
  d.ncol = w->jmax - w->jmin + 1;
  d.neigv = w->neigv;
  d.periodic = w->p.boundtype == RG_BOUND_PERIODIC;
  d.stdu = w->stdu;
  d.bmat = w->d_bmat;
  d.adiag_edge = w->d_aedge;
  d.adiag_bulk = w->d_abulk;
  d.sqmu_c = w->d_sqmu_c;
  d.sqmu_r = w->d_sqmu_r;
  d.costab = w->d_costab;
  d.expfac = w->d_expfac;
  d.jumppoly = w->d_jump;
  w->h_desc = d;
  if ((rc = upload(&w->d_desc, &d, sizeof d))) return rc;
  RG_CUDA(cudaEventCreate(&w->ev_sweep0));
  RG_CUDA(cudaEventCreate(&w->ev_sweep1));
  return RG_OK;
}

int ensure_scratch(rg_waveguide* w, size_t bytes) {
  if (bytes <= w->scratch_bytes) return RG_OK;
  cudaFree(w->d_scratch);
  w->d_scratch = nullptr;
  w->scratch_bytes = 0;
  cudaError_t e = cudaMalloc(&w->d_scratch, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return rg::fail(RG_ERR_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed");
  }
  w->scratch_bytes = bytes;
  return RG_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// The symmetric sweep is on unless RG_SYMMETRIC=0; RG_SYM_TAU overrides its
// pivot threshold (a huge value sends every item to the pivoted kernel).
bool symmetric_enabled() {
  const char* e = std::getenv("RG_SYMMETRIC");
  return !(e && std::strcmp(e, "0") == 0);
}

double symmetric_tau() {
  const char* e = std::getenv("RG_SYM_TAU");
  if (!e || !*e) return rg::kSymTau;
  char* end = nullptr;
  const double t = std::strtod(e, &end);
  return (end && *end == '\0' && t >= 0.0) ? t : rg::kSymTau;
}

// The blocked symmetric sweep forms its propagator product on the tensor
// cores unless RG_TENSOR_R=0 (then B Gs1 rides through the Gauss-Jordan
// sweep in FP64 as before).
bool tensor_r_enabled() {
  const char* e = std::getenv("RG_TENSOR_R");
  return !(e && std::strcmp(e, "0") == 0);
}

// With the tensor-core product, the levels of the 2 x 2 block inverse of the
// slice matrix (each halves an even mode count of at least 128): 2 unless
// RG_SPLIT_INVERSE is 0 or 1.
int split_inverse_levels() {
  const char* e = std::getenv("RG_SPLIT_INVERSE");
  if (e && std::strcmp(e, "0") == 0) return 0;
  if (e && std::strcmp(e, "1") == 0) return 1;
  return 2;
}

// Launch arguments for items of this one waveguide (the caller sets nreal,
// seeds or upot, outputs and the workspace).
rg::SweepArgs make_args(const rg_waveguide* w, int mode) {
  rg::SweepArgs a{};
  a.mode = mode;
  a.wgs = w->d_desc;
  a.work_counter = w->d_counter;
  a.max_M = w->nmu;
  a.max_ny = w->ny;
  a.symmetric = (w->p.boundtype == RG_BOUND_DIRICHLET && symmetric_enabled()) ? 1 : 0;
  a.sym_tau = symmetric_tau();
  a.tensor_r = tensor_r_enabled() ? 1 : 0;
  a.split_inverse = split_inverse_levels();
  return a;
}

// Plans a launch, grows the scratch to hold `off` bytes plus the per-CTA
// workspace (and the flag list of a symmetric sweep), and sets a.work and
// a.flag_list.  Pointers into the scratch below `off` must be taken after
// this call (the scratch may move).
int place_workspace(rg_waveguide* w, rg::SweepArgs& a, size_t off, int* grid) {
  int64_t stride = 0;
  int rc = rg::sweep_plan(a, w->sm_count, grid, &stride);
  if (rc) return rc;
  const int slots = *grid / (a.cluster > 0 ? a.cluster : 1);  // one workspace per cluster
  const size_t ws = align256(sizeof(double2) * (size_t)stride * slots);
  const size_t fl = a.symmetric ? align256(sizeof(int32_t) * (size_t)a.nreal) : 0;
  if ((rc = ensure_scratch(w, off + ws + fl))) return rc;
  a.work = (double2*)((char*)w->d_scratch + off);
  a.work_stride = stride;
  a.flag_list = a.symmetric ? (int32_t*)((char*)w->d_scratch + off + ws) : nullptr;
  return RG_OK;
}

// ---------------------------------------------------------------------------
// Autotuner.  For a waveguide shape (M, ny) and a batch size, candidate launch
// configurations are timed once on a short proxy guide (the same modes and
// grid, 16 slices, the same number of realizations) and the fastest is
// cached for the process.  RG_AUTOTUNE=0 disables it (the built-in
// heuristics decide).  Only choices that leave every realization's result
// bit for bit the same are tuned:
//   * above 64 modes, the blocked kernel's cluster size (CTAs per
//     realization; it changes which CTA computes an element, not its
//     arithmetic), then, for the chosen cluster size, the threads per update
//     unit of the symmetric kernel (1, 4 or 8; it changes which thread
//     updates a row, not the row's operations);
//   * up to 64 modes, the persistent CTAs per SM of the shared-memory
//     kernels (each realization is one CTA's, whatever the grid).
// The kernel itself (symmetric for Dirichlet guides, pivoted shared-memory
// for periodic ones up to 64 modes, blocked above) and the panel width of the
// blocked elimination (8; another width regroups the rank updates and
// changes the rounding) are fixed, so a realization gives the same bits in a
// batch of any size and in a single call.
// ---------------------------------------------------------------------------
struct TuneChoice {
  int force_cluster = 0;
  int force_rowsplit = 0;
  int force_per_sm = 0;
};

struct TuneKey {
  int M, ny, bucket, sms;
  bool operator<(const TuneKey& o) const {
    return std::tie(M, ny, bucket, sms) < std::tie(o.M, o.ny, o.bucket, o.sms);
  }
};

std::mutex g_tune_mutex;
std::map<TuneKey, TuneChoice> g_tune_cache;

bool autotune_enabled() {
  const char* e = std::getenv("RG_AUTOTUNE");
  return !(e && std::strcmp(e, "0") == 0);
}

int size_bucket(int n) {
  int b = 1;
  while (b < n && b < (1 << 20)) b <<= 1;
  return b;
}

void apply_choice(rg::SweepArgs& a, const TuneChoice& tc) {
  a.force_cluster = tc.force_cluster;
  a.force_rowsplit = tc.force_rowsplit;
  a.force_per_sm = tc.force_per_sm;
}

// Times one configuration on the proxy (ms); large values mean "unusable".
// seg_end > 0 stops the (blocked-kernel) sweep after that many slices, before
// the Fisher-Lee and eigenvalue stage.  *grid_out receives the planned grid.
double time_candidate(rg_waveguide* w, const rg::WgDesc* d_proxy, int n, const int32_t* d_seeds, double* d_teig,
                      int32_t* d_status, const TuneChoice& tc, int seg_end, cudaStream_t s, int* grid_out = nullptr) {
  rg::SweepArgs a = make_args(w, rg::kModeEig);
  a.wgs = d_proxy;
  a.nreal = n;
  a.n_end = seg_end;
  a.seeds = d_seeds;
  a.teig = d_teig;
  a.status = d_status;
  apply_choice(a, tc);
  int grid = 0;
  int64_t stride = 0;
  if (rg::sweep_plan(a, w->sm_count, &grid, &stride) != RG_OK) return 1e30;
  if (grid_out) *grid_out = grid;
  const size_t need = align256(sizeof(double2) * (size_t)stride * (grid / (a.cluster > 0 ? a.cluster : 1)));
  double2* ws = nullptr;
  if (cudaMalloc((void**)&ws, need + sizeof(int32_t) * (size_t)n) != cudaSuccess) {
    cudaGetLastError();
    return 1e30;
  }
  a.work = ws;
  a.work_stride = stride;
  a.flag_list = a.symmetric ? (int32_t*)((char*)ws + need) : nullptr;
  double best = 1e30;
  for (int rep = 0; rep < 2; ++rep) {
    cudaMemsetAsync(w->d_counter, 0, sizeof(int) * rg::kQueueCounters, s);
    cudaEventRecord(w->ev_sweep0, s);
    if (rg::launch_sweep(a, s, grid) != RG_OK) break;
    cudaEventRecord(w->ev_sweep1, s);
    float ms = 0.0f;
    if (cudaEventSynchronize(w->ev_sweep1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, w->ev_sweep0, w->ev_sweep1) != cudaSuccess)
      break;
    if (rep > 0) best = ms;
  }
  cudaStreamSynchronize(s);
  cudaFree(ws);
  cudaGetLastError();
  return best;
}

TuneChoice autotune(rg_waveguide* w, int n, cudaStream_t s) {
  TuneChoice def;
  if (!autotune_enabled() || n <= 0) return def;
  const bool blocked = w->nmu > rg::kMaxModesSmem;
  const TuneKey key{w->nmu, w->ny, size_bucket(n), w->sm_count};
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) return it->second;
  }
  // Proxy: the same waveguide cut to 16 slices (all disordered).  The
  // blocked kernel stops before the eigenvalue stage (at the sizes that reach
  // it that stage is a negligible part of a real guide but would dominate 16
  // slices); the shared-memory kernels run whole guides.
  rg::WgDesc pd = w->h_desc;
  pd.nx = std::min(pd.nx, 16) + 1;
  pd.nxfree = 0;
  pd.nxdiso = pd.nx;
  const int seg_end = blocked ? pd.nx - 1 : 0;
  const int np = std::min(n, 4 * w->sm_count);
  char* buf = nullptr;
  const size_t b_desc = align256(sizeof pd), b_seed = align256(sizeof(int32_t) * np);
  const size_t b_teig = align256(sizeof(double) * (size_t)np * w->neigv);
  if (cudaMalloc((void**)&buf, b_desc + 2 * b_seed + b_teig) != cudaSuccess) {
    cudaGetLastError();
    return def;
  }
  rg::WgDesc* d_pd = (rg::WgDesc*)buf;
  int32_t* d_seeds = (int32_t*)(buf + b_desc);
  int32_t* d_status = (int32_t*)(buf + b_desc + b_seed);
  double* d_teig = (double*)(buf + b_desc + 2 * b_seed);
  std::vector<int32_t> seeds(np);
  for (int k = 0; k < np; ++k) seeds[k] = k + 1;
  cudaMemcpyAsync(d_pd, &pd, sizeof pd, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d_seeds, seeds.data(), sizeof(int32_t) * np, cudaMemcpyHostToDevice, s);
  TuneChoice best = def;
  double tbest = 1e30;
  auto consider = [&](const TuneChoice& c, int* grid_out = nullptr) {
    const double t = time_candidate(w, d_pd, np, d_seeds, d_teig, d_status, c, seg_end, s, grid_out);
    if (t < tbest) {
      tbest = t;
      best = c;
    }
  };
  if (blocked) {
    for (int c = 1; c <= 8; c *= 2) consider(TuneChoice{c, 0, 0});
    const int cbest = best.force_cluster;
    if (w->p.boundtype == RG_BOUND_DIRICHLET)  // the symmetric kernel's row split
      for (int t : {1, 4, 8}) consider(TuneChoice{cbest, t, 0});
  } else {
    // CTAs per SM: the occupancy limit, then fewer (distinct grids only)
    std::vector<int> grids;
    for (int k : {0, 1, 2, 4}) {
      int gk = 0;
      rg::SweepArgs a = make_args(w, rg::kModeEig);
      a.wgs = d_pd;
      a.nreal = np;
      a.force_per_sm = k;
      int64_t stride = 0;
      if (rg::sweep_plan(a, w->sm_count, &gk, &stride) != RG_OK) continue;
      if (std::find(grids.begin(), grids.end(), gk) != grids.end()) continue;
      grids.push_back(gk);
      consider(TuneChoice{0, 0, k});
    }
  }
  cudaStreamSynchronize(s);
  cudaFree(buf);
  cudaGetLastError();
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tune_cache[key] = best;
  return best;
}

// Seed-driven batch on device buffers: one persistent launch, the potential
// of every item drawn inside the kernel.  d_seeds, d_teig, d_status are
// device pointers.  CUDA events bracket the launch for rg_last_sweep_time.
// The launch (counter reset and kernel) is captured as a CUDA graph the
// first time a given argument set is seen and replayed afterwards.
int run_seed_batch(rg_waveguide* w, const int32_t* d_seeds, int n, double* d_teig, int32_t* d_status,
                   cudaStream_t s) {
  const TuneChoice tc = autotune(w, n, s);
  rg::SweepArgs a = make_args(w, rg::kModeEig);
  a.nreal = n;
  a.seeds = d_seeds;
  a.teig = d_teig;
  a.status = d_status;
  apply_choice(a, tc);
  int grid = 0, rc;
  if ((rc = place_workspace(w, a, 0, &grid))) return rc;
  int64_t tau_bits = 0;
  std::memcpy(&tau_bits, &a.sym_tau, sizeof tau_bits);
  const int64_t key[kGraphKey] = {n, (int64_t)(intptr_t)d_seeds, (int64_t)(intptr_t)d_teig,
                                  (int64_t)(intptr_t)d_status, (int64_t)(intptr_t)a.work, grid, a.cluster,
                                  a.force_large, a.work_stride, a.symmetric, (int64_t)(intptr_t)a.flag_list,
                                  tau_bits, a.force_rowsplit, a.force_per_sm, a.tensor_r * 4 + a.split_inverse};
  if (!w->graph || std::memcmp(key, w->graph_key, sizeof key) != 0) {
    if (w->graph) cudaGraphExecDestroy(w->graph);
    w->graph = nullptr;
    cudaGraph_t gr = nullptr;
    RG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemsetAsync(w->d_counter, 0, sizeof(int) * rg::kQueueCounters, s);
    rc = (e == cudaSuccess) ? rg::launch_sweep(a, s, grid) : rg::cuda_fail(e, "graph capture");
    const cudaError_t ec = cudaStreamEndCapture(s, &gr);
    if (rc) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    RG_CUDA(ec);
    e = cudaGraphInstantiate(&w->graph, gr, 0);
    cudaGraphDestroy(gr);
    RG_CUDA(e);
    std::memcpy(w->graph_key, key, sizeof key);
  }
  // Timing events bracket the graph launch (events inside a graph cannot be timed).
  RG_CUDA(cudaEventRecord(w->ev_sweep0, s));
  RG_CUDA(cudaGraphLaunch(w->graph, s));
  RG_CUDA(cudaEventRecord(w->ev_sweep1, s));
  w->sweep_timed = true;
  const bool blocked = a.force_large || a.max_M > rg::kMaxModesSmem;
  w->last_batch.kernel = blocked ? (a.symmetric ? RG_KERNEL_BLOCKED_SYMMETRIC : RG_KERNEL_BLOCKED)
                                 : (a.symmetric ? RG_KERNEL_SYMMETRIC : RG_KERNEL_PIVOTED);
  w->last_batch.grid = grid;
  w->last_batch.cluster = a.cluster > 0 ? a.cluster : 1;
  w->last_batch.rerun = 0;
  return RG_OK;
}

int first_bad_status(const int32_t* st, int n) {
  for (int k = 0; k < n; ++k)
    if (st[k] != RG_OK) return st[k];
  return RG_OK;
}

// Single realization with either a seed or a host potential.  mode selects
// the eigenvalue path (tdistrib) or the v1 path (full t; and r when h_r is
// given: a second sweep over the slices in reverse order, whose last Gss is
// G(x_1; x_1)).  The seed's potential is drawn inside the kernel, except for
// r, whose reverse sweep needs the rows in reverse order: then it is drawn
// into scratch first.  Scratch layout: [potential | t | r | eigenvalues |
// status | seed | per-CTA workspace | flag list].
int run_single(rg_waveguide* w, const int32_t* seed, const double* h_upot, int mode, double* h_teig,
               double* h_t, double* h_tfilt, double* h_r = nullptr) {
  DeviceGuard g(w->device);
  const int M = w->nmu;
  const bool want_r = (h_r != nullptr);
  const bool materialize = !seed || want_r;
  const size_t pot = materialize ? sizeof(double) * (size_t)w->p.nxdiso * w->ny : 0;
  const int nrow = mode == rg::kModeEig ? w->imax - w->imin + 1 : M;
  const int ncol = mode == rg::kModeEig ? w->jmax - w->jmin + 1 : M;
  const size_t tbytes = sizeof(double2) * (size_t)nrow * ncol;
  const size_t rbytes = want_r ? sizeof(double2) * (size_t)M * M : 0;
  const size_t off_t = align256(pot), off_r = off_t + align256(tbytes), off_e = off_r + align256(rbytes);
  const size_t off_s = off_e + align256(sizeof(double) * w->neigv), off_seed = off_s + 256;
  const size_t off_ws = off_seed + 256;
  rg::SweepArgs a = make_args(w, mode);
  a.nreal = 1;
  int grid = 1, rc;
  if ((rc = place_workspace(w, a, off_ws, &grid))) return rc;
  char* base = (char*)w->d_scratch;
  double* d_pot = (double*)base;
  double2* d_t = (double2*)(base + off_t);
  double2* d_r = (double2*)(base + off_r);
  double* d_teig = (double*)(base + off_e);
  int32_t* d_status = (int32_t*)(base + off_s);
  int32_t* d_seed = (int32_t*)(base + off_seed);
  cudaStream_t s = w->stream;
  if (seed) RG_CUDA(cudaMemcpyAsync(d_seed, seed, sizeof(int32_t), cudaMemcpyHostToDevice, s));
  if (!materialize) {
    a.seeds = d_seed;
  } else if (seed) {
    rg::PotArgs pa{};
    pa.nxdiso = w->p.nxdiso;
    pa.ny = w->ny;
    pa.nreal = 1;
    pa.stdu = w->stdu;
    pa.seeds = d_seed;
    pa.jumppoly = w->d_jump;
    pa.upot = d_pot;
    if ((rc = rg::launch_potential(pa, s))) return rc;
    a.upot = d_pot;
    a.pot_xstride = w->ny;
    a.pot_ystride = 1;
  } else {
    // caller layout upot(nxdiso, ny), x fastest
    RG_CUDA(cudaMemcpyAsync(d_pot, h_upot, pot, cudaMemcpyHostToDevice, s));
    a.upot = d_pot;
    a.pot_xstride = 1;
    a.pot_ystride = w->p.nxdiso;
  }
  a.pot_rstride = 0;
  a.tout = (h_t || h_tfilt) ? d_t : nullptr;
  a.teig = d_teig;
  a.status = d_status;
  RG_CUDA(cudaMemsetAsync(w->d_counter, 0, sizeof(int) * rg::kQueueCounters, s));
  if ((rc = rg::launch_sweep(a, s, grid))) return rc;
  if (want_r) {
    rg::SweepArgs b = a;
    b.mode = rg::kModeRefl;
    b.tout = d_r;
    b.status = d_status + 1;
    RG_CUDA(cudaMemsetAsync(w->d_counter, 0, sizeof(int) * rg::kQueueCounters, s));
    if ((rc = rg::launch_sweep(b, s, grid))) return rc;
  }
  int32_t st[2] = {0, 0};
  RG_CUDA(cudaMemcpyAsync(st, d_status, sizeof(int32_t) * (want_r ? 2 : 1), cudaMemcpyDeviceToHost, s));
  if (h_teig) RG_CUDA(cudaMemcpyAsync(h_teig, d_teig, sizeof(double) * w->neigv, cudaMemcpyDeviceToHost, s));
  if (h_t) RG_CUDA(cudaMemcpyAsync(h_t, d_t, tbytes, cudaMemcpyDeviceToHost, s));
  if (h_tfilt) RG_CUDA(cudaMemcpyAsync(h_tfilt, d_t, tbytes, cudaMemcpyDeviceToHost, s));
  if (h_r) RG_CUDA(cudaMemcpyAsync(h_r, d_r, rbytes, cudaMemcpyDeviceToHost, s));
  RG_CUDA(cudaStreamSynchronize(s));
  const int bad = st[0] != RG_OK ? st[0] : st[1];
  if (bad != RG_OK) return rg::fail(bad, status_text(bad));
  return RG_OK;
}

}  // namespace

namespace rg {

int noalloc_view(const rg_waveguide* w, NoAllocView* out) {
  if (!w || !out) return fail(RG_ERR_INVALID_ARG, "noalloc_view: NULL argument");
  out->device = w->device;
  out->sm_count = w->sm_count;
  out->nxdiso = w->p.nxdiso;
  out->ny = w->ny;
  out->nmu = w->nmu;
  out->stdu = w->stdu;
  out->jumppoly = w->d_jump;
  out->stream = w->stream;
  out->d_desc = w->d_desc;
  const SweepArgs a = make_args(w, kModeEig);
  out->symmetric = a.symmetric;
  out->sym_tau = a.sym_tau;
  return RG_OK;
}

int green_view(const rg_waveguide* w, GreenView* out) {
  if (!w || !out) return fail(RG_ERR_INVALID_ARG, "green_view: NULL argument");
  out->device = w->device;
  out->sm_count = w->sm_count;
  out->stream = w->stream;
  out->d_desc = w->d_desc;
  out->desc = w->h_desc;
  out->d_counter = w->d_counter;
  out->nxdiso = w->p.nxdiso;
  out->nxfree = w->p.nxfree;
  out->nx = w->nx;
  out->ny = w->ny;
  out->nmu = w->nmu;
  out->neigv = w->neigv;
  out->periodic = w->p.boundtype == RG_BOUND_PERIODIC;
  out->imin = w->imin;
  out->imax = w->imax;
  out->jmin = w->jmin;
  out->jmax = w->jmax;
  out->wol = w->p.wol;
  out->stdu = w->stdu;
  out->xmesh = w->xmesh.data();
  out->ymesh = w->ymesh.data();
  out->kpmesh = w->kpmesh.data();
  out->sqmu_r = w->sqmu_r.data();
  const SweepArgs a = make_args(w, kModeEig);
  out->symmetric = a.symmetric;
  out->sym_tau = a.sym_tau;
  out->tensor_r = a.tensor_r;
  out->split_inverse = a.split_inverse;
  return RG_OK;
}

}  // namespace rg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* rg_last_error(void) { return rg::g_last_error.c_str(); }

int rg_init(const rg_params* params, rg_waveguide** out) {
  if (!params || !out) return rg::fail(RG_ERR_INVALID_ARG, "rg_init: NULL argument");
  *out = nullptr;
  if (rg::rng_selfcheck() != 0) return rg::fail(RG_ERR_INVALID_ARG, "xoshiro256 jump-ahead self-check failed");
  rg_waveguide* w = new (std::nothrow) rg_waveguide();
  if (!w) return rg::fail(RG_ERR_NOMEM, "rg_init: out of host memory");
  int rc = build_tables(w, *params);
  if (!rc) rc = upload_tables(w);
  if (rc) {
    free_device(w);
    delete w;
    return rc;
  }
  *out = w;
  return RG_OK;
}

int rg_init_copy(const rg_waveguide* src, rg_waveguide** out) {
  if (!src) return rg::fail(RG_ERR_INVALID_ARG, "rg_init_copy: NULL source");
  DeviceGuard g(src->device);
  return rg_init(&src->p, out);
}

void rg_del(rg_waveguide* w) {
  if (!w) return;
  {
    DeviceGuard g(w->device);
    if (w->stream) cudaStreamSynchronize(w->stream);
    free_device(w);
  }
  delete w;
}

int rg_get_nmu(const rg_waveguide* w) { return w ? w->nmu : -1; }
int rg_get_neigv(const rg_waveguide* w) { return w ? w->neigv : -1; }
int rg_get_nx(const rg_waveguide* w) { return w ? w->nx : -1; }
int rg_get_ny(const rg_waveguide* w) { return w ? w->ny : -1; }
int rg_get_nprop(const rg_waveguide* w) { return w ? w->nprop : -1; }

int rg_get_window(const rg_waveguide* w, int* imin, int* imax, int* jmin, int* jmax) {
  if (!w || !imin || !imax || !jmin || !jmax) return rg::fail(RG_ERR_INVALID_ARG, "rg_get_window: NULL argument");
  *imin = w->imin;
  *imax = w->imax;
  *jmin = w->jmin;
  *jmax = w->jmax;
  return RG_OK;
}

int rg_get_xmesh(const rg_waveguide* w, double* xmesh, int64_t len) {
  if (!w || !xmesh) return rg::fail(RG_ERR_INVALID_ARG, "rg_get_xmesh: NULL argument");
  if (len != w->nx) return rg::fail(RG_ERR_INVALID_ARG, "rg_get_xmesh: length must equal nx");
  std::memcpy(xmesh, w->xmesh.data(), sizeof(double) * w->nx);
  return RG_OK;
}

int rg_get_parameters(const rg_waveguide* w, rg_params* out) {
  if (!w || !out) return rg::fail(RG_ERR_INVALID_ARG, "rg_get_parameters: NULL argument");
  *out = w->p;
  return RG_OK;
}

int rg_get_scalars(const rg_waveguide* w, double* kdx, double* dos, double* stdu) {
  if (!w) return rg::fail(RG_ERR_INVALID_ARG, "rg_get_scalars: NULL handle");
  if (kdx) *kdx = w->kdx;
  if (dos) *dos = w->dos;
  if (stdu) *stdu = w->stdu;
  return RG_OK;
}

int rg_get_modes(const rg_waveguide* w, double* mumesh, double* bmat) {
  if (!w) return rg::fail(RG_ERR_INVALID_ARG, "rg_get_modes: NULL handle");
  if (mumesh) std::memcpy(mumesh, w->mumesh.data(), sizeof(cplx) * w->nmu);
  if (bmat) std::memcpy(bmat, w->bmat.data(), sizeof(cplx) * w->nmu);
  return RG_OK;
}

int rg_compute_tdistrib(rg_waveguide* w, int iseed, double* tallvals, int64_t len) {
  rg::NvtxRange nvtx_range("rg_compute_tdistrib");
  if (!w || !tallvals) return rg::fail(RG_ERR_INVALID_ARG, "rg_compute_tdistrib: NULL argument");
  // Chunk checks of src/waveguide.f90:408-421.
  const int64_t nchunk = len / w->neigv;
  if (nchunk == 0)
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid eigenvalue array length, received " + std::to_string(len) +
                                            ", expected at least " + std::to_string(w->neigv) + "...");
  if (nchunk * w->neigv != len)
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid eigenvalue array length, received " + std::to_string(len) +
                                            ", expected " + std::to_string(nchunk * w->neigv) + "...");
  if (iseed < 1 || nchunk < iseed)
    return rg::fail(RG_ERR_INVALID_ARG, "Invalid chunk index, received " + std::to_string(iseed) +
                                            ", expected in [1, " + std::to_string(nchunk) + "]...");
  const int32_t s = iseed;
  return run_single(w, &s, nullptr, rg::kModeEig, tallvals + (iseed - 1) * (int64_t)w->neigv, nullptr, nullptr);
}

int rg_refl_trans_v1_batch(rg_waveguide* w, const int32_t* seeds, int n, double* rmat, double* tmat,
                           int32_t* status) {
  rg::NvtxRange nvtx_range("rg_refl_trans_v1_batch");
  if (!w || n < 0 || (n > 0 && (!seeds || !tmat)))
    return rg::fail(RG_ERR_INVALID_ARG, "rg_refl_trans_v1_batch: invalid argument");
  if (n == 0) return RG_OK;
  DeviceGuard g(w->device);
  const int M = w->nmu;
  const size_t mm = (size_t)M * M;
  const size_t pot_per = (size_t)w->p.nxdiso * w->ny;
  const bool want_r = rmat != nullptr;
  // Realizations per launch: their potentials (drawn first, so that r's
  // reverse sweep can read the rows backwards) and t, r within ~1 GiB.
  const size_t per_item = sizeof(double) * pot_per + sizeof(double2) * mm * (want_r ? 2 : 1);
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)n, ((size_t)1 << 30) / per_item));
  const size_t b_seed = align256(sizeof(int32_t) * chunk), b_st = align256(sizeof(int32_t) * 2 * chunk);
  const size_t b_pot = align256(sizeof(double) * pot_per * chunk), b_mat = align256(sizeof(double2) * mm * chunk);
  char* buf = nullptr;
  RG_CUDA(cudaMalloc((void**)&buf, b_seed + b_st + b_pot + b_mat * (want_r ? 2 : 1)));
  int32_t* d_seed = (int32_t*)buf;
  int32_t* d_st = (int32_t*)(buf + b_seed);
  double* d_pot = (double*)(buf + b_seed + b_st);
  double2* d_t = (double2*)(buf + b_seed + b_st + b_pot);
  double2* d_r = want_r ? (double2*)(buf + b_seed + b_st + b_pot + b_mat) : nullptr;
  std::vector<int32_t> st(2 * (size_t)chunk);
  cudaStream_t s = w->stream;
  int rc = RG_OK, bad = RG_OK;
  for (int k0 = 0; !rc && k0 < n; k0 += chunk) {
    const int nk = std::min(chunk, n - k0);
    cudaError_t e = cudaMemcpyAsync(d_seed, seeds + k0, sizeof(int32_t) * nk, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      rc = rg::cuda_fail(e, "rg_refl_trans_v1_batch seeds");
      break;
    }
    rg::PotArgs pa{};
    pa.nxdiso = w->p.nxdiso;
    pa.ny = w->ny;
    pa.nreal = nk;
    pa.stdu = w->stdu;
    pa.seeds = d_seed;
    pa.jumppoly = w->d_jump;
    pa.upot = d_pot;
    if ((rc = rg::launch_potential(pa, s))) break;
    for (int pass = 0; pass < (want_r ? 2 : 1) && !rc; ++pass) {
      rg::SweepArgs a = make_args(w, pass == 0 ? rg::kModeTmat : rg::kModeRefl);
      a.nreal = nk;
      a.upot = d_pot;
      a.pot_rstride = (int64_t)pot_per;
      a.pot_xstride = w->ny;
      a.pot_ystride = 1;
      a.tout = pass == 0 ? d_t : d_r;
      a.status = d_st + (size_t)pass * chunk;
      int grid = 0;
      if ((rc = place_workspace(w, a, 0, &grid))) break;
      e = cudaMemsetAsync(w->d_counter, 0, sizeof(int) * rg::kQueueCounters, s);
      if (e != cudaSuccess) {
        rc = rg::cuda_fail(e, "rg_refl_trans_v1_batch counter");
        break;
      }
      rc = rg::launch_sweep(a, s, grid);
    }
    if (rc) break;
    e = cudaMemcpyAsync(tmat + 2 * mm * (size_t)k0, d_t, sizeof(double2) * mm * nk, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && want_r)
      e = cudaMemcpyAsync(rmat + 2 * mm * (size_t)k0, d_r, sizeof(double2) * mm * nk, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st.data(), d_st, sizeof(int32_t) * 2 * chunk, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      rc = rg::cuda_fail(e, "rg_refl_trans_v1_batch");
      break;
    }
    for (int k = 0; k < nk; ++k) {
      const int sk = st[k] != RG_OK ? st[k] : (want_r ? st[(size_t)chunk + k] : RG_OK);
      if (status) status[k0 + k] = sk;
      if (!bad && sk != RG_OK) bad = sk;
    }
  }
  cudaStreamSynchronize(s);
  cudaFree(buf);
  if (rc) return rc;
  if (bad) return rg::fail(bad, status_text(bad));
  return RG_OK;
}

int rg_tdistrib_upot(rg_waveguide* w, const double* upot, double* teigvals, double* tfilt) {
  if (!w || !upot || !teigvals) return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_upot: NULL argument");
  return run_single(w, nullptr, upot, rg::kModeEig, teigvals, nullptr, tfilt);
}

int rg_compute_refl_trans_v1(rg_waveguide* w, int iseed, double* rmat, double* tmat) {
  rg::NvtxRange nvtx_range("rg_compute_refl_trans_v1");
  if (!w || !tmat) return rg::fail(RG_ERR_INVALID_ARG, "rg_compute_refl_trans_v1: NULL argument");
  const int32_t s = iseed;
  return run_single(w, &s, nullptr, rg::kModeTmat, nullptr, tmat, nullptr, rmat);
}

int rg_refl_trans_v1_upot(rg_waveguide* w, const double* upot, double* rmat, double* tmat) {
  if (!w || !upot || !tmat) return rg::fail(RG_ERR_INVALID_ARG, "rg_refl_trans_v1_upot: NULL argument");
  return run_single(w, nullptr, upot, rg::kModeTmat, nullptr, tmat, nullptr, rmat);
}

int rg_potential(rg_waveguide* w, int iseed, double* upot) {
  if (!w || !upot) return rg::fail(RG_ERR_INVALID_ARG, "rg_potential: NULL argument");
  DeviceGuard g(w->device);
  const size_t n = (size_t)w->p.nxdiso * w->ny;
  int rc = ensure_scratch(w, align256(sizeof(double) * n) + 256);
  if (rc) return rc;
  double* d_pot = (double*)w->d_scratch;
  int32_t* d_seed = (int32_t*)((char*)w->d_scratch + align256(sizeof(double) * n));
  const int32_t s = iseed;
  RG_CUDA(cudaMemcpyAsync(d_seed, &s, sizeof s, cudaMemcpyHostToDevice, w->stream));
  rg::PotArgs pa{};
  pa.nxdiso = w->p.nxdiso;
  pa.ny = w->ny;
  pa.nreal = 1;
  pa.stdu = w->stdu;
  pa.seeds = d_seed;
  pa.jumppoly = w->d_jump;
  pa.upot = d_pot;
  if ((rc = rg::launch_potential(pa, w->stream))) return rc;
  std::vector<double> tmp(n);
  RG_CUDA(cudaMemcpyAsync(tmp.data(), d_pot, sizeof(double) * n, cudaMemcpyDeviceToHost, w->stream));
  RG_CUDA(cudaStreamSynchronize(w->stream));
  const int nxd = w->p.nxdiso, ny = w->ny;
  for (int ix = 0; ix < nxd; ++ix)
    for (int iy = 0; iy < ny; ++iy) upot[ix + (size_t)nxd * iy] = tmp[(size_t)ix * ny + iy];
  return RG_OK;
}

int rg_tdistrib_batch_device(rg_waveguide* w, const int32_t* d_seeds, int n, double* d_tallvals, int32_t* d_status,
                             void* stream) {
  rg::NvtxRange nvtx_range("rg_tdistrib_batch_device");
  if (!w || !d_seeds || !d_tallvals || !d_status || n < 0)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_batch_device: invalid argument");
  DeviceGuard g(w->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : w->stream;
  int rc = run_seed_batch(w, d_seeds, n, d_tallvals, d_status, s);
  if (rc) return rc;
  RG_CUDA(cudaStreamSynchronize(s));
  return RG_OK;
}

int rg_tdistrib_batch(rg_waveguide* w, const int32_t* seeds, int n, double* tallvals, int32_t* status) {
  rg::NvtxRange nvtx_range("rg_tdistrib_batch");
  if (!w || (n > 0 && (!seeds || !tallvals)) || n < 0)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_batch: invalid argument");
  if (n == 0) return RG_OK;
  DeviceGuard g(w->device);
  int32_t* d_seeds = nullptr;
  int32_t* d_status = nullptr;
  double* d_out = nullptr;
  const size_t ob = sizeof(double) * (size_t)n * w->neigv;
  RG_CUDA(cudaMalloc((void**)&d_seeds, sizeof(int32_t) * n));
  cudaError_t e1 = cudaMalloc((void**)&d_status, sizeof(int32_t) * n);
  cudaError_t e2 = cudaMalloc((void**)&d_out, ob);
  int rc = RG_OK;
  std::vector<int32_t> st_host;
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    cudaGetLastError();
    rc = rg::fail(RG_ERR_NOMEM, "rg_tdistrib_batch: device allocation failed");
  }
  cudaStream_t s = w->stream;
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(d_seeds, seeds, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) rc = rg::cuda_fail(e, "copy seeds");
  }
  if (!rc) rc = run_seed_batch(w, d_seeds, n, d_out, d_status, s);
  if (!rc) {
    st_host.resize(n);
    cudaError_t e = cudaMemcpyAsync(tallvals, d_out, ob, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st_host.data(), d_status, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = rg::cuda_fail(e, "rg_tdistrib_batch");
  }
  cudaFree(d_seeds);
  cudaFree(d_status);
  cudaFree(d_out);
  if (rc) return rc;
  if (status) std::memcpy(status, st_host.data(), sizeof(int32_t) * n);
  const int bad = first_bad_status(st_host.data(), n);
  if (bad) return rg::fail(bad, status_text(bad));
  return RG_OK;
}

int rg_tdistrib_multi(rg_waveguide* const* wgs, const int32_t* seeds, int n, const int64_t* offsets,
                      double* tallvals, int64_t len, int32_t* status) {
  rg::NvtxRange nvtx_range("rg_tdistrib_multi");
  if (n < 0 || (n > 0 && (!wgs || !seeds || !offsets || !tallvals)))
    return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_multi: invalid argument");
  if (n == 0) return RG_OK;
  rg_waveguide* w0 = wgs[0];
  if (!w0) return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_multi: NULL waveguide");
  // Distinct waveguides, output ranges, and kernel classes.
  std::vector<rg::WgDesc> descs;
  std::vector<const rg_waveguide*> uniq;
  std::vector<int32_t> item_wg(n);
  for (int k = 0; k < n; ++k) {
    const rg_waveguide* w = wgs[k];
    if (!w) return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_multi: NULL waveguide");
    if (w->device != w0->device) return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_multi: waveguides on different devices");
    if (offsets[k] < 0 || offsets[k] + w->neigv > len)
      return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_multi: output range of item " + std::to_string(k) +
                                              " outside tallvals");
    size_t u = 0;
    while (u < uniq.size() && uniq[u] != w) ++u;
    if (u == uniq.size()) {
      uniq.push_back(w);
      descs.push_back(w->h_desc);
    }
    item_wg[k] = (int32_t)u;
  }
  auto klass = [](int M) { return M <= 16 ? 0 : M <= 32 ? 1 : M <= rg::kMaxModesSmem ? 2 : 3; };
  // Order: by class (largest first), then by decreasing cost M^3 * nx inside a class.
  std::vector<int> order(n);
  for (int k = 0; k < n; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const rg::WgDesc& a = descs[item_wg[x]];
    const rg::WgDesc& b = descs[item_wg[y]];
    if (klass(a.M) != klass(b.M)) return klass(a.M) > klass(b.M);
    return (double)a.M * a.M * a.M * a.nx > (double)b.M * b.M * b.M * b.nx;
  });
  std::vector<int32_t> o_wg(n), o_seed(n);
  std::vector<int64_t> o_off(n);
  for (int k = 0; k < n; ++k) {
    o_wg[k] = item_wg[order[k]];
    o_seed[k] = seeds[order[k]];
    o_off[k] = offsets[order[k]];
  }
  DeviceGuard g(w0->device);
  cudaStream_t s = w0->stream;
  // Device buffers, kept on w0 for the next call (grow-only): descriptors,
  // item waveguides, seeds, statuses, output offsets, outputs, and the queue
  // counters of each class.
  const size_t b_desc = align256(sizeof(rg::WgDesc) * descs.size()), b_i32 = align256(sizeof(int32_t) * n);
  const size_t b_off = align256(sizeof(int64_t) * n), b_out = align256(sizeof(double) * (size_t)len);
  const size_t b_cnt = align256(sizeof(int) * rg::kQueueCounters * rg_waveguide::kMultiClasses);
  const size_t need = b_desc + 3 * b_i32 + b_off + b_out + b_cnt;
  if (need > w0->multi_bytes) {
    if (w0->multi_graph) cudaGraphExecDestroy(w0->multi_graph);
    w0->multi_graph = nullptr;
    w0->multi_key.clear();
    cudaFree(w0->d_multi);
    w0->d_multi = nullptr;
    w0->multi_bytes = 0;
    cudaError_t e = cudaMalloc(&w0->d_multi, need);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return rg::fail(RG_ERR_NOMEM, "rg_tdistrib_multi: device allocation of " + std::to_string(need) + " bytes failed");
    }
    w0->multi_bytes = need;
  }
  char* dbuf = (char*)w0->d_multi;
  rg::WgDesc* d_desc = (rg::WgDesc*)dbuf;
  int32_t* d_wg = (int32_t*)(dbuf + b_desc);
  int32_t* d_seed = (int32_t*)(dbuf + b_desc + b_i32);
  int32_t* d_st = (int32_t*)(dbuf + b_desc + 2 * b_i32);
  int64_t* d_off = (int64_t*)(dbuf + b_desc + 3 * b_i32);
  double* d_out = (double*)(dbuf + b_desc + 3 * b_i32 + b_off);
  int* d_cnt = (int*)(dbuf + b_desc + 3 * b_i32 + b_off + b_out);

  // One persistent launch per kernel class, each with its own workspace and
  // queue counters, so that the classes can run side by side.
  struct Cls {
    rg::SweepArgs a;
    int grid;
    size_t ws_off, ws_bytes;
  };
  std::vector<Cls> cls;
  size_t total_ws = 0;
  int rc = RG_OK;
  for (int k0 = 0; k0 < n;) {
    const int cl = klass(descs[o_wg[k0]].M);
    int k1 = k0, maxM = 0, maxny = 0;
    while (k1 < n && klass(descs[o_wg[k1]].M) == cl) {
      maxM = std::max(maxM, descs[o_wg[k1]].M);
      maxny = std::max(maxny, descs[o_wg[k1]].ny);
      ++k1;
    }
    rg::SweepArgs a{};
    a.mode = rg::kModeEig;
    a.nreal = k1 - k0;
    a.wgs = d_desc;
    a.item_wg = d_wg + k0;
    a.seeds = d_seed + k0;
    a.teig_off = d_off + k0;
    a.teig = d_out;
    a.status = d_st + k0;
    a.work_counter = d_cnt + cls.size() * rg::kQueueCounters;
    a.max_M = maxM;
    a.max_ny = maxny;
    // The symmetric kernel when the class has Dirichlet items (it hands
    // periodic ones straight to the pivoted kernel).
    bool any_dirichlet = false;
    for (int k = k0; k < k1; ++k) any_dirichlet = any_dirichlet || !descs[o_wg[k]].periodic;
    a.symmetric = (any_dirichlet && symmetric_enabled()) ? 1 : 0;
    a.sym_tau = symmetric_tau();
    a.tensor_r = tensor_r_enabled() ? 1 : 0;
    a.split_inverse = split_inverse_levels();
    if (maxM > rg::kMaxModesSmem) {
      // The blocked class's makespan is at least its longest item's time on
      // one CTA slot.  When that item's work times the slot count exceeds the
      // class's total work, spread every item over a cluster (the items are
      // ordered longest first, so the long ones start at once).
      double total = 0.0, longest = 0.0;
      for (int k = k0; k < k1; ++k) {
        const rg::WgDesc& d = descs[o_wg[k]];
        const double wk = (double)d.M * d.M * d.M * d.nx;
        total += wk;
        longest = std::max(longest, wk);
      }
      const double slots = 2.0 * w0->sm_count;  // two CTAs per SM
      int C = 1;
      while (C < 8 && longest * slots / C > total) C *= 2;
      a.force_cluster = C > 1 ? C : 0;
    }
    Cls c{a, 0, 0, 0};
    int64_t stride = 0;
    if ((rc = rg::sweep_plan(c.a, w0->sm_count, &c.grid, &stride))) return rc;
    c.a.work_stride = stride;
    const size_t ws = align256(sizeof(double2) * (size_t)stride * (c.grid / (c.a.cluster > 0 ? c.a.cluster : 1)));
    const size_t fl = c.a.symmetric ? align256(sizeof(int32_t) * (size_t)c.a.nreal) : 0;
    c.ws_off = total_ws;
    c.ws_bytes = ws;
    total_ws += ws + fl;
    cls.push_back(c);
    k0 = k1;
  }
  if ((rc = ensure_scratch(w0, total_ws))) return rc;
  for (Cls& c : cls) {
    c.a.work = (double2*)((char*)w0->d_scratch + c.ws_off);
    c.a.flag_list = c.a.symmetric ? (int32_t*)((char*)w0->d_scratch + c.ws_off + c.ws_bytes) : nullptr;
  }
  // Inputs for this call (outside the graph, which reads them from the buffers).
  cudaError_t e = cudaMemcpyAsync(d_desc, descs.data(), sizeof(rg::WgDesc) * descs.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_wg, o_wg.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_seed, o_seed.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_off, o_off.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_out, 0, sizeof(double) * (size_t)len, s);
  if (e != cudaSuccess) return rg::cuda_fail(e, "rg_tdistrib_multi upload");
  // The graph: counters reset, then every class on its own stream.
  std::vector<int64_t> key = {n, len, (int64_t)(intptr_t)w0->d_multi, (int64_t)(intptr_t)w0->d_scratch,
                              (int64_t)descs.size(), (int64_t)cls.size()};
  for (const Cls& c : cls) {
    int64_t tau_bits = 0;
    std::memcpy(&tau_bits, &c.a.sym_tau, sizeof tau_bits);
    const int64_t k[] = {(int64_t)(c.a.item_wg - d_wg), c.a.nreal, c.a.max_M, c.a.max_ny, c.a.symmetric,
                         c.a.tensor_r * 4 + c.a.split_inverse, c.a.force_cluster, c.a.cluster, c.grid, (int64_t)c.ws_off, c.a.work_stride,
                         tau_bits};
    key.insert(key.end(), std::begin(k), std::end(k));
  }
  if (!w0->multi_graph || key != w0->multi_key) {
    if (w0->multi_graph) cudaGraphExecDestroy(w0->multi_graph);
    w0->multi_graph = nullptr;
    w0->multi_key.clear();
    if (!w0->multi_fork) RG_CUDA(cudaEventCreateWithFlags(&w0->multi_fork, cudaEventDisableTiming));
    for (size_t c = 0; c < cls.size(); ++c) {
      if (!w0->multi_streams[c]) RG_CUDA(cudaStreamCreateWithFlags(&w0->multi_streams[c], cudaStreamNonBlocking));
      if (!w0->multi_join[c]) RG_CUDA(cudaEventCreateWithFlags(&w0->multi_join[c], cudaEventDisableTiming));
    }
    cudaGraph_t gr = nullptr;
    RG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    e = cudaMemsetAsync(d_cnt, 0, b_cnt, s);
    if (e == cudaSuccess) e = cudaEventRecord(w0->multi_fork, s);
    if (e != cudaSuccess) rc = rg::cuda_fail(e, "rg_tdistrib_multi capture");
    for (size_t c = 0; !rc && c < cls.size(); ++c) {
      cudaStream_t sc = w0->multi_streams[c];
      e = cudaStreamWaitEvent(sc, w0->multi_fork, 0);
      if (e != cudaSuccess) {
        rc = rg::cuda_fail(e, "rg_tdistrib_multi capture");
        break;
      }
      if ((rc = rg::launch_sweep(cls[c].a, sc, cls[c].grid))) break;
      e = cudaEventRecord(w0->multi_join[c], sc);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, w0->multi_join[c], 0);
      if (e != cudaSuccess) rc = rg::cuda_fail(e, "rg_tdistrib_multi capture");
    }
    const cudaError_t ec = cudaStreamEndCapture(s, &gr);
    if (rc) {
      if (gr) cudaGraphDestroy(gr);
      return rc;
    }
    RG_CUDA(ec);
    e = cudaGraphInstantiate(&w0->multi_graph, gr, 0);
    cudaGraphDestroy(gr);
    RG_CUDA(e);
    w0->multi_key = key;
    w0->multi_replays = 0;
  } else {
    ++w0->multi_replays;
  }
  std::vector<int32_t> st_sorted(n);
  e = cudaGraphLaunch(w0->multi_graph, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tallvals, d_out, sizeof(double) * (size_t)len, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(st_sorted.data(), d_st, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return rg::cuda_fail(e, "rg_tdistrib_multi");
  int bad = RG_OK;
  for (int k = 0; k < n; ++k) {
    if (status) status[order[k]] = st_sorted[k];
    if (!bad && st_sorted[k] != RG_OK) bad = st_sorted[k];
  }
  if (bad) return rg::fail(bad, status_text(bad));
  return RG_OK;
}

int rg_sweep_segment(rg_waveguide* w, const double* d_upot, int n, int n_begin, int n_end, const double* d_state_in,
                     double* d_state_dump, double* d_state_out, double* d_tfilt, double* d_teig, int32_t* d_status,
                     void* stream) {
  rg::NvtxRange nvtx_range("rg_sweep_segment");
  if (!w || !d_upot || !d_status || n < 0) return rg::fail(RG_ERR_INVALID_ARG, "rg_sweep_segment: invalid argument");
  if (n_begin < 0 || n_end <= n_begin || n_end > w->nx)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_sweep_segment: need 0 <= n_begin < n_end <= nx");
  if ((n_begin > 0) != (d_state_in != nullptr))
    return rg::fail(RG_ERR_INVALID_ARG, "rg_sweep_segment: a state is given exactly when n_begin > 0");
  if (n_end == w->nx && !d_teig) return rg::fail(RG_ERR_INVALID_ARG, "rg_sweep_segment: the last segment needs d_teig");
  if (n == 0) return RG_OK;
  DeviceGuard g(w->device);
  cudaStream_t s = (cudaStream_t)stream;  // taken literally: 0 is CUDA's default stream
  rg::SweepArgs a = make_args(w, rg::kModeEig);
  a.nreal = n;
  a.force_large = 1;
  a.symmetric = 0;
  a.upot = d_upot;
  a.pot_rstride = (int64_t)w->p.nxdiso * w->ny;
  a.pot_xstride = w->ny;
  a.pot_ystride = 1;
  a.n_begin = n_begin;
  a.n_end = n_end;
  a.state_in = (const double2*)d_state_in;
  a.state_dump = (double2*)d_state_dump;
  a.state_out = (double2*)d_state_out;
  a.tout = (double2*)d_tfilt;
  a.teig = d_teig;
  a.status = d_status;
  int grid = 0, rc;
  if ((rc = place_workspace(w, a, 0, &grid))) return rc;
  RG_CUDA(cudaMemsetAsync(w->d_counter, 0, sizeof(int) * rg::kQueueCounters, s));
  return rg::launch_sweep(a, s, grid);
}

int rg_adjoint_grad_rows(rg_waveguide* w, const double* d_xbar, int n, double* d_grad, int64_t grad_stride,
                         void* stream) {
  rg::NvtxRange nvtx_range("rg_adjoint_grad_rows");
  if (!w || !d_xbar || !d_grad || n < 0) return rg::fail(RG_ERR_INVALID_ARG, "rg_adjoint_grad_rows: invalid argument");
  if (w->p.boundtype != RG_BOUND_DIRICHLET)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_adjoint_grad_rows: the adjoint supports Dirichlet guides only");
  if (grad_stride < w->ny) return rg::fail(RG_ERR_INVALID_ARG, "rg_adjoint_grad_rows: grad_stride < ny");
  DeviceGuard g(w->device);
  cudaStream_t s = (cudaStream_t)stream;  // taken literally: 0 is CUDA's default stream
  return rg::launch_grad_rows(w->d_desc, w->nmu, (const double2*)d_xbar, n, d_grad, grad_stride, s);
}

int rg_last_sweep_time(rg_waveguide* w, float* ms) {
  if (!w || !ms) return rg::fail(RG_ERR_INVALID_ARG, "rg_last_sweep_time: NULL argument");
  if (!w->sweep_timed) return rg::fail(RG_ERR_INVALID_ARG, "rg_last_sweep_time: no batch timed yet");
  DeviceGuard g(w->device);
  RG_CUDA(cudaEventSynchronize(w->ev_sweep1));
  RG_CUDA(cudaEventElapsedTime(ms, w->ev_sweep0, w->ev_sweep1));
  return RG_OK;
}

int rg_last_batch_info(rg_waveguide* w, rg_batch_info* info) {
  if (!w || !info) return rg::fail(RG_ERR_INVALID_ARG, "rg_last_batch_info: NULL argument");
  if (!w->sweep_timed) return rg::fail(RG_ERR_INVALID_ARG, "rg_last_batch_info: no batch run yet");
  DeviceGuard g(w->device);
  RG_CUDA(cudaEventSynchronize(w->ev_sweep1));
  *info = w->last_batch;
  if (info->kernel == RG_KERNEL_SYMMETRIC || info->kernel == RG_KERNEL_BLOCKED_SYMMETRIC) {
    int32_t flagged = 0;
    RG_CUDA(cudaMemcpyAsync(&flagged, w->d_counter + 1, sizeof flagged, cudaMemcpyDeviceToHost, w->stream));
    RG_CUDA(cudaStreamSynchronize(w->stream));
    info->rerun = flagged;
  }
  return RG_OK;
}

int rg_histogram(const double* samples, int64_t n, const double* bins, int nbins, double* histo, double* missing) {
  rg::NvtxRange nvtx_range("rg_histogram");
  if (!bins || !histo || !missing || (n > 0 && !samples) || n < 0)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_histogram: invalid argument");
  if (nbins < 1) return rg::fail(RG_ERR_INVALID_ARG, "Invalid number of bins");
  for (int j = 1; j <= nbins; ++j)  // check_histogram, src/base_utils.f90:478-486
    if (bins[j - 1] > bins[j]) return rg::fail(RG_ERR_INVALID_ARG, "Unsorted array of bins, aborting...");
  double* d_x = nullptr;
  double* d_b = nullptr;
  unsigned long long* d_c = nullptr;
  const size_t xb = sizeof(double) * (size_t)std::max<int64_t>(n, 1);
  RG_CUDA(cudaMalloc((void**)&d_x, xb));
  cudaError_t e = cudaMalloc((void**)&d_b, sizeof(double) * (nbins + 1));
  if (e == cudaSuccess) e = cudaMalloc((void**)&d_c, sizeof(unsigned long long) * (nbins + 1));
  int rc = RG_OK;
  std::vector<unsigned long long> counts(nbins + 1, 0ULL);
  if (e == cudaSuccess && n > 0) e = cudaMemcpy(d_x, samples, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_b, bins, sizeof(double) * (nbins + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d_c, 0, sizeof(unsigned long long) * (nbins + 1));
  if (e != cudaSuccess) rc = rg::cuda_fail(e, "rg_histogram setup");
  if (!rc && n > 0) rc = rg::launch_histogram(d_x, n, d_b, nbins, d_c, 0);
  if (!rc) {
    e = cudaMemcpy(counts.data(), d_c, sizeof(unsigned long long) * (nbins + 1), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = rg::cuda_fail(e, "rg_histogram result");
  }
  cudaFree(d_x);
  cudaFree(d_b);
  cudaFree(d_c);
  if (rc) return rc;
  for (int j = 0; j < nbins; ++j) histo[j] = (double)counts[j];
  *missing = (double)counts[nbins];
  return RG_OK;
}

}  // extern "C"
