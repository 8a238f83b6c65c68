// Internal declarations shared by the host side (rg_waveguide.cpp) and the
// kernels (rg_sweep.cu).  Not part of the public C ABI.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <complex>
#include <string>
#include <vector>

#include "../../include/recurgreen.h"

namespace rg {

using cplx = std::complex<double>;

// Error plumbing: the thread-local message behind rg_last_error().
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define RG_CUDA(call)                                          \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return ::rg::cuda_fail(e_, #call); \
  } while (0)

// Switches to a handle's device for the duration of a call.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

// An NVTX range around a host-side entry point, for profilers (nsys, ncu's
// NVTX filters); a no-op when no tool is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Message of a per-realization status.
inline const char* status_text(int code) {
  switch (code) {
    case RG_ERR_SINGULAR: return "zgetrf: Matrix is numerically singular (zero or NaN pivot)";
    case RG_ERR_NOCONV: return "singular values did not converge";
    default: return "error";
  }
}

// Largest mode count the shared-memory sweep kernel handles.
constexpr int kMaxModesSmem = 64;

// One waveguide as the kernels see it: sizes and device tables, built by
// rg_init and kept in device memory for the handle's lifetime.
struct WgDesc {
  int M;        // nmu
  int ny;       // transverse grid points
  int nx;       // total slices
  int nxdiso;   // disordered slices
  int nxfree;   // free slices on each side
  int row0, nrow, col0, ncol;  // tdistrib Fisher-Lee window, 0-based start and extent
  int neigv;    // eigenvalues kept per realization
  int periodic;
  double stdu;                // standard deviation of the dimensionless potential
  const double2* bmat;        // [M] B diagonal
  const double2* adiag_edge;  // [M] A diagonal on slices 1 and nx
  const double2* adiag_bulk;  // [M] A diagonal in the bulk
  const double2* sqmu_c;      // [M] complex sqrt(mu) (tdistrib Fisher-Lee)
  const double2* sqmu_r;      // [M] sqrt(real(mu)) (v1 Fisher-Lee)
  const double* costab;       // [ny * (2M+1)] cos(pi d y_j) / ny  (Dirichlet)
  const double2* expfac;      // [ny * M] exp(2 pi i d y_j) / ny  (periodic), d = 0..M-1
  const uint64_t* jumppoly;   // [ny * 4] x^(2*nxdiso*iy) mod the xoshiro256 characteristic polynomial
};

// One launch of a sweep kernel: a queue of work items (realizations), each a
// (waveguide, seed) pair.  Device pointers.
struct SweepArgs {
  int mode;                   // kModeEig or kModeTmat
  int nreal;                  // work items in this launch
  const WgDesc* wgs;          // waveguides
  const int32_t* item_wg;     // [nreal] waveguide of each item; nullptr: all use wgs[0]
  const int32_t* seeds;       // [nreal] seeds; the potential is drawn in-kernel when upot == nullptr
  const double* upot;         // optional potentials, (r, ix, iy) at r*pot_rstride + ix*pot_xstride + iy*pot_ystride
  int64_t pot_rstride, pot_xstride, pot_ystride;
  const int64_t* teig_off;    // [nreal] offset of item r's eigenvalues in teig; nullptr: r * neigv
  double* teig;               // eigenvalues (kModeEig)
  double2* tout;              // [nreal][nrow * ncol] column-major t, optional (items of one waveguide only)
  int32_t* status;            // [nreal]
  int* work_counter;          // kQueueCounters ints, zeroed before launch: [0] the work queue,
                              // [1] items flagged by the symmetric kernel, [2] their re-run queue
  double2* work;              // per-CTA workspace in global memory
  int64_t work_stride;        // double2 elements per CTA
  int max_M, max_ny;          // largest M and ny among the items (shared-memory sizing)
  int cluster;                // CTAs per work item (large-mode kernel; set by sweep_plan)
  // Segment mode (blocked kernel only; used by the adjoint's recomputation):
  // run slices [n_begin, n_end) from a given state and dump the states.
  int n_begin, n_end;         // slice range; n_end == 0 means the whole guide
  const double2* state_in;    // [nreal][2][M][M] (Gss, Gs1) after slice n_begin-1, natural order; nullptr: fresh start
  double2* state_dump;        // [nreal][n_end-n_begin][2][M][M] (Gss, Gs1) after every slice, optional
  double2* state_out;         // [nreal][2][M][M] state after slice n_end-1, optional
  int force_large;            // 1: the pivoted blocked kernel even for max_M <= 64 (segment mode with states)
  // Symmetric sweep (Dirichlet items): the symmetric kernel (shared-memory
  // or blocked, by max_M) runs every item and appends those it cannot pivot
  // stably to flag_list; the pivoted kernel of the same class re-runs them.
  int symmetric;              // 1: symmetric kernel first (needs flag_list)
  int32_t* flag_list;         // [nreal] flagged item indices
  double sym_tau;             // smallest accepted |diagonal pivot| / max |unswept entry of its row|
  // Queue indirection of the pivoted kernel (set by launch_sweep for the re-run):
  const int32_t* item_idx;    // [count] item index of queue position q; nullptr: q itself
  const int* count_ptr;       // device-side queue length; nullptr: nreal
  int force_cluster;          // > 0: cluster size for the blocked kernels instead of the heuristic
                              // (autotuner, multi calls with long items)
  int force_rowsplit;         // > 0: threads per update unit of the blocked symmetric kernel (1, 4
                              // or 8) instead of its fewest-rows-per-thread rule (autotuner)
  int force_per_sm;           // > 0: at most this many CTAs per SM for the shared-memory kernels
                              // (autotuner); 0: the occupancy limit
  // Source slice of the Green-function column (pivoted blocked kernel, fresh
  // start): Gs1 after slice n is Z_n of solve_block_tridiag for the identity
  // source at slice inject_at (src/base_utils.f90:318-324), zero before it.
  // 0 is the usual sweep (source at slice 0, where Z_0 = Gss_0).
  int inject_at;
  // 1: the blocked symmetric kernel forms the propagator product Gss (B Gs1)
  // on the tensor cores (rg_ozaki.cuh) after inverting X on its own, instead
  // of carrying B Gs1 through the Gauss-Jordan sweep (up to 512 modes).
  // Set from RG_TENSOR_R (default on).
  int tensor_r;
  // With tensor_r, the levels (0..2) of the 2 x 2 block inverse of X in the
  // blocked symmetric kernel: each level halves an even size of at least 128
  // modes into two half-size inverses and four half-size tensor-core
  // products; the blocks left are inverted by FP64 Gauss-Jordan sweeps.
  // Set from RG_SPLIT_INVERSE (default 2).
  int split_inverse;
};

// Status the symmetric kernel leaves on an item whose diagonal pivots were
// too small; the pivoted kernel recomputes such items (never returned).
constexpr int kStatusNeedPivot = 64;
// Queue counters behind SweepArgs::work_counter.
constexpr int kQueueCounters = 3;
// Default of SweepArgs::sym_tau.
constexpr double kSymTau = 0.1;

constexpr int kModeEig = 0;   // tdistrib: filtered t -> eigenvalues of t^H t
constexpr int kModeTmat = 1;  // v1 t: full t written to tout
constexpr int kModeRefl = 2;  // v1 r: the sweep runs over the slices in reverse order, and
                              // its last Gss is G(x_1; x_1) of the guide; r goes to tout

// Potential generator arguments.
struct PotArgs {
  int nxdiso, ny, nreal;
  double stdu;
  const int32_t* seeds;        // [nreal]
  const uint64_t* jumppoly;    // [ny * 4] x^(2*nxdiso*iy) mod charpoly
  double* upot;                // [nreal][nxdiso][ny]
};

// Launchers.  All enqueue on `stream`.  A sweep launch is planned first (grid
// size and per-CTA workspace, from max_M/max_ny and the kernel's occupancy),
// then launched with a.work pointing at grid * work_stride double2 elements.
int launch_potential(const PotArgs& a, cudaStream_t stream);
int sweep_plan(SweepArgs& a, int sm_count, int* grid, int64_t* work_stride);
int launch_sweep(const SweepArgs& a, cudaStream_t stream, int grid);
// Symmetric sweep (rg_sweep_sym.cu): complex-symmetric slice matrices
// (Dirichlet), M <= kMaxModesSmem, diagonal pivoting.  launch_sweep calls it
// when a.symmetric is set and re-runs the flagged items itself.
int sweep_sym_plan(SweepArgs& a, int sm_count, int* grid, int64_t* work_stride);
int launch_sweep_sym(const SweepArgs& a, cudaStream_t stream, int grid);
// The large-mode kernel behind sweep_plan/launch_sweep for max_M > kMaxModesSmem (rg_sweep_large.cu).
int sweep_large_plan(SweepArgs& a, int sm_count, int* grid, int64_t* work_stride);
int launch_sweep_large(const SweepArgs& a, cudaStream_t stream, int grid);
// Its symmetric counterpart for Dirichlet guides (rg_sweep_large_sym.cu);
// launch_sweep re-runs the items it flags with the pivoted one.
int sweep_large_sym_plan(SweepArgs& a, int sm_count, int* grid, int64_t* work_stride);
int launch_sweep_large_sym(const SweepArgs& a, cudaStream_t stream, int grid);
// Adjoint (rg_adjoint.cu): dL/dU rows of n realizations from their slice-matrix adjoints.
int launch_grad_rows(const WgDesc* d_desc, int M, const double2* xbar, int n, double* grad, int64_t gstride,
                     cudaStream_t s);
int launch_histogram(const double* d_samples, int64_t n, const double* d_bins, int nbins,
                     unsigned long long* d_counts, cudaStream_t stream);

// xoshiro256** jump-ahead polynomials (rg_waveguide.cpp).
void jump_polynomial(uint64_t distance, uint64_t out[4]);

// Read-only view of a handle for the allocation-free entry point
// (rg_noalloc.cu): sizes, device tables and the device-resident descriptor.
struct NoAllocView {
  int device, sm_count, nxdiso, ny, nmu;
  double stdu;
  const uint64_t* jumppoly;
  cudaStream_t stream;
  const WgDesc* d_desc;
  int symmetric;   // SweepArgs::symmetric for this guide
  double sym_tau;  // SweepArgs::sym_tau
};
int noalloc_view(const rg_waveguide* w, NoAllocView* out);

// ---------------------------------------------------------------------------
// Full Green-function column (rg_green.cu, rg_green.cpp): the block
// tridiagonal solve of src/base_utils.f90:296-335 for a source at one slice,
// as a forward sweep that keeps (Gss_n, Gs1_n) = (S_n, Z_n) of every slice
// and a back-substitution X_n = Z_n - S_n B X_{n+1} applied to a few source
// vectors.
// ---------------------------------------------------------------------------

// What rg_green.cpp needs of a handle.
struct GreenView {
  int device, sm_count;
  cudaStream_t stream;
  const WgDesc* d_desc;
  WgDesc desc;      // host copy: sizes and device table pointers
  int* d_counter;   // kQueueCounters ints
  int nxdiso, nxfree, nx, ny, nmu, neigv, periodic;
  int imin, imax, jmin, jmax;  // 1-based Fisher-Lee window
  double wol, stdu;
  const double* xmesh;   // host [nx]
  const double* ymesh;   // host [ny]
  const double* kpmesh;  // host [nmu]
  const cplx* sqmu_r;    // host [nmu] sqrt(real(mu))
  int symmetric;         // the symmetric sweep is enabled for this guide (Dirichlet)
  double sym_tau;        // its pivot threshold
  int tensor_r;          // SweepArgs::tensor_r for this guide
  int split_inverse;     // SweepArgs::split_inverse for this guide
};
int green_view(const rg_waveguide* w, GreenView* out);

// Eigenvectors of t^H t per item (diagonalize_ahca, src/base_utils.f90:394-444)
// and, for the transmission-eigenstate profiles, the selection of the
// eigenvectors inside windows of T and their source vectors.
struct EigvecArgs {
  int nreal;
  const double2* a;     // item r's matrix at a + r*astride, column-major with leading dimension lda
  int64_t astride;
  int lda;
  int row0, nr, col0, nc;  // the block of a that is diagonalized (nr x nc)
  double2* work;        // per-item workspace, work_stride double2: the block and V
  int64_t work_stride;
  double* tvals;        // [nreal][nc] eigenvalues, descending (ties by index)
  double2* u;           // optional [nreal][nc][nc] eigenvectors, column-major, in tvals order
  // Selection (when wsel != nullptr): eigenvector v enters window w when
  //   centered == 0: wa[w] <= T_v <= wb[w]   (compute_tprofile, src/waveguide.f90:892)
  //   centered == 1: |T_v - wa[w]| <= wb[w]  (compute_tprofile_group, src/waveguide.f90:978)
  int nprof, centered;
  const double* wa;     // [nprof]
  const double* wb;     // [nprof]
  int M;                // length of a source vector
  const double2* sqmu;  // [M] sqrt(real(mu)); source row col0 + j is sqmu[col0 + j] * V[j][v]
  double2* wsel;        // [nreal][nc][M] source vectors of the selected eigenvectors, in tvals order
  uint32_t* member;     // [nreal][nc] bit w: in window w
  int32_t* ksel;        // [nreal] selected count
  int32_t* nt;          // [nreal][nprof] eigenvalues in each window
  double* tavg;         // optional [nreal] sum(tvals) / nc
  int32_t* status;      // [nreal]
};
int launch_eigvec(const EigvecArgs& a, cudaStream_t s);
int64_t eigvec_work_stride(int nr, int nc);

// Back-substitution over slices nx-1 .. i_lo for the source vectors of each
// item: Y_{nx-1} = Z_{nx-1} W, Y_n = Z_n W - S_n (B Y_{n+1}).
constexpr int kBackProfile = 0;  // prof[r][s][n] = sum_m |Y_n[m][s]|^2
constexpr int kBackColumns = 1;  // cols[r][n - i_lo][s][m] = Y_n[m][s] (or only n = i_lo)
struct BackArgs {
  int nreal, M, nx;
  const double2* dump;     // [nreal][nx][2][M][M]: (Gss_n, Gs1_n), row-major
  const double2* bmat;     // [M]
  const double2* src;      // item r's source vectors at src + r*src_stride, [kmax][M]
  int64_t src_stride;      // 0: every item uses the same vectors
  int kmax;
  const int32_t* kcount;   // [nreal] vectors per item; nullptr: kmax
  int i_lo;                // lowest slice, 0-based
  int out_mode;            // kBackProfile or kBackColumns
  int only_lo;             // kBackColumns: write slice i_lo only
  const double2* left;     // kBackColumns, optional: output 2i * left[m] * Y[m][s] (Fisher-Lee rows)
  double* prof;            // [nreal][kmax][nx]
  double2* cols;           // [nreal][nslices][kmax][M], nslices = only_lo ? 1 : nx - i_lo
};
int launch_back(const BackArgs& a, cudaStream_t s);

// Window sums of the per-vector profiles, normalised: out[r][w][n] =
//   sum over selected s in window w (ascending s) of prof[r][s][n], times
//   4/nt[r][w] when nt != 0 (compute_tprofile[_group], src/waveguide.f90:902,988), or
//   2/(pi wol |wb[w] - wa[w]|) for kind RG_PROFILE_ITX (src/waveguide.f90:821).
struct WindowArgs {
  int nreal, nx, kmax, nprof, kind;
  double wol;
  const double* wa;        // [nprof]
  const double* wb;        // [nprof]
  const int32_t* ksel;
  const uint32_t* member;
  const int32_t* nt;
  const double* prof;
  double* out;             // [nreal][nprof][nx]
};
int launch_windows(const WindowArgs& a, cudaStream_t s);

// compute_wavefunction's pixels (src/waveguide.f90:680-695): psi(x_n, y_j) =
// sum_m modal[j][m] Y_n[m], written with x, y and the potential as the
// (nx*ny) x 5 column-major table [x, y, Re psi, Im psi, upot].
struct WavefunArgs {
  int nx, ny, M, nxfree, nxdiso;
  const double2* y;        // [nx][M]
  const double2* modal;    // [ny][M]
  const double* xmesh;     // [nx]
  const double* ymesh;     // [ny]
  const double* upot;      // [nxdiso][ny] (x-major rows of ny)
  double* out;             // [5][nx*ny]
};
int launch_wavefun(const WavefunArgs& a, cudaStream_t s);

}  // namespace rg
