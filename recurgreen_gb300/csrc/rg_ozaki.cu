// Batched complex products with FP64 accuracy on the FP16 tensor cores, for
// the adjoint's per-slice products (rg_zgemm_batched) and for tests
// (rg_ozaki_zgemm): the device functions of rg_ozaki.cuh, which the blocked
// symmetric sweep also uses for its propagator product, behind three
// stream-ordered kernels per call -- exponents, digit planes, product.
#include <algorithm>

#include "rg_internal.h"
#include "rg_ozaki.cuh"

namespace rg {
namespace {

constexpr int kOzThreads = 256;
constexpr int kOzMaxM = 512;

// One operand of the batch: item k uses the matrix at p + (k % mod) * stride,
// as op(X) with op 0 = X, 1 = X^T, 2 = X^H; row-major or column-major.
struct ZOp {
  const double2* p;
  int64_t stride;
  int mod, op, colmajor;
};

__device__ __forceinline__ double2 zat(const ZOp& o, int item, int M, int r, int c) {
  const double2* base = o.p + (int64_t)(item % o.mod) * o.stride;
  const int i = o.op ? c : r, j = o.op ? r : c;
  double2 v = o.colmajor ? base[i + (int64_t)j * M] : base[(int64_t)i * M + j];
  if (o.op == 2) v.y = -v.y;
  return v;
}

__device__ __forceinline__ double2 zscale(const double2* s, int r, double2 v) {
  if (!s) return v;
  const double2 a = s[r];
  return make_double2(a.x * v.x - a.y * v.y, a.x * v.y + a.y * v.x);
}

struct ItemWs {
  uint4* adig;
  uint4* bdig;
  int* ea;
  int* eb;
};

__device__ __forceinline__ ItemWs item_ws(char* ws, int M, int item) {
  char* b = ws + (int64_t)item * oz::workspace_bytes(M);
  ItemWs w;
  w.adig = reinterpret_cast<uint4*>(b);
  w.bdig = w.adig + oz::operand_uint4(M);
  w.ea = reinterpret_cast<int*>(w.bdig + oz::operand_uint4(M));
  w.eb = w.ea + 16 * oz::tiles(M);
  return w;
}

// One CTA per item: exponents of the rows of op(A) (a warp per row, lanes
// along the row) and of the columns of diag(s) op(B) (a thread per column,
// rows in sequence); no atomics.
__global__ void __launch_bounds__(kOzThreads) zb_exps_kernel(int M, ZOp A, ZOp B, const double2* rowscale, char* ws) {
  const int item = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const ItemWs w = item_ws(ws, M, item);
  const int Mp = 16 * oz::tiles(M);
  for (int r = warp; r < Mp; r += nw) {
    int e = oz::kNoExp;
    if (r < M)
      for (int c = lane; c < M; c += 32) e = max(e, oz::fexp2(zat(A, item, M, r, c)));
#pragma unroll
    for (int off = 16; off; off >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, off));
    if (lane == 0) w.ea[r] = e;
  }
  for (int c = threadIdx.x; c < Mp; c += blockDim.x) {
    int e = oz::kNoExp;
    if (c < M)
      for (int k = 0; k < M; ++k) e = max(e, oz::fexp2(zscale(rowscale, k, zat(B, item, M, k, c))));
    w.eb[c] = e;
  }
}

// `per` CTAs per item write its digit planes.
__global__ void __launch_bounds__(kOzThreads) zb_split_kernel(int M, ZOp A, ZOp B, const double2* rowscale, char* ws,
                                                              int per) {
  const int item = blockIdx.x / per, t0 = (blockIdx.x % per) * blockDim.x + threadIdx.x, step = per * blockDim.x;
  const ItemWs w = item_ws(ws, M, item);
  oz::split_a(M, [&](int i, int k) { return zat(A, item, M, i, k); }, w.ea, w.adig, t0, step);
  oz::split_b(M, [&](int k, int j) { return zscale(rowscale, k, zat(B, item, M, k, j)); }, w.eb, w.bdig, t0, step);
}

// CTA (item, block of 2 x 4 output tiles): oz::gemm_block with both
// operands' digits staged in shared memory.  C = alpha (A B) + beta D.
__global__ void __launch_bounds__(kOzThreads, 2) zb_gemm_kernel(int M, char* ws, double2 alpha, ZOp D, double beta,
                                                                double2* C, int64_t strideC, int colmajor) {
  extern __shared__ uint4 stg[];
  const int T = oz::tiles(M);
  const int nbr = (T + oz::kBlkRows - 1) / oz::kBlkRows, nbc = (T + oz::kBlkCols - 1) / oz::kBlkCols;
  const int item = blockIdx.x / (nbr * nbc), rest = blockIdx.x % (nbr * nbc);
  const int ti0 = (rest / nbc) * oz::kBlkRows, tj0 = (rest % nbc) * oz::kBlkCols;
  const ItemWs w = item_ws(ws, M, item);
  double2* c = C + (int64_t)item * strideC;
  oz::gemm_block(M, ti0, tj0, false, w.adig, w.bdig, w.ea, w.eb, stg, [&](int i, int j, double re, double im) {
    double2 v = make_double2(alpha.x * re - alpha.y * im, alpha.x * im + alpha.y * re);
    if (beta != 0.0) {
      const double2 d = zat(D, item, M, i, j);
      v.x = fma(beta, d.x, v.x);
      v.y = fma(beta, d.y, v.y);
    }
    c[colmajor ? i + (int64_t)j * M : (int64_t)i * M + j] = v;
  });
}

constexpr size_t kZbGemmSmem = sizeof(uint4) * oz::kBlkStageUint4;

int launch_zgemm(int M, int nbatch, const ZOp& A, const ZOp& B, const double2* rowscale, double2 alpha, const ZOp& D,
                 double beta, double2* C, int64_t strideC, int colmajor, char* ws, cudaStream_t s) {
  const int T = oz::tiles(M);
  const int per = std::max(1, std::min(16, T * T * 32 / kOzThreads));
  zb_exps_kernel<<<nbatch, kOzThreads, 0, s>>>(M, A, B, rowscale, ws);
  zb_split_kernel<<<nbatch * per, kOzThreads, 0, s>>>(M, A, B, rowscale, ws, per);
  RG_CUDA(cudaFuncSetAttribute(zb_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZbGemmSmem));
  const int nblk = ((T + oz::kBlkRows - 1) / oz::kBlkRows) * ((T + oz::kBlkCols - 1) / oz::kBlkCols);
  zb_gemm_kernel<<<nbatch * nblk, kOzThreads, kZbGemmSmem, s>>>(M, ws, alpha, D, beta, C, strideC, colmajor);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

}  // namespace
}  // namespace rg

extern "C" int64_t rg_zgemm_workspace_bytes(int M, int nbatch) {
  if (M < 1 || M > rg::kOzMaxM || nbatch < 0) return -1;
  return rg::oz::workspace_bytes(M) * (int64_t)nbatch;
}

extern "C" int rg_zgemm_batched(int M, int nbatch, const double* a, int64_t stride_a, int mod_a, int op_a,
                                const double* b, int64_t stride_b, int mod_b, int op_b, const double* rowscale_b,
                                double alpha_re, double alpha_im, const double* d, int64_t stride_d, int mod_d,
                                double beta, double* c, int64_t stride_c, int colmajor, void* workspace,
                                int64_t workspace_bytes, void* stream) {
  using namespace rg;
  NvtxRange nvtx_range("rg_zgemm_batched");
  if (M < 1 || M > kOzMaxM || nbatch < 0 || !a || !b || !c || op_a < 0 || op_a > 2 || op_b < 0 || op_b > 2 ||
      (beta != 0.0 && !d))
    return fail(RG_ERR_INVALID_ARG, "rg_zgemm_batched: invalid argument (1 <= M <= 512, op in 0..2, D for beta != 0)");
  if (nbatch == 0) return RG_OK;
  if (!workspace || workspace_bytes < oz::workspace_bytes(M) * (int64_t)nbatch)
    return fail(RG_ERR_INVALID_ARG, "rg_zgemm_batched: workspace smaller than rg_zgemm_workspace_bytes(M, nbatch)");
  if (((uintptr_t)workspace & 15) != 0)
    return fail(RG_ERR_INVALID_ARG, "rg_zgemm_batched: workspace not 16-byte aligned");
  auto fix = [nbatch](int m) { return m <= 0 ? nbatch : m; };
  const ZOp A{(const double2*)a, stride_a, fix(mod_a), op_a, colmajor ? 1 : 0};
  const ZOp B{(const double2*)b, stride_b, fix(mod_b), op_b, colmajor ? 1 : 0};
  const ZOp D{(const double2*)(d ? d : a), d ? stride_d : 0, d ? fix(mod_d) : 1, 0, colmajor ? 1 : 0};
  return launch_zgemm(M, nbatch, A, B, (const double2*)rowscale_b, make_double2(alpha_re, alpha_im), D, beta,
                      (double2*)c, stride_c, colmajor ? 1 : 0, (char*)workspace, (cudaStream_t)stream);
}

extern "C" int rg_ozaki_zgemm(int M, const double* a, const double* b, double* c) {
  using namespace rg;
  NvtxRange nvtx_range("rg_ozaki_zgemm");
  if (M < 1 || M > kOzMaxM || !a || !b || !c)
    return fail(RG_ERR_INVALID_ARG, "rg_ozaki_zgemm: 1 <= M <= 512 and non-NULL matrices required");
  const size_t mat = sizeof(double2) * (size_t)M * M;
  const size_t wsb = (size_t)oz::workspace_bytes(M);
  char* buf = nullptr;
  RG_CUDA(cudaMalloc((void**)&buf, 3 * mat + wsb));
  double* da = (double*)buf;
  double* db = (double*)(buf + mat);
  double* dc = (double*)(buf + 2 * mat);
  cudaError_t e = cudaMemcpy(da, a, mat, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(db, b, mat, cudaMemcpyHostToDevice);
  int rc = RG_OK;
  if (e == cudaSuccess)
    rc = rg_zgemm_batched(M, 1, da, 0, 1, 0, db, 0, 1, 0, nullptr, 1.0, 0.0, nullptr, 0, 1, 0.0, dc, 0, 1,
                          buf + 3 * mat, (int64_t)wsb, nullptr);
  if (e == cudaSuccess && rc == RG_OK) e = cudaMemcpy(c, dc, mat, cudaMemcpyDeviceToHost);
  cudaFree(buf);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "rg_ozaki_zgemm");
  return RG_OK;
}
