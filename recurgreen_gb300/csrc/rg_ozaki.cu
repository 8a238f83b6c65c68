// rg_ozaki_zgemm: one complex product C = A B through the tensor-core digit
// path of rg_ozaki.cuh (the same device functions the blocked symmetric
// sweep uses for its propagator product), for tests and measurements.
#include <algorithm>
#include <vector>

#include "rg_internal.h"
#include "rg_ozaki.cuh"

namespace rg {
namespace {

constexpr int kOzThreads = 256;

// Row exponents of A (rows of a column-major M x M) and column exponents of B.
__global__ void oz_exps_kernel(int M, const double2* a, const double2* b, int* ea, int* eb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  int e1 = oz::kNoExp, e2 = oz::kNoExp;
  for (int k = 0; k < M; ++k) {
    e1 = max(e1, oz::fexp2(a[i + (int64_t)k * M]));
    e2 = max(e2, oz::fexp2(b[k + (int64_t)i * M]));
  }
  ea[i] = e1;
  eb[i] = e2;
}

__global__ void oz_split_kernel(int M, const double2* a, const double2* b, const int* ea, const int* eb, uint4* adig,
                                uint4* bdig) {
  const int step = gridDim.x * blockDim.x, t0 = blockIdx.x * blockDim.x + threadIdx.x;
  oz::split_a(M, [&](int i, int k) { return a[i + (int64_t)k * M]; }, ea, adig, t0, step);
  oz::split_b(M, [&](int k, int j) { return b[k + (int64_t)j * M]; }, eb, bdig, t0, step);
}

// CTA (ti, group): warp w computes tile (ti, group * 8 + w).
__global__ void __launch_bounds__(kOzThreads) oz_gemm_kernel(int M, const uint4* adig, const uint4* bdig,
                                                             const int* ea, const int* eb, double2* c) {
  __shared__ uint4 astage[2 * oz::kSlices * oz::kChunkTiles * 32];
  const int T = oz::tiles(M);
  const int ngroup = (T + 7) / 8;
  const int ti = blockIdx.x / ngroup, tj = (blockIdx.x % ngroup) * 8 + (threadIdx.x >> 5);
  const int64_t plane = (int64_t)T * T * 32;
  auto stage = [&](int ch) {
    __syncthreads();
    const int nk = min(oz::kChunkTiles, T - ch * oz::kChunkTiles);
    for (int e = threadIdx.x; e < 2 * oz::kSlices * oz::kChunkTiles * 32; e += blockDim.x) {
      const int lane = e & 31, kk = (e >> 5) % oz::kChunkTiles, ps = (e >> 5) / oz::kChunkTiles;
      if (kk < nk) astage[e] = __ldcg(adig + ps * plane + ((int64_t)ti * T + ch * oz::kChunkTiles + kk) * 32 + lane);
    }
    __syncthreads();
  };
  oz::gemm_tile(M, ti, tj, tj < T, bdig, ea, eb, astage, stage,
                [&](int i, int j, double re, double im) { c[i + (int64_t)j * M] = make_double2(re, im); });
}

}  // namespace
}  // namespace rg

extern "C" int rg_ozaki_zgemm(int M, const double* a, const double* b, double* c) {
  using namespace rg;
  NvtxRange nvtx_range("rg_ozaki_zgemm");
  if (M < 1 || M > 512 || !a || !b || !c)
    return fail(RG_ERR_INVALID_ARG, "rg_ozaki_zgemm: 1 <= M <= 512 and non-NULL matrices required");
  const int T = oz::tiles(M);
  const size_t mat = sizeof(double2) * (size_t)M * M;
  const size_t dig = sizeof(uint4) * (size_t)oz::operand_uint4(M);
  char* buf = nullptr;
  RG_CUDA(cudaMalloc((void**)&buf, 3 * mat + 2 * dig + 2 * sizeof(int) * M));
  double2* da = (double2*)buf;
  double2* db = da + (size_t)M * M;
  double2* dc = db + (size_t)M * M;
  uint4* adig = (uint4*)(buf + 3 * mat);
  uint4* bdig = (uint4*)(buf + 3 * mat + dig);
  int* ea = (int*)(buf + 3 * mat + 2 * dig);
  int* eb = ea + M;
  cudaError_t e = cudaMemcpy(da, a, mat, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(db, b, mat, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    oz_exps_kernel<<<(M + 127) / 128, 128>>>(M, da, db, ea, eb);
    oz_split_kernel<<<std::max(1, T * T / 2), kOzThreads>>>(M, da, db, ea, eb, adig, bdig);
    oz_gemm_kernel<<<T * ((T + 7) / 8), kOzThreads>>>(M, adig, bdig, ea, eb, dc);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(c, dc, mat, cudaMemcpyDeviceToHost);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(e, "rg_ozaki_zgemm");
  return RG_OK;
}
