// Throughput probes of the arithmetic pipes the sweep can use (diagnostics;
// no counterpart in the reference).  Each probe keeps every warp of a full
// grid busy with independent dependency chains of one instruction kind on
// register operands, so the measured rate is the pipe's, not memory's:
//   kind 0  FP64 FMA (fma.rn.f64), 8 chains per thread
//   kind 1  FP64 mma.sync m8n8k4 (DMMA), 4 accumulators per warp
//   kind 2  FP64 mma.sync m16n8k16, 4 accumulators per warp
//   kind 3  FP16 mma.sync m16n8k16 with FP32 accumulation, 4 accumulators per warp
//   kind 4  FP32 FMA (fma.rn.f32), 8 chains per thread
// The operands are small constants, so no accumulator overflows.
#include <cuda_fp16.h>

#include <algorithm>

#include "rg_internal.h"

namespace rg {
namespace {

constexpr int kProbeThreads = 256;

template <int KIND>
__global__ void __launch_bounds__(kProbeThreads) probe_kernel(int iters, double seedv, double* sink) {
  double acc = 0.0;
  if constexpr (KIND == 0) {
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seedv * (k + 1) + threadIdx.x;
    const double x = 1.0 - 1e-12, y = seedv;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = fma(a[k], x, y);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) acc += a[k];
  } else if constexpr (KIND == 4) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = (float)seedv * (k + 1) + threadIdx.x;
    const float x = 1.0f - 1e-6f, y = (float)seedv;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], x, y);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) acc += a[k];
  } else if constexpr (KIND == 1) {
    const double av = seedv, bv = seedv;
    double c[4][2];
#pragma unroll
    for (int j = 0; j < 4; ++j) c[j][0] = c[j][1] = 0.0;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(c[j][0]), "+d"(c[j][1])
                     : "d"(av), "d"(bv));
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) acc += c[j][0] + c[j][1];
  } else if constexpr (KIND == 2) {
    const double av = seedv, bv = seedv;
    double c[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) c[j][q] = 0.0;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%4,%4,%4,%4,%4,%4,%4}, "
            "{%5,%5,%5,%5}, {%0,%1,%2,%3};"
            : "+d"(c[j][0]), "+d"(c[j][1]), "+d"(c[j][2]), "+d"(c[j][3])
            : "d"(av), "d"(bv));
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) acc += c[j][0] + c[j][1] + c[j][2] + c[j][3];
  } else {
    // two halves of value ~seedv packed per register
    const __half h = __double2half(seedv);
    const unsigned short hb = __half_as_ushort(h);
    const unsigned int ab = ((unsigned int)hb << 16) | hb;
    float c[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) c[j][q] = 0.0f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%4,%4,%4}, {%4,%4}, "
            "{%0,%1,%2,%3};"
            : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
            : "r"(ab));
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) acc += c[j][0] + c[j][1] + c[j][2] + c[j][3];
  }
  if (acc == 12345.678) sink[blockIdx.x] = acc;  // never true; keeps the work alive
}

// Flops of one loop iteration of one thread.
double flops_per_thread_iter(int kind) {
  switch (kind) {
    case 0: return 16.0;                           // 8 FMA
    case 4: return 16.0;
    case 1: return 4.0 * 2 * 8 * 8 * 4 / 32.0;     // 4 m8n8k4 per warp
    case 2: return 4.0 * 2 * 16 * 8 * 16 / 32.0;   // 4 m16n8k16 per warp
    default: return 4.0 * 2 * 16 * 8 * 16 / 32.0;  // 4 m16n8k16 per warp
  }
}

}  // namespace
}  // namespace rg

extern "C" int rg_probe_rate(int kind, int iters, double* tflops) {
  using namespace rg;
  if (!tflops || kind < 0 || kind > 4 || iters < 1)
    return fail(RG_ERR_INVALID_ARG, "rg_probe_rate: kind must be 0..4, iters >= 1, tflops non-NULL");
  int dev = 0, sms = 0;
  RG_CUDA(cudaGetDevice(&dev));
  RG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 4;
  double* sink = nullptr;
  RG_CUDA(cudaMalloc((void**)&sink, sizeof(double) * blocks));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto launch = [&](int it) {
    switch (kind) {
      case 0: probe_kernel<0><<<blocks, kProbeThreads>>>(it, 1e-3, sink); break;
      case 1: probe_kernel<1><<<blocks, kProbeThreads>>>(it, 1e-3, sink); break;
      case 2: probe_kernel<2><<<blocks, kProbeThreads>>>(it, 1e-3, sink); break;
      case 3: probe_kernel<3><<<blocks, kProbeThreads>>>(it, 1e-3, sink); break;
      default: probe_kernel<4><<<blocks, kProbeThreads>>>(it, 1e-3, sink); break;
    }
  };
  launch(std::max(1, iters / 16));  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    launch(iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  const cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess) return cuda_fail(e, "rg_probe_rate");
  *tflops = flops_per_thread_iter(kind) * kProbeThreads * (double)blocks * iters / (best * 1e-3) / 1e12;
  return RG_OK;
}
