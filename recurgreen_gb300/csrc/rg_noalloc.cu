// rg_tdistrib_seed_noalloc: the seed-driven eigenvalue computation of one
// realization with no device allocation in the call.
//
// Why it exists: some callers cannot call cudaMalloc at the point where they
// need a result -- host applications that hand all device memory to their
// own pool allocator, and steady-state loops that must not take cudaMalloc's
// implicit device synchronisation.  They create the
// waveguide handle once at set-up (rg_init allocates its tables there) and
// then call this entry point, which only launches kernels on memory that
// already exists.
//
// The per-call scratch (the disorder potential of the realization, the seed,
// the work-queue counters, the symmetric sweep's flag slot and, above 64
// modes, the elimination matrices) lives
// in a file-scope __device__ array of fixed size, kNoAllocScratchBytes =
// 16 MiB.  Every GPU that loads this library
// holds that array until the process exits.  Its device address is looked up
// with cudaGetSymbolAddress once per device, on the first call made with that
// device current; make that first call before any stream capture begins.
// All calls share the one array and it keeps the previous call's contents:
// the header words that must start at zero are reset by a kernel at the start
// of every call, and calls whose work overlaps on the GPU (different streams,
// or different host threads) race on the array.
#include <mutex>

#include "rg_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;  // 16 MiB
constexpr size_t kNoAllocHeaderBytes = 256;         // seed, queue counters, flag slot

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Writes the seed and zeroes the queue counters in the header of the array:
// int32 [0] seed, [1, 1 + kQueueCounters) counters, then the flag slot.
__global__ void noalloc_header_kernel(int32_t seed) {
  int32_t* hdr = reinterpret_cast<int32_t*>(g_noalloc_scratch);
  hdr[0] = seed;  // seed read by the potential generator
  for (int k = 1; k <= rg::kQueueCounters; ++k) hdr[k] = 0;
}

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of g_noalloc_scratch on the current device (looked up once).
int noalloc_scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_seed_noalloc: device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return rg::cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[device] = p;
  }
  *out = static_cast<unsigned char*>(g_noalloc_ptr[device]);
  return RG_OK;
}

}  // namespace

extern "C" int rg_tdistrib_seed_noalloc(rg_waveguide* wg, int iseed, double* d_teigvals, int32_t* d_status,
                                        void* stream) {
  if (!wg || !d_teigvals || !d_status)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_seed_noalloc: NULL argument");
  if (iseed < 1)  // the same seeds as rg_compute_tdistrib accepts
    return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_seed_noalloc: iseed must be >= 1");
  rg::NoAllocView v{};
  int rc = rg::noalloc_view(wg, &v);
  if (rc) return rc;
  // The sweep's launch arguments: one item, the potential read from the array.
  rg::SweepArgs a{};
  a.mode = rg::kModeEig;
  a.nreal = 1;
  a.wgs = v.d_desc;
  a.max_M = v.nmu;
  a.max_ny = v.ny;
  a.teig = d_teigvals;
  a.status = d_status;
  a.symmetric = v.symmetric;
  a.sym_tau = v.sym_tau;
  int grid = 1;
  int64_t stride = 0;
  if ((rc = rg::sweep_plan(a, v.sm_count, &grid, &stride))) return rc;
  // Above 64 modes the elimination also needs its matrices in the array.
  const bool large = v.nmu > rg::kMaxModesSmem;
  const size_t pot_doubles = (size_t)v.nxdiso * (size_t)v.ny;
  const size_t pot_bytes = (pot_doubles * sizeof(double) + 255) & ~(size_t)255;
  const size_t ws_bytes = large ? sizeof(double2) * (size_t)stride * (grid / a.cluster) : 0;
  if (pot_bytes + ws_bytes > kNoAllocScratchBytes - kNoAllocHeaderBytes)
    return rg::fail(RG_ERR_INVALID_ARG,
                    "rg_tdistrib_seed_noalloc: nxdiso*ny = " + std::to_string(pot_doubles) +
                        " potential doubles" + (large ? " plus the elimination workspace" : "") +
                        " exceed the fixed scratch capacity of 16 MiB; use rg_compute_tdistrib");
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) return rg::cuda_fail(e, "cudaGetDevice");
  if (cur != v.device)
    return rg::fail(RG_ERR_INVALID_ARG, "rg_tdistrib_seed_noalloc: make the handle's device current first");
  unsigned char* base = nullptr;
  if ((rc = noalloc_scratch_address(cur, &base))) return rc;
  int32_t* d_seed = reinterpret_cast<int32_t*>(base);
  int* d_counter = reinterpret_cast<int*>(base) + 1;
  int32_t* d_flag = reinterpret_cast<int32_t*>(base) + 1 + rg::kQueueCounters;
  double* d_pot = reinterpret_cast<double*>(base + kNoAllocHeaderBytes);
  cudaStream_t s = stream ? (cudaStream_t)stream : v.stream;

  noalloc_header_kernel<<<1, 1, 0, s>>>((int32_t)iseed);
  e = cudaGetLastError();
  if (e != cudaSuccess) return rg::cuda_fail(e, "noalloc_header_kernel");
  rg::PotArgs pa{};
  pa.nxdiso = v.nxdiso;
  pa.ny = v.ny;
  pa.nreal = 1;
  pa.stdu = v.stdu;
  pa.seeds = d_seed;
  pa.jumppoly = v.jumppoly;
  pa.upot = d_pot;
  if ((rc = rg::launch_potential(pa, s))) return rc;
  a.upot = d_pot;
  a.pot_rstride = 0;
  a.pot_xstride = v.ny;
  a.pot_ystride = 1;
  a.work_counter = d_counter;
  a.flag_list = a.symmetric ? d_flag : nullptr;
  a.work = large ? reinterpret_cast<double2*>(base + kNoAllocHeaderBytes + pot_bytes) : nullptr;
  a.work_stride = large ? stride : 0;
  return rg::launch_sweep(a, s, grid);
}
