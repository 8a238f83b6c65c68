// Full Green-function column: the kernels behind the transmission-eigenstate
// profiles (compute_tprofile, compute_tprofile_group, compute_itx_profile,
// src/waveguide.f90:764-997), the deposition matrix (compute_deposition,
// src/waveguide.f90:710-745) and the wavefunction (compute_wavefunction,
// src/waveguide.f90:636-698).
//
// The reference solves the block tridiagonal system for every slice with
// solve_block_tridiag (src/base_utils.f90:296-335): a forward loop S_n =
// inv(A_n - B S_{n-1} B), Z_n = S_n (I_n - B Z_{n-1}) and a backward loop
// X_n = Z_n - S_n B X_{n+1}, each block M x M.  Here the forward loop is the
// pivoted blocked sweep kernel (its state after slice n is (Gss, Gs1) =
// (S_n, Z_n), kept for every slice), and the backward loop runs only on the
// few source vectors W the caller needs: X_n W for the eigenvectors of t^H t
// inside a window of T, or one column for the deposition and the
// wavefunction.  That cuts the backward work from 8 M^3 to 16 M^2 k per slice
// for k vectors, and the profiles |X_n W|^2 come out of the same loop.
#include <algorithm>

#include "rg_device.cuh"

namespace rg {
namespace {

constexpr int kNT = 256;
constexpr int kKC = 8;  // source vectors per CTA of the back-substitution (one warp each in the reduction)

// One-sided Jacobi on the nv columns (length L) of A, with the right
// rotations accumulated in V (nv x nv): at convergence A_0 V = A has
// orthogonal columns, so A_0^H A_0 = V diag(|a_v|^2) V^H.  Both matrices are
// column-major in per-item global memory owned by this CTA (written and read
// by its threads only, ordered by __syncthreads).  Same rotation and
// convergence rule as tt_eigenvalues.  Returns false after 60 sweeps.
__device__ bool jacobi_with_vectors(double2* A, int lda, int L, int nv, double2* V, int* rot) {
  constexpr int NW = kNT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int NP = (nv + 1) & ~1;
  const double tol = 2.220446049250313e-16 * L;
  int sweep = 0;
  for (; sweep < 60; ++sweep) {
    if (threadIdx.x == 0) *rot = 0;
    __syncthreads();
    for (int rr = 0; rr < NP - 1; ++rr) {
      for (int pk = warp; pk < NP / 2; pk += NW) {
        const int pos1 = pk, pos2 = NP - 1 - pk;
        const int vp = pos1 == 0 ? 0 : ((pos1 - 1 + rr) % (NP - 1)) + 1;
        const int vq = ((pos2 - 1 + rr) % (NP - 1)) + 1;
        if (vp >= nv || vq >= nv) continue;
        double2* xp = A + (int64_t)vp * lda;
        double2* xq = A + (int64_t)vq * lda;
        double al = 0.0, be = 0.0, gr = 0.0, gi = 0.0;
        for (int i = lane; i < L; i += 32) {
          const double2 u = xp[i], w = xq[i];
          al = fma(u.x, u.x, fma(u.y, u.y, al));
          be = fma(w.x, w.x, fma(w.y, w.y, be));
          gr = fma(u.x, w.x, fma(u.y, w.y, gr));
          gi = fma(u.x, w.y, fma(-u.y, w.x, gi));
        }
#pragma unroll
        for (int off = 16; off; off >>= 1) {
          al += __shfl_xor_sync(0xffffffffu, al, off);
          be += __shfl_xor_sync(0xffffffffu, be, off);
          gr += __shfl_xor_sync(0xffffffffu, gr, off);
          gi += __shfl_xor_sync(0xffffffffu, gi, off);
        }
        const double ga = sqrt(gr * gr + gi * gi);
        if (ga > tol * sqrt(al * be) && ga > 1e-300) {
          if (lane == 0) *rot = 1;
          const double zeta = (be - al) / (2.0 * ga);
          const double t = fabs(zeta) > 1e100 ? 0.5 / zeta
                                              : copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
          const double2 ph = make_double2(gr / ga, -gi / ga);
          for (int i = lane; i < L; i += 32) {
            const double2 u = xp[i];
            const double2 w = cmul(ph, xq[i]);
            xp[i] = make_double2(c * u.x - s * w.x, c * u.y - s * w.y);
            xq[i] = make_double2(s * u.x + c * w.x, s * u.y + c * w.y);
          }
          double2* yp = V + (int64_t)vp * nv;
          double2* yq = V + (int64_t)vq * nv;
          for (int i = lane; i < nv; i += 32) {
            const double2 u = yp[i];
            const double2 w = cmul(ph, yq[i]);
            yp[i] = make_double2(c * u.x - s * w.x, c * u.y - s * w.y);
            yq[i] = make_double2(s * u.x + c * w.x, s * u.y + c * w.y);
          }
        }
      }
      __syncthreads();
    }
    if (!*rot) break;
    __syncthreads();
  }
  return sweep < 60;
}

// One CTA per item: the block of t, Jacobi with vectors, eigenvalues in
// descending order with their eigenvectors, then the window selection.
__global__ void __launch_bounds__(kNT) eigvec_kernel(EigvecArgs a) {
  extern __shared__ double sh[];
  double* tv = sh;                        // [nc] |a_v|^2 by column
  int* order = (int*)(tv + a.nc);         // [nc] column of rank k
  int* rankof = order + a.nc;             // [nc] rank of column v
  __shared__ int s_rot, s_k;
  const int r = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NW = kNT / 32;
  const int nr = a.nr, nc = a.nc;
  double2* A = a.work + (int64_t)r * a.work_stride;
  double2* V = A + (int64_t)nr * nc;
  const double2* src = a.a + (int64_t)r * a.astride;
  for (int64_t e = tid; e < (int64_t)nr * nc; e += kNT) {
    const int i = (int)(e % nr), j = (int)(e / nr);
    A[e] = src[(int64_t)(a.col0 + j) * a.lda + a.row0 + i];
  }
  for (int64_t e = tid; e < (int64_t)nc * nc; e += kNT)
    V[e] = make_double2((e % nc) == (e / nc) ? 1.0 : 0.0, 0.0);
  __syncthreads();
  const bool ok = jacobi_with_vectors(A, nr, nr, nc, V, &s_rot);
  for (int v = warp; v < nc; v += NW) {
    const double2* x = A + (int64_t)v * nr;
    double s = 0.0;
    for (int i = lane; i < nr; i += 32) s = fma(x[i].x, x[i].x, fma(x[i].y, x[i].y, s));
#pragma unroll
    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) tv[v] = s;
  }
  __syncthreads();
  for (int v = tid; v < nc; v += kNT) {
    const double t = tv[v];
    int k = 0;
    for (int j = 0; j < nc; ++j) k += (tv[j] > t || (tv[j] == t && j < v)) ? 1 : 0;
    order[k] = v;
    rankof[v] = k;
    a.tvals[(int64_t)r * nc + k] = t;
  }
  __syncthreads();
  if (a.u) {
    double2* u = a.u + (int64_t)r * nc * nc;
    for (int64_t e = tid; e < (int64_t)nc * nc; e += kNT) {
      const int i = (int)(e % nc), k = (int)(e / nc);
      u[e] = V[(int64_t)order[k] * nc + i];
    }
  }
  if (a.wsel) {
    // Selection in rank order (the reference's loop over iv of tvals).
    if (tid == 0) {
      int k = 0;
      for (int w = 0; w < a.nprof; ++w) a.nt[(int64_t)r * a.nprof + w] = 0;
      double sum = 0.0;
      for (int q = 0; q < nc; ++q) {
        const double t = tv[order[q]];
        sum += t;
        uint32_t bits = 0;
        for (int w = 0; w < a.nprof; ++w) {
          const bool in = a.centered ? (fabs(t - a.wa[w]) <= a.wb[w]) : (a.wa[w] <= t && t <= a.wb[w]);
          if (in) {
            bits |= 1u << w;
            a.nt[(int64_t)r * a.nprof + w] += 1;
          }
        }
        if (bits) {
          a.member[(int64_t)r * nc + k] = bits;
          rankof[k] = order[q];  // reused: column of selected vector k
          ++k;
        }
      }
      s_k = k;
      a.ksel[r] = k;
      if (a.tavg) a.tavg[r] = sum / nc;
    }
    __syncthreads();
    const int k = s_k;
    double2* ws = a.wsel + (int64_t)r * nc * a.M;
    for (int64_t e = tid; e < (int64_t)k * a.M; e += kNT) {
      const int s = (int)(e / a.M), m = (int)(e % a.M);
      const int j = m - a.col0;
      ws[e] = (j >= 0 && j < nc) ? cmul(a.sqmu[m], V[(int64_t)rankof[s] * nc + j]) : make_double2(0.0, 0.0);
    }
  }
  if (tid == 0) a.status[r] = ok ? RG_OK : RG_ERR_NOCONV;
}

// Back-substitution.  Block (chunk, item): the nv <= kKC source vectors
// s0 .. s0+nv-1 of item blockIdx.y.  The M*nv outputs are dealt to the
// threads, e = tid + kNT*j -> row m = e / nv, vector v = e % nv, so the FP64
// work is 16 M^2 nv per slice whatever nv is (an FP64 warp instruction costs
// the same with idle lanes; whole idle warps cost nothing).  Ysh holds
// B Y_{n+1} and Wsh the source vectors, [M][kKC]; Psh the |Y|^2 terms of
// the profile, summed per vector in a fixed order.
template <int JMAX>
__global__ void __launch_bounds__(kNT) back_kernel(BackArgs a) {
  extern __shared__ double2 shb[];
  const int M = a.M;
  double2* Ysh = shb;
  double2* Wsh = shb + M * kKC;
  double* Psh = (double*)(Wsh + M * kKC);
  const int r = blockIdx.y;
  const int kr = a.kcount ? a.kcount[r] : a.kmax;
  const int s0 = blockIdx.x * kKC;
  if (s0 >= kr) return;  // uniform over the block
  const int nv = min(kKC, kr - s0);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nout = M * nv;  // <= kNT * JMAX (checked by the launcher)
  for (int e = tid; e < M * kKC; e += kNT) {
    const int m = e / kKC, vv = e % kKC;
    Wsh[e] = vv < nv ? a.src[(int64_t)r * a.src_stride + (int64_t)(s0 + vv) * M + m] : make_double2(0.0, 0.0);
    Ysh[e] = make_double2(0.0, 0.0);
  }
  __syncthreads();
  const int64_t mm = (int64_t)M * M;
  const int nslices = a.only_lo ? 1 : a.nx - a.i_lo;
  int mj[JMAX], vj[JMAX];  // row and vector of output j (the divisions once, outside the slice loop)
#pragma unroll
  for (int j = 0; j < JMAX; ++j) {
    const int e = tid + kNT * j;
    mj[j] = e < nout ? e / nv : 0;
    vj[j] = e < nout ? e % nv : 0;
  }
  for (int n = a.nx - 1; n >= a.i_lo; --n) {
    const double2* S = a.dump + ((int64_t)r * a.nx + n) * 2 * mm;
    const double2* Z = S + mm;
    const bool first = (n == a.nx - 1);
    double2 acc[JMAX];
#pragma unroll
    for (int j = 0; j < JMAX; ++j) acc[j] = make_double2(0.0, 0.0);
    if (tid < nout) {
      for (int c = 0; c < M; ++c) {
#pragma unroll
        for (int j = 0; j < JMAX; ++j) {
          if (tid + kNT * j < nout) {
            const int m = mj[j], v = vj[j];
            const double2 wc = Wsh[c * kKC + v];
            const double2 z = __ldg(Z + (int64_t)m * M + c);
            acc[j] = make_double2(fma(z.x, wc.x, fma(-z.y, wc.y, acc[j].x)), fma(z.x, wc.y, fma(z.y, wc.x, acc[j].y)));
            if (!first) {
              const double2 yc = Ysh[c * kKC + v];
              const double2 sv = __ldg(S + (int64_t)m * M + c);
              acc[j] = make_double2(fma(-sv.x, yc.x, fma(sv.y, yc.y, acc[j].x)),
                                    fma(-sv.x, yc.y, fma(-sv.y, yc.x, acc[j].y)));
            }
          }
        }
      }
    }
    __syncthreads();  // every thread has read Ysh
#pragma unroll
    for (int j = 0; j < JMAX; ++j) {
      if (tid + kNT * j < nout) {
        const int m = mj[j], v = vj[j];
        const double2 y = acc[j];
        Ysh[m * kKC + v] = cmul(a.bmat[m], y);
        Psh[m * kKC + v] = fma(y.x, y.x, y.y * y.y);
        if (a.out_mode == kBackColumns && (!a.only_lo || n == a.i_lo)) {
          const int64_t sl = a.only_lo ? 0 : n - a.i_lo;
          double2 o = y;
          if (a.left) {
            const double2 q = cmul(a.left[m], y);
            o = make_double2(-2.0 * q.y, 2.0 * q.x);
          }
          a.cols[(((int64_t)r * nslices + sl) * a.kmax + s0 + v) * M + m] = o;
        }
      }
    }
    __syncthreads();  // Ysh and Psh complete
    if (a.out_mode == kBackProfile) {
      for (int v = warp; v < nv; v += kNT / 32) {  // warp v sums vector v over the rows
        double p = 0.0;
        for (int m = lane; m < M; m += 32) p += Psh[m * kKC + v];
#pragma unroll
        for (int off = 16; off; off >>= 1) p += __shfl_xor_sync(0xffffffffu, p, off);
        if (lane == 0) a.prof[((int64_t)r * a.kmax + s0 + v) * a.nx + n] = p;
      }
    }
  }
}

__global__ void windows_kernel(WindowArgs a) {
  const int64_t total = (int64_t)a.nreal * a.nprof * a.nx;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(e % a.nx);
    const int w = (int)((e / a.nx) % a.nprof);
    const int r = (int)(e / ((int64_t)a.nx * a.nprof));
    const int k = a.ksel[r];
    double s = 0.0;
    for (int q = 0; q < k; ++q)
      if ((a.member[(int64_t)r * a.kmax + q] >> w) & 1u) s += a.prof[((int64_t)r * a.kmax + q) * a.nx + n];
    if (a.kind == RG_PROFILE_ITX) {
      s = (s * 2.0) / ((3.141592653589793 * a.wol) * fabs(a.wb[w] - a.wa[w]));
    } else {
      const int nt = a.nt[(int64_t)r * a.nprof + w];
      if (nt != 0) s = s * (4.0 / nt);
    }
    a.out[e] = s;
  }
}

__global__ void wavefun_kernel(WavefunArgs a) {
  const int64_t rows = (int64_t)a.nx * a.ny;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < rows; e += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(e / a.ny), j = (int)(e % a.ny);
    const double2* y = a.y + (int64_t)n * a.M;
    const double2* md = a.modal + (int64_t)j * a.M;
    double re = 0.0, im = 0.0;
    for (int m = 0; m < a.M; ++m) {
      const double2 c = md[m], g = y[m];
      re = fma(c.x, g.x, fma(-c.y, g.y, re));
      im = fma(c.x, g.y, fma(c.y, g.x, im));
    }
    const int id = n - a.nxfree;
    a.out[e] = a.xmesh[n];
    a.out[rows + e] = a.ymesh[j];
    a.out[2 * rows + e] = re;
    a.out[3 * rows + e] = im;
    a.out[4 * rows + e] = (id >= 0 && id < a.nxdiso) ? a.upot[(int64_t)id * a.ny + j] : 0.0;
  }
}

template <int JMAX>
int launch_back_t(const BackArgs& a, cudaStream_t s) {
  const size_t smem = (2 * sizeof(double2) + sizeof(double)) * (size_t)a.M * kKC;
  RG_CUDA(cudaFuncSetAttribute(back_kernel<JMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const dim3 grid((a.kmax + kKC - 1) / kKC, a.nreal);
  back_kernel<JMAX><<<grid, kNT, smem, s>>>(a);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

}  // namespace

int64_t eigvec_work_stride(int nr, int nc) {
  return (((int64_t)nr * nc + (int64_t)nc * nc) + 15) & ~(int64_t)15;
}

int launch_eigvec(const EigvecArgs& a, cudaStream_t s) {
  if (a.nreal <= 0) return RG_OK;
  if (a.nc < 1 || a.nr < 1 || a.nprof > 32) return fail(RG_ERR_INVALID_ARG, "eigvec: invalid sizes");
  const size_t smem = sizeof(double) * a.nc + sizeof(int) * 2 * a.nc;
  RG_CUDA(cudaFuncSetAttribute(eigvec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  eigvec_kernel<<<a.nreal, kNT, smem, s>>>(a);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

int launch_back(const BackArgs& a, cudaStream_t s) {
  if (a.nreal <= 0 || a.kmax <= 0) return RG_OK;
  if (a.i_lo < 0 || a.i_lo >= a.nx) return fail(RG_ERR_INVALID_ARG, "back-substitution: slice out of range");
  const int J = (a.M * kKC + kNT - 1) / kNT;
  if ((2 * sizeof(double2) + sizeof(double)) * (size_t)a.M * kKC > 200 * 1024)
    return fail(RG_ERR_INVALID_ARG, "back-substitution: too many modes");
  if (J <= 2) return launch_back_t<2>(a, s);
  if (J <= 4) return launch_back_t<4>(a, s);
  if (J <= 8) return launch_back_t<8>(a, s);
  if (J <= 16) return launch_back_t<16>(a, s);
  return launch_back_t<32>(a, s);
}

int launch_windows(const WindowArgs& a, cudaStream_t s) {
  const int64_t total = (int64_t)a.nreal * a.nprof * a.nx;
  if (total <= 0) return RG_OK;
  const int grid = (int)std::min<int64_t>((total + 255) / 256, 4096);
  windows_kernel<<<grid, 256, 0, s>>>(a);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

int launch_wavefun(const WavefunArgs& a, cudaStream_t s) {
  const int64_t rows = (int64_t)a.nx * a.ny;
  if (rows <= 0) return RG_OK;
  const int grid = (int)std::min<int64_t>((rows + 255) / 256, 4096);
  wavefun_kernel<<<grid, 256, 0, s>>>(a);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

}  // namespace rg
