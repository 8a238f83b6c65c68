// GB300 (sm_103a) kernels of the recursive Green-function sweep.
//
//   potential_kernel  -- the disorder U(x, y) of each seed, drawn with the
//                        gfortran-style xoshiro256** stream of the reference
//                        (src/random_normal.f90:40-67), one thread per
//                        transverse point using jump-ahead polynomials.
//   sweep_kernel      -- one realization per CTA, persistent over a work
//                        queue: per slice the projection of U onto the modes
//                        (src/waveguide.f90:377-380), then a pivoted complex
//                        Gauss-Jordan elimination that yields both
//                        Gss = inv(A - B Gss B) and Gs1 = -Gss B Gs1
//                        (src/waveguide.f90:426-440, src/base_utils.f90:235-274),
//                        Fisher-Lee t (src/waveguide.f90:443-445, :510) and the
//                        eigenvalues of t^H t by one-sided Jacobi
//                        (src/waveguide.f90:448-449, src/base_utils.f90:341-380).
//   histogram_kernel  -- histogram with the exact edge semantics of
//                        src/base_utils.f90:491-516.
//
// Everything is IEEE FP64.  On GB300 the FP64 pipe (about 1 TFLOP/s for the
// whole chip) is the roofline of the sweep; shared memory, registers and HBM
// have ample headroom, so the kernel keeps each slice matrix resident in
// shared memory and spends its FP64 operations only on the elimination.
#include <algorithm>

#include "rg_device.cuh"

namespace rg {
namespace {

// Thread (iy, r): column iy of realization r.  The reference stream is
// upot(ix, iy) = normal[ix + iy * nxdiso] (reshape, src/waveguide.f90:372),
// each normal consuming two uniforms, so column iy starts 2*nxdiso*iy draws
// into the stream: the state is advanced by the jump polynomial for that
// distance (x^d mod the characteristic polynomial, evaluated by Horner).
__global__ void potential_kernel(PotArgs a) {
  const int iy = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (iy >= a.ny || r >= a.nreal) return;
  Xoshiro st = jump_state(seeded_state(a.seeds[r]), a.jumppoly + 4 * (int64_t)iy);
  double* out = a.upot + (int64_t)r * a.nxdiso * a.ny + iy;
  for (int ix = 0; ix < a.nxdiso; ++ix) out[(int64_t)ix * a.ny] = scaled_normal(a.stdu, st);
}

// ---------------------------------------------------------------------------
// Sweep kernel
// ---------------------------------------------------------------------------
//
// One work item (a realization of one waveguide) per CTA; persistent CTAs
// take items from a work counter, so one launch can mix waveguides of
// different sizes up to MCAP modes.  Per slice the kernel solves X Y = R for
// the slice matrix X = A_n - V_n - B Gss B and the right-hand side
// R = B Gs1 by Gauss-Jordan elimination, which leaves inv(X) = Gss in W and
// Y in R, so the new propagator is Gs1 = -Y.
//
// W (M x M complex) lives in shared memory (row stride LDW = MCAP + 1);
// R (M x M complex) lives in registers: thread (warp w, lane l) owns
// rows w + NW*a and columns l + 32*b.  Keeping R out of shared memory halves
// the footprint so two realizations share an SM, and the serial phases of
// one (pivot search, reciprocal, slice assembly) overlap the other's FP64
// elimination work.
//
// Pivoting is implicit: rows are never swapped.  Step k takes, among rows
// not yet used, the largest max(|re|, |im|) in column k (compared as integer
// bit patterns, so the search costs no FP64 instructions), scales that row
// and eliminates column k from every other row.  After M steps row piv[a] of
// R holds row a of Y, and W holds inv(X) with permuted rows and columns.  The
// next slice keeps every R row in place: physical row q then carries logical
// row pinv[q], so R is only rescaled by B, and W is rebuilt by a gather that
// stays inside each row.
//
// The disorder is drawn in the kernel: each transverse column iy has its own
// xoshiro256** state (jumped to the column's start in the reference stream)
// in the CTA's workspace, advanced by two draws per disordered slice.
template <int MCAP>
struct SweepSmem {
  static constexpr int LDW = MCAP + 1;
  static size_t bytes(int max_ny) {
    const int nyp = (max_ny + 1) & ~1;
    return sizeof(double2) * ((size_t)MCAP * LDW + 3 * MCAP) + sizeof(double) * (2 * MCAP + 2 + nyp) +
           sizeof(int) * 5 * MCAP;
  }
};

// Per-CTA workspace of the shared-memory kernel: generator states only.
inline int64_t small_stride(int max_ny) { return ((2 * (int64_t)max_ny) + 15) & ~(int64_t)15; }

template <int MCAP, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) sweep_kernel(SweepArgs a) {
  constexpr int NW = NT / 32;
  constexpr int LDW = SweepSmem<MCAP>::LDW;
  constexpr int AMAX = (MCAP + NW - 1) / NW;  // rows per warp
  constexpr int CB = (MCAP + 31) / 32;        // column blocks per lane
  constexpr int TMAX = (MCAP * MCAP + NT - 1) / NT;
  extern __shared__ double2 smem[];
  double2* W = smem;                           // [MCAP][LDW]
  double2* colbuf = W + MCAP * LDW;            // [MCAP] column k before the update
  double2* rowW = colbuf + MCAP;               // [MCAP] scaled pivot row of W
  double2* rowR = rowW + MCAP;                 // [MCAP] scaled pivot row of R
  double* cc = (double*)(rowR + MCAP);         // [2*MCAP+2] projection coefficients
  double* urow = cc + (2 * MCAP + 2);          // [max_ny] potential of the slice
  int* piv = (int*)(urow + ((a.max_ny + 1) & ~1));  // [MCAP] pivot row of column k
  int* pinv = piv + MCAP;                      // [MCAP] column of which row q was pivot
  int* sinv = pinv + MCAP;                     // [MCAP] physical row of logical row c
  int* colmap = sinv + MCAP;                   // [MCAP] W column holding Gss column c
  int* used = colmap + MCAP;                   // [MCAP]
  __shared__ int s_r, s_p, s_status, s_rot;
  __shared__ double2 s_d;
  __shared__ WgDesc wd;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint64_t* gen = (uint64_t*)(a.work + (int64_t)blockIdx.x * a.work_stride);  // [max_ny][4]
  const bool draw = (a.upot == nullptr);
  const bool tmat = (a.mode == kModeTmat);
  const bool refl = (a.mode == kModeRefl);
  double2 R[AMAX][CB];

  for (;;) {
    if (tid == 0) {
      const int q = atomicAdd(a.work_counter, 1);
      const int nq = a.count_ptr ? *a.count_ptr : a.nreal;
      s_r = q < nq ? (a.item_idx ? a.item_idx[q] : q) : -1;
      if (s_r >= 0) wd = a.wgs[a.item_wg ? a.item_wg[s_r] : 0];
    }
    __syncthreads();
    const int r = s_r;  // item index (queue position mapped through item_idx)
    if (r < 0) break;
    const int M = wd.M, ny = wd.ny, nx = wd.nx;
    if (tid == 0) s_status = RG_OK;
    for (int c = tid; c < M; c += NT) {
      sinv[c] = c;
      used[c] = 0;
    }
#pragma unroll
    for (int ai = 0; ai < AMAX; ++ai)
#pragma unroll
      for (int b = 0; b < CB; ++b)
        R[ai][b] = make_double2((warp + NW * ai) == (lane + 32 * b) ? 1.0 : 0.0, 0.0);
    if (draw) {
      for (int iy = tid; iy < ny; iy += NT) {
        const Xoshiro st = jump_state(seeded_state(a.seeds[r]), wd.jumppoly + 4 * (int64_t)iy);
        gen[4 * iy + 0] = st.s0;
        gen[4 * iy + 1] = st.s1;
        gen[4 * iy + 2] = st.s2;
        gen[4 * iy + 3] = st.s3;
      }
    }
    const double* U = draw ? nullptr : a.upot + (int64_t)r * a.pot_rstride;
    __syncthreads();

    for (int n = 0; n < nx; ++n) {
      const int id = (refl ? nx - 1 - n : n) - wd.nxfree;  // slice of the guide swept at step n
      const bool dis = (id >= 0 && id < wd.nxdiso);
      if (dis) {
        // 1. This slice's potential row (drawn or loaded) and its projection.
        if (draw) {
          for (int iy = tid; iy < ny; iy += NT) {
            Xoshiro st{gen[4 * iy], gen[4 * iy + 1], gen[4 * iy + 2], gen[4 * iy + 3]};
            urow[iy] = scaled_normal(wd.stdu, st);
            gen[4 * iy + 0] = st.s0;
            gen[4 * iy + 1] = st.s1;
            gen[4 * iy + 2] = st.s2;
            gen[4 * iy + 3] = st.s3;
          }
        } else {
          for (int j = tid; j < ny; j += NT) urow[j] = U[(int64_t)id * a.pot_xstride + (int64_t)j * a.pot_ystride];
        }
        __syncthreads();
        if (!wd.periodic) {
          // cc[d] = (1/ny) sum_j U_j cos(pi d y_j), d = 0..2M, so that
          // (modal^T diag(U) modal)[a][c] = cc[|a-c|] - cc[a+c+2].
          const int nd = 2 * M + 1;
          for (int d = tid; d < nd; d += NT) {
            const double* ct = wd.costab + d;
            double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
            int j = 0;
            for (; j + 4 <= ny; j += 4) {
              s0 = fma(ct[(int64_t)(j + 0) * nd], urow[j + 0], s0);
              s1 = fma(ct[(int64_t)(j + 1) * nd], urow[j + 1], s1);
              s2 = fma(ct[(int64_t)(j + 2) * nd], urow[j + 2], s2);
              s3 = fma(ct[(int64_t)(j + 3) * nd], urow[j + 3], s3);
            }
            for (; j < ny; ++j) s0 = fma(ct[(int64_t)j * nd], urow[j], s0);
            cc[d] = (s0 + s1) + (s2 + s3);
          }
        } else {
          // f[d] = (1/ny) sum_j U_j exp(2 pi i d y_j), d = 0..M-1, so that
          // (modal^H diag(U) modal)[a][c] = f[c-a] (c >= a), conj(f[a-c]) else.
          for (int d = tid; d < M; d += NT) {
            const double2* et = wd.expfac + d;
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < ny; ++j) {
              const double2 e = et[(int64_t)j * M];
              sr = fma(e.x, urow[j], sr);
              si = fma(e.y, urow[j], si);
            }
            cc[2 * d] = sr;
            cc[2 * d + 1] = si;
          }
        }
        __syncthreads();
      }

      // 2. Assemble X = A_n - V_n - B Gss B in physical row order (W), and
      //    R = B Gs1 (identity on the first slice; registers, in place).
      const double2* adiag = (n == 0 || n == nx - 1) ? wd.adiag_edge : wd.adiag_bulk;
      const double rsign = (n == 1) ? 1.0 : -1.0;  // Gs1 = +Y after slice 1, -Y after later slices
#pragma unroll
      for (int ai = 0; ai < AMAX; ++ai) {
        const int q = warp + NW * ai;
        if (q < M) {
          const int al = (n == 0) ? q : pinv[q];  // logical row carried by physical row q
          const double2 ba = wd.bmat[al];
          double2 v[CB];
#pragma unroll
          for (int b = 0; b < CB; ++b) {
            const int c = lane + 32 * b;
            double2 x = make_double2(0.0, 0.0);
            if (c < M) {
              if (al == c) x = adiag[c];
              if (dis) {
                double2 vac;
                if (!wd.periodic) {
                  const int dd = al > c ? al - c : c - al;
                  vac = make_double2(cc[dd] - cc[al + c + 2], 0.0);
                } else {
                  vac = (c >= al) ? make_double2(cc[2 * (c - al)], cc[2 * (c - al) + 1])
                                  : make_double2(cc[2 * (al - c)], -cc[2 * (al - c) + 1]);
                }
                x = csub(x, vac);
              }
              if (n > 0) x = csub(x, cmul(cmul(ba, W[q * LDW + colmap[c]]), wd.bmat[c]));
              if (n > 0) R[ai][b] = cmul(ba, cscale(rsign, R[ai][b]));
            }
            v[b] = x;
          }
          __syncwarp();
#pragma unroll
          for (int b = 0; b < CB; ++b) {
            const int c = lane + 32 * b;
            if (c < M) W[q * LDW + c] = v[b];
          }
        }
      }
      __syncthreads();

      // 3. Gauss-Jordan elimination, three barriers per step:
      //    A: warp 0 finds the pivot row p of column k and d = 1/X[p][k];
      //    B: the scaled pivot rows of W and R go to shared memory;
      //    C: every thread updates its W and R elements.
      for (int k = 0; k < M; ++k) {
        if (warp == 0) {
          unsigned long long best = 0ULL;
          int bi = 0x7fffffff;
          for (int i = lane; i < M; i += 32) {
            const double2 x = W[i * LDW + k];
            colbuf[i] = x;
            const unsigned long long key = used[i] ? 0ULL : pivot_key(x);
            if (key > best) {
              best = key;
              bi = i;
            }
          }
#pragma unroll
          for (int off = 16; off; off >>= 1) {
            const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, off);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ob > best || (ob == best && oi < bi)) {
              best = ob;
              bi = oi;
            }
          }
          if (lane == 0) {
            double2 d = make_double2(0.0, 0.0);
            if (best == 0ULL) {  // zero or NaN column: numerically singular
              s_status = RG_ERR_SINGULAR;
              bi = 0;
              while (bi < M - 1 && used[bi]) ++bi;
            } else {
              const double2 z = colbuf[bi];
              const double rden = 1.0 / fma(z.x, z.x, z.y * z.y);
              d = make_double2(z.x * rden, -z.y * rden);
            }
            used[bi] = 1;
            piv[k] = bi;
            pinv[bi] = k;
            s_p = bi;
            s_d = d;
          }
        }
        __syncthreads();
        const int p = s_p;
        const double2 d = s_d;
        for (int J = tid; J < M; J += NT) rowW[J] = (J == k) ? d : cmul(W[p * LDW + J], d);
        if (warp == p % NW) {
          const int ap = p / NW;
#pragma unroll
          for (int b = 0; b < CB; ++b) {
            const int j = lane + 32 * b;
            double2 val = R[0][b];
#pragma unroll
            for (int ai = 1; ai < AMAX; ++ai)
              if (ai == ap) val = R[ai][b];
            if (j < M) rowR[j] = cmul(val, d);
          }
        }
        __syncthreads();
        double2 rw[CB], rr[CB];
#pragma unroll
        for (int b = 0; b < CB; ++b) {
          const int J = lane + 32 * b;
          rw[b] = (J < M) ? rowW[J] : make_double2(0.0, 0.0);
          rr[b] = (J < M) ? rowR[J] : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int ai = 0; ai < AMAX; ++ai) {
          const int i = warp + NW * ai;
          if (i < M) {
            const double2 f = colbuf[i];
            const bool isp = (i == p);
            double2 wv[CB];
#pragma unroll
            for (int b = 0; b < CB; ++b) {
              const int J = lane + 32 * b;
              wv[b] = (J < M && J != k) ? W[i * LDW + J] : make_double2(0.0, 0.0);
            }
#pragma unroll
            for (int b = 0; b < CB; ++b) {
              const int J = lane + 32 * b;
              wv[b] = isp ? rw[b] : cfms(wv[b], f, rw[b]);
              R[ai][b] = isp ? rr[b] : cfms(R[ai][b], f, rr[b]);
              if (J < M) W[i * LDW + J] = wv[b];
            }
          }
        }
        __syncthreads();
      }

      // 4. Permutation bookkeeping for the next slice.
      for (int c = tid; c < M; c += NT) {
        const int cm = pinv[sinv[c]];
        sinv[c] = piv[c];
        colmap[c] = cm;
        used[c] = 0;
      }
      __syncthreads();
    }

    if (refl) {
      // 5'. Reflection: after the reverse sweep W holds G(x_1; x_1) with
      //     G11[a][c] = W[piv[a]][colmap[c]];  r = -1 + 2i sqmu_a G11 sqmu_c
      //     with sqrt(real(mu)) (src/waveguide.f90:510-512).
      double2* rout = a.tout + (int64_t)r * M * M;
      for (int e = tid; e < M * M; e += NT) {
        const int i = e % M, j = e / M;
        const double2 v = cmul(cmul(wd.sqmu_r[i], W[piv[i] * LDW + colmap[j]]), wd.sqmu_r[j]);
        rout[e] = make_double2((i == j ? -1.0 : 0.0) - 2.0 * v.y, 2.0 * v.x);
      }
      __syncthreads();
      if (tid == 0) a.status[r] = s_status;
      continue;
    }

    // 5. Fisher-Lee: Gs1[a][j] = sign * R[piv[a]][j]; t = 2i sqmu_a Gs1 sqmu_j.
    //    R goes to shared memory (physical rows), t is formed in registers
    //    and then stored over it for the eigenvalue stage.
#pragma unroll
    for (int ai = 0; ai < AMAX; ++ai) {
      const int q = warp + NW * ai;
#pragma unroll
      for (int b = 0; b < CB; ++b) {
        const int j = lane + 32 * b;
        if (q < M && j < M) W[q * LDW + j] = R[ai][b];
      }
    }
    __syncthreads();
    const double gsign = (nx >= 2) ? -1.0 : 1.0;
    const int row0 = tmat ? 0 : wd.row0, col0 = tmat ? 0 : wd.col0;
    const int nrow = tmat ? M : wd.nrow, ncol = tmat ? M : wd.ncol;
    const double2* sqmu = tmat ? wd.sqmu_r : wd.sqmu_c;
    double2* tout = a.tout ? a.tout + (int64_t)r * nrow * ncol : nullptr;
    double2 tv[TMAX];
#pragma unroll
    for (int s = 0; s < TMAX; ++s) {
      const int e = tid + NT * s;
      tv[s] = make_double2(0.0, 0.0);
      if (e < nrow * ncol) {
        const int i = e % nrow, j = e / nrow;
        const int gi = row0 + i, gj = col0 + j;
        const double2 g = cscale(gsign, W[piv[gi] * LDW + gj]);
        const double2 v = cmul(cmul(sqmu[gi], g), sqmu[gj]);
        tv[s] = make_double2(-2.0 * v.y, 2.0 * v.x);  // (0, 2) * v
        if (tout) tout[e] = tv[s];
      }
    }
    __syncthreads();

    if (!tmat) {
#pragma unroll
      for (int s = 0; s < TMAX; ++s) {
        const int e = tid + NT * s;
        if (e < nrow * ncol) W[(e % nrow) * LDW + e / nrow] = tv[s];
      }
      __syncthreads();
      // 6. Eigenvalues of t^H t, sorted descending into teig.
      const int64_t obase = a.teig_off ? a.teig_off[r] : (int64_t)r * wd.neigv;
      if (!tt_eigenvalues<NT>(W, LDW, nrow, ncol, wd.neigv, cc, &s_rot, a.teig + obase) && tid == 0)
        s_status = RG_ERR_NOCONV;
    }
    __syncthreads();
    if (tid == 0) a.status[r] = s_status;
  }
}

// ---------------------------------------------------------------------------
// Histogram
// ---------------------------------------------------------------------------
__global__ void histogram_kernel(const double* __restrict__ x, int64_t n, const double* __restrict__ bins,
                                 int nbins, unsigned long long* counts) {
  extern __shared__ unsigned long long hs[];  // [nbins + 1]; the last slot counts missing samples
  for (int i = threadIdx.x; i <= nbins; i += blockDim.x) hs[i] = 0ULL;
  __syncthreads();
  const double b0 = bins[0], bn = bins[nbins];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[e];
    if (v < b0 || bn < v) {
      atomicAdd(&hs[nbins], 1ULL);
    } else if (v == bn) {
      atomicAdd(&hs[nbins - 1], 1ULL);
    } else if (v == v) {  // NaN is neither counted nor missing
      int lo = 1, hi = nbins;  // first edge index in [1, nbins] with v < bins[idx]
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (v < bins[mid]) hi = mid;
        else lo = mid + 1;
      }
      atomicAdd(&hs[lo - 1], 1ULL);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= nbins; i += blockDim.x)
    if (hs[i]) atomicAdd(&counts[i], hs[i]);
}

template <int MCAP, int NT, int MINB>
int plan_t(SweepArgs& a, int sm_count, int* grid, int64_t* stride) {
  a.cluster = 1;
  const size_t smem = SweepSmem<MCAP>::bytes(a.max_ny);
  RG_CUDA(cudaFuncSetAttribute(sweep_kernel<MCAP, NT, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_kernel<MCAP, NT, MINB>, NT, smem));
  if (per_sm < 1) return fail(RG_ERR_INVALID_ARG, "sweep kernel does not fit on an SM (ny too large?)");
  if (a.force_per_sm > 0 && a.force_per_sm < per_sm) per_sm = a.force_per_sm;
  int g = per_sm * sm_count;
  if (g > a.nreal) g = a.nreal;
  *grid = g < 1 ? 1 : g;
  *stride = small_stride(a.max_ny);
  return RG_OK;
}

template <int MCAP, int NT, int MINB>
int launch_t(const SweepArgs& a, cudaStream_t stream, int grid) {
  sweep_kernel<MCAP, NT, MINB><<<grid, NT, SweepSmem<MCAP>::bytes(a.max_ny), stream>>>(a);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

}  // namespace

int launch_potential(const PotArgs& a, cudaStream_t stream) {
  if (a.nreal <= 0) return RG_OK;
  dim3 block(128), grid((a.ny + 127) / 128, a.nreal);
  potential_kernel<<<grid, block, 0, stream>>>(a);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

// Kernel choice: the blocked kernel when forced or above kMaxModesSmem
// modes; otherwise the pivoted shared-memory kernel, preceded by the
// symmetric kernel when a.symmetric is set.  Both shared-memory kernels then
// run on the same grid and per-CTA workspace (the larger of their plans).
int sweep_plan(SweepArgs& a, int sm_count, int* grid, int64_t* work_stride) {
  if (a.force_large || a.max_M > kMaxModesSmem) {
    // The symmetric blocked kernel, unless segment states are asked for (the
    // adjoint's recomputation forces the pivoted one); the pivoted re-run
    // uses the same cluster size, grid and workspace.
    if (!a.symmetric || a.force_large || a.state_in || a.state_dump || a.state_out || a.inject_at) {
      a.symmetric = 0;
      return sweep_large_plan(a, sm_count, grid, work_stride);
    }
    int rc = sweep_large_sym_plan(a, sm_count, grid, work_stride);
    if (rc) return rc;
    SweepArgs b = a;
    b.symmetric = 0;
    b.force_cluster = a.cluster;
    int g2 = 0;
    int64_t s2 = 0;
    if ((rc = sweep_large_plan(b, sm_count, &g2, &s2))) return rc;
    if (b.cluster != a.cluster) {  // the pivoted kernel cannot run clusters of this size
      a.symmetric = 0;
      return sweep_large_plan(a, sm_count, grid, work_stride);
    }
    *grid = std::max(*grid, g2);
    *work_stride = std::max(*work_stride, s2);
    return RG_OK;
  }
  // The shared-memory kernels run whole guides from slice 0 and keep no
  // per-slice states (the symmetric one keeps them when launched directly).
  if (a.n_end != 0 || a.state_in || a.state_dump || a.state_out || a.inject_at)
    return fail(RG_ERR_INVALID_ARG, "sweep: segment arguments need the blocked kernel (force_large)");
  int rc;
  if (a.max_M <= 16) rc = plan_t<16, 64, 8>(a, sm_count, grid, work_stride);
  else if (a.max_M <= 32) rc = plan_t<32, 128, 4>(a, sm_count, grid, work_stride);
  else rc = plan_t<64, 256, 2>(a, sm_count, grid, work_stride);
  if (rc || !a.symmetric) return rc;
  int g2 = 0;
  int64_t s2 = 0;
  if ((rc = sweep_sym_plan(a, sm_count, &g2, &s2))) return rc;
  *grid = std::max(*grid, g2);
  *work_stride = std::max(*work_stride, s2);
  return RG_OK;
}

int launch_sweep(const SweepArgs& a, cudaStream_t stream, int grid) {
  if (a.nreal <= 0) return RG_OK;
  const bool blocked = a.force_large || a.max_M > kMaxModesSmem;
  if (!a.symmetric) {
    if (blocked) return launch_sweep_large(a, stream, grid);
  } else if (!a.flag_list) {
    return fail(RG_ERR_INVALID_ARG, "symmetric sweep: no flag list");
  }
  const SweepArgs* p = &a;
  SweepArgs rerun;
  if (a.symmetric) {
    int rc = blocked ? launch_sweep_large_sym(a, stream, grid) : launch_sweep_sym(a, stream, grid);
    if (rc) return rc;
    // The pivoted kernel takes the flagged items: queue length in counter 1,
    // its own queue position in counter 2.
    rerun = a;
    rerun.symmetric = 0;
    rerun.item_idx = a.flag_list;
    rerun.count_ptr = a.work_counter + 1;
    rerun.work_counter = a.work_counter + 2;
    p = &rerun;
    if (blocked) return launch_sweep_large(rerun, stream, grid);
  }
  if (a.max_M <= 16) return launch_t<16, 64, 8>(*p, stream, grid);
  if (a.max_M <= 32) return launch_t<32, 128, 4>(*p, stream, grid);
  return launch_t<64, 256, 2>(*p, stream, grid);
}

int launch_histogram(const double* d_samples, int64_t n, const double* d_bins, int nbins,
                     unsigned long long* d_counts, cudaStream_t stream) {
  const size_t smem = sizeof(unsigned long long) * (nbins + 1);
  if (smem > 200 * 1024) return fail(RG_ERR_INVALID_ARG, "too many histogram bins");
  if (smem > 48 * 1024)
    RG_CUDA(cudaFuncSetAttribute(histogram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t blocks = (n + 255) / 256;
  if (blocks > 1024) blocks = 1024;
  if (blocks < 1) blocks = 1;
  histogram_kernel<<<(int)blocks, 256, smem, stream>>>(d_samples, n, d_bins, nbins, d_counts);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

}  // namespace rg
