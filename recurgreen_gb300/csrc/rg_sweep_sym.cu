// Symmetric recursive Green sweep for Dirichlet guides of up to 64 modes.
//
// With Dirichlet modes the slice matrix X_n = A_n - V_n - B Gss B is complex
// symmetric (A and B diagonal, V real symmetric, and Gss = inv(X_{n-1}) is
// symmetric in turn), so Gss can be formed by a symmetric Gauss-Jordan sweep
// that keeps only the upper triangle of W: step k pivots on the diagonal
// element (p, p) of largest max(|re|, |im|) among the indices not yet swept.
// After sweeping the set S the in-place matrix satisfies
// M[i][j] = M[j][i] when i and j are both in S or both outside it, and
// M[i][j] = -M[j][i] otherwise, so the triangle plus the swept flags
// determine it.  Sweeping p with d = 1/M[p][p] and r_k = M[p][k]:
//   g_i = M[i][p] = r_i (i unswept) or -r_i (i swept),
//   M[i][j] -= g_i d r_j            (i, j != p),
//   M[p][j]  = d r_j,  M[i][p] = -g_i d,  M[p][p] = d,
//   R[i]    -= g_i d R[p],  R[p] = d R[p].
// When every index is swept, W = inv(X) in natural order and R = inv(X) R,
// with no row or column permutation to track.  The W update costs half of
// the general elimination's, so a slice costs 12 M^3 instead of 16 M^3 FP64
// flops (src/waveguide.f90:426-440 does 16 M^3: zgetrf+zgetri and a matmul).
//
// Diagonal pivoting is not partial pivoting: if a pivot's magnitude falls
// below sym_tau times the largest unswept entry of its row, the item is
// flagged (kStatusNeedPivot), its index appended to a.flag_list, and it is
// recomputed by the pivoted kernel, which launch_sweep starts on that list.
#include "rg_device.cuh"

namespace rg {
namespace {

template <int MCAP>
struct SymSmem {
  static constexpr int LDW = MCAP + 1;
  static constexpr int TRI = MCAP * (MCAP + 1) / 2;
  static size_t bytes(int max_ny) {
    const int nyp = (max_ny + 1) & ~1;
    return sizeof(double2) * ((size_t)MCAP * LDW + 3 * MCAP) + sizeof(double) * (2 * MCAP + 2 + nyp) +
           sizeof(int) * (TRI + MCAP);
  }
};

inline int64_t sym_stride(int max_ny) { return ((2 * (int64_t)max_ny) + 15) & ~(int64_t)15; }

template <int MCAP, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) sweep_sym_kernel(SweepArgs a) {
  constexpr int NW = NT / 32;
  constexpr int LDW = SymSmem<MCAP>::LDW;
  constexpr int TRI = SymSmem<MCAP>::TRI;
  constexpr int AMAX = (MCAP + NW - 1) / NW;  // R rows per warp
  constexpr int CB = (MCAP + 31) / 32;        // R column blocks per lane
  constexpr int SMAX = (TRI + NT - 1) / NT;   // triangle elements per thread
  constexpr int TMAX = (MCAP * MCAP + NT - 1) / NT;
  extern __shared__ double2 smem[];
  double2* W = smem;                           // [MCAP][LDW], upper triangle used
  double2* gcol = W + MCAP * LDW;              // [MCAP] g_i = M[i][p]
  double2* rowW = gcol + MCAP;                 // [MCAP] d r_j (new row p of W)
  double2* rowR = rowW + MCAP;                 // [MCAP] d R[p]
  double* cc = (double*)(rowR + MCAP);         // [2*MCAP+2] projection coefficients
  double* urow = cc + (2 * MCAP + 2);          // [max_ny] potential of the slice
  int* tri = (int*)(urow + ((a.max_ny + 1) & ~1));  // [TRI] (i << 16) | j of triangle element e
  int* used = tri + TRI;                       // [MCAP] swept flags
  __shared__ int s_r, s_p, s_status, s_rot, s_M;
  __shared__ double2 s_d;
  __shared__ WgDesc wd;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  uint64_t* gen = (uint64_t*)(a.work + (int64_t)blockIdx.x * a.work_stride);  // [max_ny][4]
  const bool draw = (a.upot == nullptr);
  const bool tmat = (a.mode == kModeTmat);
  const bool refl = (a.mode == kModeRefl);
  double2 R[AMAX][CB];
  if (tid == 0) s_M = -1;

  for (;;) {
    if (tid == 0) {
      s_r = atomicAdd(a.work_counter, 1);
      if (s_r < a.nreal) wd = a.wgs[a.item_wg ? a.item_wg[s_r] : 0];
    }
    __syncthreads();
    const int r = s_r;
    if (r >= a.nreal) break;
    const int M = wd.M, ny = wd.ny, nx = wd.nx;
    const int T = M * (M + 1) / 2;
    if (s_M != M) {  // triangle index table for this size
      for (int i = tid; i < M; i += NT) {
        const int base = i * M - i * (i - 1) / 2;  // elements of rows 0..i-1
        for (int j = i; j < M; ++j) tri[base + (j - i)] = (i << 16) | j;
      }
    }
    __syncthreads();
    if (tid == 0) {
      s_M = M;
      s_status = wd.periodic ? kStatusNeedPivot : RG_OK;  // periodic X is Hermitian, not symmetric
    }
    // R starts as the identity source at slice 0, or as zero when the source
    // is at a later slice (a.inject_at).
    const double one = a.inject_at > 0 ? 0.0 : 1.0;
#pragma unroll
    for (int ai = 0; ai < AMAX; ++ai)
#pragma unroll
      for (int b = 0; b < CB; ++b)
        R[ai][b] = make_double2((warp + NW * ai) == (lane + 32 * b) ? one : 0.0, 0.0);
    if (draw) {
      // Each generator state is set up by the thread that draws from it (the
      // pair (j, ny-1-j) of the projection step).
      for (int j = tid; j < (ny >> 1) + (ny & 1); j += NT) {
        for (int h2 = 0; h2 < 2; ++h2) {
          const int iy = h2 == 0 ? j : ny - 1 - j;
          if (h2 == 1 && iy == j) break;
          const Xoshiro st = jump_state(seeded_state(a.seeds[r]), wd.jumppoly + 4 * (int64_t)iy);
          gen[4 * iy + 0] = st.s0;
          gen[4 * iy + 1] = st.s1;
          gen[4 * iy + 2] = st.s2;
          gen[4 * iy + 3] = st.s3;
        }
      }
    }
    const double* U = draw ? nullptr : a.upot + (int64_t)r * a.pot_rstride;
    __syncthreads();

    for (int n = 0; n < nx; ++n) {
      if (s_status == kStatusNeedPivot) break;  // the pivoted kernel redoes this item
      const int id = (refl ? nx - 1 - n : n) - wd.nxfree;
      const bool dis = (id >= 0 && id < wd.nxdiso);
      if (dis) {
        // 1. This slice's potential row and its projection coefficients
        //    cc[d] = sum_j costab[j][d] U_j.  The transverse grid is symmetric
        //    (y_{ny-1-j} = 1 - y_j) and cos(pi d (1 - y)) = (-1)^d cos(pi d y),
        //    so the points pair up: urow[j] = U_j + U_j', urow[j'] = U_j - U_j'
        //    (j < ny/2, j' = ny-1-j), and even d sums costab[j][d] urow[j],
        //    odd d sums costab[j][d] urow[j'], over half the points.
        const int h = ny >> 1;
        for (int j = tid; j < h + (ny & 1); j += NT) {
          const int jp = ny - 1 - j;
          double u0 = 0.0, u1 = 0.0;
          if (draw) {
            Xoshiro st{gen[4 * j], gen[4 * j + 1], gen[4 * j + 2], gen[4 * j + 3]};
            u0 = scaled_normal(wd.stdu, st);
            gen[4 * j + 0] = st.s0;
            gen[4 * j + 1] = st.s1;
            gen[4 * j + 2] = st.s2;
            gen[4 * j + 3] = st.s3;
            if (jp != j) {
              Xoshiro sq{gen[4 * jp], gen[4 * jp + 1], gen[4 * jp + 2], gen[4 * jp + 3]};
              u1 = scaled_normal(wd.stdu, sq);
              gen[4 * jp + 0] = sq.s0;
              gen[4 * jp + 1] = sq.s1;
              gen[4 * jp + 2] = sq.s2;
              gen[4 * jp + 3] = sq.s3;
            }
          } else {
            u0 = U[(int64_t)id * a.pot_xstride + (int64_t)j * a.pot_ystride];
            u1 = U[(int64_t)id * a.pot_xstride + (int64_t)jp * a.pot_ystride];
          }
          if (jp == j) {
            urow[j] = u0;  // middle point of an odd grid
          } else {
            urow[j] = u0 + u1;
            urow[jp] = u0 - u1;
          }
        }
        __syncthreads();
        // Coefficients d < NT/2 take one thread each in the first half of the
        // CTA (one warp per SMSP); d = NT/2 = 2*MCAP, present when M = MCAP,
        // takes one warp of the second half with a shuffle reduction.
        const int nd = 2 * M + 1;
        if (tid < NT / 2) {
          for (int d = tid; d < nd && d < NT / 2; d += NT / 2) {
            const double* ct = wd.costab + d;
            const double* up = (d & 1) ? urow + (ny - 1) : urow;
            const int us = (d & 1) ? -1 : 1;
            double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
            int j = 0;
            for (; j + 4 <= h; j += 4) {
              s0 = fma(ct[(int64_t)(j + 0) * nd], up[us * (j + 0)], s0);
              s1 = fma(ct[(int64_t)(j + 1) * nd], up[us * (j + 1)], s1);
              s2 = fma(ct[(int64_t)(j + 2) * nd], up[us * (j + 2)], s2);
              s3 = fma(ct[(int64_t)(j + 3) * nd], up[us * (j + 3)], s3);
            }
            for (; j < h; ++j) s0 = fma(ct[(int64_t)j * nd], up[us * j], s0);
            if (ny & 1) s1 = fma(ct[(int64_t)h * nd], urow[h], s1);
            cc[d] = (s0 + s1) + (s2 + s3);
          }
        } else if (warp == NW / 2 && nd > NT / 2) {
          const int d = NT / 2;  // even
          const double* ct = wd.costab + d;
          double s0 = 0.0;
          for (int j = lane; j < h; j += 32) s0 = fma(ct[(int64_t)j * nd], urow[j], s0);
          if ((ny & 1) && lane == 0) s0 = fma(ct[(int64_t)h * nd], urow[h], s0);
#pragma unroll
          for (int off = 16; off; off >>= 1) s0 += __shfl_xor_sync(0xffffffffu, s0, off);
          if (lane == 0) cc[d] = s0;
        }
        __syncthreads();
      }

      // 2. X = A_n - V_n - B Gss B on the upper triangle, in place (each
      //    element is read and written by one thread), and R = B Gs1.
      const double2* adiag = (n == 0 || n == nx - 1) ? wd.adiag_edge : wd.adiag_bulk;
      const double rsign = (n == 1) ? 1.0 : -1.0;
      const int arot = (tid + NT - 32 * (n % NW)) % NT;  // the partial chunk rotates over the warps
#pragma unroll
      for (int s = 0; s < SMAX; ++s) {
        const int e = arot + NT * s;
        if (e < T) {
          const int i = tri[e] >> 16, j = tri[e] & 0xffff;
          double2 x = (i == j) ? adiag[i] : make_double2(0.0, 0.0);
          if (dis) x = csub(x, make_double2(cc[j - i] - cc[i + j + 2], 0.0));
          if (n > 0) x = csub(x, cmul(cmul(wd.bmat[i], W[i * LDW + j]), wd.bmat[j]));
          W[i * LDW + j] = x;
        }
      }
      if (n > 0 && n == a.inject_at) {
        // The identity source at this slice: Z_n = S_n I, stored as R = -S_n
        // (Gs1 = -R after slice 0), so the right-hand side is -I.
#pragma unroll
        for (int ai = 0; ai < AMAX; ++ai)
#pragma unroll
          for (int b = 0; b < CB; ++b)
            R[ai][b] = make_double2((warp + NW * ai) == (lane + 32 * b) ? -1.0 : 0.0, 0.0);
      } else if (n > 0) {
#pragma unroll
        for (int ai = 0; ai < AMAX; ++ai) {
          const int q = warp + NW * ai;
          if (q < M) {
            const double2 bq = wd.bmat[q];
#pragma unroll
            for (int b = 0; b < CB; ++b) R[ai][b] = cmul(bq, cscale(rsign, R[ai][b]));
          }
        }
      }
      for (int c = tid; c < M; c += NT) used[c] = 0;
      __syncthreads();

      // 3. Symmetric Gauss-Jordan, three barriers per step.  Phase A runs on
      //    warp k % NW and the partial chunk of the triangle update on warp
      //    (k + 2) % NW, so their extra FP64 work rotates over the SMSPs.
      for (int k = 0; k < M; ++k) {
        if (warp == k % NW) {
          // A. pivot: the largest unswept diagonal element
          unsigned long long best = 0ULL;
          int bi = 0x7fffffff;
          for (int i = lane; i < M; i += 32) {
            const unsigned long long key = used[i] ? 0ULL : pivot_key(W[i * LDW + i]);
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
          bool singular = (best == 0ULL);
          if (singular) {  // zero or NaN diagonal: let the pivoted kernel decide
            bi = 0;
            while (bi < M - 1 && used[bi]) ++bi;
          }
          const int p = bi;
          double2 d = make_double2(0.0, 0.0);
          if (lane == 0 && !singular) {
            const double2 z = W[p * LDW + p];
            const double rden = 1.0 / fma(z.x, z.x, z.y * z.y);
            d = make_double2(z.x * rden, -z.y * rden);
          }
          d.x = __shfl_sync(0xffffffffu, d.x, 0);
          d.y = __shfl_sync(0xffffffffu, d.y, 0);
          // row p: r_j = M[p][j]; g_j = M[j][p]
          unsigned long long offmax = 0ULL;
          for (int j = lane; j < M; j += 32) {
            double2 rj, gj;
            if (j < p) {
              const double2 u = W[j * LDW + p];
              rj = used[j] ? make_double2(-u.x, -u.y) : u;
              gj = u;
            } else {
              const double2 u = W[p * LDW + j];
              rj = u;
              gj = used[j] ? make_double2(-u.x, -u.y) : u;
            }
            if (j != p && !used[j]) {
              const unsigned long long kk = pivot_key(rj);
              offmax = kk > offmax ? kk : offmax;
            }
            gcol[j] = gj;
            rowW[j] = (j == p) ? d : cmul(d, rj);
          }
#pragma unroll
          for (int off = 16; off; off >>= 1) {
            const unsigned long long o = __shfl_xor_sync(0xffffffffu, offmax, off);
            offmax = o > offmax ? o : offmax;
          }
          __syncwarp();  // every lane has read used[] before lane 0 marks p
          if (lane == 0) {
            const double zmag = __longlong_as_double((long long)best);
            const double omag = __longlong_as_double((long long)offmax);
            if (singular || zmag < a.sym_tau * omag) s_status = kStatusNeedPivot;
            used[p] = 1;
            s_p = p;
            s_d = d;
          }
        }
        __syncthreads();
        const int p = s_p;
        const double2 d = s_d;
        if (warp == p % NW) {  // B. the scaled pivot row of R
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
        // C. W triangle and R rows.  One FMA form for every element, with
        //    selected operands (rowW[p] = d):
        //      (i, j), i, j != p:  W - g_i rowW[j]
        //      (p, j):             rowW[j] - 0 * rowW[j]
        //      (i, p), i < p:      0 - g_i d
        const int crot = (tid + NT - 32 * ((k + 2) % NW)) % NT;
#pragma unroll
        for (int s = 0; s < SMAX; ++s) {
          const int e = crot + NT * s;
          if (e < T) {
            const int i = tri[e] >> 16, j = tri[e] & 0xffff;
            const double2 rj = rowW[j];
            const double2 w = (i == p) ? rj : (j == p) ? make_double2(0.0, 0.0) : W[i * LDW + j];
            const double2 f = (i == p) ? make_double2(0.0, 0.0) : gcol[i];
            W[i * LDW + j] = cfms(w, f, rj);
          }
        }
        double2 rr[CB];
#pragma unroll
        for (int b = 0; b < CB; ++b) {
          const int J = lane + 32 * b;
          rr[b] = (J < M) ? rowR[J] : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int ai = 0; ai < AMAX; ++ai) {
          const int i = warp + NW * ai;
          if (i < M) {
            const double2 g = gcol[i];
            const bool isp = (i == p);
#pragma unroll
            for (int b = 0; b < CB; ++b) R[ai][b] = isp ? rr[b] : cfms(R[ai][b], g, rr[b]);
          }
        }
        __syncthreads();
      }
      if (a.state_dump) {
        // The state after this slice, natural order: Gss = W (symmetric) and
        // Gs1 = sign * R, the solve_block_tridiag pair (S_n, Z_n).
        double2* d1 = a.state_dump + ((int64_t)r * nx + n) * 2 * M * M;
        for (int e = tid; e < M * M; e += NT) {
          const int i = e / M, j = e % M;
          d1[e] = i <= j ? W[i * LDW + j] : W[j * LDW + i];
        }
        const double gs = (n == 0) ? 1.0 : -1.0;
#pragma unroll
        for (int ai = 0; ai < AMAX; ++ai) {
          const int q = warp + NW * ai;
#pragma unroll
          for (int b = 0; b < CB; ++b) {
            const int j = lane + 32 * b;
            if (q < M && j < M) d1[(int64_t)M * M + q * M + j] = cscale(gs, R[ai][b]);
          }
        }
        __syncthreads();  // W is read before the next slice overwrites it
      }
    }

    if (s_status == kStatusNeedPivot) {
      __syncthreads();
      if (tid == 0) {
        a.status[r] = s_status;
        a.flag_list[atomicAdd(a.work_counter + 1, 1)] = r;
      }
      continue;
    }

    if (refl) {
      // Reflection from the reverse sweep: G11 = W (symmetric, upper triangle),
      // r = -1 + 2i sqrt(real mu) G11 sqrt(real mu) (src/waveguide.f90:510-512).
      double2* rout = a.tout + (int64_t)r * M * M;
      for (int e = tid; e < M * M; e += NT) {
        const int i = e % M, j = e / M;
        const double2 gij = i <= j ? W[i * LDW + j] : W[j * LDW + i];
        const double2 v = cmul(cmul(wd.sqmu_r[i], gij), wd.sqmu_r[j]);
        rout[e] = make_double2((i == j ? -1.0 : 0.0) - 2.0 * v.y, 2.0 * v.x);
      }
      __syncthreads();
      if (tid == 0) a.status[r] = s_status;
      continue;
    }

    // 5. Fisher-Lee from R (natural order): Gs1 = sign * R, t = 2i sqmu Gs1 sqmu.
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
        const double2 g = cscale(gsign, W[gi * LDW + gj]);
        const double2 v = cmul(cmul(sqmu[gi], g), sqmu[gj]);
        tv[s] = make_double2(-2.0 * v.y, 2.0 * v.x);
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
      if (!tt_eigenvalues<NT>(W, LDW, nrow, ncol, wd.neigv, cc, &s_rot, a.teig + obase) && tid == 0 &&
          s_status == RG_OK)
        s_status = RG_ERR_NOCONV;
    }
    __syncthreads();
    if (tid == 0) a.status[r] = s_status;
  }
}

template <int MCAP, int NT, int MINB>
int plan_sym_t(SweepArgs& a, int sm_count, int* grid, int64_t* stride) {
  const size_t smem = SymSmem<MCAP>::bytes(a.max_ny);
  RG_CUDA(cudaFuncSetAttribute(sweep_sym_kernel<MCAP, NT, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  int per_sm = 0;
  RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_sym_kernel<MCAP, NT, MINB>, NT, smem));
  if (per_sm < 1) return fail(RG_ERR_INVALID_ARG, "symmetric sweep kernel does not fit on an SM (ny too large?)");
  if (a.force_per_sm > 0 && a.force_per_sm < per_sm) per_sm = a.force_per_sm;
  int g = per_sm * sm_count;
  if (g > a.nreal) g = a.nreal;
  *grid = g < 1 ? 1 : g;
  *stride = sym_stride(a.max_ny);
  a.cluster = 1;
  return RG_OK;
}

template <int MCAP, int NT, int MINB>
int launch_sym_t(const SweepArgs& a, cudaStream_t stream, int grid) {
  sweep_sym_kernel<MCAP, NT, MINB><<<grid, NT, SymSmem<MCAP>::bytes(a.max_ny), stream>>>(a);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

}  // namespace

int sweep_sym_plan(SweepArgs& a, int sm_count, int* grid, int64_t* work_stride) {
  if (a.max_M <= 16) return plan_sym_t<16, 64, 8>(a, sm_count, grid, work_stride);
  if (a.max_M <= 32) return plan_sym_t<32, 128, 4>(a, sm_count, grid, work_stride);
  if (a.max_M <= kMaxModesSmem) return plan_sym_t<64, 256, 2>(a, sm_count, grid, work_stride);
  return fail(RG_ERR_INVALID_ARG, "symmetric sweep kernel: too many modes");
}

int launch_sweep_sym(const SweepArgs& a, cudaStream_t stream, int grid) {
  if (a.nreal <= 0) return RG_OK;
  if (a.max_M <= 16) return launch_sym_t<16, 64, 8>(a, stream, grid);
  if (a.max_M <= 32) return launch_sym_t<32, 128, 4>(a, stream, grid);
  return launch_sym_t<64, 256, 2>(a, stream, grid);
}

}  // namespace rg
