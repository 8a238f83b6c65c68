// Recursive Green sweep for many modes (M > 64): the slice matrices no longer
// fit in shared memory, so W (the slice matrix inverted in place) and R (the
// propagator right-hand side) live in a workspace in global memory
// (L2-resident when the batch allows), and Gauss-Jordan runs blocked:
//
//   for each panel of NB columns
//     load the panel (M x NB) into shared memory,
//     factor it: NB pivoted elimination steps restricted to the panel,
//       recording the multipliers u_k (x <- x + u_k x[p_k] is step k),
//     apply the NB steps to every other column at once:
//       z = (I - L)^-1 x[p_0..p_NB-1]  (L[k][l] = u_l[p_k], l < k),
//       x += U z                       (a rank-NB update, one column per thread),
//     store the panel back.
//
// Same mathematics as the shared-memory kernel (src/waveguide.f90:426-445:
// Gss = inv(A - B Gss B), Gs1 = -Gss B Gs1, Fisher-Lee), with the same implicit
// pivoting and permutation bookkeeping; each matrix element is read and
// written once per panel instead of once per step, so memory traffic is
// 1/NB of the unblocked elimination.  The disorder is drawn in-kernel, one
// xoshiro256** state per transverse column kept in the workspace, so the
// Nx x ny potential of a large guide never goes through HBM.
//
// A work item can be spread over a thread-block cluster of C CTAs (C SMs).
// Every CTA of the cluster factors each panel itself (same input, same code,
// same result, so no pivot data is exchanged), the rank-NB update, slice
// assembly, disorder draws and eigenvalue rotations are split across the
// CTAs, and a cluster barrier separates the phases.  Data another CTA wrote
// is read with ld.global.cg (L2, never a stale L1 line).
#include <cooperative_groups.h>

#include "rg_device.cuh"

namespace cg = cooperative_groups;

namespace rg {
namespace {

constexpr int kLargeNT = 256;
constexpr int kLargeNB = 8;
constexpr int kMaxCluster = 8;
constexpr int kMaxRowSplit = 8;  // threads sharing one column's rows in the rank-NB update

struct LargeSmem {
  static size_t bytes(int M, int ny) {
    const int nyp = (ny + 1) & ~1;
    return sizeof(double2) * (2 * (size_t)M * kLargeNB + kLargeNB * kLargeNB + M + kLargeNB +
                               (kLargeNT / 2) * kLargeNB) +
           sizeof(double) * (2 * M + 2 + nyp) + sizeof(int) * 5 * M;
  }
};

// Workspace of one cluster, in double2 units: W (two buffers), R, t,
// generator states (ny x 4 uint64) and the drawn potential row (ny doubles).
inline int64_t large_stride(int M, int ny) {
  const int64_t mm = (int64_t)M * M;
  return ((4 * mm + 2 * (int64_t)ny + (ny + 1) / 2) + 15) & ~(int64_t)15;
}

__global__ void __launch_bounds__(kLargeNT, 2) sweep_large_kernel(SweepArgs a) {
  constexpr int NT = kLargeNT, NB = kLargeNB, NW = NT / 32;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int MX = a.max_M;
  extern __shared__ double2 sm[];
  double2* P = sm;                          // [M][NB] current panel
  double2* Ub = P + MX * NB;                // [M][NB] multipliers of the panel's steps
  double2* Lt = Ub + MX * NB;               // [NB][NB] Lt[k][l] = u_l[p_k], l < k
  double2* colf = Lt + NB * NB;             // [M] panel column before the step
  double2* rowp = colf + MX;                // [NB] scaled pivot row inside the panel
  double2* zsh = rowp + NB;                 // [NT/2][NB] z of the columns of a chunk (row split)
  double* cc = (double*)(zsh + (NT / 2) * NB);  // [2M+2] projection coefficients
  double* urow = cc + (2 * MX + 2);         // [ny] potential of the slice
  int* piv = (int*)(urow + ((a.max_ny + 1) & ~1));
  int* pinv = piv + MX;
  int* sinv = pinv + MX;
  int* colmap = sinv + MX;
  int* used = colmap + MX;
  __shared__ int s_r, s_p, s_status, s_rot;
  __shared__ double2 s_d;
  __shared__ unsigned long long s_key[NW];
  __shared__ int s_idx[NW];
  __shared__ WgDesc wd;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ctid = rank * NT + tid, CNT = C * NT;  // thread index and count in the cluster
  const bool draw = (a.upot == nullptr);
  const bool tmat = (a.mode == kModeTmat);
  const bool refl = (a.mode == kModeRefl);

  for (;;) {
    if (rank == 0 && tid == 0) {
      const int q = atomicAdd(a.work_counter, 1);
      const int nq = a.count_ptr ? *a.count_ptr : a.nreal;
      s_r = q < nq ? (a.item_idx ? a.item_idx[q] : q) : -1;
      if (s_r >= 0) wd = a.wgs[a.item_wg ? a.item_wg[s_r] : 0];
    }
    cluster.sync();
    if (rank != 0 && tid == 0) {
      s_r = *cluster.map_shared_rank(&s_r, 0);
      if (s_r >= 0) wd = *cluster.map_shared_rank(&wd, 0);
    }
    cluster.sync();  // rank 0's shared memory has been read before any CTA can leave the loop
    const int r = s_r;  // item index (queue position mapped through item_idx)
    if (r < 0) break;
    const int M = wd.M, ny = wd.ny;
    const int64_t mm = (int64_t)M * M;
    double2* ws = a.work + (int64_t)(blockIdx.x / C) * a.work_stride;
    double2* const Wb0 = ws;
    double2* const Wb1 = ws + mm;
    double2* Rg = ws + 2 * mm;
    double2* Tg = ws + 3 * mm;
    uint64_t* gen = (uint64_t*)(ws + 4 * mm);     // [ny][4]
    double* urow_g = (double*)(gen + 4 * ny);     // [ny] drawn row, shared by the cluster
    if (tid == 0) s_status = RG_OK;
    for (int c = tid; c < M; c += NT) {
      sinv[c] = c;
      used[c] = 0;
    }
    const int nb = a.n_begin, ne = a.n_end > 0 ? a.n_end : wd.nx;
    if (a.state_in) {
      // Resume after slice nb-1 from a natural-order state: Gss goes to the
      // buffer the first slice reads, R holds Y with Gs1 = rsign * Y.
      const double2* sin = a.state_in + (int64_t)r * 2 * mm;
      const double rs = (nb == 1) ? 1.0 : -1.0;
      for (int64_t e = ctid; e < mm; e += CNT) {
        Wb0[e] = sin[e];
        Rg[e] = cscale(rs, sin[mm + e]);
      }
      for (int c = tid; c < M; c += NT) {
        pinv[c] = c;
        colmap[c] = c;
      }
    } else {
      // Source at slice 0: R = I.  A later source slice starts from R = 0.
      const double one = a.inject_at > 0 ? 0.0 : 1.0;
      for (int64_t e = ctid; e < mm; e += CNT) Rg[e] = make_double2((e / M) == (e % M) ? one : 0.0, 0.0);
    }
    if (draw) {
      for (int iy = ctid; iy < ny; iy += CNT) {
        const Xoshiro st = jump_state(seeded_state(a.seeds[r]), wd.jumppoly + 4 * (int64_t)iy);
        gen[4 * iy + 0] = st.s0;
        gen[4 * iy + 1] = st.s1;
        gen[4 * iy + 2] = st.s2;
        gen[4 * iy + 3] = st.s3;
      }
    }
    const double* U = draw ? nullptr : a.upot + (int64_t)r * a.pot_rstride;
    cluster.sync();

    int cur = 0;
    for (int n = nb; n < ne; ++n) {
      const int id = (refl ? wd.nx - 1 - n : n) - wd.nxfree;  // slice of the guide swept at step n
      const bool dis = (id >= 0 && id < wd.nxdiso);
      if (dis) {
        // 1. This slice's potential row (drawn or loaded) and its projection.
        if (draw) {
          for (int iy = ctid; iy < ny; iy += CNT) {
            Xoshiro st{gen[4 * iy], gen[4 * iy + 1], gen[4 * iy + 2], gen[4 * iy + 3]};
            urow_g[iy] = scaled_normal(wd.stdu, st);
            gen[4 * iy + 0] = st.s0;
            gen[4 * iy + 1] = st.s1;
            gen[4 * iy + 2] = st.s2;
            gen[4 * iy + 3] = st.s3;
          }
          cluster.sync();
          for (int j = tid; j < ny; j += NT) urow[j] = __ldcg(urow_g + j);
        } else {
          for (int j = tid; j < ny; j += NT) urow[j] = U[(int64_t)id * a.pot_xstride + (int64_t)j * a.pot_ystride];
        }
        __syncthreads();
        if (!wd.periodic) {
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

      // 2. Assemble X = A_n - V_n - B Gss B (physical row order) into the
      //    other W buffer, and R = B Gs1 in place (elements split over the cluster).
      double2* Wold = cur ? Wb1 : Wb0;
      double2* W = cur ? Wb0 : Wb1;
      cur ^= 1;
      const double2* adiag = (n == 0 || n == wd.nx - 1) ? wd.adiag_edge : wd.adiag_bulk;
      const double rsign = (n == 1) ? 1.0 : -1.0;
      // At the source slice s > 0 the right-hand side is the identity source:
      // Z_s = S_s I, and the stored R carries Gs1 = -R, so R's right-hand
      // side is -I in the physical rows (row q of W is physical row pinv[q]).
      const bool source = (n > 0 && n == a.inject_at);
      for (int64_t e = ctid; e < mm; e += CNT) {
        const int q = (int)(e / M), c = (int)(e % M);
        const int al = (n == 0) ? q : pinv[q];
        double2 x = (al == c) ? adiag[c] : make_double2(0.0, 0.0);
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
        if (n > 0) {
          x = csub(x, cmul(cmul(wd.bmat[al], __ldcg(Wold + (int64_t)q * M + colmap[c])), wd.bmat[c]));
          Rg[e] = source ? make_double2(al == c ? -1.0 : 0.0, 0.0)
                         : cmul(wd.bmat[al], cscale(rsign, __ldcg(Rg + e)));
        }
        W[e] = x;
      }
      cluster.sync();

      // 3. Blocked Gauss-Jordan with implicit partial pivoting.
      for (int k0 = 0; k0 < M; k0 += NB) {
        const int nbk = min(NB, M - k0);
        for (int e = tid; e < M * nbk; e += NT) {
          const int i = e / nbk, l = e % nbk;
          P[i * NB + l] = __ldcg(W + (int64_t)i * M + k0 + l);
        }
        __syncthreads();
        for (int kk = 0; kk < nbk; ++kk) {
          // a. pivot: largest max(|re|,|im|) among unused rows (ties: lowest row)
          unsigned long long best = 0ULL;
          int bi = 0x7fffffff;
          for (int i = tid; i < M; i += NT) {
            const unsigned long long key = used[i] ? 0ULL : pivot_key(P[i * NB + kk]);
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
            s_key[warp] = best;
            s_idx[warp] = bi;
          }
          __syncthreads();
          if (warp == 0) {
            best = lane < NW ? s_key[lane] : 0ULL;
            bi = lane < NW ? s_idx[lane] : 0x7fffffff;
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
                const double2 z = P[bi * NB + kk];
                const double rden = 1.0 / fma(z.x, z.x, z.y * z.y);
                d = make_double2(z.x * rden, -z.y * rden);
              }
              used[bi] = 1;
              piv[k0 + kk] = bi;
              pinv[bi] = k0 + kk;
              s_p = bi;
              s_d = d;
            }
          }
          __syncthreads();
          const int p = s_p;
          const double2 d = s_d;
          // b. multipliers u_k and the scaled pivot row of the panel
          for (int i = tid; i < M; i += NT) {
            const double2 f = P[i * NB + kk];
            colf[i] = f;
            const double2 fd = cmul(f, d);
            Ub[i * NB + kk] = (i == p) ? make_double2(d.x - 1.0, d.y) : make_double2(-fd.x, -fd.y);
          }
          if (tid < nbk) rowp[tid] = (tid == kk) ? d : cmul(P[p * NB + tid], d);
          __syncthreads();
          // c. eliminate inside the panel
          for (int e = tid; e < M * nbk; e += NT) {
            const int i = e / nbk, l = e % nbk;
            if (i == p) {
              P[i * NB + l] = rowp[l];
            } else {
              const double2 w = (l == kk) ? make_double2(0.0, 0.0) : P[i * NB + l];
              P[i * NB + l] = cfms(w, colf[i], rowp[l]);
            }
          }
          __syncthreads();
        }
        for (int e = tid; e < nbk * nbk; e += NT) {
          const int k = e / nbk, l = e % nbk;
          Lt[k * NB + l] = (l < k) ? Ub[piv[k0 + k] * NB + l] : make_double2(0.0, 0.0);
        }
        __syncthreads();
        // d. the panel's steps applied to every other column of [W | R].
        //    Columns are dealt round-robin to the cluster's CTAs (jj = rank +
        //    C*c); when a CTA has fewer columns than threads, T threads share
        //    a column's rows and its z comes through shared memory.
        const int ntrail = 2 * M - nbk;
        const int ncl = (ntrail - rank + C - 1) / C;
        int T = 1;
        while (T < kMaxRowSplit && ncl * T * 2 <= NT) T *= 2;
        const int NCH = NT / T;  // columns per chunk
        const int cs = tid % NCH, sub = tid / NCH;
        for (int c0 = 0; c0 < ncl; c0 += NCH) {
          const int c = c0 + cs;
          const bool active = c < ncl;
          const int jj = rank + C * c;
          const int j = jj < k0 ? jj : jj + nbk;
          double2* col = active ? ((j < M) ? W + j : Rg + (j - M)) : nullptr;
          double2 z[NB];
#pragma unroll
          for (int k = 0; k < NB; ++k) z[k] = make_double2(0.0, 0.0);
          if (active && sub == 0) {
#pragma unroll
            for (int k = 0; k < NB; ++k) {
              if (k < nbk) {
                double2 v = __ldcg(col + (int64_t)piv[k0 + k] * M);
#pragma unroll
                for (int l = 0; l < k; ++l) v = cfms(v, make_double2(-Lt[k * NB + l].x, -Lt[k * NB + l].y), z[l]);
                z[k] = v;
              }
            }
            if (T > 1) {
#pragma unroll
              for (int k = 0; k < NB; ++k) zsh[cs * NB + k] = z[k];
            }
          }
          if (T > 1) {
            __syncthreads();  // z is read before any pivot row of these columns changes
            if (active) {
#pragma unroll
              for (int k = 0; k < NB; ++k) z[k] = zsh[cs * NB + k];
            }
          }
          if (active) {
            if (nbk == NB) {
              for (int i = sub; i < M; i += T) {
                double2 x = __ldcg(col + (int64_t)i * M);
                const double2* ui = Ub + i * NB;
#pragma unroll
                for (int k = 0; k < NB; ++k) {
                  const double2 u = ui[k];
                  x = cfms(x, make_double2(-u.x, -u.y), z[k]);
                }
                col[(int64_t)i * M] = x;
              }
            } else {
              for (int i = sub; i < M; i += T) {
                double2 x = __ldcg(col + (int64_t)i * M);
                const double2* ui = Ub + i * NB;
                for (int k = 0; k < nbk; ++k) {
                  const double2 u = ui[k];
                  x = cfms(x, make_double2(-u.x, -u.y), z[k]);
                }
                col[(int64_t)i * M] = x;
              }
            }
          }
          if (T > 1) __syncthreads();  // zsh is reused by the next chunk
        }
        if (rank == 0) {
          for (int e = tid; e < M * nbk; e += NT) {
            const int i = e / nbk, l = e % nbk;
            W[(int64_t)i * M + k0 + l] = P[i * NB + l];
          }
        }
        cluster.sync();
      }

      // 4. Permutation bookkeeping for the next slice.
      for (int c = tid; c < M; c += NT) {
        const int cm = pinv[sinv[c]];
        sinv[c] = piv[c];
        colmap[c] = cm;
        used[c] = 0;
      }
      __syncthreads();
      // Segment mode: the natural-order state after this slice,
      // Gss[a][c] = W[piv[a]][colmap[c]] and Gs1[a][j] = sign * R[piv[a]][j].
      const bool last = (n == ne - 1);
      if (a.state_dump || (a.state_out && last)) {
        const double2* Wn = cur ? Wb1 : Wb0;
        const double gs = (n == 0) ? 1.0 : -1.0;
        double2* d1 = a.state_dump ? a.state_dump + ((int64_t)r * (ne - nb) + (n - nb)) * 2 * mm : nullptr;
        double2* d2 = (a.state_out && last) ? a.state_out + (int64_t)r * 2 * mm : nullptr;
        for (int64_t e = ctid; e < mm; e += CNT) {
          const int ar = (int)(e / M), c = (int)(e % M);
          const double2 gss = __ldcg(Wn + (int64_t)piv[ar] * M + colmap[c]);
          const double2 gs1 = cscale(gs, __ldcg(Rg + (int64_t)piv[ar] * M + c));
          if (d1) {
            d1[e] = gss;
            d1[mm + e] = gs1;
          }
          if (d2) {
            d2[e] = gss;
            d2[mm + e] = gs1;
          }
        }
        cluster.sync();  // R is rescaled in place by the next slice
      }
    }

    if (ne < wd.nx) {  // a partial sweep (segment): no Fisher-Lee stage
      __syncthreads();
      if (rank == 0 && tid == 0) a.status[r] = s_status;
      cluster.sync();
      continue;
    }

    if (refl) {
      // 5'. Reflection: the reverse sweep's last Gss is G(x_1; x_1):
      //     G11[a][c] = W[piv[a]][colmap[c]];  r = -1 + 2i sqmu_a G11 sqmu_c.
      const double2* Wl = cur ? Wb1 : Wb0;  // buffer the last slice was inverted in
      double2* rout = a.tout + (int64_t)r * M * M;
      for (int e = ctid; e < M * M; e += CNT) {
        const int i = e % M, j = e / M;
        const double2 v = cmul(cmul(wd.sqmu_r[i], __ldcg(Wl + (int64_t)piv[i] * M + colmap[j])), wd.sqmu_r[j]);
        rout[e] = make_double2((i == j ? -1.0 : 0.0) - 2.0 * v.y, 2.0 * v.x);
      }
      __syncthreads();
      if (rank == 0 && tid == 0) a.status[r] = s_status;
      cluster.sync();
      continue;
    }

    // 5. Fisher-Lee: t = 2i sqmu_a Gs1 sqmu_j with Gs1[a][j] = sign * R[piv[a]][j];
    //    t goes to the workspace, column-major (ld = nrow).
    const double gsign = (wd.nx >= 2) ? -1.0 : 1.0;
    const int row0 = tmat ? 0 : wd.row0, col0 = tmat ? 0 : wd.col0;
    const int nrow = tmat ? M : wd.nrow, ncol = tmat ? M : wd.ncol;
    const double2* sqmu = tmat ? wd.sqmu_r : wd.sqmu_c;
    double2* tout = a.tout ? a.tout + (int64_t)r * nrow * ncol : nullptr;
    for (int e = ctid; e < nrow * ncol; e += CNT) {
      const int i = e % nrow, j = e / nrow;
      const int gi = row0 + i, gj = col0 + j;
      const double2 g = cscale(gsign, __ldcg(Rg + (int64_t)piv[gi] * M + gj));
      const double2 v = cmul(cmul(sqmu[gi], g), sqmu[gj]);
      const double2 t = make_double2(-2.0 * v.y, 2.0 * v.x);
      Tg[e] = t;
      if (tout) tout[e] = t;
    }
    cluster.sync();

    if (!tmat) {
      // 6. Eigenvalues of t^H t: one-sided Jacobi on the vectors of the
      //    smaller dimension (columns of t, or its rows), in the workspace;
      //    the pairs of a round are split over the cluster's warps.
      const bool bycol = nrow >= ncol;
      const int nv = bycol ? ncol : nrow;
      const int L = bycol ? nrow : ncol;
      const int es = bycol ? 1 : nrow;
      const int vs = bycol ? nrow : 1;
      const int NP = (nv + 1) & ~1;
      const double tol = 2.220446049250313e-16 * L;
      int* rot0 = cluster.map_shared_rank(&s_rot, 0);
      int sweep = 0;
      for (; sweep < 60; ++sweep) {
        if (rank == 0 && tid == 0) s_rot = 0;
        cluster.sync();
        for (int rr = 0; rr < NP - 1; ++rr) {
          for (int pk = rank * NW + warp; pk < NP / 2; pk += C * NW) {
            const int pos1 = pk, pos2 = NP - 1 - pk;
            const int vp = pos1 == 0 ? 0 : ((pos1 - 1 + rr) % (NP - 1)) + 1;
            const int vq = ((pos2 - 1 + rr) % (NP - 1)) + 1;
            if (vp >= nv || vq >= nv) continue;
            double2* xp = Tg + (int64_t)vp * vs;
            double2* xq = Tg + (int64_t)vq * vs;
            double al = 0.0, be = 0.0, gr = 0.0, gi = 0.0;
            for (int i = lane; i < L; i += 32) {
              const double2 u = __ldcg(xp + (int64_t)i * es), w = __ldcg(xq + (int64_t)i * es);
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
              if (lane == 0) atomicOr(rot0, 1);
              const double zeta = (be - al) / (2.0 * ga);
              const double t = fabs(zeta) > 1e100 ? 0.5 / zeta
                                                  : copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
              const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
              const double2 ph = make_double2(gr / ga, -gi / ga);
              for (int i = lane; i < L; i += 32) {
                const double2 u = __ldcg(xp + (int64_t)i * es);
                const double2 w = cmul(ph, __ldcg(xq + (int64_t)i * es));
                xp[(int64_t)i * es] = make_double2(c * u.x - s * w.x, c * u.y - s * w.y);
                xq[(int64_t)i * es] = make_double2(s * u.x + c * w.x, s * u.y + c * w.y);
              }
            }
          }
          cluster.sync();
        }
        const int any = *rot0;
        cluster.sync();  // every CTA has read the flag before rank 0 clears it
        if (!any) break;
      }
      if (sweep == 60 && tid == 0) s_status = RG_ERR_NOCONV;
      if (rank == 0) {
        for (int k = warp; k < nv; k += NW) {
          const double2* xk = Tg + (int64_t)k * vs;
          double s = 0.0;
          for (int i = lane; i < L; i += 32) {
            const double2 u = __ldcg(xk + (int64_t)i * es);
            s = fma(u.x, u.x, fma(u.y, u.y, s));
          }
#pragma unroll
          for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
          if (lane == 0) cc[k] = s;
        }
        __syncthreads();
        const int64_t obase = a.teig_off ? a.teig_off[r] : (int64_t)r * wd.neigv;
        for (int k = tid; k < nv; k += NT) {
          const double tk = cc[k];
          int rank_k = 0;
          for (int j = 0; j < nv; ++j) {
            const double tj = cc[j];
            rank_k += (tj > tk || (tj == tk && j < k)) ? 1 : 0;
          }
          if (rank_k < wd.neigv) a.teig[obase + rank_k] = tk;
        }
      }
    }
    __syncthreads();
    if (rank == 0 && tid == 0) a.status[r] = s_status;
    cluster.sync();  // the cluster finishes this item before rank 0 takes the next
  }
}

}  // namespace

// Cluster size: spread an item over several SMs when there are fewer items
// than CTA slots, so a small batch (or one large realization) still fills
// the GPU; full batches run one CTA per item (no redundant panel work).
int sweep_large_plan(SweepArgs& a, int sm_count, int* grid, int64_t* work_stride) {
  const size_t smem = LargeSmem::bytes(a.max_M, a.max_ny);
  if (smem > 227 * 1024) return fail(RG_ERR_INVALID_ARG, "too many modes or transverse points for the large-mode kernel");
  RG_CUDA(cudaFuncSetAttribute(sweep_large_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_large_kernel, kLargeNT, smem));
  if (per_sm < 1) return fail(RG_ERR_INVALID_ARG, "large-mode sweep kernel does not fit on an SM");
  const int slots = per_sm * sm_count;
  int C = 1;
  if (a.force_cluster > 0) {
    while (C < kMaxCluster && C < a.force_cluster) C *= 2;
  } else {
    while (C < kMaxCluster && (int64_t)a.nreal * C * 2 <= slots) C *= 2;
  }
  int nclusters = slots / C;
  if (C > 1) {
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = C;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.gridDim = dim3(C * 64);
    cfg.blockDim = dim3(kLargeNT);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int maxc = 0;
    RG_CUDA(cudaOccupancyMaxActiveClusters(&maxc, sweep_large_kernel, &cfg));
    if (maxc < 1) {
      C = 1;
      nclusters = slots;
    } else {
      nclusters = maxc;
    }
  }
  if (nclusters > a.nreal) nclusters = a.nreal;
  if (nclusters < 1) nclusters = 1;
  a.cluster = C;
  *grid = nclusters * C;
  *work_stride = large_stride(a.max_M, a.max_ny);
  return RG_OK;
}

int launch_sweep_large(const SweepArgs& a, cudaStream_t stream, int grid) {
  if (a.nreal <= 0) return RG_OK;
  const size_t smem = LargeSmem::bytes(a.max_M, a.max_ny);
  const int C = a.cluster > 0 ? a.cluster : 1;
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute attr{};
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = C;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kLargeNT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  RG_CUDA(cudaLaunchKernelEx(&cfg, sweep_large_kernel, a));
  return RG_OK;
}

}  // namespace rg
