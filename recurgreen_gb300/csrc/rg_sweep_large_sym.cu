// Symmetric blocked sweep for Dirichlet guides of more than 64 modes.
//
// The slice matrix X_n = A_n - V_n - B Gss B of a Dirichlet guide is complex
// symmetric, so its inverse is formed by a symmetric Gauss-Jordan sweep on
// the upper triangle (the shared-memory version and its sign rule are in
// rg_sweep_sym.cu), here blocked for matrices that live in global memory
// (L2-resident when the batch allows):
//
//   for each panel of NB diagonal pivots
//     for each step k of the panel (left-looking)
//       p_k = the unswept index with the largest current diagonal |dg_i|,
//       x   = column p_k at the panel start (upper triangle plus sign rule),
//             plus the panel's earlier steps: x += U z, z = (I - L)^-1 x[p],
//       u_k = -x d (u_k[p_k] = d - 1), d = 1 / x[p_k],
//       dg_i += u_k[i] x[i] for the unswept i;
//     every other column j of [W | R] gets x += U z with z = (I - L)^-1 x[p]
//       (a rank-NB update, rows i <= j only for W: half the work),
//     pivot column p_k becomes u_k + e_{p_k} with the later steps applied.
//
// A slice costs 12 M^3 + O(M^2) FP64 flops instead of the pivoted blocked
// kernel's 16 M^3 (src/waveguide.f90:426-440: zgetrf+zgetri and a matmul).
// W and R stay in natural order, so there is no permutation bookkeeping.
// The z of a W column comes from the panel's raw pivot columns, which each
// CTA keeps in its own staging area: no column reads another column's
// storage during the update.  A cluster barrier separates each panel's
// factorisation (whose column fetches read W anywhere) from its update, and
// another ends the update.
//
// With tensor_r the sweep inverts X alone (4 M^3 +
// O(M^2) FP64 flops) and then forms the new right-hand side B Gs1 <- X^-1
// (B Gs1) as one complex product on the FP16 tensor cores with FP64
// accuracy (rg_ozaki.cuh: 8 M^3 of the slice's flops leave the FP64 pipe):
// the row exponents of X^-1 and column exponents of B Gs1 are reduced over
// the cluster, the cluster writes both operands' digit planes to its
// workspace, and each CTA computes 16 x 128 column groups of the product,
// row tile by row tile, with its 8 warps.
//
// A diagonal pivot below sym_tau times the largest unswept entry of its
// column flags the realization (kStatusNeedPivot, appended to flag_list);
// launch_sweep then re-runs the flagged ones with the pivoted blocked kernel.
// Periodic items (Hermitian, not symmetric) are flagged at once.  Segment
// mode supports a stop after n_end slices (no Fisher-Lee stage); a whole
// sweep can keep the state of every slice (state_dump) and start its source
// at a later slice (inject_at), not resume from a state.
#include <cooperative_groups.h>

#include "rg_device.cuh"
#include "rg_ozaki.cuh"

namespace cg = cooperative_groups;

namespace rg {
namespace {

constexpr int kSymNT = 256;
constexpr int kSymNB = 8;
constexpr int kSymMaxCluster = 8;
constexpr int kSymMaxRowSplit = 8;
// The 2 x 2 block inverse for even mode counts from this size up.
constexpr int kSplitMinModes = 128;
// Gauss-Jordan blocks of at most this many modes are eliminated in shared
// memory (gj_small): [n][n+1] matrix, two [n] vectors, [n] flags and the
// n(n+1)/2 triangle index, within the product staging area.
constexpr int kSmallGJ = 64;

// The pivot column (panel phase) and the chunk's z values (update phase)
// share one region: they are never live at the same time.
//
// With tensor_r the products' two digit stages (72 KB) and, between
// products, the shared-memory Gauss-Jordan blocks overlay the start of this
// area (dead during either), and two arrays of 16-padded exponents follow.
constexpr size_t kSmallGJBytes = sizeof(double2) * (kSmallGJ * (kSmallGJ + 1) + 2 * kSmallGJ) +
                                 sizeof(int) * (kSmallGJ + kSmallGJ * (kSmallGJ + 1) / 2);
struct LargeSymSmem {
  __host__ __device__ static size_t shared_region(int M) {
    const size_t z = (size_t)(kSymNT / 4) * 2 * kSymNB;
    return (size_t)M > z ? (size_t)M : z;
  }
  static size_t base(int M) {
    return sizeof(double2) * ((size_t)M * kSymNB + kSymNB * kSymNB + (size_t)M + kSymNB + shared_region(M)) +
           sizeof(double) * (2 * (size_t)M + 2) + sizeof(int) * 3 * (size_t)M;
  }
  // the products' staged digits, or a shared-memory Gauss-Jordan block
  static constexpr size_t kStage =
      sizeof(uint4) * oz::kBlkStageUint4 > kSmallGJBytes ? sizeof(uint4) * oz::kBlkStageUint4 : kSmallGJBytes;
  __host__ __device__ static size_t exps_offset(int M) {
    const size_t b = sizeof(double2) * ((size_t)M * kSymNB + kSymNB * kSymNB + (size_t)M + kSymNB + shared_region(M)) +
                     sizeof(double) * (2 * (size_t)M + 2) + sizeof(int) * 3 * (size_t)M;
    return ((b > kStage ? b : kStage) + 15) & ~(size_t)15;
  }
  static size_t bytes(int M, bool tensor) {
    return tensor ? exps_offset(M) + sizeof(int) * 2 * 16 * (size_t)oz::tiles(M) : base(M);
  }
};

// Workspace of one cluster, in double2 units: W, R, t (M x M each), the
// generator states (ny x 4 uint64), the paired potential row (ny doubles)
// and each CTA's raw pivot columns (kSymMaxCluster x NB x M).
// With tensor_r the digit planes of both product operands and the cluster's
// exponent exchange area ([kSymMaxCluster][2][16 T] ints) follow.
__host__ __device__ inline int64_t large_sym_base_stride(int M, int ny) {
  const int64_t mm = (int64_t)M * M;
  const int64_t urow = ((int64_t)ny + 1) / 2;
  return ((3 * mm + 2 * (int64_t)ny + urow + (int64_t)kSymMaxCluster * kSymNB * M) + 15) & ~(int64_t)15;
}
// Then the 2 x 2 block inverse's buffers: three h x h (h = M / 2) for the
// first level, three (h/2) x (h/2) for the second.
__host__ __device__ inline int64_t large_sym_schur_offset(int M, int ny) {
  const int64_t ex = ((int64_t)kSymMaxCluster * 2 * 16 * oz::tiles(M) * 4 + 15) / 16;
  return (large_sym_base_stride(M, ny) + 2 * oz::operand_uint4(M) + ex + 15) & ~(int64_t)15;
}
inline int64_t large_sym_stride(int M, int ny, bool tensor) {
  if (!tensor) return large_sym_base_stride(M, ny);
  return (large_sym_schur_offset(M, ny) + 3 * (int64_t)(M / 2) * (M / 2) + 3 * (int64_t)(M / 4) * (M / 4) + 15) &
         ~(int64_t)15;
}

// Levels of the 2 x 2 block inverse for M modes, at most `want`: a level
// halves an even size of at least kSplitMinModes.
__host__ __device__ inline int split_depth(int want, int M) {
  int d = 0;
  while (d < want && d < 2 && M >= kSplitMinModes && (M % 2) == 0) {
    ++d;
    M >>= 1;
  }
  return d;
}

// The steps of the symmetric inverse for 0, 1 and 2 block levels: code =
// op * 4 + frame (frame 0: X itself; 1: frame 0's block A, inverted in place
// in its buffer; 2: frame 0's Schur complement S, likewise).
enum : int { kInvGJ, kInvCopyA, kInvGJA, kInvT, kInvS, kInvGJS, kInvY12, kInvY11, kInvY22 };
#define RG_INV(op, f) (unsigned char)((op) * 4 + (f))
__constant__ unsigned char kInvSteps[3][22] = {
    {RG_INV(kInvGJ, 0)},
    {RG_INV(kInvCopyA, 0), RG_INV(kInvGJA, 0), RG_INV(kInvT, 0), RG_INV(kInvS, 0), RG_INV(kInvGJS, 0),
     RG_INV(kInvY12, 0), RG_INV(kInvY11, 0), RG_INV(kInvY22, 0)},
    {RG_INV(kInvCopyA, 0),
     RG_INV(kInvCopyA, 1), RG_INV(kInvGJA, 1), RG_INV(kInvT, 1), RG_INV(kInvS, 1), RG_INV(kInvGJS, 1),
     RG_INV(kInvY12, 1), RG_INV(kInvY11, 1), RG_INV(kInvY22, 1),
     RG_INV(kInvT, 0), RG_INV(kInvS, 0),
     RG_INV(kInvCopyA, 2), RG_INV(kInvGJA, 2), RG_INV(kInvT, 2), RG_INV(kInvS, 2), RG_INV(kInvGJS, 2),
     RG_INV(kInvY12, 2), RG_INV(kInvY11, 2), RG_INV(kInvY22, 2),
     RG_INV(kInvY12, 0), RG_INV(kInvY11, 0), RG_INV(kInvY22, 0)}};
#undef RG_INV
__constant__ int kInvStepCount[3] = {1, 8, 22};

__device__ __forceinline__ double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }

// An operand of a cluster product: entry (r, c) is p[r ld + c + off], or,
// with trans, p[c ld + r + off], or, with sym, the symmetric matrix stored
// as the upper triangle at p (row stride ld).
struct Opnd {
  const double2* p;
  int64_t ld, off;
  int sym, trans;
};

__device__ __forceinline__ double2 opnd_at(const Opnd& o, int r, int c) {
  if (o.sym) return __ldcg(o.p + (r <= c ? (int64_t)r * o.ld + c : (int64_t)c * o.ld + r));
  return o.trans ? __ldcg(o.p + (int64_t)c * o.ld + r + o.off) : __ldcg(o.p + (int64_t)r * o.ld + c + o.off);
}

// Where one output tile of a cluster product goes:
//   dst[i ld + j + off] = sign C_ij + aux(i, j)   (only i <= j when upper),
// aux(i, j) = 0, or aux[i aux_ld + j + aux_off], or, with aux_sym, the
// symmetric matrix stored as the upper triangle at aux (row stride aux_ld).
struct TileOut {
  double2* dst;
  int64_t ld, off;
  double sign;
  const double2* aux;
  int64_t aux_ld, aux_off;
  int aux_sym, upper;
};

// One CTA's 2 x 4 block of 16 x 16 output tiles of a cluster product (warp
// w: row tile ti0 + w/4, column tile tj0 + w%4; both operands' digits staged
// in shared memory per chunk).  The output description o lives in shared
// memory, so none of its fields holds a register through the tensor-core
// loop.  Not inlined: one copy of the loop, with its own register
// allocation, serves all of a slice's products.
__device__ __noinline__ void block_product(int Mb, int ti0, int tj0, const uint4* adig, const uint4* bdig,
                                           const int* ea, const int* eb, uint4* stage, const TileOut* o) {
  oz::gemm_block(Mb, ti0, tj0, o->upper != 0, adig, bdig, ea, eb, stage, [&](int i, int j, double re, double im) {
    if (o->upper && i > j) return;
    const double sg = o->sign;
    double2 v = make_double2(sg * re, sg * im);
    if (o->aux) {
      const double2 x = o->aux_sym ? __ldcg(o->aux + (i <= j ? (int64_t)i * o->aux_ld + j : (int64_t)j * o->aux_ld + i))
                                   : __ldcg(o->aux + (int64_t)i * o->aux_ld + j + o->aux_off);
      v.x += x.x;
      v.y += x.y;
    }
    o->dst[(int64_t)i * o->ld + j + o->off] = v;
  });
}

// Where a cluster product keeps its state: the CTA's exponent arrays in
// shared memory, the cluster's partial exponents and both operands' digit
// planes in the workspace, and the CTA's staging area.
struct ZgemmCtx {
  int* ea_s;
  int* eb_s;
  int* expart;
  uint4* adig;
  uint4* bdig;
  uint4* stage;
};

// A cluster-wide complex product C = A B of two Mb x Mb operands on the
// tensor cores (rg_ozaki.cuh): exponents reduced over the cluster, digit
// planes in the workspace, then CTA tasks (blocks of 2 x 4 output tiles,
// both operands' digits staged in shared memory; with out.upper, blocks
// wholly below the diagonal are skipped).  The operands are read only in
// the first two phases, so out may overwrite them.  Called by every thread
// of the cluster; ends with a cluster barrier.  Not inlined: the slice's
// five products share one copy.
__device__ __noinline__ void cluster_zgemm(const ZgemmCtx c, const int Mb, const Opnd A, const Opnd B,
                                           const TileOut out) {
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks(), rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, ctid = rank * kSymNT + tid, CNT = C * kSymNT;
  auto getA = [&](int i, int k) { return opnd_at(A, i, k); };
  auto getB = [&](int k, int j) { return opnd_at(B, k, j); };
  const int T = oz::tiles(Mb);
  for (int i = tid; i < 16 * T; i += kSymNT) {
    c.ea_s[i] = oz::kNoExp;
    c.eb_s[i] = oz::kNoExp;
  }
  __syncthreads();
  for (int64_t e = ctid; e < (int64_t)Mb * Mb; e += CNT) {
    const int i = (int)(e / Mb), j = (int)(e % Mb);
    atomicMax(c.ea_s + i, oz::fexp2(getA(i, j)));
    atomicMax(c.eb_s + j, oz::fexp2(getB(i, j)));
  }
  __syncthreads();
  int* mine = c.expart + rank * 32 * T;
  for (int i = tid; i < 16 * T; i += kSymNT) {
    mine[i] = c.ea_s[i];
    mine[16 * T + i] = c.eb_s[i];
  }
  cluster.sync();
  for (int i = tid; i < 16 * T; i += kSymNT) {
    int x = oz::kNoExp, y = oz::kNoExp;
    for (int r = 0; r < C; ++r) {
      x = max(x, __ldcg(c.expart + r * 32 * T + i));
      y = max(y, __ldcg(c.expart + r * 32 * T + 16 * T + i));
    }
    c.ea_s[i] = x;
    c.eb_s[i] = y;
  }
  __syncthreads();
  oz::split_a(Mb, getA, c.ea_s, c.adig, ctid, CNT);
  oz::split_b(Mb, getB, c.eb_s, c.bdig, ctid, CNT);
  __shared__ TileOut s_out;
  if (tid == 0) s_out = out;
  cluster.sync();  // every digit is written before any CTA reads them (and s_out is set)
  const int nbr = (T + oz::kBlkRows - 1) / oz::kBlkRows, nbc = (T + oz::kBlkCols - 1) / oz::kBlkCols;
  int k = 0;
  for (int bi = 0; bi < nbr; ++bi)
    for (int bj = 0; bj < nbc; ++bj) {
      const int ti0 = bi * oz::kBlkRows, tj0 = bj * oz::kBlkCols;
      if (out.upper && ti0 > tj0 + oz::kBlkCols - 1) continue;
      if (k++ % C == rank) block_product(Mb, ti0, tj0, c.adig, c.bdig, c.ea_s, c.eb_s, c.stage, &s_out);
    }
  cluster.sync();
}

__global__ void __launch_bounds__(kSymNT, 2) sweep_large_sym_kernel(SweepArgs a) {
  constexpr int NT = kSymNT, NB = kSymNB, NW = NT / 32;
  cg::cluster_group cluster = cg::this_cluster();
  const int C = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int MX = a.max_M;
  extern __shared__ double2 sm[];
  double2* Ub = sm;                         // [M][NB] u_k of the panel's steps
  double2* Lt = Ub + MX * NB;               // [NB][NB] Lt[k][l] = u_l[p_k], l < k
  double2* dg = Lt + NB * NB;               // [M] current diagonal
  double2* zc = dg + MX;                    // [NB] z of the panel's earlier steps for the pivot column
  double2* colb = zc + NB;                  // [M] current pivot column (panel phase)
  double2* zsh = colb;                      // [NT/4][2][NB] z of the units of a chunk (update phase)
  double* cc = (double*)(colb + LargeSymSmem::shared_region(MX));  // [2M+2] projection coefficients
  int* piv = (int*)(cc + 2 * MX + 2);       // [M] pivot of step k
  int* used = piv + MX;                     // [M] swept
  int* used0 = used + MX;                   // [M] swept at the start of the panel
  __shared__ int s_r, s_p, s_status, s_rot;
  __shared__ unsigned long long s_key[NW], s_cmx[NW], s_cmax;
  __shared__ int s_idx[NW];
  __shared__ WgDesc wd;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ctid = rank * NT + tid, CNT = C * NT;
  const bool draw = (a.upot == nullptr);
  const bool tmat = (a.mode == kModeTmat);
  const bool refl = (a.mode == kModeRefl);
  // the propagator product on the tensor cores
  const bool gemm_on = a.tensor_r != 0;
  uint4* stage = reinterpret_cast<uint4*>(sm);  // overlays the panel arrays during the product
  int* ea_s = reinterpret_cast<int*>(reinterpret_cast<char*>(sm) + LargeSymSmem::exps_offset(MX));
  int* eb_s = ea_s + 16 * oz::tiles(MX);

  // Block argmax of the diagonal keys over the unswept indices (ties: lowest
  // index) together with a max of per-thread values `cm`; results in s_p and s_cmax.
  auto reduce_pivot = [&](unsigned long long best, int bi, unsigned long long cm) {
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      const unsigned long long oc = __shfl_xor_sync(0xffffffffu, cm, off);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
      cm = oc > cm ? oc : cm;
    }
    if (lane == 0) {
      s_key[warp] = best;
      s_idx[warp] = bi;
      s_cmx[warp] = cm;
    }
    __syncthreads();
    if (warp == 0) {
      best = lane < NW ? s_key[lane] : 0ULL;
      bi = lane < NW ? s_idx[lane] : 0x7fffffff;
      cm = lane < NW ? s_cmx[lane] : 0ULL;
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        const unsigned long long oc = __shfl_xor_sync(0xffffffffu, cm, off);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
        cm = oc > cm ? oc : cm;
      }
      if (lane == 0) {
        s_p = (best == 0ULL) ? -1 : bi;  // -1: no usable diagonal left
        s_cmax = cm;
      }
    }
    __syncthreads();
  };

  for (;;) {
    if (rank == 0 && tid == 0) {
      s_r = atomicAdd(a.work_counter, 1);
      if (s_r < a.nreal) wd = a.wgs[a.item_wg ? a.item_wg[s_r] : 0];
    }
    cluster.sync();
    if (rank != 0 && tid == 0) {
      s_r = *cluster.map_shared_rank(&s_r, 0);
      if (s_r < a.nreal) wd = *cluster.map_shared_rank(&wd, 0);
    }
    cluster.sync();  // rank 0's shared memory has been read before any CTA can leave the loop
    const int r = s_r;
    if (r >= a.nreal) break;
    const int M = wd.M, ny = wd.ny;
    const int64_t mm = (int64_t)M * M;
    double2* ws = a.work + (int64_t)(blockIdx.x / C) * a.work_stride;
    double2* W = ws;                              // upper triangle, W[i * M + j], i <= j
    double2* Rg = ws + mm;
    double2* Tg = ws + 2 * mm;
    uint64_t* gen = (uint64_t*)(ws + 3 * mm);     // [ny][4]
    double* urow_g = (double*)(gen + 4 * ny);     // [ny] paired potential row
    double2* PR = (double2*)(urow_g + ((ny + 1) & ~1)) + (int64_t)rank * NB * M;  // [NB][M] this CTA's raw pivot columns
    uint4* adig = reinterpret_cast<uint4*>(ws + large_sym_base_stride(M, ny));  // product digit planes
    uint4* bdig = adig + oz::operand_uint4(M);
    int* expart = reinterpret_cast<int*>(bdig + oz::operand_uint4(M));  // [C][2][16 T] partial exponents
    // the 2 x 2 block inverse's levels (0: one Gauss-Jordan elimination) and
    // buffers: A^-1, T = A^-1 B, S^-1 (h x h each, h = M / 2), then the same
    // for the half-size blocks (M / 4 each)
    const int split_levels = split_depth(gemm_on ? a.split_inverse : 0, M);
    double2* Wa = ws + large_sym_schur_offset(M, ny);
    double2* Tb = Wa + (int64_t)(M / 2) * (M / 2);
    double2* Ws = Tb + (int64_t)(M / 2) * (M / 2);
    double2* Wa2 = Ws + (int64_t)(M / 2) * (M / 2);
    double2* Tb2 = Wa2 + (int64_t)(M / 4) * (M / 4);
    double2* Ws2 = Tb2 + (int64_t)(M / 4) * (M / 4);
    if (tid == 0) s_status = wd.periodic ? kStatusNeedPivot : RG_OK;  // periodic X is Hermitian, not symmetric
    const double one = a.inject_at > 0 ? 0.0 : 1.0;  // the source at slice 0, or zero until inject_at
    for (int64_t e = ctid; e < mm; e += CNT) Rg[e] = make_double2((e / M) == (e % M) ? one : 0.0, 0.0);
    if (draw) {
      // Each generator state is set up by the thread that draws from it (the
      // pair (j, ny-1-j) below), so it is only ever read and written from one
      // SM: a state written by another CTA could be read through a stale L1
      // line when the cluster takes its next item.
      for (int j = ctid; j < (ny >> 1) + (ny & 1); j += CNT) {
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
    const int ne = a.n_end > 0 ? a.n_end : wd.nx;
    cluster.sync();
    // Rank 0's status decides for the whole cluster (every CTA computes the
    // same flags from the same data; reading one copy makes the decision
    // uniform by construction).  It is read right after a cluster barrier,
    // and rank 0 writes it again only after the next one.
    const int* status0 = cluster.map_shared_rank(&s_status, 0);

    for (int n = 0; n < ne; ++n) {
      if (*status0 == kStatusNeedPivot) break;
      const int id = (refl ? wd.nx - 1 - n : n) - wd.nxfree;
      const bool dis = (id >= 0 && id < wd.nxdiso);
      if (dis) {
        // 1. The slice's potential, paired (j, ny-1-j) as sum and difference
        //    (the transverse grid is symmetric and cos(pi d (1 - y)) =
        //    (-1)^d cos(pi d y)), then the projection over half the points.
        const int h = ny >> 1;
        for (int j = ctid; j < h + (ny & 1); j += CNT) {
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
            urow_g[j] = u0;
          } else {
            urow_g[j] = u0 + u1;
            urow_g[jp] = u0 - u1;
          }
        }
        cluster.sync();
        const int nd = 2 * M + 1;
        for (int d = tid; d < nd; d += NT) {
          const double* ct = wd.costab + d;
          const double* up = (d & 1) ? urow_g + (ny - 1) : urow_g;
          const int us = (d & 1) ? -1 : 1;
          double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
          int j = 0;
          for (; j + 4 <= h; j += 4) {
            s0 = fma(ct[(int64_t)(j + 0) * nd], __ldcg(up + us * (j + 0)), s0);
            s1 = fma(ct[(int64_t)(j + 1) * nd], __ldcg(up + us * (j + 1)), s1);
            s2 = fma(ct[(int64_t)(j + 2) * nd], __ldcg(up + us * (j + 2)), s2);
            s3 = fma(ct[(int64_t)(j + 3) * nd], __ldcg(up + us * (j + 3)), s3);
          }
          for (; j < h; ++j) s0 = fma(ct[(int64_t)j * nd], __ldcg(up + us * j), s0);
          if (ny & 1) s1 = fma(ct[(int64_t)h * nd], __ldcg(urow_g + h), s1);
          cc[d] = (s0 + s1) + (s2 + s3);
        }
        __syncthreads();
      }

      // 2. X = A_n - V_n - B Gss B on the upper triangle, in place, and
      //    R = B Gs1 (elements split over the cluster).
      const double2* adiag = (n == 0 || n == wd.nx - 1) ? wd.adiag_edge : wd.adiag_bulk;
      const double rsign = (n == 1) ? 1.0 : -1.0;
      for (int64_t e = ctid; e < mm; e += CNT) {
        const int i = (int)(e / M), j = (int)(e % M);
        if (i <= j) {
          double2 x = (i == j) ? adiag[i] : make_double2(0.0, 0.0);
          if (dis) x = csub(x, make_double2(cc[j - i] - cc[i + j + 2], 0.0));
          if (n > 0) x = csub(x, cmul(cmul(wd.bmat[i], __ldcg(W + e)), wd.bmat[j]));
          W[e] = x;
        }
        // At the source slice the right-hand side is -I (Gs1 = -R after slice 0).
        if (n > 0)
          Rg[e] = (n == a.inject_at) ? make_double2(i == j ? -1.0 : 0.0, 0.0)
                                     : cmul(wd.bmat[i], cscale(rsign, __ldcg(Rg + e)));
      }
      cluster.sync();
      // 3. Blocked symmetric Gauss-Jordan of the M x M symmetric matrix whose
      //    upper triangle is stored at W (row stride M): W becomes its inverse
      //    (and, without the tensor-core product, the R columns Rg become
      //    X^-1 Rg).  Ends with a cluster barrier.
      auto gj = [&](double2* W, const int M) {
        unsigned long long best = 0ULL;
        int bi = 0x7fffffff;
        for (int i = tid; i < M; i += NT) {
          const double2 x = __ldcg(W + (int64_t)i * M + i);
          dg[i] = x;
          used[i] = 0;
          const unsigned long long k = pivot_key(x);
          if (k > best) {
            best = k;
            bi = i;
          }
        }
        reduce_pivot(best, bi, 0ULL);

        // 3. Blocked symmetric Gauss-Jordan.
        for (int k0 = 0; k0 < M; k0 += NB) {
          const int nbk = min(NB, M - k0);
          for (int i = tid; i < M; i += NT) used0[i] = used[i];
          __syncthreads();
          for (int kk = 0; kk < nbk; ++kk) {
            int p = s_p;
            if (p < 0) {  // zero or NaN diagonal everywhere left: the pivoted kernel decides
              if (tid == 0) s_status = kStatusNeedPivot;
              p = 0;
              while (p < M - 1 && used[p]) ++p;
            }
            // a. column p at the panel start: W[i][p] above the diagonal, and
            //    below it M[i][p] = +-W[p][i], minus when i was swept before the panel
            for (int i = tid; i < M; i += NT) {
              double2 v;
              if (i <= p) {
                v = __ldcg(W + (int64_t)i * M + p);
              } else {
                v = __ldcg(W + (int64_t)p * M + i);
                if (used0[i]) v = cneg(v);
              }
              PR[(int64_t)kk * M + i] = v;
              colb[i] = v;
            }
            __syncthreads();
            if (kk > 0) {
              // b. the panel's earlier steps: z_m = x[p_m] + sum_{l<m} u_l[p_m] z_l, x += U z
              if (tid == 0) {
                for (int m = 0; m < kk; ++m) {
                  const int pm = piv[k0 + m];
                  double2 v = colb[pm];
                  for (int l = 0; l < m; ++l) v = cfms(v, cneg(Ub[pm * NB + l]), zc[l]);
                  zc[m] = v;
                }
              }
              __syncthreads();
              for (int i = tid; i < M; i += NT) {
                double2 x = colb[i];
                for (int m = 0; m < kk; ++m) x = cfms(x, cneg(Ub[i * NB + m]), zc[m]);
                colb[i] = x;
              }
              __syncthreads();
            }
            // c. reciprocal, multipliers, diagonal update; the next pivot and the
            //    largest unswept entry of this column in one reduction
            const double2 z = colb[p];
            const double rden = 1.0 / fma(z.x, z.x, z.y * z.y);
            const double2 d = make_double2(z.x * rden, -z.y * rden);
            unsigned long long nbest = 0ULL, cm = 0ULL;
            int nbi = 0x7fffffff;
            for (int i = tid; i < M; i += NT) {
              const double2 g = colb[i];
              double2 u;
              if (i == p) {
                u = make_double2(d.x - 1.0, d.y);
              } else {
                u = cneg(cmul(g, d));
              }
              Ub[i * NB + kk] = u;
              if (!used[i] && i != p) {
                const unsigned long long kc = pivot_key(g);
                cm = kc > cm ? kc : cm;
                const double2 nd2 = cfms(dg[i], cneg(u), g);  // dg + u g
                dg[i] = nd2;
                const unsigned long long kd = pivot_key(nd2);
                if (kd > nbest) {
                  nbest = kd;
                  nbi = i;
                }
              }
            }
            reduce_pivot(nbest, nbi, cm);
            if (tid == 0) {
              const double zmag = __longlong_as_double((long long)pivot_key(z));
              const double omag = __longlong_as_double((long long)s_cmax);
              if (!(zmag > 0.0) || zmag < a.sym_tau * omag) s_status = kStatusNeedPivot;
              used[p] = 1;
              piv[k0 + kk] = p;
            }
            __syncthreads();
          }
          for (int e = tid; e < nbk * nbk; e += NT) {
            const int k = e / nbk, l = e % nbk;
            Lt[k * NB + l] = (l < k) ? Ub[piv[k0 + k] * NB + l] : make_double2(0.0, 0.0);
          }
          // The panel's column fetches read W anywhere (row p_k lies in other
          // columns), so no CTA of the cluster may start writing W until every
          // CTA has finished factoring the panel.
          if (C > 1) cluster.sync();
          else __syncthreads();

          // d. The panel applied to every column of [W | R]: a column gets
          //    x += U z over its rows (i <= j for W, all for R), with
          //    z = (I - L)^-1 x[p] from its pivot rows (for W, the panel's raw
          //    pivot columns with the sign rule), and the panel's pivot column
          //    m is u_m + e_{p_m} with the later steps applied.
          auto column_z = [&](int kind, int j, int mcol, const double2* col, double2* zz) {
  #pragma unroll
            for (int k = 0; k < NB; ++k) zz[k] = make_double2(0.0, 0.0);
            if (kind == 1) {
  #pragma unroll
              for (int l = 0; l < NB; ++l) {
                if (l > mcol && l < nbk) {
                  double2 v = Lt[l * NB + mcol];
  #pragma unroll
                  for (int q = 0; q < NB; ++q)
                    if (q > mcol && q < l) v = cfms(v, cneg(Lt[l * NB + q]), zz[q]);
                  zz[l] = v;
                }
              }
            } else {
              const double sg = (kind == 0 && used0[j]) ? -1.0 : 1.0;
  #pragma unroll
              for (int m = 0; m < NB; ++m) {
                if (m < nbk) {
                  double2 v = (kind == 0) ? cscale(sg, __ldcg(PR + (int64_t)m * M + j))
                                          : __ldcg(col + (int64_t)piv[k0 + m] * M);
  #pragma unroll
                  for (int l = 0; l < m; ++l) v = cfms(v, cneg(Lt[m * NB + l]), zz[l]);
                  zz[m] = v;
                }
              }
            }
          };
          // The rows of a unit as one sequence of virtual rows v = sub, sub+T,
          // ... < lena + lenb: v < lena is row v of column a, the rest row
          // v - lena of column b.  A pair unit has M+1 virtual rows and an R
          // unit M, so the threads of a warp (consecutive units) run the same
          // trip count and their FP64 instructions keep every lane busy.
          struct Col {
            int kind, j, mcol, len;
            double2* col;
          };
          auto unit_rows = [&](const Col& A, const double2* za, const Col& B, const double2* zb, int sub, int T) {
            const int tot = A.len + B.len;
            // the starting value of virtual row v and where it goes
            auto load = [&](int v, int* irow, double2** dst) {
              const bool inA = v < A.len;
              const Col& c = inA ? A : B;
              const int i = inA ? v : v - A.len;
              *irow = i;
              *dst = c.col + (int64_t)i * M;
              if (c.kind == 1) {
                double2 x = Ub[i * NB + c.mcol];
                if (i == c.j) x.x += 1.0;
                return x;
              }
              return __ldcg(*dst);
            };
            int v = sub;
            for (; v < tot; v += T) {
              int i;
              double2* d;
              double2 x = load(v, &i, &d);
              const bool a0 = v < A.len;
              const double2* ui = Ub + i * NB;
  #pragma unroll
              for (int k = 0; k < NB; ++k)
                if (k < nbk) x = cfms(x, cneg(ui[k]), a0 ? za[k] : zb[k]);
              *d = x;
            }
          };
          // Which kind of W column j is: 1 if it is pivot mcol of this panel.
          auto w_kind = [&](int j, int* mcol) {
            *mcol = -1;
            if (used[j] && !used0[j]) {
              for (int m = 0; m < nbk; ++m)
                if (piv[k0 + m] == j) *mcol = m;
              return 1;
            }
            return 0;
          };
          // Units: the W column pairs (q, M-1-q), M+1 rows together, then the
          // R columns (M rows), dealt round-robin to the cluster's CTAs.  T
          // threads share a unit's rows (T = 1, 4 or 8, whichever gives the
          // fewest rows per thread); with T > 1 the unit's z vectors (two for
          // a pair) come through shared memory, [NT/4][2][NB] at most.
          const int P = (M + 1) / 2;
          const int ucta = (P + (gemm_on ? 0 : M) - rank + C - 1) / C;  // R columns only without the product
          int T = 1;
          if (a.force_rowsplit == 1 || a.force_rowsplit == 4 || a.force_rowsplit == 8) {
            T = a.force_rowsplit;  // the autotuner's choice (the same arithmetic per element)
          } else {
            int best = ((ucta + NT - 1) / NT) * (M + 1);
            for (int t = 4; t <= kSymMaxRowSplit; t *= 2) {
              const int rows = ((ucta + NT / t - 1) / (NT / t)) * ((M + 1 + t - 1) / t);
              if (rows < best) {
                best = rows;
                T = t;
              }
            }
          }
          const int NCH = NT / T;
          const int cs = tid % NCH, sub = tid / NCH;
          for (int c0 = 0; c0 < ucta; c0 += NCH) {
            const int c = c0 + cs;
            const bool active = c < ucta;
            const int u = rank + C * c;
            int ka = 0, kb = 0, ja = 0, jb = 0, ma = -1, mb = -1, lena = 0, lenb = 0;
            double2* cola = nullptr;
            double2* colb2 = nullptr;
            if (active) {
              if (u < P) {
                ja = u;
                jb = M - 1 - u;
                lena = ja + 1;
                lenb = (jb != ja) ? jb + 1 : 0;
                cola = W + ja;
                colb2 = W + jb;
                ka = w_kind(ja, &ma);
                if (lenb) kb = w_kind(jb, &mb);
              } else {
                ka = 2;
                ja = u - P;
                lena = M;
                cola = Rg + ja;
              }
            }
            const Col A{ka, ja, ma, lena, cola};
            const Col B{kb, jb, mb, lenb, colb2 ? colb2 : cola};
            double2 za[NB], zb[NB];
  #pragma unroll
            for (int k = 0; k < NB; ++k) zb[k] = make_double2(0.0, 0.0);
            if (T == 1) {
              if (active) {
                column_z(ka, ja, ma, cola, za);
                if (lenb) column_z(kb, jb, mb, colb2, zb);
                unit_rows(A, za, B, zb, 0, 1);
              }
            } else {
              if (active && sub < 2 && (sub == 0 || lenb)) {
                double2 zz[NB];
                if (sub == 0) column_z(ka, ja, ma, cola, zz);
                else column_z(kb, jb, mb, colb2, zz);
  #pragma unroll
                for (int k = 0; k < NB; ++k) zsh[(cs * 2 + sub) * NB + k] = zz[k];
              }
              __syncthreads();  // z is read before any row of these columns changes
              if (active) {
  #pragma unroll
                for (int k = 0; k < NB; ++k) za[k] = zsh[(cs * 2) * NB + k];
                if (lenb) {
  #pragma unroll
                  for (int k = 0; k < NB; ++k) zb[k] = zsh[(cs * 2 + 1) * NB + k];
                }
                unit_rows(A, za, B, zb, sub, T);
              }
              __syncthreads();  // zsh is reused by the next chunk
            }
          }
          cluster.sync();
        }
      };
      // Symmetric Gauss-Jordan of an n x n block (n <= kSmallGJ, upper
      // triangle at P, row stride n) in shared memory: every CTA of the
      // cluster eliminates the whole block on its own copy (no cluster
      // barrier per step; the block's FP64 work is small), rank 0 writes the
      // inverse back.  Step k pivots on the largest unswept diagonal element
      // (ties: lowest index); with d = 1/M[p][p], r_j = M[p][j] and
      // g_i = M[i][p] (the swept/unswept sign rule of the blocked sweep),
      //   M[i][j] -= g_i d r_j (i, j != p),  M[p][j] = d r_j,
      //   M[i][p] = -g_i d,  M[p][p] = d.
      // A pivot below sym_tau times the largest unswept entry of its row
      // flags the realization.  Ends with a cluster barrier.
      auto gj_small = [&](double2* P, const int nb) {
        const int ld = nb + 1, ntri = nb * (nb + 1) / 2;
        double2* Sw = reinterpret_cast<double2*>(stage);  // [nb][ld], upper triangle
        double2* gcol = Sw + nb * ld;                      // [nb] g_i
        double2* roww = gcol + nb;                         // [nb] d r_j
        int* sused = reinterpret_cast<int*>(roww + nb);    // [nb] swept flags
        int* tri = sused + nb;                             // [ntri] (i << 16) | j
        __syncthreads();  // the staging area's previous contents have been used
        for (int e = tid; e < nb * nb; e += NT) {
          const int i = e / nb, j = e % nb;
          if (i <= j) Sw[i * ld + j] = __ldcg(P + (int64_t)i * nb + j);
        }
        for (int i = tid; i < nb; i += NT) {
          sused[i] = 0;
          const int base = i * nb - i * (i - 1) / 2;  // triangle elements of rows < i
          for (int j = i; j < nb; ++j) tri[base + j - i] = (i << 16) | j;
        }
        cluster.sync();  // every CTA has read P before rank 0 overwrites it
        for (int k = 0; k < nb; ++k) {
          if (warp == k % NW) {
            unsigned long long best = 0ULL;
            int bi = 0x7fffffff;
            for (int i = lane; i < nb; i += 32) {
              const unsigned long long key = sused[i] ? 0ULL : pivot_key(Sw[i * ld + i]);
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
            const bool singular = (best == 0ULL);
            if (singular) {  // zero or NaN diagonal everywhere left: the pivoted kernel decides
              bi = 0;
              while (bi < nb - 1 && sused[bi]) ++bi;
            }
            const int pk = bi;
            double2 d = make_double2(0.0, 0.0);
            if (!singular) {
              const double2 z = Sw[pk * ld + pk];
              const double rden = 1.0 / fma(z.x, z.x, z.y * z.y);
              d = make_double2(z.x * rden, -z.y * rden);
            }
            unsigned long long offmax = 0ULL;
            for (int j = lane; j < nb; j += 32) {
              double2 rj, gjv;
              if (j < pk) {
                const double2 u = Sw[j * ld + pk];
                rj = sused[j] ? cneg(u) : u;
                gjv = u;
              } else {
                const double2 u = Sw[pk * ld + j];
                rj = u;
                gjv = sused[j] ? cneg(u) : u;
              }
              if (j != pk && !sused[j]) {
                const unsigned long long kk2 = pivot_key(rj);
                offmax = kk2 > offmax ? kk2 : offmax;
              }
              gcol[j] = gjv;
              roww[j] = (j == pk) ? d : cmul(d, rj);
            }
#pragma unroll
            for (int off = 16; off; off >>= 1) {
              const unsigned long long o2 = __shfl_xor_sync(0xffffffffu, offmax, off);
              offmax = o2 > offmax ? o2 : offmax;
            }
            __syncwarp();  // every lane has read sused[] before lane 0 marks pk
            if (lane == 0) {
              const double zmag = __longlong_as_double((long long)best);
              const double omag = __longlong_as_double((long long)offmax);
              if (singular || zmag < a.sym_tau * omag) s_status = kStatusNeedPivot;
              sused[pk] = 1;
              s_p = pk;
            }
          }
          __syncthreads();
          const int pk = s_p;
          for (int e = tid; e < ntri; e += NT) {
            const int i = tri[e] >> 16, j = tri[e] & 0xffff;
            const double2 rj = roww[j];
            const double2 w = (i == pk) ? rj : (j == pk) ? make_double2(0.0, 0.0) : Sw[i * ld + j];
            const double2 f = (i == pk) ? make_double2(0.0, 0.0) : gcol[i];
            Sw[i * ld + j] = cfms(w, f, rj);
          }
          __syncthreads();
        }
        if (rank == 0)
          for (int e = tid; e < ntri; e += NT) {
            const int i = tri[e] >> 16, j = tri[e] & 0xffff;
            P[(int64_t)i * nb + j] = Sw[i * ld + j];
          }
        cluster.sync();
      };
      const ZgemmCtx zc{ea_s, eb_s, expart, adig, bdig, stage};
      auto wsym = [&](const double2* Wb, int Mb, int i, int j) {  // symmetric matrix from its upper triangle
        return __ldcg(Wb + (i <= j ? (int64_t)i * Mb + j : (int64_t)j * Mb + i));
      };

      // X^-1 by its 2 x 2 block form, X = [[A, B], [B^T, D]] with h x h
      // blocks, two half-size inverses and four half-size products on the
      // tensor cores:
      //   T = A^-1 B,  S = D - B^T T,  Y12 = -T S^-1,  Y11 = A^-1 - Y12 T^T,
      //   Y22 = S^-1,
      // with, at two levels, the half-size inverses of A and S in the same
      // form.  The steps (kInvSteps) act on frames: frame 0 splits X (at W,
      // row stride M) with the buffers Wa, Tb, Ws; frames 1 and 2 split A^-1's
      // block Wa and S's block Ws (row stride h) with Wa2, Tb2, Ws2.  Every
      // Gauss-Jordan block goes through the one call below.  A small pivot in
      // a block flags the realization as the full elimination does.
      {
        const int nsteps = kInvStepCount[split_levels];
        for (int st = 0; st < nsteps; ++st) {
          const int code = kInvSteps[split_levels][st];
          const int op = code >> 2, f = code & 3;
          double2* P = f == 0 ? W : (f == 1 ? Wa : Ws);
          const int nP = f == 0 ? M : M >> 1;  // also P's row stride
          double2* Ha = f == 0 ? Wa : Wa2;
          double2* Hb = f == 0 ? Tb : Tb2;
          double2* Hs = f == 0 ? Ws : Ws2;
          const int h = nP >> 1;
          const int64_t hh = (int64_t)h * h;
          if (op == kInvGJ || op == kInvGJA || op == kInvGJS) {
            double2* Q = op == kInvGJ ? W : (op == kInvGJA ? Ha : Hs);
            const int nq = op == kInvGJ ? M : h;
            if (nq <= kSmallGJ) gj_small(Q, nq);
            else gj(Q, nq);
          } else if (op == kInvCopyA) {  // A into Ha (upper triangle)
            for (int64_t e = ctid; e < hh; e += CNT) {
              const int i = (int)(e / h), j = (int)(e % h);
              if (i <= j) Ha[e] = __ldcg(P + (int64_t)i * nP + j);
            }
            cluster.sync();
          } else if (op == kInvT) {
            cluster_zgemm(zc, h, Opnd{Ha, h, 0, 1, 0}, Opnd{P, nP, h, 0, 0}, TileOut{Hb, h, 0, 1.0, nullptr, 0, 0, 0, 0});
          } else if (op == kInvS) {
            cluster_zgemm(zc, h, Opnd{P, nP, h, 0, 1}, Opnd{Hb, h, 0, 0, 0},
                          TileOut{Hs, h, 0, -1.0, P, nP, (int64_t)h * nP + h, 0, 1});
          } else if (op == kInvY12) {
            cluster_zgemm(zc, h, Opnd{Hb, h, 0, 0, 0}, Opnd{Hs, h, 0, 1, 0}, TileOut{P, nP, h, -1.0, nullptr, 0, 0, 0, 0});
          } else if (op == kInvY11) {
            cluster_zgemm(zc, h, Opnd{P, nP, h, 0, 0}, Opnd{Hb, h, 0, 0, 1}, TileOut{P, nP, 0, -1.0, Ha, h, 0, 1, 1});
          } else {  // kInvY22: Y22 = S^-1
            for (int64_t e = ctid; e < hh; e += CNT) {
              const int i = (int)(e / h), j = (int)(e % h);
              if (i <= j) P[(int64_t)(h + i) * nP + h + j] = __ldcg(Hs + e);
            }
            cluster.sync();
          }
        }
      }

      if (gemm_on) {
        // 4. B Gs1 <- X^-1 (B Gs1) on the tensor cores (rg_ozaki.cuh).
        if (n < a.inject_at) {
          // before the source slice the right-hand side is zero and stays zero
        } else if (n == a.inject_at) {
          // X^-1 (+-I) at the source slice: the full symmetric inverse itself
          // (+I at slice 0, -I at a later source slice)
          const double sg = n == 0 ? 1.0 : -1.0;
          for (int64_t e = ctid; e < mm; e += CNT) {
            const int i = (int)(e / M), j = (int)(e % M);
            Rg[e] = cscale(sg, wsym(W, M, i, j));
          }
          cluster.sync();  // the new right-hand side is complete before the next slice
        } else {
          // the result overwrites B Gs1 in place (its digits are already taken)
          cluster_zgemm(zc, M, Opnd{W, M, 0, 1, 0}, Opnd{Rg, M, 0, 0, 0}, TileOut{Rg, M, 0, 1.0, nullptr, 0, 0, 0, 0});
        }
      }
      if (a.state_dump && *status0 != kStatusNeedPivot) {
        // The state after this slice, natural order: Gss = W (symmetric,
        // upper triangle) and Gs1 = sign * R, the solve_block_tridiag pair
        // (S_n, Z_n).
        double2* d1 = a.state_dump + ((int64_t)r * wd.nx + n) * 2 * mm;
        const double gs = (n == 0) ? 1.0 : -1.0;
        for (int64_t e = ctid; e < mm; e += CNT) {
          const int i = (int)(e / M), j = (int)(e % M);
          d1[e] = __ldcg(W + (i <= j ? (int64_t)i * M + j : (int64_t)j * M + i));
          d1[mm + e] = cscale(gs, __ldcg(Rg + e));
        }
        cluster.sync();  // W and R are read before the next slice rewrites them
      }
    }

    if (*status0 == kStatusNeedPivot) {
      cluster.sync();  // every CTA has read the flag before rank 0 moves on
      if (rank == 0 && tid == 0) {
        a.status[r] = kStatusNeedPivot;
        a.flag_list[atomicAdd(a.work_counter + 1, 1)] = r;
      }
      cluster.sync();
      continue;
    }
    if (ne < wd.nx) {  // stopped early (timing proxy): no Fisher-Lee stage
      __syncthreads();
      if (rank == 0 && tid == 0) a.status[r] = s_status;
      cluster.sync();
      continue;
    }

    if (refl) {
      // Reflection from the reverse sweep: G11 = W (symmetric, upper triangle),
      // r = -1 + 2i sqrt(real mu) G11 sqrt(real mu) (src/waveguide.f90:510-512).
      double2* rout = a.tout + (int64_t)r * M * M;
      for (int e = ctid; e < M * M; e += CNT) {
        const int i = e % M, j = e / M;
        const double2 gij = __ldcg(W + (i <= j ? (int64_t)i * M + j : (int64_t)j * M + i));
        const double2 v = cmul(cmul(wd.sqmu_r[i], gij), wd.sqmu_r[j]);
        rout[e] = make_double2((i == j ? -1.0 : 0.0) - 2.0 * v.y, 2.0 * v.x);
      }
      __syncthreads();
      if (rank == 0 && tid == 0) a.status[r] = s_status;
      cluster.sync();
      continue;
    }

    // 5. Fisher-Lee from R (natural order): t = 2i sqmu Gs1 sqmu, Gs1 = sign R,
    //    into the workspace, column-major (ld = nrow).
    const double gsign = (wd.nx >= 2) ? -1.0 : 1.0;
    const int row0 = tmat ? 0 : wd.row0, col0 = tmat ? 0 : wd.col0;
    const int nrow = tmat ? M : wd.nrow, ncol = tmat ? M : wd.ncol;
    const double2* sqmu = tmat ? wd.sqmu_r : wd.sqmu_c;
    double2* tout = a.tout ? a.tout + (int64_t)r * nrow * ncol : nullptr;
    for (int e = ctid; e < nrow * ncol; e += CNT) {
      const int i = e % nrow, j = e / nrow;
      const int gi = row0 + i, gj = col0 + j;
      const double2 g = cscale(gsign, __ldcg(Rg + (int64_t)gi * M + gj));
      const double2 v = cmul(cmul(sqmu[gi], g), sqmu[gj]);
      const double2 t = make_double2(-2.0 * v.y, 2.0 * v.x);
      Tg[e] = t;
      if (tout) tout[e] = t;
    }
    cluster.sync();

    if (!tmat) {
      // 6. Eigenvalues of t^H t: one-sided Jacobi on the vectors of the
      //    smaller dimension, in the workspace; the pairs of a round are
      //    split over the cluster's warps.
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
      if (sweep == 60 && tid == 0 && s_status == RG_OK) s_status = RG_ERR_NOCONV;
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

// Same cluster-size policy as the pivoted blocked kernel (sweep_large_plan).
int sweep_large_sym_plan(SweepArgs& a, int sm_count, int* grid, int64_t* work_stride) {
  if (a.max_M > 512) a.tensor_r = 0;  // the product's int64 fold is sized for M <= 512
  const bool tensor = a.tensor_r != 0;
  const size_t smem = LargeSymSmem::bytes(a.max_M, tensor);
  if (smem > 227 * 1024) return fail(RG_ERR_INVALID_ARG, "too many modes for the symmetric large-mode kernel");
  RG_CUDA(cudaFuncSetAttribute(sweep_large_sym_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_large_sym_kernel, kSymNT, smem));
  if (per_sm < 1) return fail(RG_ERR_INVALID_ARG, "symmetric large-mode sweep kernel does not fit on an SM");
  const int slots = per_sm * sm_count;
  int C = 1;
  if (a.force_cluster > 0) {
    while (C < kSymMaxCluster && C < a.force_cluster) C *= 2;
  } else {
    while (C < kSymMaxCluster && (int64_t)a.nreal * C * 2 <= slots) C *= 2;
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
    cfg.blockDim = dim3(kSymNT);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int maxc = 0;
    RG_CUDA(cudaOccupancyMaxActiveClusters(&maxc, sweep_large_sym_kernel, &cfg));
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
  *work_stride = large_sym_stride(a.max_M, a.max_ny, tensor);
  return RG_OK;
}

int launch_sweep_large_sym(const SweepArgs& a, cudaStream_t stream, int grid) {
  if (a.nreal <= 0) return RG_OK;
  const size_t smem = LargeSymSmem::bytes(a.max_M, a.tensor_r != 0);
  const int C = a.cluster > 0 ? a.cluster : 1;
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute attr{};
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = C;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kSymNT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  RG_CUDA(cudaLaunchKernelEx(&cfg, sweep_large_sym_kernel, a));
  return RG_OK;
}

}  // namespace rg
