// Complex FP64 matrix products on the FP16 tensor cores (Ozaki splitting).
//
// C = A B for M x M complex matrices (M <= 512), computed with mma.sync
// m16n8k16 (FP16 inputs, FP32 accumulation) to FP64 accuracy:
//
//  * every row i of A gets the exponent ea_i of its largest |re| or |im|
//    (|A_ik| < 2^ea_i), every column j of B the exponent eb_j likewise;
//  * each entry is written as a 53-bit fixed-point integer relative to that
//    power of two (rounded to nearest), X = |A_ik| 2^(53-ea_i) < 2^53, and
//    cut into six balanced base-512 digits (from the least significant up,
//    a digit of 256 or more becomes digit - 512 with a carry into the next;
//    the top one takes the last carry), so |d_p| <= 256 and
//        A_ik = 2^ea_i sum_p d_p 2^(-8-9p),  p = 0..5
//    (each digit exact in FP16, each product of two below 2^16);
//  * C_ij = 2^(ea_i + eb_j) sum_l v_l 2^(-16-9l) with
//        v_l = sum_{p+q=l} sum_k a_p(i,k) b_q(k,j),
//    and levels l <= 6 kept (26 digit pairs; the first dropped level lies
//    near 2^-53 K relative to 2^(ea_i+eb_j), an FP64 product's own error
//    bound);
//  * v_l is accumulated in FP32 over chunks of 16 complex k: at most
//    6 pairs x 32 real products x 2^16 = 12,582,912 < 2^24 per level, so
//    every partial sum is an integer below 2^24 and the accumulation is
//    exact; after each chunk the levels are folded into two int64 sums,
//    hi = sum_{l<=2} v_l 2^(9(2-l)) and lo = sum_{l>=3} v_l 2^(9(6-l)),
//    which are exact too (|hi| < 2^46, |lo| < 2^56 for M <= 512);
//  * finally C_ij = 2^(ea_i+eb_j) (hi 2^-34 + lo 2^-70), one rounding.
//
// The result is the correctly rounded value of the digit sum, so it does
// not depend on how tiles are spread over warps or CTAs, and it equals an
// exact integer model of the same steps bit for bit.  Its error is that of
// the dropped digit pairs and the 2^-53 rounding of the inputs, i.e.
// normwise at the level of an FP64 product (2^-53 K |A_i| |B_j| at worst).
//
// Layouts ("fragment-native", so a lane loads its mma operand with one
// 16-byte access).  With T = ceil(M/16) tiles per dimension:
//   A digits  uint4 [2 parts][6 slices][T row tiles][T k tiles][32 lanes]
//             lane (g = lane/4, t = lane%4) of tile (ti, tk) holds the halves
//             (A[g][2t], A[g][2t+1]), (A[g+8][2t], A[g+8][2t+1]),
//             (A[g][2t+8], A[g][2t+9]), (A[g+8][2t+8], A[g+8][2t+9])
//             of the 16 x 16 tile: the m16n8k16 A fragment (row-major);
//   B digits  uint4 [2 parts][6 slices][T col tiles][T k tiles][32 lanes]
//             lane holds (B[2t][g], B[2t+1][g]), (B[2t+8][g], B[2t+9][g]) of
//             columns 0..7 of the tile, then the same for columns 8..15: two
//             m16n8k16 B fragments (column-major);
//   accumulators: c0 = C[g][2t], c1 = C[g][2t+1], c2 = C[g+8][2t], c3 = C[g+8][2t+1].
// Rows/columns beyond M are zero digits.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

namespace rg {
namespace oz {

constexpr int kSlices = 6;      // digits per entry
constexpr int kDigitBits = 9;   // base 2^9, balanced digits in [-256, 256]
constexpr int kFixedBits = 53;  // fixed-point bits of an entry
constexpr int kLmax = 6;        // highest level kept
constexpr int kHiLevels = 3;    // levels 0..2 fold into hi, 3..6 into lo
constexpr int kNoExp = -4096;   // exponent of zero rows
// C = 2^(ea+eb) (hi kHiScale + lo kLoScale)
constexpr double kHiScale = 0x1p-34;  // 2^-(16 + 9 (kHiLevels - 1))
constexpr double kLoScale = 0x1p-70;  // 2^-(16 + 9 kLmax)

__host__ __device__ inline int tiles(int M) { return (M + 15) >> 4; }
// uint4 elements of one operand's digits
__host__ __device__ inline int64_t operand_uint4(int M) {
  const int64_t T = tiles(M);
  return 2LL * kSlices * T * T * 32;
}
// bytes of both operands' digits plus the exponents (2 x M ints, 16-byte padded)
__host__ __device__ inline int64_t workspace_bytes(int M) {
  return 2 * 16 * operand_uint4(M) + (((int64_t)2 * tiles(M) * 16 * 4 + 15) & ~15LL);
}

// frexp exponent of |x| (|x| < 2^e), kNoExp for zeros and subnormals.
__device__ __forceinline__ int fexp(double x) {
  const int eb = (int)((__double_as_longlong(x) >> 52) & 0x7ff);
  return eb == 0 ? kNoExp : eb - 1022;
}

__device__ __forceinline__ int fexp2(double2 v) { return max(fexp(v.x), fexp(v.y)); }

// |x| 2^(53-e) rounded to nearest, as an integer below 2^53 (e >= fexp(x)).
__device__ __forceinline__ uint64_t fixed53(double x, int e) {
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const int eb = (int)((bits >> 52) & 0x7ff);
  if (eb == 0) return 0;
  const uint64_t m = (bits & ((1ULL << 52) - 1)) | (1ULL << 52);
  const int rs = e - (eb - 1022);  // |x| 2^(53-e) = m 2^-rs, rs >= 0
  if (rs == 0) return m;
  if (rs > 54) return 0;
  return (m + (1ULL << (rs - 1))) >> rs;
}

// The six balanced base-512 digits of X < 2^53, d[0] the most significant:
// X = sum_p d[p] 2^(9(5-p)), |d[p]| <= 256.
__device__ __forceinline__ void balanced_digits(uint64_t X, int d[kSlices]) {
  int carry = 0;
#pragma unroll
  for (int p = kSlices - 1; p > 0; --p) {
    const int t = (int)((X >> (kDigitBits * (kSlices - 1 - p))) & 511u) + carry;
    carry = t >= 256 ? 1 : 0;
    d[p] = t - (carry << 9);
  }
  d[0] = (int)(X >> (kDigitBits * (kSlices - 1))) + carry;
}

// Two signed digits as FP16 halves (lo = first); the entries' signs n0, n1
// multiply them.  A magnitude m <= 256 is made exact in FP16 as
// (1024 + m) - 1024, then the sign bit is set.
__device__ __forceinline__ uint32_t digit_pair(int d0, bool n0, int d1, bool n1) {
  const uint32_t m0 = (uint32_t)abs(d0), m1 = (uint32_t)abs(d1);
  const uint32_t biased = (0x6400u | m0) | ((0x6400u | m1) << 16);
  __half2 h;
  memcpy(&h, &biased, 4);
  h = __hsub2(h, __floats2half2_rn(1024.0f, 1024.0f));
  uint32_t r;
  memcpy(&r, &h, 4);
  // the sign of a zero digit does not matter (its products are +-0)
  return r ^ ((n0 != (d0 < 0) ? 0x8000u : 0u) | (n1 != (d1 < 0) ? 0x80000000u : 0u));
}

// Writes the 12 uint4 (2 parts x 6 slices) of one lane of one tile from its
// 8 complex entries v[0..7] in fragment order (see the layout above) and
// the row (A) or column (B) exponents of each entry: for A, entries 0,1,4,5
// lie on row g and 2,3,6,7 on row g+8; for B, entries 0..3 on column g and
// 4..7 on column g+8.  dst points at [part 0][slice 0][this tile][lane];
// `plane` is the uint4 stride between slices.
__device__ __forceinline__ void write_digits(const double2 v[8], const int e[8], uint4* dst, int64_t plane) {
  uint32_t rw[kSlices][4], iw[kSlices][4];
#pragma unroll
  for (int w = 0; w < 4; ++w) {
    int dr0[kSlices], dr1[kSlices], di0[kSlices], di1[kSlices];
    balanced_digits(fixed53(v[2 * w].x, e[2 * w]), dr0);
    balanced_digits(fixed53(v[2 * w + 1].x, e[2 * w + 1]), dr1);
    balanced_digits(fixed53(v[2 * w].y, e[2 * w]), di0);
    balanced_digits(fixed53(v[2 * w + 1].y, e[2 * w + 1]), di1);
#pragma unroll
    for (int p = 0; p < kSlices; ++p) {
      rw[p][w] = digit_pair(dr0[p], v[2 * w].x < 0.0, dr1[p], v[2 * w + 1].x < 0.0);
      iw[p][w] = digit_pair(di0[p], v[2 * w].y < 0.0, di1[p], v[2 * w + 1].y < 0.0);
    }
  }
#pragma unroll
  for (int p = 0; p < kSlices; ++p) {
    __stcg(dst + p * plane, make_uint4(rw[p][0], rw[p][1], rw[p][2], rw[p][3]));
    __stcg(dst + (kSlices + p) * plane, make_uint4(iw[p][0], iw[p][1], iw[p][2], iw[p][3]));
  }
}

// Digit planes of A: entries A(i, k) = getA(i, k) (zero outside M x M),
// exponents ea[i].  Task = (row tile, k tile, lane), spread over
// [task0, ntask) with stride `step`.
template <class GetA>
__device__ void split_a(int M, GetA getA, const int* ea, uint4* dig, int task0, int step) {
  const int T = tiles(M);
  const int64_t plane = (int64_t)T * T * 32;
  const int ntask = T * T * 32;
  for (int task = task0; task < ntask; task += step) {
    const int lane = task & 31, tk = (task >> 5) % T, ti = (task >> 5) / T;
    const int g = lane >> 2, t = lane & 3;
    const int r0 = ti * 16 + g, r1 = r0 + 8;
    const int cs[4] = {tk * 16 + 2 * t, tk * 16 + 2 * t + 1, tk * 16 + 2 * t + 8, tk * 16 + 2 * t + 9};
    double2 v[8];
    int e[8];
    const int rows[8] = {r0, r0, r1, r1, r0, r0, r1, r1};
    const int cols[8] = {cs[0], cs[1], cs[0], cs[1], cs[2], cs[3], cs[2], cs[3]};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const bool in = rows[k] < M && cols[k] < M;
      v[k] = in ? getA(rows[k], cols[k]) : make_double2(0.0, 0.0);
      e[k] = rows[k] < M ? ea[rows[k]] : 0;
    }
    write_digits(v, e, dig + ((int64_t)ti * T + tk) * 32 + lane, plane);
  }
}

// Digit planes of B: entries B(k, j) = getB(k, j), exponents eb[j].
template <class GetB>
__device__ void split_b(int M, GetB getB, const int* eb, uint4* dig, int task0, int step) {
  const int T = tiles(M);
  const int64_t plane = (int64_t)T * T * 32;
  const int ntask = T * T * 32;
  for (int task = task0; task < ntask; task += step) {
    const int lane = task & 31, tk = (task >> 5) % T, tj = (task >> 5) / T;
    const int g = lane >> 2, t = lane & 3;
    const int c0 = tj * 16 + g, c1 = c0 + 8;
    const int ks[4] = {tk * 16 + 2 * t, tk * 16 + 2 * t + 1, tk * 16 + 2 * t + 8, tk * 16 + 2 * t + 9};
    double2 v[8];
    int e[8];
    const int rows[8] = {ks[0], ks[1], ks[2], ks[3], ks[0], ks[1], ks[2], ks[3]};
    const int cols[8] = {c0, c0, c0, c0, c1, c1, c1, c1};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const bool in = rows[k] < M && cols[k] < M;
      v[k] = in ? getB(rows[k], cols[k]) : make_double2(0.0, 0.0);
      e[k] = cols[k] < M ? eb[cols[k]] : 0;
    }
    write_digits(v, e, dig + ((int64_t)tj * T + tk) * 32 + lane, plane);
  }
}

__device__ __forceinline__ void mma16816(float c[4], const uint4& a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void cp_async16(uint4* smem_dst, const uint4* gsrc) {
  const unsigned saddr = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// all but the most recently committed group complete
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// ---------------------------------------------------------------------------
// The CTA-blocked product: a CTA of 8 warps computes a 2 x 4 block of 16 x 16
// complex tiles (warp w: row tile ti0 + w/4, column tile tj0 + w%4).  Both
// operands' digits for the block and one k tile -- A for 2 row tiles, B for 4
// column tiles, 36 KB -- are staged in shared memory with cp.async, two
// stages deep (stg: kBlkStageUint4 uint4 = 72 KB), so the copy of k tile
// t + 1 runs while the tensor cores work on k tile t and the loop reads no
// global memory; every staged A digit serves 4 tiles and every B digit 2.
// The level sums of a k tile are folded after it.  With
// `upper`, warps whose tile lies wholly below the diagonal (ti > tj) skip the
// products (their outputs are not wanted).  out(i, j, re, im) stores C_ij
// (called for i, j < M only).
// ---------------------------------------------------------------------------
constexpr int kBlkRows = 2, kBlkCols = 4;
constexpr int kBlkAUint4 = kBlkRows * 2 * kSlices * 32;                 // one stage's A digits
constexpr int kBlkOneUint4 = (kBlkRows + kBlkCols) * 2 * kSlices * 32;  // one stage
constexpr int kBlkStageUint4 = 2 * kBlkOneUint4;                       // two stages

template <class Out>
__device__ void gemm_block(int M, int ti0, int tj0, bool upper, const uint4* adig, const uint4* bdig, const int* ea,
                           const int* eb, uint4* stg, Out out) {
  const int T = tiles(M);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wr = warp / kBlkCols, wc = warp % kBlkCols;
  const int ti = ti0 + wr, tj = tj0 + wc;
  const bool active = ti < T && tj < T && !(upper && ti > tj);
  const int64_t plane = (int64_t)T * T * 32;
  long long hi[16], lo[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) hi[k] = lo[k] = 0;
  // stage element e = (tile * 2 kSlices + part * kSlices + slice) * 32 + lane,
  // the A tiles first, then the B tiles
  auto fetch = [&](int tk, uint4* dst) {
    for (int e = tid; e < kBlkOneUint4; e += blockDim.x) {
      const int isB = e >= kBlkAUint4;
      const int f = isB ? e - kBlkAUint4 : e;
      const int ln = f & 31, ps = (f >> 5) % (2 * kSlices), tile = (f >> 5) / (2 * kSlices);
      const int t = isB ? tj0 + tile : ti0 + tile;
      if (t < T) cp_async16(dst + e, (isB ? bdig : adig) + ps * plane + ((int64_t)t * T + tk) * 32 + ln);
    }
    cp_async_commit();
  };
  __syncthreads();  // the stages' previous contents have been used
  fetch(0, stg);
  for (int tk = 0; tk < T; ++tk) {
    const uint4* cur = stg + (tk & 1) * kBlkOneUint4;
    if (tk + 1 < T) {
      fetch(tk + 1, stg + ((tk + 1) & 1) * kBlkOneUint4);
      cp_async_wait_one();
    } else {
      cp_async_wait_all();
    }
    __syncthreads();  // k tile tk is in `cur` for every warp
    if (active) {
      const uint4* Aw = cur + wr * 2 * kSlices * 32 + lane;
      const uint4* Bw = cur + kBlkAUint4 + wc * 2 * kSlices * 32 + lane;
#pragma unroll 1
      for (int l = 0; l <= kLmax; ++l) {
        float acc[4][4];  // [re n0, re n1, im n0, im n1][4]
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int w = 0; w < 4; ++w) acc[u][w] = 0.0f;
        const int p0 = max(0, l - (kSlices - 1)), p1 = min(l, kSlices - 1);
#pragma unroll 1
        for (int p = p0; p <= p1; ++p) {
          const int q = l - p;
          const uint4 var = Aw[p * 32], vai = Aw[(kSlices + p) * 32];
          const uint4 vb = Bw[q * 32], vc = Bw[(kSlices + q) * 32];
          // re += Ar Br - Ai Bi; im += Ar Bi + Ai Br
          mma16816(acc[0], var, vb.x, vb.y);
          mma16816(acc[0], vai, vc.x ^ 0x80008000u, vc.y ^ 0x80008000u);
          mma16816(acc[1], var, vb.z, vb.w);
          mma16816(acc[1], vai, vc.z ^ 0x80008000u, vc.w ^ 0x80008000u);
          mma16816(acc[2], var, vc.x, vc.y);
          mma16816(acc[2], vai, vb.x, vb.y);
          mma16816(acc[3], var, vc.z, vc.w);
          mma16816(acc[3], vai, vb.z, vb.w);
        }
        const bool in_hi = l < kHiLevels;
        const int sh = in_hi ? kDigitBits * (kHiLevels - 1 - l) : kDigitBits * (kLmax - l);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int w = 0; w < 4; ++w) {
            const long long v = (long long)__float2int_rn(acc[u][w]) << sh;
            if (in_hi) hi[u * 4 + w] += v;
            else lo[u * 4 + w] += v;
          }
      }
    }
    __syncthreads();  // every warp is done with `cur` before it is refilled
  }
  if (!active) return;
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int n = 0; n < 2; ++n)
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const int i = ti * 16 + g + ((w & 2) ? 8 : 0);
      const int j = tj * 16 + n * 8 + 2 * t + (w & 1);
      if (i < M && j < M) {
        const int e = ea[i] + eb[j];
        const double re = fma((double)hi[n * 4 + w], kHiScale, (double)lo[n * 4 + w] * kLoScale);
        const double im = fma((double)hi[8 + n * 4 + w], kHiScale, (double)lo[8 + n * 4 + w] * kLoScale);
        out(i, j, scalbn(re, e), scalbn(im, e));
      }
    }
}

}  // namespace oz
}  // namespace rg
