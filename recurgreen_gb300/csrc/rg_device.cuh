// Device helpers shared by the sweep kernels: complex FP64 arithmetic, the
// gfortran-style xoshiro256** generator and the integer pivot key.
#pragma once

#include "rg_internal.h"

namespace rg {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// w - f * r with four FMAs.
__device__ __forceinline__ double2 cfms(double2 w, double2 f, double2 r) {
  return make_double2(fma(-f.x, r.x, fma(f.y, r.y, w.x)), fma(-f.x, r.y, fma(-f.y, r.x, w.y)));
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

struct Xoshiro {
  uint64_t s0, s1, s2, s3;
  __device__ __forceinline__ void step() {
    const uint64_t t = s1 << 17;
    s2 ^= s0;
    s3 ^= s1;
    s1 ^= s2;
    s0 ^= s3;
    s2 ^= t;
    s3 = rotl64(s3, 45);
  }
  __device__ __forceinline__ uint64_t next() {
    const uint64_t r = rotl64(s1 * 5, 7) * 9;
    step();
    return r;
  }
};

// Seed array of random_seed(put=) from the ANSI-C LCG (randi_ansic,
// src/random_normal.f90:20-31), scrambled into the 256-bit state the way
// gfortran's runtime does it (last put element first, XOR keys).
__device__ __forceinline__ Xoshiro seeded_state(int32_t seed) {
  uint32_t s = (uint32_t)seed, put[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    s = 1103515245u * s + 12345u;
    put[i] = s;
  }
  const uint64_t k0 = 0xbd0c5b6e50c2df49ULL, k1 = 0xd46061cd46e1df38ULL;
  const uint64_t k2 = 0xbb4f4d4ed6103544ULL, k3 = 0x114a583d0756ad39ULL;
  Xoshiro x;
  x.s0 = ((uint64_t)put[7] | ((uint64_t)put[6] << 32)) ^ k0;
  x.s1 = ((uint64_t)put[5] | ((uint64_t)put[4] << 32)) ^ k1;
  x.s2 = ((uint64_t)put[3] | ((uint64_t)put[2] << 32)) ^ k2;
  x.s3 = ((uint64_t)put[1] | ((uint64_t)put[0] << 32)) ^ k3;
  return x;
}

__device__ __forceinline__ unsigned long long pivot_key(double2 x) {
  const unsigned long long a = (unsigned long long)__double_as_longlong(x.x) & 0x7fffffffffffffffULL;
  const unsigned long long b = (unsigned long long)__double_as_longlong(x.y) & 0x7fffffffffffffffULL;
  const unsigned long long m = a > b ? a : b;
  return m > 0x7ff0000000000000ULL ? 0ULL : m;  // NaN never wins
}

// Advances st by the jump polynomial poly (4 words, bit i = coefficient of
// x^i): the state after d steps is poly(T) applied to st when
// poly = x^d mod the characteristic polynomial of the xoshiro256 map T.
__device__ __forceinline__ Xoshiro jump_state(Xoshiro st, const uint64_t* poly) {
  Xoshiro acc{0, 0, 0, 0};
  for (int w = 0; w < 4; ++w) {
    const uint64_t pw = poly[w];
    for (int b = 0; b < 64; ++b) {
      if ((pw >> b) & 1ULL) {
        acc.s0 ^= st.s0;
        acc.s1 ^= st.s1;
        acc.s2 ^= st.s2;
        acc.s3 ^= st.s3;
      }
      st.step();
    }
  }
  return acc;
}

// One scaled normal from two draws: random_number's real(8) conversion (top
// 53 bits) and Box-Muller as src/random_normal.f90:63-65, times stdu
// (src/waveguide.f90:371).
__device__ __forceinline__ double scaled_normal(double stdu, Xoshiro& st) {
  const double twopi = 2.0 * 3.141592653589793;
  const double u1 = (double)(st.next() >> 11) * 0x1.0p-53;
  const double u2 = (double)(st.next() >> 11) * 0x1.0p-53;
  return stdu * (sqrt(-2.0 * log(u1)) * cos(twopi * u2));
}

// Eigenvalues of t^H t for the nrow x ncol matrix t held in shared memory at
// W[i * LDW + j], by one-sided (Hestenes) Jacobi on the vectors of the smaller
// dimension: columns of t if nrow >= ncol, else rows (the singular values of
// t^T equal those of t).  The largest neigv of T_k = |v_k|^2 go to out in
// descending order.  Every thread of the NT-thread block calls this; cc
// (min(nrow, ncol) doubles) and *rot are shared scratch.  Returns false when
// 60 sweeps did not converge (the same value in every thread).
template <int NT>
__device__ bool tt_eigenvalues(double2* W, int LDW, int nrow, int ncol, int neigv, double* cc, int* rot,
                               double* out) {
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool bycol = nrow >= ncol;
  const int nv = bycol ? ncol : nrow;
  const int L = bycol ? nrow : ncol;
  const int es = bycol ? LDW : 1;  // element stride inside a vector
  const int vs = bycol ? 1 : LDW;  // stride between vectors
  const int NP = (nv + 1) & ~1;
  const double tol = 2.220446049250313e-16 * L;
  int sweep = 0;
  for (; sweep < 60; ++sweep) {
    if (threadIdx.x == 0) *rot = 0;
    __syncthreads();
    for (int rr = 0; rr < NP - 1; ++rr) {
      // round-robin pairing: position 0 fixed, the others rotate
      for (int pk = warp; pk < NP / 2; pk += NW) {
        const int pos1 = pk, pos2 = NP - 1 - pk;
        const int vp = pos1 == 0 ? 0 : ((pos1 - 1 + rr) % (NP - 1)) + 1;
        const int vq = ((pos2 - 1 + rr) % (NP - 1)) + 1;
        if (vp >= nv || vq >= nv) continue;
        double2* xp = W + vp * vs;
        double2* xq = W + vq * vs;
        double al = 0.0, be = 0.0, gr = 0.0, gi = 0.0;
        for (int i = lane; i < L; i += 32) {
          const double2 u = xp[i * es], w = xq[i * es];
          al = fma(u.x, u.x, fma(u.y, u.y, al));
          be = fma(w.x, w.x, fma(w.y, w.y, be));
          gr = fma(u.x, w.x, fma(u.y, w.y, gr));   // re(conj(u) w)
          gi = fma(u.x, w.y, fma(-u.y, w.x, gi));  // im(conj(u) w)
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
          const double2 ph = make_double2(gr / ga, -gi / ga);  // exp(-i phi), gamma = |gamma| exp(i phi)
          for (int i = lane; i < L; i += 32) {
            const double2 u = xp[i * es];
            const double2 w = cmul(ph, xq[i * es]);
            xp[i * es] = make_double2(c * u.x - s * w.x, c * u.y - s * w.y);
            xq[i * es] = make_double2(s * u.x + c * w.x, s * u.y + c * w.y);
          }
        }
      }
      __syncthreads();
    }
    if (!*rot) break;
    __syncthreads();
  }
  // T_k = |v_k|^2, ranked in descending order (ties by index).
  for (int k = warp; k < nv; k += NW) {
    const double2* xk = W + k * vs;
    double s = 0.0;
    for (int i = lane; i < L; i += 32) {
      const double2 u = xk[i * es];
      s = fma(u.x, u.x, fma(u.y, u.y, s));
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) cc[k] = s;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nv; k += NT) {
    const double tk = cc[k];
    int rank = 0;
    for (int j = 0; j < nv; ++j) {
      const double tj = cc[j];
      rank += (tj > tk || (tj == tk && j < k)) ? 1 : 0;
    }
    if (rank < neigv) out[rank] = tk;
  }
  return sweep < 60;
}

}  // namespace rg
