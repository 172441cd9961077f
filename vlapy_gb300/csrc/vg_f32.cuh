// FP32 delta-f device building blocks shared by the single-run and the
// batched-sweep kernels.
//
// The state is g = f - f0(v) in FP32 with a fixed x-independent background
// f0 (the x-average of the initial f).  Keeping the small deviation instead
// of f keeps FP32 rounding relative to the perturbation, not to f0:
//   * v-kick:   FFT_v(g') = P . FFT_v(g) + (P - 1) . FFT_v(f0), P = exp(i th),
//               with P - 1 = (-2 sin^2(th/2), sin th) free of cancellation;
//   * x-drift:  f0 has no x dependence, so only g moves;
//   * density:  1 - n = -trapz(g) - (trapz(f0) - 1), the second term in FP64;
//   * collisions: A g' = g - (A - I) f0, where (A - I) f0 is evaluated from
//               FP64-precomputed stencils of f0 and the row moments.
// Phases m * a (a per column / per row, formed in FP64) are evaluated as an
// exact FP32 product plus its FMA residual, so a phase of hundreds of radians
// is still accurate to ~1e-7 absolute.
#pragma once

#include "vg_fft.cuh"

namespace vg {

// ---- double-float (TwoSum) accumulation --------------------------------
struct df32 {
  float hi, lo;
};
__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (b.hi - bb);
  const float lo = (a.lo + b.lo) + err;
  const float hi = s + lo;
  return {hi, lo - (hi - s)};
}
__device__ __forceinline__ df32 df_shfl_xor(df32 a, int m) {
  return {__shfl_xor_sync(0xffffffffu, a.hi, m), __shfl_xor_sync(0xffffffffu, a.lo, m)};
}
__device__ __forceinline__ df32 df_warp_sum(df32 a) {
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) a = df_add(a, df_shfl_xor(a, m));
  return a;
}
__device__ __forceinline__ double df_to_double(df32 a) { return (double)a.hi + (double)a.lo; }
// double-float product (TwoProd by FMA); accurate to ~1e-14 relative
__device__ __forceinline__ df32 df_mul(df32 a, df32 b) {
  const float p = a.hi * b.hi;
  const float e = fmaf(a.hi, b.hi, -p) + fmaf(a.hi, b.lo, a.lo * b.hi);
  const float hi = p + e;
  return {hi, e - (hi - p)};
}
__device__ __forceinline__ float df_round(df32 a) { return a.hi + a.lo; }

// ---- accurate phases ---------------------------------------------------
struct Ang {
  float hi, lo;  // a = hi + lo (FP64 angle per unit index, split)
};
__device__ __forceinline__ Ang split_angle(double a) {
  const float h = (float)a;
  return {h, (float)(a - (double)h)};
}
// double-float product a * b of two (hi, lo) splits, as an angle per unit index
__device__ __forceinline__ Ang mul_angle(float2 a, float2 b) {
  const float p = a.x * b.x;
  const float e = fmaf(a.x, b.x, -p) + fmaf(a.x, b.y, a.y * b.x);
  const float h = p + e;
  return {h, e - (h - p)};
}
// sin/cos of m * a to ~1e-7 absolute for |m a| up to ~1e4
__device__ __forceinline__ void sincos_m(float m, Ang a, float& s, float& c) {
  const float p = m * a.hi;
  const float e = fmaf(m, a.hi, -p) + m * a.lo;
  float s0, c0;
  sincosf(p, &s0, &c0);
  s = fmaf(c0, e, s0);
  c = fmaf(-s0, e, c0);
}

// ---- CTA-wide reductions of NQ double-float values ----------------------
// red: shared scratch of (blockDim.x / 32) * NQ df32.  Every thread gets the
// totals.  Must be called by all threads of the CTA.
template <int NQ>
__device__ __forceinline__ void block_df_sum(df32 (&v)[NQ], df32* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) v[q] = df_warp_sum(v[q]);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) red[wid * NQ + q] = v[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    df32 t = {0.f, 0.f};
    for (int w = 0; w < nw; ++w) t = df_add(t, red[w * NQ + q]);
    v[q] = t;
  }
  __syncthreads();
}

// Same, restricted to the G threads of one group (G a multiple of 32 or a
// divisor of 32); red holds (G/32 rounded up) * NQ entries per group.  Within
// a warp the partial sums are added in FP32 (a thread's partial covers a few
// terms, the tree five levels: ~5e-7 relative), across warps in double-float.
// LEADER: only thread 0 of the group needs the totals (the other threads'
// v are left partial), so only it adds up the warps' sums.
template <int NQ, bool LEADER = false, typename Sync = CtaSync>
__device__ __forceinline__ void group_df_sum(df32 (&v)[NQ], df32* red, int G, int t, const Sync& sync = Sync()) {
  if (G >= 32) {
    const int lane = t & 31, wid = t >> 5, nw = G >> 5;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      float x = v[q].hi + v[q].lo;
#pragma unroll
      for (int m = 16; m > 0; m >>= 1) x += __shfl_xor_sync(0xffffffffu, x, m);
      v[q] = {x, 0.f};
    }
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) red[wid * NQ + q] = v[q];
    }
    sync();
    if (!LEADER || t == 0) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        df32 tt = {0.f, 0.f};
        for (int w = 0; w < nw; ++w) tt = df_add(tt, red[w * NQ + q]);
        v[q] = tt;
      }
    }
    sync();
  } else {
    // groups smaller than a warp: shuffle within the aligned sub-warp
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      for (int m = G >> 1; m > 0; m >>= 1) v[q] = df_add(v[q], df_shfl_xor(v[q], m));
    sync();
    sync();
  }
}

// ---- tridiagonal solve: partition (interior Thomas) + PCR ---------------
// Solves rows j = 0..N-1: l(j) x[j-1] + b x[j] + u(j) x[j+1] = x_in[j]
// (l(0) and u(N-1) ignored).  x is one component of a padded complex-float
// sequence in shared memory (element j at float offset 2*sp<float>(j)); thread
// t of G owns the contiguous chunk [t*m, t*m+m), m = N/G >= 2.
// red: shared scratch of 4 * 2G floats.  All threads of the CTA must call it.
// The system is diagonally dominant with pivots of order one, so its divides
// use the fast intrinsic (__fdividef, within 2 ulp there).
template <int M, typename LFn, typename UFn, typename Sync = CtaSync>
__device__ __forceinline__ void partition_solve(float* x, int t, int G, float b, LFn lf, UFn uf,
                                                float* red, const Sync& sync = Sync()) {
  const int s = t * M, e = s + M - 1;
  float y[M > 2 ? M - 2 : 1], al[M > 2 ? M - 2 : 1], be[M > 2 ? M - 2 : 1];
  float r_s = x[2 * sp<float>(s)], r_e = x[2 * sp<float>(e)];
  float RA0, RB0, RC0, RD0, RA1, RB1, RC1, RD1;
  const float l_s = (s == 0) ? 0.f : lf(s);
  const float u_s = uf(s);
  const float l_e = lf(e);
  const float u_e = (e == G * M - 1) ? 0.f : uf(e);
  if (M > 2) {
    // interior Thomas with three right-hand sides: data, x_s influence, x_e influence
    float cp[M > 2 ? M - 2 : 1];
#pragma unroll
    for (int i = 0; i < M - 2; ++i) {
      const int j = s + 1 + i;
      const float lj = lf(j), uj = uf(j);
      const float den = (i == 0) ? b : b - lj * cp[i - 1];
      const float inv = __fdividef(1.f, den);
      cp[i] = uj * inv;
      const float rj = x[2 * sp<float>(j)];
      y[i] = (i == 0) ? rj * inv : (rj - lj * y[i - 1]) * inv;
      al[i] = (i == 0) ? -lj * inv : (-lj * al[i - 1]) * inv;
      const float bsrc = (i == M - 3) ? -uj : 0.f;
      be[i] = (i == 0) ? bsrc * inv : (bsrc - lj * be[i - 1]) * inv;
    }
#pragma unroll
    for (int i = M - 4; i >= 0; --i) {
      y[i] -= cp[i] * y[i + 1];
      al[i] -= cp[i] * al[i + 1];
      be[i] -= cp[i] * be[i + 1];
    }
    RA0 = l_s;
    RB0 = b + u_s * al[0];
    RC0 = u_s * be[0];
    RD0 = r_s - u_s * y[0];
    RA1 = l_e * al[M - 3];
    RB1 = b + l_e * be[M - 3];
    RC1 = u_e;
    RD1 = r_e - l_e * y[M - 3];
  } else {
    RA0 = l_s;
    RB0 = b;
    RC0 = u_s;
    RD0 = r_s;
    RA1 = l_e;
    RB1 = b;
    RC1 = u_e;
    RD1 = r_e;
  }
  // PCR on the 2G boundary unknowns (x_s, x_e of every chunk)
  const int NR = 2 * G;
  float* A = red;
  float* B = red + NR;
  float* C = red + 2 * NR;
  float* D = red + 3 * NR;
  A[2 * t] = RA0;
  B[2 * t] = RB0;
  C[2 * t] = RC0;
  D[2 * t] = RD0;
  A[2 * t + 1] = RA1;
  B[2 * t + 1] = RB1;
  C[2 * t + 1] = RC1;
  D[2 * t + 1] = RD1;
  sync();
  for (int st = 1; st < NR; st <<= 1) {
    float na[2], nb[2], nc[2], nd[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int i = 2 * t + q;
      const int lo = i - st, hi = i + st;
      float ai = A[i], bi = B[i], ci = C[i], di = D[i];
      float k1 = 0.f, k2 = 0.f;
      na[q] = 0.f;
      nc[q] = 0.f;
      if (lo >= 0) {
        k1 = __fdividef(ai, B[lo]);
        na[q] = -A[lo] * k1;
        bi -= C[lo] * k1;
        di -= D[lo] * k1;
      }
      if (hi < NR) {
        k2 = __fdividef(ci, B[hi]);
        nc[q] = -C[hi] * k2;
        bi -= A[hi] * k2;
        di -= D[hi] * k2;
      }
      nb[q] = bi;
      nd[q] = di;
    }
    sync();
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int i = 2 * t + q;
      A[i] = na[q];
      B[i] = nb[q];
      C[i] = nc[q];
      D[i] = nd[q];
    }
    sync();
  }
  const float xs = __fdividef(D[2 * t], B[2 * t]);
  const float xe = __fdividef(D[2 * t + 1], B[2 * t + 1]);
  x[2 * sp<float>(s)] = xs;
  x[2 * sp<float>(e)] = xe;
  if (M > 2) {
#pragma unroll
    for (int i = 0; i < M - 2; ++i) x[2 * sp<float>(s + 1 + i)] = y[i] + al[i] * xs + be[i] * xe;
  }
  sync();
}

}  // namespace vg
