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

// ---- sums over the lanes of a warp row by transposition -----------------
// d[0..R) on each of the L lanes of a row (L a power of two <= 32, rows the
// aligned L-lane blocks of the warp): after the call the lanes hold the row
// totals of d[IDX..IDX+CNT), CNT = max(1, R / L), with IDX returned through
// idx.  Each level sends half of the remaining values to the partner lane
// and keeps the other half (R/2 + R/4 + ... shuffles instead of R log2 L);
// once one value is left the levels are plain butterflies, whose duplicate
// lanes clear `writer`, so exactly one lane of a row holds each total with
// writer set.  All 32 lanes of the warp must call it.
template <int R, int L>
__device__ __forceinline__ void lane_transpose_sum(float (&d)[R], int lane, int& idx, bool& writer) {
  idx = 0;
  writer = true;
  int cnt = R;
#pragma unroll
  for (int m = L / 2; m >= 1; m >>= 1) {
    const bool hi = (lane & m) != 0;
    if (cnt > 1) {
      const int h = cnt / 2;
#pragma unroll
      for (int q = 0; q < R / 2; ++q) {
        if (q < h) {
          const float send = hi ? d[q] : d[q + h];
          const float keep = hi ? d[q + h] : d[q];
          d[q] = keep + __shfl_xor_sync(0xffffffffu, send, m);
        }
      }
      if (hi) idx += h;
      cnt = h;
    } else {
      d[0] += __shfl_xor_sync(0xffffffffu, d[0], m);
      if (hi) writer = false;
    }
  }
}

// The same for R double-float values over the whole warp (L = 32): the
// writer lane with index idx holds the warp total of d[idx] in d[0] (R a
// power of two <= 32).
template <int R>
__device__ __forceinline__ void warp_transpose_sum_df(df32 (&d)[R], int lane, int& idx, bool& writer) {
  idx = 0;
  writer = true;
  int cnt = R;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    const bool hi = (lane & m) != 0;
    if (cnt > 1) {
      const int h = cnt / 2;
#pragma unroll
      for (int q = 0; q < R / 2; ++q) {
        if (q < h) {
          const df32 send = hi ? d[q] : d[q + h];
          const df32 keep = hi ? d[q + h] : d[q];
          d[q] = df_add(keep, df_shfl_xor(send, m));
        }
      }
      if (hi) idx += h;
      cnt = h;
    } else {
      d[0] = df_add(d[0], df_shfl_xor(d[0], m));
      if (hi) writer = false;
    }
  }
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
// divisor of 32); red holds (G/32 rounded up) * NQ entries per group (none
// for G < 32).  Within a warp the partial sums are added in FP32 (a thread's
// partial covers a few terms, the tree at most five levels: ~5e-7 relative),
// across warps in double-float.
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
    // groups smaller than a warp: FP32 shuffles within the aligned sub-warp
    // (at most four levels over per-thread partials, as within a warp above)
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      float x = v[q].hi + v[q].lo;
#pragma unroll
      for (int m = 16; m > 0; m >>= 1)
        if (m < G) x += __shfl_xor_sync(0xffffffffu, x, m);
      v[q] = {x, 0.f};
    }
    sync();
    sync();
  }
}

// ---- tridiagonal solve: partition (interior Thomas) + reduced system -----
// Solves rows j = 0..N-1: l(j) x[j-1] + b x[j] + u(j) x[j+1] = x_in[j]
// (l(0) and u(N-1) ignored).  x is one component of a padded complex-float
// sequence in shared memory (element j at float offset 2*sp<float, PS>(j),
// PS = row_pad_shift(M), the layout of the row kernels); thread
// t of the G threads of a group owns the contiguous chunk [t*M, t*M+M),
// M >= 2.  Each chunk is reduced by an interior Thomas sweep to two equations
// in its end values x_s, x_e (the 2G-row boundary system).  One cyclic-
// reduction step folds the x_s rows into the x_e rows, PCR solves the G
// remaining rows (one per thread), and the x_s follow by back-substitution.
// The neighbour rows move by shuffles when the group is one warp or less,
// otherwise through red (2 x G float4, 16-byte aligned, double-buffered: one
// group sync per exchange).  All threads of the group must call it.
// The system is diagonally dominant with pivots of order one, so its divides
// use the fast intrinsic (__fdividef, within 2 ulp there).
template <int M, int G, typename LFn, typename UFn, typename Sync = CtaSync>
__device__ __forceinline__ void partition_solve(float* x, int t, float b, LFn lf, UFn uf, float* red,
                                                const Sync& sync = Sync()) {
  const int s = t * M, e = s + M - 1;
  // the x_e influence vector needs no array: its source is the last interior
  // row only, so the forward sweep leaves it zero above that row and
  // back-substitution makes it be[i] = -cp[i] be[i+1] from be_last.  The
  // data solution y lives in place of the right-hand side in x (registers
  // hold the x_s influence al and the pivots cp).
  float al[M > 2 ? M - 2 : 1], cp[M > 2 ? M - 2 : 1];
  float be_last = 0.f, be0 = 0.f, y_last = 0.f, y0 = 0.f;
  float r_s = x[2 * sp<float, row_pad_shift(M)>(s)], r_e = x[2 * sp<float, row_pad_shift(M)>(e)];
  float RA0, RB0, RC0, RD0, RA1, RB1, RC1, RD1;
  const float l_s = (s == 0) ? 0.f : lf(s);
  const float u_s = uf(s);
  const float l_e = lf(e);
  const float u_e = (e == G * M - 1) ? 0.f : uf(e);
  if (M > 2) {
    // interior Thomas with three right-hand sides: data, x_s influence, x_e influence
#pragma unroll
    for (int i = 0; i < M - 2; ++i) {
      const int j = s + 1 + i;
      const float lj = lf(j), uj = uf(j);
      const float den = (i == 0) ? b : b - lj * cp[i - 1];
      const float inv = __fdividef(1.f, den);
      cp[i] = uj * inv;
      const float rj = x[2 * sp<float, row_pad_shift(M)>(j)];
      y_last = (i == 0) ? rj * inv : (rj - lj * y_last) * inv;
      x[2 * sp<float, row_pad_shift(M)>(j)] = y_last;
      al[i] = (i == 0) ? -lj * inv : (-lj * al[i - 1]) * inv;
      if (i == M - 3) be_last = -uj * inv;
    }
    be0 = be_last;
    y0 = y_last;
#pragma unroll
    for (int i = M - 4; i >= 0; --i) {
      float* xj = x + 2 * sp<float, row_pad_shift(M)>(s + 1 + i);
      y0 = *xj - cp[i] * y0;
      *xj = y0;
      al[i] -= cp[i] * al[i + 1];
      be0 = -cp[i] * be0;
    }
    RA0 = l_s;
    RB0 = b + u_s * al[0];
    RC0 = u_s * be0;
    RD0 = r_s - u_s * y0;
    RA1 = l_e * al[M - 3];
    RB1 = b + l_e * be_last;
    RC1 = u_e;
    RD1 = r_e - l_e * y_last;
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
  // the boundary rows: row 2t (x_s: RA0 x_e(t-1) + RB0 x_s + RC0 x_e = RD0) and
  // row 2t+1 (x_e: RA1 x_s + RB1 x_e + RC1 x_s(t+1) = RD1)
  constexpr bool SHFL = G <= 32;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned mask = G >= 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(unsigned)(G - 1)));
  float4* buf = reinterpret_cast<float4*>(red);
  int ph = 0;
  // publish this thread's row, then fetch the row of thread t + d (meaningful
  // for 0 <= t + d < G); d is the same on every thread of the group
  auto publish = [&](const float4& v) {
    if constexpr (!SHFL) {
      buf[ph * G + t] = v;
      sync();
    }
  };
  auto fetch = [&](const float4& own, int d) -> float4 {
    if constexpr (SHFL) {
      float4 r;
      if (d > 0) {
        r.x = __shfl_down_sync(mask, own.x, d, G);
        r.y = __shfl_down_sync(mask, own.y, d, G);
        r.z = __shfl_down_sync(mask, own.z, d, G);
        r.w = __shfl_down_sync(mask, own.w, d, G);
      } else {
        r.x = __shfl_up_sync(mask, own.x, -d, G);
        r.y = __shfl_up_sync(mask, own.y, -d, G);
        r.z = __shfl_up_sync(mask, own.z, -d, G);
        r.w = __shfl_up_sync(mask, own.w, -d, G);
      }
      return r;
    } else {
      const int src = t + d;
      return (src >= 0 && src < G) ? buf[ph * G + src] : own;
    }
  };
  auto done = [&]() {
    if constexpr (!SHFL) ph ^= 1;
  };
  // cyclic reduction: row 2t+1 without x_s(t) (own row 2t) and x_s(t+1)
  // (row 2t+2, thread t+1's first row)
  float A, B, C, D;
  {
    const float4 r0 = make_float4(RA0, RB0, RC0, RD0);
    publish(r0);
    const float4 n0 = fetch(r0, 1);
    done();
    const bool up = t + 1 < G;
    const float k1 = __fdividef(RA1, RB0);
    const float k2 = up ? __fdividef(RC1, n0.y) : 0.f;
    A = -RA0 * k1;
    B = RB1 - RC0 * k1 - (up ? n0.x * k2 : 0.f);
    C = up ? -n0.z * k2 : 0.f;
    D = RD1 - RD0 * k1 - (up ? n0.w * k2 : 0.f);
  }
  // PCR on the G rows in x_e(t)
#pragma unroll
  for (int st = 1; st < G; st <<= 1) {
    const float4 me = make_float4(A, B, C, D);
    publish(me);
    const float4 lo = fetch(me, -st), hi = fetch(me, st);
    done();
    float nA = 0.f, nC = 0.f, nB = B, nD = D;
    if (t >= st) {
      const float k1 = __fdividef(A, lo.y);
      nA = -lo.x * k1;
      nB -= lo.z * k1;
      nD -= lo.w * k1;
    }
    if (t + st < G) {
      const float k2 = __fdividef(C, hi.y);
      nC = -hi.z * k2;
      nB -= hi.x * k2;
      nD -= hi.w * k2;
    }
    A = nA;
    B = nB;
    C = nC;
    D = nD;
  }
  const float xe = __fdividef(D, B);
  // back-substitution: x_s(t) from row 2t with x_e(t-1) and x_e(t)
  float xe_lo;
  {
    const float4 v = make_float4(xe, 0.f, 0.f, 0.f);
    publish(v);
    xe_lo = fetch(v, -1).x;
  }
  const float xs = __fdividef(RD0 - (t > 0 ? RA0 * xe_lo : 0.f) - RC0 * xe, RB0);
  x[2 * sp<float, row_pad_shift(M)>(s)] = xs;
  x[2 * sp<float, row_pad_shift(M)>(e)] = xe;
  if (M > 2) {
    float bi = be_last;
#pragma unroll
    for (int i = M - 3; i >= 0; --i) {
      if (i < M - 3) bi = -cp[i] * bi;
      float* xj = x + 2 * sp<float, row_pad_shift(M)>(s + 1 + i);
      *xj = *xj + al[i] * xs + bi * xe;
    }
  }
  sync();
}

}  // namespace vg
