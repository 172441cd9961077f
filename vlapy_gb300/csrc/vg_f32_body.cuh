// Device bodies of the FP32 delta-f step shared by the single-run kernels
// (vg_step_f32.cu) and the batched sweep (vg_sweep.cu): one column tile of
// the x-drift, and one row-pair group of the row pass (kick, collide,
// measure, kick).
#pragma once

#include "vg_f32.cuh"
#include "vg_f32_plan.cuh"
#include "vg_internal.cuh"

namespace vg {

constexpr int COL32_PAD = 1;

// One column tile [NX x W] at column c0: x-drift by exp(i m (-dkx dt) v_col)
// and the tile's trapz-weighted density partials added into dacc[x].
// smem: W/2 padded sequences of NX complex floats.
template <int NX, int R>
__device__ __forceinline__ void col_tile(float* __restrict__ g, int nv, int c0, int W, float2 kdt,
                                         const float2* __restrict__ vhl, const cx<float>* __restrict__ tw,
                                         unsigned char* smem, df32* dacc) {
  constexpr int G = NX / R;
  constexpr int LD = sp_len<float>(NX) + COL32_PAD;
  cx<float>* s = reinterpret_cast<cx<float>*>(smem);
  float* sf = reinterpret_cast<float*>(smem);
  const int grp = threadIdx.x / G, t = threadIdx.x - grp * G;
  cx<float>* sg = s + (size_t)grp * LD;
  const float scale = 1.f / NX;
  // the tile in 16-byte vectors when W and nv are multiples of 4 floats
  // (then so are c0 and every row start), else float by float
  const bool vec = ((W | nv) & 3) == 0;
  const int total = NX * W, total4 = vec ? total / 4 : 0;
  for (int q = threadIdx.x; q < total4; q += blockDim.x) {
    const int x = q / (W / 4), c = 4 * (q - x * (W / 4));
    const float4 v = *reinterpret_cast<const float4*>(g + (size_t)x * nv + c0 + c);
    sf[2 * ((c >> 1) * LD + sp<float>(x))] = v.x;
    sf[2 * ((c >> 1) * LD + sp<float>(x)) + 1] = v.y;
    sf[2 * (((c >> 1) + 1) * LD + sp<float>(x))] = v.z;
    sf[2 * (((c >> 1) + 1) * LD + sp<float>(x)) + 1] = v.w;
  }
  if (!vec)
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
      const int x = q / W, c = q - x * W;
      sf[2 * ((c >> 1) * LD + sp<float>(x)) + (c & 1)] = g[(size_t)x * nv + c0 + c];
    }
  __syncthreads();
  block_fft<float, NX, false, R>(sg, t, tw);
  // theta(m) = m * (-dkx dt) v_col (kx = m dkx on the bins m <= NX/2); the angle
  // per unit m is the double-float product of kdt = -dkx dt and v (both split)
  const Ang aa = mul_angle(kdt, vhl[c0 + 2 * grp]);
  const Ang ab = mul_angle(kdt, vhl[c0 + 2 * grp + 1]);
  {
    // phases exp(i m a) for this thread's bins m = t, t+G, ...: one sincos for
    // the start, one for the step, complex products in between
    float sa, ca, sb, cb, sga, cga, sgb, cgb;
    sincos_m((float)t, aa, sa, ca);
    sincos_m((float)t, ab, sb, cb);
    sincos_m((float)G, aa, sga, cga);
    sincos_m((float)G, ab, sgb, cgb);
    two_real_rotate<float>(sg, NX, t, G, [&](int, float& pca, float& psa, float& pcb, float& psb) {
      pca = ca * scale;
      psa = sa * scale;
      pcb = cb * scale;
      psb = sb * scale;
      const float na = sa * cga + ca * sga, nca = ca * cga - sa * sga;
      const float nb = sb * cgb + cb * sgb, ncb = cb * cgb - sb * sgb;
      sa = na;
      ca = nca;
      sb = nb;
      cb = ncb;
    });
  }
  __syncthreads();
  block_fft<float, NX, true, R>(sg, t, tw);
  // density partial sums (trapz weights: 1/2 at the two v end points): the
  // tpx threads of an x point (consecutive lanes) share its W columns and
  // add their sums by shuffles
  const int tpx = (int)blockDim.x >= NX ? (int)blockDim.x / NX : 1;
  if (tpx > 1 && tpx <= 32) {
    const int x = threadIdx.x / tpx, part = threadIdx.x - x * tpx;
    float acc = 0.f;
    for (int c = part; c < W; c += tpx) {
      const int col = c0 + c;
      const float w = (col == 0 || col == nv - 1) ? 0.5f : 1.f;
      acc = fmaf(w, sf[2 * ((c >> 1) * LD + sp<float>(x)) + (c & 1)], acc);
    }
    for (int m = tpx >> 1; m > 0; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
    if (part == 0) dacc[x] = df_add(dacc[x], {acc, 0.f});
  } else {
    for (int x = threadIdx.x; x < NX; x += blockDim.x) {
      float acc = 0.f;
      for (int c = 0; c < W; ++c) {
        const int col = c0 + c;
        const float w = (col == 0 || col == nv - 1) ? 0.5f : 1.f;
        acc = fmaf(w, sf[2 * ((c >> 1) * LD + sp<float>(x)) + (c & 1)], acc);
      }
      dacc[x] = df_add(dacc[x], {acc, 0.f});
    }
  }
  for (int q = threadIdx.x; q < total4; q += blockDim.x) {
    const int x = q / (W / 4), c = 4 * (q - x * (W / 4));
    float4 v;
    v.x = sf[2 * ((c >> 1) * LD + sp<float>(x))];
    v.y = sf[2 * ((c >> 1) * LD + sp<float>(x)) + 1];
    v.z = sf[2 * (((c >> 1) + 1) * LD + sp<float>(x))];
    v.w = sf[2 * (((c >> 1) + 1) * LD + sp<float>(x)) + 1];
    *reinterpret_cast<float4*>(g + (size_t)x * nv + c0 + c) = v;
  }
  if (!vec)
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
      const int x = q / W, c = q - x * W;
      g[(size_t)x * nv + c0 + c] = sf[2 * ((c >> 1) * LD + sp<float>(x)) + (c & 1)];
    }
  __syncthreads();
}


// Moment slot q of one row (0..5: n, j, T, q, fv4, vN; 6: trapz(f^2);
// 7: trapz(f log f)) from the raw double-float sums the row pass leaves in
// its [8]-double slots: dv * sum + the background's share, in FP64.
__device__ __forceinline__ double row_moment(const double* __restrict__ slots, int q, const RowConsts& rc) {
  const df32 m = reinterpret_cast<const df32*>(slots)[q];
  const double sum = (double)m.hi + (double)m.lo;
  return q < 7 ? rc.dv * sum + rc.f0m[q] : rc.dv * sum;
}

// rotation of one packed row pair with the delta-f background term; the 1/N of
// the inverse transform is folded in.  ha/hb: half-angle per kv index.
template <int N, int PS = pad_shift<float>()>
__device__ __forceinline__ void kick_rotate(cx<float>* s, int t, int G, Ang ha, Ang hb,
                                            const cx<float>* __restrict__ F0) {
  const float sc = 1.f / N;
  // half-angle rotations h(k) = exp(i k a / 2) for this thread's bins k = t, t+G, ...
  // by one sincos for the start and one for the step, then complex products
  float sa, ca, sb, cb, sga, cga, sgb, cgb;
  sincos_m((float)t, ha, sa, ca);
  sincos_m((float)t, hb, sb, cb);
  sincos_m((float)G, ha, sga, cga);
  sincos_m((float)G, hb, sgb, cgb);
  for (int k = t; k <= N / 2; k += G) {
    // P = (1 - 2 sin^2, 2 sin cos) of the half angle; P - 1 = (-2 sin^2, 2 sin cos)
    const float pa_m1r = -2.f * sa * sa, pa_i = 2.f * sa * ca, pa_r = 1.f + pa_m1r;
    const float pb_m1r = -2.f * sb * sb, pb_i = 2.f * sb * cb, pb_r = 1.f + pb_m1r;
    const cx<float> f0 = F0[k];
    if (k == 0 || 2 * k == N) {
      const cx<float> z = s[sp<float, PS>(k)];
      // real bins: only Re(P) survives
      s[sp<float, PS>(k)] = {(pa_r * z.x + pa_m1r * f0.x) * sc, (pb_r * z.y + pb_m1r * f0.x) * sc};
    } else {
      const cx<float> zk = s[sp<float, PS>(k)], zm = s[sp<float, PS>(N - k)];
      const cx<float> fa = {(zk.x + zm.x) * 0.5f, (zk.y - zm.y) * 0.5f};
      const cx<float> fb = {(zk.y + zm.y) * 0.5f, (zm.x - zk.x) * 0.5f};
      const cx<float> ga = {(pa_r * fa.x - pa_i * fa.y + pa_m1r * f0.x - pa_i * f0.y) * sc,
                            (pa_r * fa.y + pa_i * fa.x + pa_m1r * f0.y + pa_i * f0.x) * sc};
      const cx<float> gb = {(pb_r * fb.x - pb_i * fb.y + pb_m1r * f0.x - pb_i * f0.y) * sc,
                            (pb_r * fb.y + pb_i * fb.x + pb_m1r * f0.y + pb_i * f0.x) * sc};
      s[sp<float, PS>(k)] = {ga.x - gb.y, ga.y + gb.x};
      s[sp<float, PS>(N - k)] = {ga.x + gb.y, gb.x - ga.y};
    }
    const float na = sa * cga + ca * sga, nca = ca * cga - sa * sga;
    const float nb = sb * cgb + cb * sgb, ncb = cb * cgb - sb * sgb;
    sa = na;
    ca = nca;
    sb = nb;
    cb = ncb;
  }
}

// the kick with the row pair in registers at either end (IO bit 0: io holds
// the pair's elements t + i G on entry and s need not; bit 1: they end in io;
// the row pass uses IO = 3, both)
template <int N, int R, int IO, typename Sync>
__device__ __forceinline__ void kick_io(cx<float>* s, int t, float hk, float ea, float eb,
                                        const cx<float>* __restrict__ F0, const cx<float>* __restrict__ tw,
                                        const Sync& sync, cx<float> (&io)[R]) {
  constexpr int G = N / R;
  constexpr int PS = row_pad_shift(R);
  block_fft_io<float, N, false, R, IO & 1, Sync, PS>(s, t, tw, sync, io);
  // theta(k) = -kv_k dt e = k * (-dkv dt e); hk = -dkv dt / 2 gives the half
  // angle for P - 1.  The kick angle stays O(10) rad, so an FP32 product is
  // accurate to ~1e-6 rad here
  const Ang ha = {hk * ea, 0.f};
  const Ang hb = {hk * eb, 0.f};
  kick_rotate<N, PS>(s, t, G, ha, hb, F0);
  sync();
  block_fft_io<float, N, true, R, IO & 2, Sync, PS>(s, t, tw, sync, io);
}

// Per-row collision scalars from the row's raw moment sums (sum w g v^p,
// p = 0, 1, 2), in double-float; each FP32 coefficient is rounded once:
// out = {-vth/dv^2, 1 + 2 nudt vth/dv^2, vbar, nudt vth, nudt vbar}.
__device__ __forceinline__ void collision_scalars(const RowConsts& rc, float2 nudt2, int dougherty, df32 s0,
                                                  df32 s1, df32 s2, float* out) {
  const df32 dv = {rc.dv2f.x, rc.dv2f.y};
  const df32 M0 = df_add(df_mul(dv, s0), {rc.f0m2f[0].x, rc.f0m2f[0].y});
  const df32 M1 = df_add(df_mul(dv, s1), {rc.f0m2f[1].x, rc.f0m2f[1].y});
  const df32 M2 = df_add(df_mul(dv, s2), {rc.f0m2f[2].x, rc.f0m2f[2].y});
  // DG: vbar = trapz(f v), v0t^2 = trapz(f (v - vbar)^2) = M2 + vbar^2 (M0 - 2)
  // LB: v0t^2 = trapz(f v^2), no drift
  const df32 vbar = dougherty ? M1 : df32{0.f, 0.f};
  const df32 vth = dougherty ? df_add(M2, df_mul(df_mul(vbar, vbar), df_add(M0, {-2.f, 0.f}))) : M2;
  const df32 nd = {nudt2.x, nudt2.y};
  const df32 a = df_mul(vth, {rc.idv2f.x, rc.idv2f.y});  // vth / dv^2
  const df32 na = df_mul(nd, a);
  out[0] = -df_round(a);
  out[1] = df_round(df_add({1.f, 0.f}, {2.f * na.hi, 2.f * na.lo}));
  out[2] = df_round(vbar);
  out[3] = df_round(df_mul(nd, vth));
  out[4] = df_round(df_mul(nd, vbar));
}

// Fokker-Planck step, in delta-f form, of both rows of a packed pair (row a
// in the real parts of s, row b in the imaginary parts).  The moments and the
// right-hand sides of the two rows share one pass over the pair (one 8-byte
// access per element, one load of each constant) and one reduction; the two
// tridiagonal solves run one after the other.
template <int N, int R, typename Sync = CtaSync>
__device__ __forceinline__ void collide_pair(cx<float>* s, int t, const RowConsts& rc, float2 nudt2, float nudt_f,
                                             int dougherty, df32* red, float* pcr, const Sync& sync = Sync()) {
  constexpr int G = N / R;
  // moments of g: sum w g, sum w g v, sum w g v^2 of each row.  The
  // elementwise parts give consecutive threads consecutive j, so the constant
  // vectors load coalesced; only the tridiagonal solves work on chunks
  df32 mv[6];
  {
    float m[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int j = t + i * G;
      const float w = (j == 0 || j == N - 1) ? 0.5f : 1.f;
      const cx<float> z = s[sp<float, row_pad_shift(R)>(j)];
      const float vj = rc.v[j];
      const float ga = w * z.x, gb = w * z.y;
      m[0] += ga;
      m[1] = fmaf(ga, vj, m[1]);
      m[2] = fmaf(ga * vj, vj, m[2]);
      m[3] += gb;
      m[4] = fmaf(gb, vj, m[4]);
      m[5] = fmaf(gb * vj, vj, m[5]);
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) mv[q] = {m[q], 0.f};
  }
  group_df_sum<6, true>(mv, red, G, t, sync);
  // per-row scalars in double-float by one thread; the group reads them back
  float* sc = reinterpret_cast<float*>(red);
  if (t == 0) {
    collision_scalars(rc, nudt2, dougherty, mv[0], mv[1], mv[2], sc);
    collision_scalars(rc, nudt2, dougherty, mv[3], mv[4], mv[5], sc + 5);
  }
  sync();
  float sa[5], sb[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    sa[q] = sc[q];
    sb[q] = sc[5 + q];
  }
  const float nu = nudt_f;
  const float cm = nu;
  const float i2dv = rc.i2dv;
  sync();
  // right-hand sides: g - (A - I) f0 with (A - I) f0 = nudt (-vth S + Mv - vbar D)
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int j = t + i * G;
    const float S = rc.S[j], Mv = rc.Mv[j], D = rc.D[j];
    cx<float> z = s[sp<float, row_pad_shift(R)>(j)];
    z.x -= -sa[3] * S + cm * Mv - sa[4] * D;
    z.y -= -sb[3] * S + cm * Mv - sb[4] * D;
    s[sp<float, row_pad_shift(R)>(j)] = z;
  }
  sync();
  // off-diagonals at v[j -+ 1] of the uniform grid v[j] = v[0] + j dv,
  // formed in registers (within an FP32 ulp of the tabulated grid)
  const float v0 = rc.v0f, dvf = rc.dvf;
  float* x = reinterpret_cast<float*>(s);
  {
    const float Af = sa[0], vb = sa[2];
    auto lf = [&](int j) { return nu * (Af + (fmaf((float)(j - 1), dvf, v0) - vb) * i2dv); };
    auto uf = [&](int j) { return nu * (Af - (fmaf((float)(j + 1), dvf, v0) - vb) * i2dv); };
    partition_solve<R, G>(x, t, sa[1], lf, uf, pcr, sync);
  }
  {
    const float Af = sb[0], vb = sb[2];
    auto lf = [&](int j) { return nu * (Af + (fmaf((float)(j - 1), dvf, v0) - vb) * i2dv); };
    auto uf = [&](int j) { return nu * (Af - (fmaf((float)(j + 1), dvf, v0) - vb) * i2dv); };
    partition_solve<R, G>(x + 1, t, sb[1], lf, uf, pcr, sync);
  }
}

// One row-pair group of the row pass: load, [kick dt1], [collide], [moments
// and x-mode partials], [kick dt2], store.  grp_base: this group's shared
// memory (row32_group_bytes); macc: the CTA's mode accumulators [n_modes][N].
// NPOW: how many power moments sum w g v^p (p < NPOW) the storage needs (6:
// n, j, T, q, fv4, vN; the batched sweep's series need only p < 3); the
// slots of the others are left unwritten.  KICK_ONLY: the leading half kick
// of a step sequence alone (registers in from global memory, out to it).
template <int N, int R, typename Sync = CtaSync, int NPOW = 6, bool KICK_ONLY = false>
__device__ __forceinline__ void row_pair(const RowArgs& a, int pair, unsigned char* grp_base, cx<float>* macc,
                                         int P, int grp, int t, const Sync& sync = Sync()) {
  constexpr int G = N / R;
  cx<float>* s = reinterpret_cast<cx<float>*>(grp_base);
  constexpr size_t seq_bytes = row32_seq_bytes(N, R);
  static_assert(seq_bytes % 16 == 0 && row32_group_bytes(N, R) % 16 == 0 &&
                    seq_bytes + 8 * G * sizeof(float) + round16((G / 32 + 1) * 9 * sizeof(df32)) ==
                        row32_group_bytes(N, R),
                "row-pair group layout and its host-side size disagree");
  float* pcr = reinterpret_cast<float*>(grp_base + seq_bytes);
  df32* red = reinterpret_cast<df32*>(grp_base + seq_bytes + 8 * G * sizeof(float));
  const int nm = a.n_modes;
  const int ra = 2 * pair, rb = ra + 1;
  const bool va = ra < a.nx, vb = rb < a.nx;
  float* ga = a.g + (size_t)ra * N;
  float* gbp = a.g + (size_t)rb * N;
  const bool kicks = a.hk1 != 0.f || a.hk2 != 0.f;
  const float ea = (kicks && va) ? a.e32[ra] : 0.f, eb = (kicks && vb) ? a.e32[rb] : 0.f;
  if constexpr (KICK_ONLY) {
    cx<float> io[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int n = t + i * G;
      io[i] = {va ? ga[n] : 0.f, vb ? gbp[n] : 0.f};
    }
    if (a.hk1 != 0.f) kick_io<N, R, 3>(s, t, a.hk1, ea, eb, a.F0, a.tw, sync, io);
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int n = t + i * G;
      if (va) ga[n] = io[i].x;
      if (vb) gbp[n] = io[i].y;
    }
    sync();
  } else {
  // both kicks run the same code (registers in, registers out), once each in
  // a loop the compiler keeps rolled, so the kernel holds one copy of the
  // kick's FFTs instead of four differently specialised ones (instruction-
  // cache pressure); the collision and the moments sit between the two
#pragma unroll 1
  for (int kpass = 0; kpass < 2; ++kpass) {
    const float hk = kpass == 0 ? a.hk1 : a.hk2;
    // the pair's elements t + i G, exactly what the first FFT pass reads: from
    // global memory before the first kick, from shared memory before the
    // second (io is defined afresh in every pass, so it is dead in between)
    cx<float> io[R];
    if (kpass == 0) {
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int n = t + i * G;
        io[i] = {va ? ga[n] : 0.f, vb ? gbp[n] : 0.f};
      }
    } else {
#pragma unroll
      for (int i = 0; i < R; ++i) io[i] = s[sp<float, row_pad_shift(R)>(t + i * G)];
    }
    if (hk != 0.f) {
      kick_io<N, R, 3>(s, t, hk, ea, eb, a.F0, a.tw, sync, io);
    }
    if (kpass == 1) {
      // the last FFT pass left elements t + i G in registers: the store
      // pattern, so they go straight back to global memory
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int n = t + i * G;
        if (va) ga[n] = io[i].x;
        if (vb) gbp[n] = io[i].y;
      }
      break;
    }
    // the pair into shared memory for the collision and the moments (after
    // every thread's last kick pass has read it)
    sync();
#pragma unroll
    for (int i = 0; i < R; ++i) s[sp<float, row_pad_shift(R)>(t + i * G)] = io[i];
    sync();
    if (a.fp) {
      collide_pair<N, R>(s, t, *a.rc, a.nudt2, a.nudt_f, a.dougherty, red, pcr, sync);
    }
    if (a.want_mom) {
      // sums of w g v^p (p < NPOW), sum w g^2, sum w g f0, sum w f log f for
      // both rows: [0, NQ) row a, [NQ, 2 NQ) row b
      static_assert(NPOW >= 1 && NPOW <= 6, "power moments");
      constexpr int NQ = NPOW + 3;
      float sa[NQ] = {0}, sb[NQ] = {0};
  #pragma unroll
      for (int i = 0; i < R; ++i) {
        const int j = t + i * G;  // consecutive threads, consecutive j: coalesced loads
        const float w = (j == 0 || j == N - 1) ? 0.5f : 1.f;
        const float vj = a.rc->v[j], f0j = a.rc->f0[j];
        const cx<float> z = s[sp<float, row_pad_shift(R)>(j)];
        float pa = w * z.x, pb = w * z.y;
  #pragma unroll
        for (int p = 0; p < NPOW; ++p) {
          sa[p] += pa;
          sb[p] += pb;
          if (p + 1 < NPOW) {
            pa *= vj;
            pb *= vj;
          }
        }
        sa[NPOW] = fmaf(w * z.x, z.x, sa[NPOW]);
        sb[NPOW] = fmaf(w * z.y, z.y, sb[NPOW]);
        sa[NPOW + 1] = fmaf(w * z.x, f0j, sa[NPOW + 1]);
        sb[NPOW + 1] = fmaf(w * z.y, f0j, sb[NPOW + 1]);
        // f log f by the fast logarithm (3 ulp; NaN for f < 0 as in FP64)
        const float fa = z.x + f0j, fb = z.y + f0j;
        sa[NPOW + 2] = fmaf(w * fa, __logf(fa), sa[NPOW + 2]);
        sb[NPOW + 2] = fmaf(w * fb, __logf(fb), sb[NPOW + 2]);
      }
      df32 m2[2 * NQ];
  #pragma unroll
      for (int q = 0; q < NQ; ++q) {
        m2[q] = {sa[q], 0.f};
        m2[NQ + q] = {sb[q], 0.f};
      }
      // one reduction of both rows where red has the room (9 slots per warp
      // and one more warp's worth; a group inside one warp needs none), else
      // one per row
      constexpr int NW = G >= 32 ? G / 32 : 1;
      if constexpr (G < 32 || 2 * NQ * NW <= 9 * (G / 32 + 1)) {
        group_df_sum<2 * NQ, true>(m2, red, G, t, sync);
      } else {
        df32 ma[NQ], mb[NQ];
  #pragma unroll
        for (int q = 0; q < NQ; ++q) {
          ma[q] = m2[q];
          mb[q] = m2[NQ + q];
        }
        group_df_sum<NQ, true>(ma, red, G, t, sync);
        group_df_sum<NQ, true>(mb, red, G, t, sync);
  #pragma unroll
        for (int q = 0; q < NQ; ++q) {
          m2[q] = ma[q];
          m2[NQ + q] = mb[q];
        }
      }
      if (t == 0) {
        // raw sums; the storage kernels form dv * sum + trapz(f0 ...) in FP64.
        // Each array is indexed by constants only, so it stays in registers.
        auto put = [&](int o, int row) {
          df32* out = reinterpret_cast<df32*>(a.mom + (size_t)row * MOM_STRIDE);
  #pragma unroll
          for (int p = 0; p < NPOW; ++p) out[p] = m2[o + p];
          // sum w (g^2 + 2 g f0)
          out[6] = df_add(m2[o + NPOW], {2.f * m2[o + NPOW + 1].hi, 2.f * m2[o + NPOW + 1].lo});
          out[7] = m2[o + NPOW + 2];
        };
        if (va) put(0, ra);
        if (vb) put(NQ, rb);
      }
      // x-Fourier modes of f (the f0 part of mode 0 is added in the reduction);
      // the groups of a CTA hold different rows but add into the same bins,
      // so they take turns
      // (only with a CTA-wide sync: the turns are CTA barriers)
      if (Sync::cta_wide && nm > 0) {
        for (int gq = 0; gq < P; ++gq) {
          if (gq == grp) {
            for (int mq = 0; mq < nm; ++mq) {
              float swa = 0.f, cwa = 0.f, swb = 0.f, cwb = 0.f;
              if (va) sincospif(-2.f * (float)((mq * ra) % a.nx) / (float)a.nx, &swa, &cwa);
              if (vb) sincospif(-2.f * (float)((mq * rb) % a.nx) / (float)a.nx, &swb, &cwb);
              for (int i = 0; i < R; ++i) {
                const int n = t + i * G;
                const cx<float> z = s[sp<float, row_pad_shift(R)>(n)];
                cx<float>& acc = macc[(size_t)mq * N + n];
                acc.x += z.x * cwa + z.y * cwb;
                acc.y += z.x * swa + z.y * swb;
              }
            }
          }
          __syncthreads();
        }
      }
    }
  }
  sync();
  }
}


}  // namespace vg
