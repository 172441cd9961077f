// FP32 delta-f time step of one run: the throughput path.
//
// Per leapfrog step the state g[nx][nv] (FP32) crosses HBM twice:
//   k_col_f32   x-drift (FFT along x per column pair) + density partials
//   k_dens_f32  per-x reduction of the partials (double-float)
//   k_field_f32 Poisson solve: 1 - n in FP64, FFT in FP32, + driver
//   k_row_f32   half kick(E_{n+1}) -> Fokker-Planck -> storage moments and
//               x-mode partials -> half kick(E_{n+1}) of the next step
//   k_store_f32 fields, series and stored modes of the step
// The first half kick of a batch runs once as a row pass of its own; the
// last step of a batch skips the trailing kick, so the state handed back is
// the reference's f after its collision step.
#include "vg_f32.cuh"
#include "vg_internal.cuh"
#include "vg_f32_plan.cuh"

namespace vg {

// ---------------------------------------------------------------------------
// x-drift of column tiles
// ---------------------------------------------------------------------------

constexpr int COL32_PAD = 1;

// One column tile [NX x W] at column c0: x-drift by exp(i m (-dkx dt) v_col)
// and the tile's trapz-weighted density partials added into dacc[x].
// smem: W/2 padded sequences of NX complex floats.
template <int NX, int R>
__device__ __forceinline__ void col_tile(float* __restrict__ g, int nv, int c0, int W, double phi_unit,
                                         const double* __restrict__ v, const cx<float>* __restrict__ tw,
                                         unsigned char* smem, df32* dacc) {
  constexpr int G = NX / R;
  constexpr int LD = sp_len<float>(NX) + COL32_PAD;
  cx<float>* s = reinterpret_cast<cx<float>*>(smem);
  float* sf = reinterpret_cast<float*>(smem);
  const int grp = threadIdx.x / G, t = threadIdx.x - grp * G;
  cx<float>* sg = s + (size_t)grp * LD;
  const float scale = 1.f / NX;
  const int total = NX * W;
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    const int x = q / W, c = q - x * W;
    sf[2 * ((c >> 1) * LD + sp<float>(x)) + (c & 1)] = g[(size_t)x * nv + c0 + c];
  }
  __syncthreads();
  block_fft<float, NX, false, R>(sg, t, tw);
  // theta(m) = m * (-dkx dt v_col): kx = m dkx on the bins m <= NX/2
  const Ang aa = split_angle(phi_unit * v[c0 + 2 * grp]);
  const Ang ab = split_angle(phi_unit * v[c0 + 2 * grp + 1]);
  two_real_rotate<float>(sg, NX, t, G, [&](int m, float& ca, float& sa, float& cb, float& sb) {
    sincos_m((float)m, aa, sa, ca);
    sincos_m((float)m, ab, sb, cb);
    ca *= scale;
    sa *= scale;
    cb *= scale;
    sb *= scale;
  });
  __syncthreads();
  block_fft<float, NX, true, R>(sg, t, tw);
  // density partial sums (trapz weights: 1/2 at the two v end points)
  for (int x = threadIdx.x; x < NX; x += blockDim.x) {
    float acc = 0.f;
    for (int c = 0; c < W; ++c) {
      const int col = c0 + c;
      const float w = (col == 0 || col == nv - 1) ? 0.5f : 1.f;
      acc = fmaf(w, sf[2 * ((c >> 1) * LD + sp<float>(x)) + (c & 1)], acc);
    }
    dacc[x] = df_add(dacc[x], {acc, 0.f});
  }
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    const int x = q / W, c = q - x * W;
    g[(size_t)x * nv + c0 + c] = sf[2 * ((c >> 1) * LD + sp<float>(x)) + (c & 1)];
  }
  __syncthreads();
}

template <int NX, int R>
__global__ void __launch_bounds__((NX / R) * col32_seqs(NX, R)) k_col_f32(
    float* __restrict__ g, int nv, int ntiles, int W, double phi_unit,
    const double* __restrict__ v, const cx<float>* __restrict__ tw, float2* __restrict__ dpart) {
  constexpr int LD = sp_len<float>(NX) + COL32_PAD;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int S = W / 2;
  df32* dacc = reinterpret_cast<df32*>(smem_raw + (size_t)S * LD * sizeof(cx<float>));
  for (int x = threadIdx.x; x < NX; x += blockDim.x) dacc[x] = {0.f, 0.f};
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
    col_tile<NX, R>(g, nv, tile * W, W, phi_unit, v, tw, smem_raw, dacc);
  for (int x = threadIdx.x; x < NX; x += blockDim.x)
    dpart[(size_t)blockIdx.x * NX + x] = make_float2(dacc[x].hi, dacc[x].lo);
}

// ---------------------------------------------------------------------------
// density reduction and field solve
// ---------------------------------------------------------------------------

__global__ void k_dens_f32(const float2* __restrict__ dpart, int npart, int nx, double dv, double c0,
                           double* __restrict__ rho) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= nx) return;
  df32 acc = {0.f, 0.f};
  for (int p = 0; p < npart; ++p) {
    const float2 v = dpart[(size_t)p * nx + x];
    acc = df_add(acc, {v.x, v.y});
  }
  // 1 - n = -(dv sum g) - (trapz(f0) - 1), in FP64
  rho[x] = -(dv * df_to_double(acc)) - c0;
}

// driver: scalar envelope in FP64, phase k x - w t reduced mod 2 pi in FP64,
// sine in FP32 (the driver amplitude is small; this is the FP32 path)
__device__ __forceinline__ float pulse_sum_f32(const vg_pulse* __restrict__ P, int np, double t, double x) {
  float total = 0.f;
  for (int i = 0; i < np; ++i) {
    const vg_pulse q = P[i];
    double amp;
    if (q.envelope == VG_ENV_SIN2) {
      if (t < 0.0 || t > q.t_R) continue;
      const double sn = sin(3.141592653589793 * t / q.t_R);
      amp = q.a0 * sn * sn;
    } else {
      amp = 0.5 * (tanh((t - q.t_L) / q.t_wL) - tanh((t - q.t_R) / q.t_wR)) * q.k0 * q.a0;
    }
    double arg = q.k0 * x - q.w0 * t;
    arg -= 6.283185307179586 * rint(arg * 0.15915494309189535);
    total += (float)amp * sinf((float)arg);
  }
  return total;
}

template <int NX>
__global__ void __launch_bounds__(fft_threads<float>(NX)) k_field_f32(
    const double* __restrict__ rho, const double* __restrict__ inv_kx, const double* __restrict__ driver,
    int use_pulses, const vg_pulse* __restrict__ P, int np, const double* __restrict__ x, const double* t_ptr,
    double t_host, int nadd, double a0, double a1, double a2, double a3, double a4,
    const cx<float>* __restrict__ tw, double* __restrict__ e) {
  constexpr int G = fft_threads<float>(NX);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<float>* s = reinterpret_cast<cx<float>*>(smem_raw);
  const int t = threadIdx.x;
  for (int n = t; n < NX; n += G) s[sp<float>(n)] = {(float)rho[n], 0.f};
  __syncthreads();
  block_fft<float, NX, false>(s, t, tw);
  const float sc = 1.f / NX;
  for (int k = t; k < NX; k += G) {
    const cx<float> z = s[sp<float>(k)];
    const float ik = (float)inv_kx[k] * sc;
    s[sp<float>(k)] = {-ik * z.y, ik * z.x};
  }
  __syncthreads();
  block_fft<float, NX, true>(s, t, tw);
  double tt = t_ptr ? *t_ptr : t_host;
  const double adds[5] = {a0, a1, a2, a3, a4};
  for (int i = 0; i < nadd; ++i) tt += adds[i];
  for (int n = t; n < NX; n += G) {
    float drv = 0.f;
    if (driver) drv = (float)driver[n];
    else if (use_pulses) drv = pulse_sum_f32(P, np, tt, x[n]);
    e[n] = (double)(drv + s[sp<float>(n)].x);
  }
}

// ---------------------------------------------------------------------------
// row pass: kick / collide / measure / kick
// ---------------------------------------------------------------------------

// rotation of one packed row pair with the delta-f background term; the 1/N of
// the inverse transform is folded in.  ha/hb: half-angle per kv index.
template <int N>
__device__ __forceinline__ void kick_rotate(cx<float>* s, int t, int G, Ang ha, Ang hb,
                                            const cx<float>* __restrict__ F0) {
  const float sc = 1.f / N;
  for (int k = t; k <= N / 2; k += G) {
    float sa, ca, sb, cb;
    sincos_m((float)k, ha, sa, ca);
    sincos_m((float)k, hb, sb, cb);
    // P = (1 - 2 sin^2, 2 sin cos) of the half angle; P - 1 = (-2 sin^2, 2 sin cos)
    const float pa_m1r = -2.f * sa * sa, pa_i = 2.f * sa * ca, pa_r = 1.f + pa_m1r;
    const float pb_m1r = -2.f * sb * sb, pb_i = 2.f * sb * cb, pb_r = 1.f + pb_m1r;
    const cx<float> f0 = F0[k];
    if (k == 0 || 2 * k == N) {
      const cx<float> z = s[sp<float>(k)];
      // real bins: only Re(P) survives
      s[sp<float>(k)] = {(pa_r * z.x + pa_m1r * f0.x) * sc, (pb_r * z.y + pb_m1r * f0.x) * sc};
      continue;
    }
    const cx<float> zk = s[sp<float>(k)], zm = s[sp<float>(N - k)];
    const cx<float> fa = {(zk.x + zm.x) * 0.5f, (zk.y - zm.y) * 0.5f};
    const cx<float> fb = {(zk.y + zm.y) * 0.5f, (zm.x - zk.x) * 0.5f};
    const cx<float> ga = {(pa_r * fa.x - pa_i * fa.y + pa_m1r * f0.x - pa_i * f0.y) * sc,
                          (pa_r * fa.y + pa_i * fa.x + pa_m1r * f0.y + pa_i * f0.x) * sc};
    const cx<float> gb = {(pb_r * fb.x - pb_i * fb.y + pb_m1r * f0.x - pb_i * f0.y) * sc,
                          (pb_r * fb.y + pb_i * fb.x + pb_m1r * f0.y + pb_i * f0.x) * sc};
    s[sp<float>(k)] = {ga.x - gb.y, ga.y + gb.x};
    s[sp<float>(N - k)] = {ga.x + gb.y, gb.x - ga.y};
  }
}

template <int N, int R>
__device__ __forceinline__ void kick(cx<float>* s, int t, double dkv, double dt, double ea, double eb,
                                     const cx<float>* __restrict__ F0, const cx<float>* __restrict__ tw) {
  constexpr int G = N / R;
  block_fft<float, N, false, R>(s, t, tw);
  // theta(k) = -kv_k dt e = k * (-dkv dt e); half angle for P - 1
  const Ang ha = split_angle(-0.5 * dkv * dt * ea);
  const Ang hb = split_angle(-0.5 * dkv * dt * eb);
  kick_rotate<N>(s, t, G, ha, hb, F0);
  __syncthreads();
  block_fft<float, N, true, R>(s, t, tw);
}

// Fokker-Planck step of one row stored at x (stride 2 floats) in delta-f form.
template <int N, int R>
__device__ __forceinline__ void collide_row(float* x, int t, const RowConsts& rc, double nudt, int dougherty,
                                            df32* red, float* pcr) {
  constexpr int G = N / R;
  // moments of g over the thread's chunk: sum w g, sum w g v, sum w g v^2
  df32 mv[3];
  {
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int j = t * R + i;
      const float w = (j == 0 || j == N - 1) ? 0.5f : 1.f;
      const float gv = w * x[2 * sp<float>(j)];
      const float vj = rc.v[j];
      a0 += gv;
      a1 = fmaf(gv, vj, a1);
      a2 = fmaf(gv * vj, vj, a2);
    }
    mv[0] = {a0, 0.f};
    mv[1] = {a1, 0.f};
    mv[2] = {a2, 0.f};
  }
  group_df_sum<3>(mv, red, G, t);
  const double M0 = rc.dv * df_to_double(mv[0]) + rc.f0m[0];
  const double M1 = rc.dv * df_to_double(mv[1]) + rc.f0m[1];
  const double M2 = rc.dv * df_to_double(mv[2]) + rc.f0m[2];
  // DG: vbar = trapz(f v), v0t^2 = trapz(f (v - vbar)^2) = M2 + vbar^2 (M0 - 2)
  // LB: v0t^2 = trapz(f v^2), no drift
  const double vbar = dougherty ? M1 : 0.0;
  const double vth = dougherty ? M2 + vbar * vbar * (M0 - 2.0) : M2;
  const float Af = (float)(-vth / rc.dv_sq);
  const float bdiag = (float)(1.0 + nudt * (2.0 * vth / rc.dv_sq));
  const float nu = (float)nudt;
  const float vb = (float)vbar;
  const float i2dv = (float)(0.5 / rc.dv);
  // right-hand side: g - (A - I) f0 with (A - I) f0 = nudt (-vth S + Mv - vbar D)
  const float cs = (float)(nudt * vth), cm = nu, cd = (float)(nudt * vbar);
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int j = t * R + i;
    x[2 * sp<float>(j)] -= -cs * rc.S[j] + cm * rc.Mv[j] - cd * rc.D[j];
  }
  __syncthreads();
  auto lf = [&](int j) { return nu * (Af + (rc.v[j - 1] - vb) * i2dv); };
  auto uf = [&](int j) { return nu * (Af - (rc.v[j + 1] - vb) * i2dv); };
  partition_solve<R>(x, t, G, bdiag, lf, uf, pcr);
}

// One row-pair group of the row pass: load, [kick dt1], [collide], [moments
// and x-mode partials], [kick dt2], store.  grp_base: this group's shared
// memory (row32_group_bytes); macc: the CTA's mode accumulators [n_modes][N].
template <int N, int R>
__device__ __forceinline__ void row_pair(const RowArgs& a, int pair, unsigned char* grp_base, cx<float>* macc,
                                         int P, int grp, int t) {
  constexpr int G = N / R;
  cx<float>* s = reinterpret_cast<cx<float>*>(grp_base);
  const size_t seq_bytes = (size_t)sp_len<float>(N) * sizeof(cx<float>) + 16;
  float* pcr = reinterpret_cast<float*>(grp_base + seq_bytes);
  df32* red = reinterpret_cast<df32*>(grp_base + seq_bytes + 8 * G * sizeof(float));
  const int nm = a.n_modes;
  const int ra = 2 * pair, rb = ra + 1;
  const bool va = ra < a.nx, vb = rb < a.nx;
  float* ga = a.g + (size_t)ra * N;
  float* gbp = a.g + (size_t)rb * N;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int n = t + i * G;
    s[sp<float>(n)] = {va ? ga[n] : 0.f, vb ? gbp[n] : 0.f};
  }
  __syncthreads();
  const bool kicks = a.dt1 != 0.0 || a.dt2 != 0.0;
  const double ea = (kicks && va) ? a.e[ra] : 0.0, eb = (kicks && vb) ? a.e[rb] : 0.0;
  if (a.dt1 != 0.0) kick<N, R>(s, t, a.rc.dkv, a.dt1, ea, eb, a.F0, a.tw);
  float* sx = reinterpret_cast<float*>(s);
  if (a.fp) {
    collide_row<N, R>(sx, t, a.rc, a.nudt, a.dougherty, red, pcr);
    collide_row<N, R>(sx + 1, t, a.rc, a.nudt, a.dougherty, red, pcr);
  }
  if (a.want_mom) {
    // n, j, T, q, fv4, vN (sums of w g v^p), sum w g^2, sum w g f0, sum w f log f
    df32 mv[9], mw[9];
    float sa[9] = {0}, sb[9] = {0};
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int j = t * R + i;
      const float w = (j == 0 || j == N - 1) ? 0.5f : 1.f;
      const float vj = a.rc.v[j], f0j = a.rc.f0[j];
      const cx<float> z = s[sp<float>(j)];
      float pa = w * z.x, pb = w * z.y;
#pragma unroll
      for (int p = 0; p < 6; ++p) {
        sa[p] += pa;
        sb[p] += pb;
        pa *= vj;
        pb *= vj;
      }
      sa[6] = fmaf(w * z.x, z.x, sa[6]);
      sb[6] = fmaf(w * z.y, z.y, sb[6]);
      sa[7] = fmaf(w * z.x, f0j, sa[7]);
      sb[7] = fmaf(w * z.y, f0j, sb[7]);
      const float fa = z.x + f0j, fb = z.y + f0j;
      sa[8] = fmaf(w * fa, logf(fa), sa[8]);
      sb[8] = fmaf(w * fb, logf(fb), sb[8]);
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      mv[q] = {sa[q], 0.f};
      mw[q] = {sb[q], 0.f};
    }
    group_df_sum<9>(mv, red, G, t);
    group_df_sum<9>(mw, red, G, t);
    if (t == 0) {
      for (int r = 0; r < 2; ++r) {
        const int row = r ? rb : ra;
        if (!(r ? vb : va)) continue;
        const df32* m = r ? mw : mv;
        double* out = a.mom + (size_t)row * MOM_STRIDE;
        for (int p = 0; p < 6; ++p) out[p] = a.rc.dv * df_to_double(m[p]) + a.rc.f0m[p];
        out[6] = a.rc.dv * (df_to_double(m[6]) + 2.0 * df_to_double(m[7])) + a.rc.f0m[6];
        out[7] = a.rc.dv * df_to_double(m[8]);
      }
    }
    // x-Fourier modes of f (the f0 part of mode 0 is added in the reduction);
    // the groups of a CTA hold different rows but add into the same bins,
    // so they take turns
    if (nm > 0) {
      for (int gq = 0; gq < P; ++gq) {
        if (gq == grp) {
          for (int mq = 0; mq < nm; ++mq) {
            float swa = 0.f, cwa = 0.f, swb = 0.f, cwb = 0.f;
            if (va) sincospif(-2.f * (float)((mq * ra) % a.nx) / (float)a.nx, &swa, &cwa);
            if (vb) sincospif(-2.f * (float)((mq * rb) % a.nx) / (float)a.nx, &swb, &cwb);
            for (int i = 0; i < R; ++i) {
              const int n = t + i * G;
              const cx<float> z = s[sp<float>(n)];
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
  if (a.dt2 != 0.0) kick<N, R>(s, t, a.rc.dkv, a.dt2, ea, eb, a.F0, a.tw);
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int n = t + i * G;
    const cx<float> z = s[sp<float>(n)];
    if (va) ga[n] = z.x;
    if (vb) gbp[n] = z.y;
  }
  __syncthreads();
}

template <int N, int R>
__global__ void __launch_bounds__(row32_block(N, R)) k_row_f32(RowArgs a) {
  constexpr int G = N / R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int P = blockDim.x / G;
  const int grp = threadIdx.x / G, t = threadIdx.x - grp * G;
  const size_t grp_bytes = row32_group_bytes(N, R);
  cx<float>* macc = reinterpret_cast<cx<float>*>(smem_raw + (size_t)P * grp_bytes);  // [n_modes][N]
  const int nm = a.want_mom ? a.n_modes : 0;
  for (int q = threadIdx.x; q < nm * N; q += blockDim.x) macc[q] = {0.f, 0.f};
  const int npairs = (a.nx + 1) / 2;
  const int ngroups = (npairs + P - 1) / P;
  for (int pg = blockIdx.x; pg < ngroups; pg += gridDim.x)
    row_pair<N, R>(a, pg * P + grp, smem_raw + (size_t)grp * grp_bytes, macc, P, grp, t);
  if (nm > 0) {
    __syncthreads();
    for (int q = threadIdx.x; q < nm * N; q += blockDim.x)
      a.mpart[(size_t)blockIdx.x * nm * N + q] = macc[q];
  }
}

// ---------------------------------------------------------------------------
// storage of one step: fields, series and stored modes
// ---------------------------------------------------------------------------

__global__ void k_store_fields_f32(const double* __restrict__ mom, const double* __restrict__ e,
                                   const double* __restrict__ de, int nx, int i, vg_history h) {
  __shared__ df32 red[32 * 7];
  const size_t off = (size_t)i * nx;
  df32 acc[7];
  for (int q = 0; q < 7; ++q) acc[q] = {0.f, 0.f};
  for (int n = threadIdx.x; n < nx; n += blockDim.x) {
    const double* m = mom + (size_t)n * MOM_STRIDE;
    if (h.fields[0]) h.fields[0][off + n] = e[n];
    if (h.fields[1]) h.fields[1][off + n] = de ? de[n] : 0.0;
    for (int q = 0; q < 6; ++q)
      if (h.fields[2 + q]) h.fields[2 + q][off + n] = m[q];
    const double src[7] = {m[0], m[1], m[2], e[n] * e[n], de ? de[n] * de[n] : 0.0, m[6], m[7]};
    for (int q = 0; q < 7; ++q) {
      const float hi = (float)src[q];
      acc[q] = df_add(acc[q], {hi, (float)(src[q] - (double)hi)});
    }
  }
  block_df_sum<7>(acc, red);
  if (threadIdx.x < 7 && h.series[threadIdx.x]) h.series[threadIdx.x][i] = df_to_double(acc[threadIdx.x]) / nx;
}

__global__ void k_store_modes_f32(const cx<float>* __restrict__ mpart, int npart, int nm, int nv, int nx,
                                  const double* __restrict__ f0, int n_slots, int i, cx<float>* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nv) return;
  cx<float>* dst = out + (size_t)i * n_slots * nv;
  for (int m = 0; m < nm && m < n_slots; ++m) {
    df32 re = {0.f, 0.f}, im = {0.f, 0.f};
    for (int p = 0; p < npart; ++p) {
      const cx<float> z = mpart[((size_t)p * nm + m) * nv + j];
      re = df_add(re, {z.x, 0.f});
      im = df_add(im, {z.y, 0.f});
    }
    double zr = df_to_double(re), zi = df_to_double(im);
    if (m == 0) zr += (double)nx * f0[j];
    const cx<float> z = {(float)zr, (float)zi};
    if (nm == 1) {
      for (int sl = 0; sl < n_slots; ++sl) dst[(size_t)sl * nv + j] = z;
    } else {
      dst[(size_t)m * nv + j] = z;
    }
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

namespace {

template <int NX>
cudaError_t col_n(const vg_plan& p, float* g, double dt, cudaStream_t s) {
  constexpr int R = col32_radix(NX);
  constexpr int G = NX / R;
  int S = col32_seqs(NX, R);
  if (2 * S > p.nv) S = p.nv / 2;
  const int W = 2 * S;
  const int ntiles = p.nv / W;
  const size_t smem = (size_t)S * (sp_len<float>(NX) + COL32_PAD) * sizeof(cx<float>) + (size_t)NX * sizeof(df32);
  cudaError_t err = ensure_smem((const void*)k_col_f32<NX, R>, smem);
  if (err != cudaSuccess) return err;
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_col_f32<NX, R>, S * G, smem);
  int grid = (occ > 0 ? occ : 1) * p.f32->n_sm;
  if (grid > p.f32->col_grid_max) grid = p.f32->col_grid_max;
  if (grid > ntiles) grid = ntiles;
  k_col_f32<NX, R><<<grid, S * G, smem, s>>>(g, p.nv, ntiles, W, -p.f32->dkx * dt, p.v, p.tw32, p.f32->dpart);
  p.f32->npart = grid;
  return cudaGetLastError();
}

template <int NX>
cudaError_t field_n(const vg_plan& p, const double* driver, const FieldTime& ft, double* e, cudaStream_t s) {
  constexpr int G = fft_threads<float>(NX);
  const size_t smem = (size_t)sp_len<float>(NX) * sizeof(cx<float>);
  cudaError_t err = ensure_smem((const void*)k_field_f32<NX>, smem);
  if (err != cudaSuccess) return err;
  k_field_f32<NX><<<1, G, smem, s>>>(p.rho, p.inv_kx, driver, ft.use_pulses, p.pulses, p.n_pulses, p.x, ft.t_ptr,
                                     ft.t_host, ft.nadd, ft.add[0], ft.add[1], ft.add[2], ft.add[3], ft.add[4],
                                     p.tw32, e);
  return cudaGetLastError();
}

template <int N>
cudaError_t row_n(const vg_plan& p, RowArgs a, cudaStream_t s) {
  constexpr int R = row32_radix(N);
  constexpr int G = N / R;
  const int block = row32_block(N, R);
  const int P = block / G;
  const int npairs = (p.nx + 1) / 2;
  const int ngroups = (npairs + P - 1) / P;
  const size_t smem = (size_t)P * row32_group_bytes(N, R) + (size_t)a.n_modes * N * sizeof(cx<float>);
  cudaError_t err = ensure_smem((const void*)k_row_f32<N, R>, smem);
  if (err != cudaSuccess) return err;
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_row_f32<N, R>, block, smem);
  int grid = (occ > 0 ? occ : 1) * p.f32->n_sm;
  if (grid > p.f32->row_grid_max) grid = p.f32->row_grid_max;
  if (grid > ngroups) grid = ngroups;
  k_row_f32<N, R><<<grid, block, smem, s>>>(a);
  p.f32->mgrid = grid;
  return cudaGetLastError();
}

}  // namespace

#define VG_F32_POW2_CASES(M) M(1) M(2) M(3) M(4) M(5) M(6) M(7) M(8) M(9) M(10) M(11) M(12) M(13)

cudaError_t launch_col_f32(const vg_plan& p, float* g, double dt, cudaStream_t s) {
  switch (ilog2(p.nx)) {
#define CASE(L) case L: return col_n<(1 << L)>(p, g, dt, s);
    VG_F32_POW2_CASES(CASE)
#undef CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_poisson_only_f32(const vg_plan& p, const double* rho, const double* driver,
                                    const FieldTime& ft, double* e, cudaStream_t s) {
  if (rho != p.rho) {
    cudaError_t err = cudaMemcpyAsync(p.rho, rho, (size_t)p.nx * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (err != cudaSuccess) return err;
  }
  switch (ilog2(p.nx)) {
#define CASE(L) case L: return field_n<(1 << L)>(p, driver, ft, e, s);
    VG_F32_POW2_CASES(CASE)
#undef CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_field_f32(const vg_plan& p, const double* driver, const FieldTime& ft, double* e,
                             cudaStream_t s) {
  k_dens_f32<<<div_up(p.nx, 128), 128, 0, s>>>(p.f32->dpart, p.f32->npart, p.nx, p.dv, p.f32->c0, p.rho);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  return launch_poisson_only_f32(p, p.rho, driver, ft, e, s);
}

// density of the current state by rows (stand-alone field solve / density):
// out = n (as_density) or 1 - n
__global__ void k_dens_rows_f32(const float* __restrict__ g, int nv, double dv, double n0, double c0,
                                int as_density, double* __restrict__ out) {
  __shared__ df32 red[32];
  const size_t r = blockIdx.x;
  float acc = 0.f;
  df32 a[1] = {{0.f, 0.f}};
  for (int j = threadIdx.x; j < nv; j += blockDim.x) {
    const float w = (j == 0 || j == nv - 1) ? 0.5f : 1.f;
    acc = w * g[r * nv + j];
    a[0] = df_add(a[0], {acc, 0.f});
  }
  block_df_sum<1>(a, red);
  if (threadIdx.x == 0) {
    const double sg = dv * df_to_double(a[0]);
    out[r] = as_density ? sg + n0 : -sg - c0;
  }
}

cudaError_t launch_dens_rows_f32(const vg_plan& p, const float* g, double* out, int as_density, cudaStream_t s) {
  k_dens_rows_f32<<<p.nx, 256, 0, s>>>(g, p.nv, p.dv, p.f32->rc.f0m[0], p.f32->c0, as_density, out);
  return cudaGetLastError();
}

// stored_f[i] = g + f0 as float64 (store-all rule)
__global__ void k_store_all_f32(const float* __restrict__ g, const double* __restrict__ f0, int nx, int nv,
                                double* __restrict__ out) {
  const size_t n = (size_t)nx * nv;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    out[q] = (double)g[q] + f0[q % nv];
}

cudaError_t launch_row_f32(const vg_plan& p, float* g, const double* e, double dt1, double dt2, int fp, int mom,
                           int n_modes, cudaStream_t s) {
  RowArgs a;
  a.g = g;
  a.nx = p.nx;
  a.e = e;
  a.dt1 = dt1;
  a.dt2 = dt2;
  a.fp = fp && p.collision != VG_COLL_NONE;
  a.dougherty = p.collision == VG_COLL_DG;
  a.nudt = p.nudt;
  a.want_mom = mom;
  a.mom = p.mom;
  a.n_modes = mom ? n_modes : 0;
  a.mpart = p.f32->mpart;
  a.F0 = p.f32->F0;
  a.tw = p.tw32;
  a.rc = p.f32->rc;
  switch (ilog2(p.nv)) {
#define CASE(L) case L: return row_n<(1 << L)>(p, a, s);
    VG_F32_POW2_CASES(CASE)
#undef CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_store_f32(const vg_plan& p, const float* g, const double* e, const double* de,
                             const vg_history& h, int i, int n_modes, cudaStream_t s) {
  k_store_fields_f32<<<1, 256, 0, s>>>(p.mom, e, de, p.nx, i, h);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  if (h.stored_f && h.store_all) {
    const size_t n = (size_t)p.nx * p.nv;
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_store_all_f32<<<blocks, 256, 0, s>>>(g, p.f_bg, p.nx, p.nv, static_cast<double*>(h.stored_f) + (size_t)i * n);
    return cudaGetLastError();
  }
  if (h.stored_f && !h.store_all && n_modes > 0) {
    k_store_modes_f32<<<div_up(p.nv, 128), 128, 0, s>>>(p.f32->mpart, p.f32->mgrid, n_modes, p.nv, p.nx, p.f_bg,
                                                        h.n_slots, i, static_cast<cx<float>*>(h.stored_f));
    err = cudaGetLastError();
  }
  return err;
}

}  // namespace vg
