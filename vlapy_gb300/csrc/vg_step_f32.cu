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
#include <algorithm>

#include "vg_f32_body.cuh"
#include "vg_internal.cuh"

namespace vg {

// ---------------------------------------------------------------------------
// x-drift of column tiles
// ---------------------------------------------------------------------------

template <int NX, int R>
__global__ void __launch_bounds__((NX / R) * col32_seqs(NX, R)) k_col_f32(
    float* __restrict__ g, int nv, int ntiles, int W, float2 kdt,
    const float2* __restrict__ vhl, const cx<float>* __restrict__ tw, float2* __restrict__ dpart) {
  constexpr int LD = sp_len<float>(NX) + COL32_PAD;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int S = W / 2;
  df32* dacc = reinterpret_cast<df32*>(smem_raw + (size_t)S * LD * sizeof(cx<float>));
  for (int x = threadIdx.x; x < NX; x += blockDim.x) dacc[x] = {0.f, 0.f};
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
    col_tile<NX, R>(g, nv, tile * W, W, kdt, vhl, tw, smem_raw, dacc);
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
    const cx<float>* __restrict__ tw, double* __restrict__ e, float* __restrict__ e32, int* flags) {
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
    const float en = drv + s[sp<float>(n)].x;
    e[n] = (double)en;
    e32[n] = en;
    if (flags && !isfinite(en)) atomicOr(flags, VG_FLAG_NONFINITE);
  }
}

// ---------------------------------------------------------------------------
// row pass: kick / collide / measure / kick
// ---------------------------------------------------------------------------

// KICK: a launch that only kicks (no collision, no moments, no trailing
// kick), a lighter instantiation at two CTAs per SM
// (radix 32: two CTAs of 128 registers a thread per SM)
template <int N, int R, bool KICK = false>
__global__ void __launch_bounds__(row32_block(N, R), (KICK || R == 32) ? 2 : 1) k_row_f32(RowArgs a) {
  constexpr int G = N / R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int P = blockDim.x / G;
  const int grp = threadIdx.x / G, t = threadIdx.x - grp * G;
  const size_t grp_bytes = row32_group_bytes(N, R);
  const int nm = a.want_mom ? a.n_modes : 0;
  // x-mode accumulators [n_modes][N]: in shared memory, or (long rows, where
  // they would crowd the row-pair groups out) in this CTA's slice of the
  // mode partials, where they stay in L2; element n is only touched by the
  // threads t = n mod G, in turns of the CTA's groups
  cx<float>* macc = a.macc_global ? a.mpart + (size_t)blockIdx.x * nm * N
                                  : reinterpret_cast<cx<float>*>(smem_raw + (size_t)P * grp_bytes);
  for (int q = threadIdx.x; q < nm * N; q += blockDim.x) macc[q] = {0.f, 0.f};
  const int npairs = (a.nx + 1) / 2;
  const int ngroups = (npairs + P - 1) / P;
  for (int pg = blockIdx.x; pg < ngroups; pg += gridDim.x)
    row_pair<N, R, CtaSync, 6, KICK>(a, pg * P + grp, smem_raw + (size_t)grp * grp_bytes, macc, P, grp, t);
  if (nm > 0 && !a.macc_global) {
    __syncthreads();
    for (int q = threadIdx.x; q < nm * N; q += blockDim.x)
      a.mpart[(size_t)blockIdx.x * nm * N + q] = macc[q];
  }
}

// ---------------------------------------------------------------------------
// storage of one step: fields, series and stored modes
// ---------------------------------------------------------------------------

// fields of one step and the series partial sums of this CTA's rows (rows
// blockIdx.x * blockDim.x + threadIdx.x, stride the whole grid); spart[b][q]
// is CTA b's double-float partial of series q
__global__ void k_store_fields_f32(const double* __restrict__ mom, RowConsts rc, const double* __restrict__ e,
                                   const double* __restrict__ de, int nx, int i, vg_history h,
                                   float2* __restrict__ spart) {
  __shared__ df32 red[32 * 7];
  const size_t off = (size_t)i * nx;
  df32 acc[7];
  for (int q = 0; q < 7; ++q) acc[q] = {0.f, 0.f};
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nx; n += gridDim.x * blockDim.x) {
    const double* slots = mom + (size_t)n * MOM_STRIDE;
    double m[8];
    for (int q = 0; q < 8; ++q) m[q] = row_moment(slots, q, rc);
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
  if (threadIdx.x < 7) spart[blockIdx.x * 7 + threadIdx.x] = make_float2(acc[threadIdx.x].hi, acc[threadIdx.x].lo);
}

// the series of one step: the CTAs' partials added in CTA order (one thread
// per series, so the sum is the same on every run)
__global__ void k_store_series_f32(const float2* __restrict__ spart, int nb, int nx, int i, vg_history h) {
  const int q = threadIdx.x;
  if (q >= 7 || !h.series[q]) return;
  df32 acc = {0.f, 0.f};
  for (int b = 0; b < nb; ++b) acc = df_add(acc, {spart[b * 7 + q].x, spart[b * 7 + q].y});
  h.series[q][i] = df_to_double(acc) / nx;
}

// stored x-modes of one step: thread (j, m) adds mode m of velocity j over
// the row kernel's per-CTA partials, in four interleaved double-float chains
// (partials p = 0, 4, 8, ... in the first, and so on) joined in a fixed order
// stored x modes of one step: the CTAs' mode partials summed in double-float.
// A block is 32 bins x STORE_MODE_SPLIT slice ranges: thread (jx, gy) sums
// the slices of range gy for bin j (consecutive jx, consecutive j: coalesced),
// then the ranges are added in order (deterministic)
constexpr int STORE_MODE_SPLIT = 8;
__global__ void __launch_bounds__(32 * STORE_MODE_SPLIT) k_store_modes_f32(
    const cx<float>* __restrict__ mpart, int npart, int nm, int nv, int nx, const double* __restrict__ f0,
    int n_slots, int i, cx<float>* __restrict__ out) {
  __shared__ df32 part_re[STORE_MODE_SPLIT][32], part_im[STORE_MODE_SPLIT][32];
  const int jx = threadIdx.x & 31, gy = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + jx;
  const int m = blockIdx.y;
  const bool live = j < nv && m < nm && m < n_slots;
  df32 re[2] = {{0.f, 0.f}, {0.f, 0.f}}, im[2] = {{0.f, 0.f}, {0.f, 0.f}};
  if (live) {
    const int per = (npart + STORE_MODE_SPLIT - 1) / STORE_MODE_SPLIT;
    const int p0 = gy * per, p1 = min(npart, p0 + per);
    int p = p0, u = 0;
    for (; p < p1; ++p, u ^= 1) {
      const cx<float> z = mpart[((size_t)p * nm + m) * nv + j];
      re[u] = df_add(re[u], {z.x, 0.f});
      im[u] = df_add(im[u], {z.y, 0.f});
    }
  }
  part_re[gy][jx] = df_add(re[0], re[1]);
  part_im[gy][jx] = df_add(im[0], im[1]);
  __syncthreads();
  if (gy != 0 || !live) return;
  df32 rs = part_re[0][jx], is = part_im[0][jx];
  for (int q = 1; q < STORE_MODE_SPLIT; ++q) {
    rs = df_add(rs, part_re[q][jx]);
    is = df_add(is, part_im[q][jx]);
  }
  cx<float>* dst = out + (size_t)i * n_slots * nv;
  double zr = df_to_double(rs), zi = df_to_double(is);
  if (m == 0) zr += (double)nx * f0[j];
  const cx<float> z = {(float)zr, (float)zi};
  if (nm == 1) {
    for (int sl = 0; sl < n_slots; ++sl) dst[(size_t)sl * nv + j] = z;
  } else {
    dst[(size_t)m * nv + j] = z;
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
  k_col_f32<NX, R><<<grid, S * G, smem, s>>>(g, p.nv, ntiles, W, split_f2(-p.f32->dkx * dt), p.f32->vhl, p.tw32,
                                             p.f32->dpart);
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
                                     p.tw32, e, p.f32->e32, p.flags);
  return cudaGetLastError();
}

template <int N, bool KICK>
cudaError_t row_nk(const vg_plan& p, RowArgs a, cudaStream_t s) {
  constexpr int R = row32_radix(N);
  constexpr int G = N / R;
  const int block = row32_block(N, R);
  const int P = block / G;
  const int npairs = (p.nx + 1) / 2;
  const int ngroups = (npairs + P - 1) / P;
  const size_t mode_bytes = (size_t)(a.want_mom ? a.n_modes : 0) * N * sizeof(cx<float>);
  a.macc_global = (size_t)P * row32_group_bytes(N, R) + mode_bytes > ((size_t)100 << 10) ? 1 : 0;
  const size_t smem = (size_t)P * row32_group_bytes(N, R) + (a.macc_global ? 0 : mode_bytes);
  cudaError_t err = ensure_smem((const void*)k_row_f32<N, R, KICK>, smem);
  if (err != cudaSuccess) return err;
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_row_f32<N, R, KICK>, block, smem);
  int grid = (occ > 0 ? occ : 1) * p.f32->n_sm;
  if (grid > p.f32->row_grid_max) grid = p.f32->row_grid_max;
  if (grid > ngroups) grid = ngroups;
  k_row_f32<N, R, KICK><<<grid, block, smem, s>>>(a);
  p.f32->mgrid = grid;
  return cudaGetLastError();
}

template <int N>
cudaError_t row_n(const vg_plan& p, RowArgs a, cudaStream_t s) {
  const bool kick_only = !a.fp && !a.want_mom && a.hk2 == 0.f;
  return kick_only ? row_nk<N, true>(p, a, s) : row_nk<N, false>(p, a, s);
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

__global__ void k_e_to_f32(const double* __restrict__ e, int nx, float* __restrict__ e32) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nx; i += gridDim.x * blockDim.x) e32[i] = (float)e[i];
}

cudaError_t launch_e_to_f32(const vg_plan& p, const double* e, cudaStream_t s) {
  k_e_to_f32<<<div_up(p.nx, 256), 256, 0, s>>>(e, p.nx, p.f32->e32);
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
  (void)e;  // the kicks read the FP32 copy p.f32->e32 (written by the field solve or launch_e_to_f32)
  RowArgs a;
  a.g = g;
  a.nx = p.nx;
  a.e32 = p.f32->e32;
  a.dt1 = dt1;
  a.dt2 = dt2;
  a.hk1 = (float)(-0.5 * p.f32->dkv * dt1);
  a.hk2 = (float)(-0.5 * p.f32->dkv * dt2);
  a.fp = fp && p.collision != VG_COLL_NONE;
  a.dougherty = p.collision == VG_COLL_DG;
  a.nudt2 = split_f2(p.nudt);
  a.nudt_f = (float)p.nudt;
  a.want_mom = mom;
  a.mom = p.mom;
  a.n_modes = mom ? n_modes : 0;
  a.mpart = p.f32->mpart;
  a.macc_global = 0;
  a.F0 = p.f32->F0;
  a.tw = p.tw32;
  a.rc = p.f32->rc_dev;
  switch (ilog2(p.nv)) {
#define CASE(L) case L: return row_n<(1 << L)>(p, a, s);
    VG_F32_POW2_CASES(CASE)
#undef CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_store_f32(const vg_plan& p, const float* g, const double* e, const double* de,
                             const vg_history& h, int i, int n_modes, cudaStream_t s) {
  const int nb = std::min(F32_STORE_MAX_CTAS, (p.nx + 255) / 256);
  k_store_fields_f32<<<nb, 256, 0, s>>>(p.mom, p.f32->rc, e, de, p.nx, i, h, p.f32->spart);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  k_store_series_f32<<<1, 32, 0, s>>>(p.f32->spart, nb, p.nx, i, h);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  if (h.stored_f && h.store_all) {
    const size_t n = (size_t)p.nx * p.nv;
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_store_all_f32<<<blocks, 256, 0, s>>>(g, p.f_bg, p.nx, p.nv, static_cast<double*>(h.stored_f) + (size_t)i * n);
    return cudaGetLastError();
  }
  if (h.stored_f && !h.store_all && n_modes > 0) {
    k_store_modes_f32<<<dim3(div_up(p.nv, 32), n_modes), 32 * STORE_MODE_SPLIT, 0, s>>>(
        p.f32->mpart, p.f32->mgrid, n_modes, p.nv, p.nx, p.f_bg, h.n_slots, i, static_cast<cx<float>*>(h.stored_f));
    err = cudaGetLastError();
  }
  return err;
}

}  // namespace vg
