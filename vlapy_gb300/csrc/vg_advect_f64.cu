// FP64 advection kernels: the exponential integrators in v (rows) and x
// (columns) of vlapy/core/vlasov.py:83-140, as shared-memory FFTs.
//
// v-advection (rows).  One group of N/R threads owns a PAIR of rows packed as
// z = f[a] + i f[b]; one complex FFT of length nv transforms both rows, the
// bins of each row are separated by Hermitian symmetry, rotated by
// exp(i (-kv dt) e_row) and recombined, and one inverse FFT returns both rows.
// The whole row pair stays in shared memory between the two transforms: f is
// read once and written once per call.
//
// x-advection (columns).  One CTA owns a tile of all nx rows by W adjacent v
// columns; pairs of columns are packed the same way and transformed along x,
// rotated by exp(i (-kx dt) v_col).  Loads/stores are row segments of W
// contiguous doubles (coalesced), transposed through shared memory.
#include "vg_internal.cuh"

namespace vg {

template <int N>
__global__ void __launch_bounds__(row_block<double>(N)) k_edfdv_f64(double* __restrict__ f, int nrows,
                                                    const double* __restrict__ e,
                                                    const double* __restrict__ kv, double dt,
                                                    const cx<double>* __restrict__ tw) {
  constexpr int R = fft_radix<double>(N);
  constexpr int G = N / R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int P = blockDim.x / G;
  const int g = threadIdx.x / G, t = threadIdx.x - g * G;
  cx<double>* s = reinterpret_cast<cx<double>*>(smem_raw) + (size_t)g * sp_len<double>(N);
  const int pair = blockIdx.x * P + g;
  const int ra = 2 * pair, rb = ra + 1;
  const bool va = ra < nrows, vb = rb < nrows;
  double* fa = f + (size_t)ra * N;
  double* fb = f + (size_t)rb * N;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int n = t + i * G;
    s[sp<double>(n)] = {va ? fa[n] : 0.0, vb ? fb[n] : 0.0};
  }
  __syncthreads();
  block_fft<double, N, false>(s, t, tw);
  const double ea = va ? e[ra] : 0.0, eb = vb ? e[rb] : 0.0;
  // theta = ((-kv) * dt) * e, the imaginary part of (-1j * kv * dt * e)
  two_real_rotate<double>(s, N, t, G, [&](int k, double& ca, double& sa, double& cb, double& sb) {
    const double ph = -kv[k] * dt;
    sincos(ph * ea, &sa, &ca);
    sincos(ph * eb, &sb, &cb);
  });
  __syncthreads();
  block_fft<double, N, true>(s, t, tw);
  const double sc = 1.0 / N;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int n = t + i * G;
    const cx<double> z = s[sp<double>(n)];
    if (va) fa[n] = z.x * sc;
    if (vb) fb[n] = z.y * sc;
  }
}

// pad one element per sequence so column-pair sequences start in different banks
constexpr int COL_PAD = 1;

template <int NX>
__global__ void __launch_bounds__(col_seqs<double>(NX) * fft_threads<double>(NX)) k_vdfdx_f64(double* __restrict__ f, int nv, int W,
                                                    const double* __restrict__ kx,
                                                    const double* __restrict__ v, double dt,
                                                    const cx<double>* __restrict__ tw) {
  constexpr int R = fft_radix<double>(NX);
  constexpr int G = NX / R;
  constexpr int LD = sp_len<double>(NX) + COL_PAD;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<double>* s = reinterpret_cast<cx<double>*>(smem_raw);
  double* sd = reinterpret_cast<double*>(smem_raw);
  const int c0 = blockIdx.x * W;
  const int total = NX * W;
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    const int x = q / W, c = q - x * W;
    const int col = c0 + c;
    const double val = col < nv ? f[(size_t)x * nv + col] : 0.0;
    sd[2 * ((c >> 1) * LD + sp<double>(x)) + (c & 1)] = val;
  }
  __syncthreads();
  const int g = threadIdx.x / G, t = threadIdx.x - g * G;
  cx<double>* sg = s + (size_t)g * LD;
  block_fft<double, NX, false>(sg, t, tw);
  const int ca_col = c0 + 2 * g, cb_col = ca_col + 1;
  const double vva = ca_col < nv ? v[ca_col] : 0.0;
  const double vvb = cb_col < nv ? v[cb_col] : 0.0;
  // theta = ((-kx) * dt) * v, the imaginary part of (-1j * kx * dt * v)
  two_real_rotate<double>(sg, NX, t, G, [&](int m, double& ca, double& sa, double& cb, double& sb) {
    const double ph = -kx[m] * dt;
    sincos(ph * vva, &sa, &ca);
    sincos(ph * vvb, &sb, &cb);
  });
  __syncthreads();
  block_fft<double, NX, true>(sg, t, tw);
  const double sc = 1.0 / NX;
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    const int x = q / W, c = q - x * W;
    const int col = c0 + c;
    if (col < nv) f[(size_t)x * nv + col] = sd[2 * ((c >> 1) * LD + sp<double>(x)) + (c & 1)] * sc;
  }
}

namespace {

template <int N>
cudaError_t edfdv_n(const vg_plan& p, double* f, const double* e, double dt, cudaStream_t s) {
  constexpr int G = fft_threads<double>(N);
  const int P = row_block<double>(N) / G;
  const int pairs = (p.nx + 1) / 2;
  const int blocks = div_up(pairs, P);
  const size_t smem = (size_t)P * sp_len<double>(N) * sizeof(cx<double>);
  cudaError_t err = ensure_smem((const void*)k_edfdv_f64<N>, smem);
  if (err != cudaSuccess) return err;
  k_edfdv_f64<N><<<blocks, P * G, smem, s>>>(f, p.nx, e, p.kv, dt, p.tw64);
  return cudaGetLastError();
}

template <int NX>
cudaError_t vdfdx_n(const vg_plan& p, double* f, double dt, cudaStream_t s) {
  constexpr int G = fft_threads<double>(NX);
  int S = col_seqs<double>(NX);
  if (2 * S > p.nv) S = p.nv / 2;
  const int W = 2 * S;
  const size_t smem = (size_t)S * (sp_len<double>(NX) + COL_PAD) * sizeof(cx<double>);
  cudaError_t err = ensure_smem((const void*)k_vdfdx_f64<NX>, smem);
  if (err != cudaSuccess) return err;
  k_vdfdx_f64<NX><<<div_up(p.nv, W), S * G, smem, s>>>(f, p.nv, W, p.kx, p.v, dt, p.tw64);
  return cudaGetLastError();
}

}  // namespace

#define VG_POW2_CASES(M, ...) \
  M(1, __VA_ARGS__) M(2, __VA_ARGS__) M(3, __VA_ARGS__) M(4, __VA_ARGS__) M(5, __VA_ARGS__) \
  M(6, __VA_ARGS__) M(7, __VA_ARGS__) M(8, __VA_ARGS__) M(9, __VA_ARGS__) M(10, __VA_ARGS__) \
  M(11, __VA_ARGS__) M(12, __VA_ARGS__) M(13, __VA_ARGS__)

cudaError_t launch_edfdv_f64(const vg_plan& p, double* f, const double* e, double dt, cudaStream_t s) {
  switch (ilog2(p.nv)) {
#define CASE(L, ...) case L: return edfdv_n<(1 << L)>(p, f, e, dt, s);
    VG_POW2_CASES(CASE, 0)
#undef CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_vdfdx_f64(const vg_plan& p, double* f, double dt, cudaStream_t s) {
  switch (ilog2(p.nx)) {
#define CASE(L, ...) case L: return vdfdx_n<(1 << L)>(p, f, dt, s);
    VG_POW2_CASES(CASE, 0)
#undef CASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vg
