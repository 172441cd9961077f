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
#include "vg_f64_body.cuh"

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

template <int NX>
__global__ void __launch_bounds__(col_seqs<double>(NX) * fft_threads<double>(NX)) k_vdfdx_f64(double* __restrict__ f, int nv, int W,
                                                    const double* __restrict__ kx,
                                                    const double* __restrict__ v, double dt,
                                                    const cx<double>* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  vdfdx_tile_body<NX>(f, nv, blockIdx.x * W, W, kx, v, dt, tw, smem_raw);
}

// Exponential advection of lines whose length N is not a power of two, by
// direct DFTs (the reference's scipy.fft transforms any length; O(N^2) work
// per line here).  Line l is the row l of f for the v step (elements
// contiguous) or the column l for the x step (elements nv apart):
//   F_k = sum_n f_n w^(n k),  w = exp(-2 pi i / N),
//   G_k = exp(i theta_k) F_k,  theta_k = ((-kw[k]) * dt) * c_l,
//   f_n <- Re (1/N) sum_k G_k w^(-n k),
// with kw = kv, c_l = e[l] (v step) or kw = kx, c_l = v[l] (x step), the
// phase the reference evaluates (vlapy/core/vlasov.py:106-108, 136-138).  One
// CTA per line; shared memory holds the line, G and the N twiddles w^q,
// q = (n k) mod N, each from sincospi(2 q / N).
__global__ void k_dft_advect_f64(double* __restrict__ f, int N, int n_lines, long long elem_stride,
                                 long long line_stride, const double* __restrict__ kw,
                                 const double* __restrict__ c, double dt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* line = reinterpret_cast<double*>(smem_raw);
  cx<double>* G = reinterpret_cast<cx<double>*>(line + N + (N & 1));
  cx<double>* W = G + N;
  const int l = blockIdx.x;
  if (l >= n_lines) return;
  double* fl = f + (long long)l * line_stride;
  for (int q = threadIdx.x; q < N; q += blockDim.x) {
    double sn, cs;
    sincospi(2.0 * (double)q / (double)N, &sn, &cs);
    W[q] = {cs, -sn};
    line[q] = fl[(long long)q * elem_stride];
  }
  __syncthreads();
  const double cl = c[l];
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    double zr = 0.0, zi = 0.0;
    int q = 0;
    for (int n = 0; n < N; ++n) {
      const cx<double> w = W[q];
      zr += line[n] * w.x;
      zi += line[n] * w.y;
      q += k;
      if (q >= N) q -= N;
    }
    double sa, ca;
    sincos(((-kw[k]) * dt) * cl, &sa, &ca);
    G[k] = {ca * zr - sa * zi, ca * zi + sa * zr};
  }
  __syncthreads();
  const double sc = 1.0 / N;
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    double acc = 0.0;
    int q = 0;
    for (int k = 0; k < N; ++k) {
      // Re(G_k conj(w^(n k)))
      const cx<double> w = W[q];
      acc += G[k].x * w.x + G[k].y * w.y;
      q += n;
      if (q >= N) q -= N;
    }
    fl[(long long)n * elem_stride] = acc * sc;
  }
}

static size_t dft_advect_smem(int n) { return ((size_t)n + (n & 1) + 4 * (size_t)n) * sizeof(double); }

namespace {

cudaError_t dft_advect(double* f, int N, int n_lines, long long elem_stride, long long line_stride,
                       const double* kw, const double* c, double dt, cudaStream_t s) {
  const size_t smem = dft_advect_smem(N);
  cudaError_t err = ensure_smem((const void*)k_dft_advect_f64, smem);
  if (err != cudaSuccess) return err;
  k_dft_advect_f64<<<n_lines, 256, smem, s>>>(f, N, n_lines, elem_stride, line_stride, kw, c, dt);
  return cudaGetLastError();
}

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
  if (!p.nv_pow2) return dft_advect(f, p.nv, p.nx, 1, p.nv, p.kv, e, dt, s);
  switch (ilog2(p.nv)) {
#define CASE(L, ...) case L: return edfdv_n<(1 << L)>(p, f, e, dt, s);
    VG_POW2_CASES(CASE, 0)
#undef CASE
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_vdfdx_f64(const vg_plan& p, double* f, double dt, cudaStream_t s) {
  if (!p.nx_pow2) return dft_advect(f, p.nx, p.nv, p.nv, 1, p.kx, p.v, dt, s);
  switch (ilog2(p.nx)) {
#define CASE(L, ...) case L: return vdfdx_n<(1 << L)>(p, f, dt, s);
    VG_POW2_CASES(CASE, 0)
#undef CASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vg
