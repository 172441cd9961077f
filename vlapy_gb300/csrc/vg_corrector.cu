// Learned coarse-velocity corrector: a small 1-D convolutional network along
// v, trained on the GPU by the kernels of this file.
//
// Each x row of a coarse run (nv = 128 velocity cells) after one coarse step
// is normalised by its RMS s and fed with the cell-centred velocity as a
// second channel to four conv1d layers (kernel 5, zero padding 2, 64 channels,
// ReLU after the first three).  The output is the correction towards the
// restricted fine-grid state in units of s: g <- g + s * net(g / s, v / vmax).
//
// Every layer is an implicit GEMM on the BF16 tensor cores with FP32
// accumulation (mma.sync.m16n8k16): positions x output channels, with K =
// 5 taps x input channels, each tap a row-shifted view of one activation tile
// in shared memory.  The backward pass is a second implicit GEMM with the
// transposed, tap-flipped weights for the data gradient (ReLU mask fused) and
// a third one, reducing over positions, for the weight gradients.  Weights
// are kept in FP32 (Adam state too) and copied to BF16 for the GEMMs.
// Activations are channels-last BF16 [row][128][C].
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "vg_internal.cuh"

namespace vg {

constexpr int CP = 128;             // positions per row
constexpr int CHALO = 2;            // kernel 5
constexpr int CROWS = CP + 2 * CHALO;
constexpr int CORR_THREADS = 128;   // 4 warps, 32 positions each
constexpr int CORR_ROWS_PER_CTA = 8;
constexpr int L1_IN = 16, HID = 64, L4_OUT = 8;  // channel counts with padding

// parameter layout (FP32, PyTorch conv1d order [C_out][C_in][5] then bias)
__host__ __device__ constexpr int w_size(int cout, int cin) { return cout * cin * 5; }
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + w_size(HID, L1_IN);
constexpr int OFF_W2 = OFF_B1 + HID, OFF_B2 = OFF_W2 + w_size(HID, HID);
constexpr int OFF_W3 = OFF_B2 + HID, OFF_B3 = OFF_W3 + w_size(HID, HID);
constexpr int OFF_W4 = OFF_B3 + HID, OFF_B4 = OFF_W4 + w_size(1, HID);
constexpr int N_PARAMS = OFF_B4 + 1;

// byte offset of (row, col) in a shared tile with C bf16 channels per row;
// 16-byte chunks are XOR-swizzled with the row so that ldmatrix rows fall
// in distinct banks
template <int C>
__device__ __forceinline__ int swz(int row, int col) {
  constexpr int RB = C * 2;
  const int chunk = col >> 3;
  int sw = chunk;
  if (RB >= 128) sw = chunk ^ (row & 7);
  else if (RB == 32) sw = chunk ^ ((row >> 2) & 1);
  return row * RB + sw * 16 + (col & 7) * 2;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, uint32_t a) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, uint32_t a) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}
__device__ __forceinline__ void ldsm_x2(uint32_t& r0, uint32_t& r1, uint32_t a) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0, %1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}
__device__ __forceinline__ void mma_bf16(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// copy n bf16 channels of `rows` consecutive positions from global [p][C] into
// a swizzled tile starting at tile row r0 (16-byte vectors)
template <int C>
__device__ __forceinline__ void load_tile(unsigned char* tile, int r0, const __nv_bfloat16* __restrict__ src,
                                          int rows) {
  constexpr int VPR = C / 8;  // 16-byte vectors per row
  for (int q = threadIdx.x; q < rows * VPR; q += blockDim.x) {
    const int r = q / VPR, v = q - r * VPR;
    const uint4 val = reinterpret_cast<const uint4*>(src + (size_t)r * C)[v];
    *reinterpret_cast<uint4*>(tile + swz<C>(r0 + r, v * 8)) = val;
  }
}
template <int C>
__device__ __forceinline__ void zero_rows(unsigned char* tile, int r0, int rows) {
  constexpr int VPR = C / 8;
  for (int q = threadIdx.x; q < rows * VPR; q += blockDim.x) {
    const int r = q / VPR, v = q - r * VPR;
    *reinterpret_cast<uint4*>(tile + swz<C>(r0 + r, v * 8)) = make_uint4(0, 0, 0, 0);
  }
}

// MODE 0: out = relu(conv + b) (bf16); MODE 1: out[p] = conv + b, channel 0
// only (fp32); MODE 2: out = conv * (mask > 0) (bf16, no bias).
// Weights W: bf16 [5][COUT][CIN] (for MODE 2: transposed, tap-flipped).
template <int CIN, int COUT, int MODE>
__global__ void __launch_bounds__(CORR_THREADS) k_conv(const __nv_bfloat16* __restrict__ x,
                                                      const __nv_bfloat16* __restrict__ w,
                                                      const float* __restrict__ bias,
                                                      const __nv_bfloat16* __restrict__ mask, void* out,
                                                      int rows) {
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* wt = smem;                                  // [5 * COUT][CIN]
  unsigned char* xt = smem + (size_t)5 * COUT * CIN * 2;     // [CROWS][CIN]
  // weights once per CTA
  {
    constexpr int VPR = CIN / 8;
    for (int q = threadIdx.x; q < 5 * COUT * VPR; q += blockDim.x) {
      const int r = q / VPR, v = q - r * VPR;
      *reinterpret_cast<uint4*>(wt + swz<CIN>(r, v * 8)) = reinterpret_cast<const uint4*>(w + (size_t)r * CIN)[v];
    }
  }
  zero_rows<CIN>(xt, 0, CHALO);
  zero_rows<CIN>(xt, CHALO + CP, CHALO);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tig = lane & 3;
  constexpr int NT = COUT / 8;
  const int row0 = blockIdx.x * CORR_ROWS_PER_CTA;
  for (int rr = 0; rr < CORR_ROWS_PER_CTA; ++rr) {
    const int row = row0 + rr;
    if (row >= rows) break;
    __syncthreads();
    load_tile<CIN>(xt, CHALO, x + (size_t)row * CP * CIN, CP);
    __syncthreads();
    float acc[2][NT][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[mt][nt][q] = 0.f;
#pragma unroll
    for (int t = 0; t < 5; ++t) {
#pragma unroll
      for (int kc = 0; kc < CIN / 16; ++kc) {
        uint32_t a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          const int p0 = warp * 32 + mt * 16;
          // A row r (position p0 + r) reads tile row p0 + r + t (tap shift)
          const int trow = p0 + (lane & 15) + t;
          const int tcol = kc * 16 + (lane >> 4) * 8;
          ldsm_x4(a[mt][0], a[mt][1], a[mt][2], a[mt][3], smem_u32(xt + swz<CIN>(trow, tcol)));
        }
        if (NT == 1) {
          uint32_t b0, b1;
          const int l = lane & 15;
          const int wrow = t * COUT + (l & 7);
          const int wcol = kc * 16 + (l >> 3) * 8;
          ldsm_x2(b0, b1, smem_u32(wt + swz<CIN>(wrow, wcol)));
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) mma_bf16(acc[mt][0], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b0, b1);
        } else {
#pragma unroll
          for (int np = 0; np < NT / 2; ++np) {
            uint32_t b0, b1, b2, b3;
            const int m = lane >> 3, i = lane & 7;
            const int wrow = t * COUT + np * 16 + i + (m >> 1) * 8;
            const int wcol = kc * 16 + (m & 1) * 8;
            ldsm_x4(b0, b1, b2, b3, smem_u32(wt + swz<CIN>(wrow, wcol)));
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
              mma_bf16(acc[mt][2 * np], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b0, b1);
              mma_bf16(acc[mt][2 * np + 1], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b2, b3);
            }
          }
        }
      }
    }
    // epilogue
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int p = warp * 32 + mt * 16 + g + half * 8;
        const size_t base = ((size_t)row * CP + p);
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
          const int o = nt * 8 + 2 * tig;
          float v0 = acc[mt][nt][2 * half], v1 = acc[mt][nt][2 * half + 1];
          if (MODE == 1) {
            if (nt == 0 && tig == 0) static_cast<float*>(out)[base] = v0 + bias[0];
          } else {
            if (MODE == 0) {
              v0 = fmaxf(v0 + bias[o], 0.f);
              v1 = fmaxf(v1 + bias[o + 1], 0.f);
            } else {
              const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(mask + base * COUT + o);
              if (!(__bfloat162float(mk.x) > 0.f)) v0 = 0.f;
              if (!(__bfloat162float(mk.y) > 0.f)) v1 = 0.f;
            }
            *reinterpret_cast<__nv_bfloat162*>(static_cast<__nv_bfloat16*>(out) + base * COUT + o) =
                __floats2bfloat162_rn(v0, v1);
          }
        }
      }
    }
  }
}

// Weight gradients of one tap t (grid.y) over a chunk of rows (grid.x):
// part[chunk][t][o][c] = sum_rows sum_p dy[row][p][o] * x[row][p + t - 2][c].
// dy has COUTP >= 16 channels (zero beyond the layer's real outputs).  The
// centre-tap CTAs also sum dy over positions for the bias gradient:
// bpart[chunk][o].
template <int CIN, int COUTP>
__global__ void __launch_bounds__(CORR_THREADS) k_wgrad(const __nv_bfloat16* __restrict__ x,
                                                       const __nv_bfloat16* __restrict__ dy, int rows,
                                                       int rows_per_chunk, float* __restrict__ part,
                                                       float* __restrict__ bpart) {
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* yt = smem;                               // [CP][COUTP]
  unsigned char* xt = smem + (size_t)CP * COUTP * 2;      // [CROWS][CIN]
  const int t = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tig = lane & 3;
  constexpr int NT = CIN / 8;
  const bool active = warp * 16 < COUTP;
  float acc[NT][4];
#pragma unroll
  for (int nt = 0; nt < NT; ++nt)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
  zero_rows<CIN>(xt, 0, CHALO);
  zero_rows<CIN>(xt, CHALO + CP, CHALO);
  const int r_begin = blockIdx.x * rows_per_chunk;
  const int r_end = min(rows, r_begin + rows_per_chunk);
  const bool bias_sum = (t == 2) && (int)threadIdx.x < COUTP;
  float bsum = 0.f;
  for (int row = r_begin; row < r_end; ++row) {
    __syncthreads();
    load_tile<COUTP>(yt, 0, dy + (size_t)row * CP * COUTP, CP);
    load_tile<CIN>(xt, CHALO, x + (size_t)row * CP * CIN, CP);
    __syncthreads();
    if (bias_sum) {
      float rs = 0.f;
      for (int p = 0; p < CP; ++p)
        rs += __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(yt + swz<COUTP>(p, threadIdx.x)));
      bsum += rs;
    }
    if (active) {
#pragma unroll 2
      for (int ks = 0; ks < CP / 16; ++ks) {
        const int p0 = ks * 16;
        uint32_t a0, a1, a2, a3;
        {
          const int m = lane >> 3, i = lane & 7;
          const int yrow = p0 + i + (m >> 1) * 8;
          const int ycol = warp * 16 + (m & 1) * 8;
          ldsm_x4_t(a0, a1, a2, a3, smem_u32(yt + swz<COUTP>(yrow, ycol)));
        }
#pragma unroll
        for (int np = 0; np < NT / 2; ++np) {
          uint32_t b0, b1, b2, b3;
          const int m = lane >> 3, i = lane & 7;
          const int xrow = p0 + t + i + (m & 1) * 8;
          const int xcol = np * 16 + (m >> 1) * 8;
          ldsm_x4_t(b0, b1, b2, b3, smem_u32(xt + swz<CIN>(xrow, xcol)));
          mma_bf16(acc[2 * np], a0, a1, a2, a3, b0, b1);
          mma_bf16(acc[2 * np + 1], a0, a1, a2, a3, b2, b3);
        }
      }
    }
  }
  if (bias_sum) bpart[(size_t)blockIdx.x * COUTP + threadIdx.x] = bsum;
  if (active) {
    float* dst = part + ((size_t)blockIdx.x * 5 + t) * COUTP * CIN;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const int o = warp * 16 + g, c = nt * 8 + 2 * tig;
      dst[(size_t)o * CIN + c] = acc[nt][0];
      dst[(size_t)o * CIN + c + 1] = acc[nt][1];
      dst[(size_t)(o + 8) * CIN + c] = acc[nt][2];
      dst[(size_t)(o + 8) * CIN + c + 1] = acc[nt][3];
    }
  }
}

// dW[o][c][t] (PyTorch order, FP32) and db[o]: sums over the chunks in a
// fixed order (deterministic)
__global__ void k_wgrad_reduce(const float* __restrict__ part, const float* __restrict__ bpart, int nchunks,
                               int coutp, int cin, int cout, float* __restrict__ dw, float* __restrict__ db) {
  const int n = cout * cin * 5;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n + cout; q += gridDim.x * blockDim.x) {
    float s = 0.f;
    if (q < n) {
      const int t = q % 5, c = (q / 5) % cin, o = q / (5 * cin);
      for (int k = 0; k < nchunks; ++k) s += part[(((size_t)k * 5 + t) * coutp + o) * cin + c];
      dw[q] = s;
    } else {
      const int o = q - n;
      for (int k = 0; k < nchunks; ++k) s += bpart[(size_t)k * coutp + o];
      db[o] = s;
    }
  }
}

// mean over each group of `group_rows` consecutive rows (the x-mean of a
// run when a group is one run's x rows), accumulated in FP64: a run's x-mean
// can exceed its x-varying part by 1e3 or more (the coarse grid's slow
// collisional drift of the background), so an FP32 mean would leave errors
// comparable to the deviations it is subtracted from.  out[group][p].
__global__ void k_group_mean(const float* __restrict__ g, int group_rows, double* __restrict__ out) {
  const int grp = blockIdx.x, p = threadIdx.x;  // blockDim = CP
  const float* src = g + (size_t)grp * group_rows * CP + p;
  double acc = 0.0;
  for (int r = 0; r < group_rows; ++r) acc += (double)src[(size_t)r * CP];
  out[(size_t)grp * CP + p] = acc / (double)group_rows;
}

// deviation of g[q] (row `row`, position p) from its group mean, rounded once
__device__ __forceinline__ float deviation(float gq, const double* __restrict__ gmean, int group_rows, int row,
                                           int p) {
  return group_rows > 0 ? (float)((double)gq - gmean[(size_t)(row / group_rows) * CP + p]) : gq;
}

// features [row][p][16]: d / s, v / vmax, the row's scalar feature (the
// collision-rate channel), d_prev / s, zeros; d = g minus its group mean
// (or g itself without groups), d_prev the same of the row before the
// coarse step (zero channel without it), s = RMS of d over the row
__global__ void k_features(const float* __restrict__ g, const double* __restrict__ gmean,
                           const float* __restrict__ gp, const double* __restrict__ pmean, int group_rows,
                           const float* __restrict__ row_feat, int rows, float vmax, __nv_bfloat16* __restrict__ x0,
                           float* __restrict__ scale) {
  __shared__ float red[CP];
  const int row = blockIdx.x;
  const int p = threadIdx.x;  // blockDim = CP
  const size_t q = (size_t)row * CP + p;
  const float val = deviation(g[q], gmean, group_rows, row, p);
  const float prev = gp ? deviation(gp[q], pmean, group_rows, row, p) : 0.f;
  red[p] = val * val;
  __syncthreads();
  for (int m = CP / 2; m > 0; m >>= 1) {
    if (p < m) red[p] += red[p + m];
    __syncthreads();
  }
  const float s = sqrtf(red[0] / CP) + 1e-30f;
  if (p == 0) scale[row] = s;
  const float dv = 2.f * vmax / CP;
  const float v = __fadd_rn(-vmax, __fmul_rn(dv, (float)p + 0.5f));
  __nv_bfloat16* dst = x0 + q * L1_IN;
  dst[0] = __float2bfloat16(val / s);
  dst[1] = __float2bfloat16(v / vmax);
  dst[2] = __float2bfloat16(row_feat ? row_feat[row] : 0.f);
  dst[3] = __float2bfloat16(prev / s);
#pragma unroll
  for (int c = 4; c < L1_IN; ++c) dst[c] = __float2bfloat16(0.f);
}

// Orthogonal projection of one row (one value per thread, blockDim = CP)
// onto the complement of the v-Fourier modes |m| < M of the 128-point row:
// v - sum_q <v, b_q> b_q over the orthonormal basis b_q (1, cos, sin of
// 2 pi m j / 128 for 0 < m < M).  basis [nq][CP], basis_t [CP][nq_pad].
// All threads of the CTA must call it; sh and coef are [CP] shared arrays.
__device__ __forceinline__ float high_pass(float v, const float* __restrict__ basis,
                                           const float* __restrict__ basis_t, int nq, float* sh, float* coef) {
  const int p = threadIdx.x;
  if (nq == 0) return v;
  sh[p] = v;
  __syncthreads();
  if (p < nq) {
    float a = 0.f;
    for (int j = 0; j < CP; ++j) a = fmaf(sh[j], basis_t[j * CP + p], a);
    coef[p] = a;
  }
  __syncthreads();
  float r = v;
  for (int q = 0; q < nq; ++q) r = fmaf(-coef[q], basis[q * CP + p], r);
  __syncthreads();
  return r;
}

// loss = mean((P (pred - want))^2) over rows x positions, P the projection
// onto the corrected modes (|m| >= M) and want = ((target - tmean) - (g -
// gmean)) / (s tau) the correction in units of the row RMS s times a global
// scale tau (means only with groups); dy4 channel 0 = d loss / d pred =
// 2 P (pred - want) / n.  One row at a time per CTA, blockDim = CP.
__global__ void k_loss(const float* __restrict__ pred, const float* __restrict__ g, const float* __restrict__ target,
                       const double* __restrict__ gmean, const double* __restrict__ tmean, int group_rows,
                       const float* __restrict__ scale, float tau, const float* __restrict__ basis,
                       const float* __restrict__ basis_t, int nq, int rows, __nv_bfloat16* __restrict__ dy4,
                       float* __restrict__ loss_part) {
  __shared__ float sh[CP], coef[CP];
  const int p = threadIdx.x;
  const float inv_n = 1.f / ((float)rows * CP);
  float acc = 0.f;
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const size_t q = (size_t)row * CP + p;
    const float diff = deviation(target[q], tmean, group_rows, row, p) - deviation(g[q], gmean, group_rows, row, p);
    const float want = diff / (scale[row] * tau);
    const float d = high_pass(pred[q] - want, basis, basis_t, nq, sh, coef);
    acc += d * d;
    __nv_bfloat16* dst = dy4 + q * 16;
    dst[0] = __float2bfloat16(2.f * d * inv_n);
#pragma unroll
    for (int c = 1; c < 16; ++c) dst[c] = __float2bfloat16(0.f);
  }
  sh[p] = acc;
  __syncthreads();
  for (int m = CP / 2; m > 0; m >>= 1) {
    if (p < m) sh[p] += sh[p + m];
    __syncthreads();
  }
  if (p == 0) loss_part[blockIdx.x] = sh[0];
}

// g_out = m + P'd + (Pd + c) * min(1, |Pd| / |Pd + c|) per row, with m the
// group mean (0 without groups), d = g - m, P the projection onto the
// corrected modes |m| >= M, P' = 1 - P, and c = P(s tau pred) the network's
// correction: the low modes, which carry the density and the field, are
// never touched, and the corrected high part is never longer in L2 norm
// than the coarse step left it, so repeated corrections cannot feed energy
// into a run.  blockDim = CP, one row per CTA.
__global__ void k_apply(const float* __restrict__ g, const double* __restrict__ gmean, int group_rows,
                        const float* __restrict__ pred, const float* __restrict__ scale, float tau,
                        const float* __restrict__ basis, const float* __restrict__ basis_t, int nq,
                        float* __restrict__ out) {
  __shared__ float r_old[CP], r_new[CP];
  const int row = blockIdx.x, p = threadIdx.x;
  const size_t q = (size_t)row * CP + p;
  const float d = deviation(g[q], gmean, group_rows, row, p);
  const float dh = high_pass(d, basis, basis_t, nq, r_old, r_new);
  const float c = high_pass((scale[row] * tau) * pred[q], basis, basis_t, nq, r_old, r_new);
  const float hn = dh + c;
  r_old[p] = dh * dh;
  r_new[p] = hn * hn;
  __syncthreads();
  for (int k = CP / 2; k > 0; k >>= 1) {
    if (p < k) {
      r_old[p] += r_old[p + k];
      r_new[p] += r_new[p + k];
    }
    __syncthreads();
  }
  const float factor = r_new[0] > r_old[0] ? sqrtf(r_old[0] / r_new[0]) : 1.f;
  const float dn = (d - dh) + hn * factor;
  // g - d is the group mean rounded to FP32 next to g; adding the corrected
  // deviation in FP64 keeps the x-varying part exact to FP32
  out[q] = group_rows > 0 ? (float)(gmean[(size_t)(row / group_rows) * CP + p] + (double)dn) : dn;
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ grad, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const float gq = grad[q];
    const float mq = b1 * m[q] + (1.f - b1) * gq;
    const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
    m[q] = mq;
    v[q] = vq;
    w[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + eps);
  }
}

// BF16 GEMM operands of one layer from its FP32 [cout][cin][5] weights:
// fwd[t][o][c] with frows >= cout rows (zero beyond cout) and, for the data
// gradient, bwd[t][c][o] = W[o][c][4 - t] with bcols >= cout columns
__global__ void k_pack(const float* __restrict__ w, int cout, int cin, int frows, int bcols,
                       __nv_bfloat16* __restrict__ fwd, __nv_bfloat16* __restrict__ bwd) {
  const int P = frows > bcols ? frows : bcols;
  const int n = 5 * P * cin;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int c = q % cin, o = (q / cin) % P, t = q / (cin * P);
    const float val = o < cout ? w[((size_t)o * cin + c) * 5 + t] : 0.f;
    if (fwd && o < frows) fwd[((size_t)t * frows + o) * cin + c] = __float2bfloat16(val);
    if (bwd && o < bcols) bwd[((size_t)(4 - t) * cin + c) * bcols + o] = __float2bfloat16(val);
  }
}

}  // namespace vg

using namespace vg;

struct vg_corrector {
  int max_rows;
  int wg_chunks;   // row chunks of the weight-gradient pass
  float* params;   // FP32 master [N_PARAMS], PyTorch conv1d order
  float* grads;
  float* adam_m;
  float* adam_v;
  long long step;
  // BF16 GEMM operands
  __nv_bfloat16 *w1f, *w2f, *w3f, *w4f;  // fwd [5][rows][cin]
  __nv_bfloat16 *w2b, *w3b, *w4b;        // bwd [5][cin][cols]
  // activations and gradients, channels-last [rows][128][C]
  __nv_bfloat16 *x0, *a1, *a2, *a3, *dy4, *d3, *d2, *d1;
  float *pred, *scale, *part, *bpart, *loss_part;
  double *gmean, *tmean, *pmean;  // group means [groups][128]
  float vmax, tau;
  int protect_modes;      // M: the modes |m| < M are never corrected
  int nq;                 // 2M - 1 basis functions (0 when M = 0)
  float *basis, *basis_t; // [nq][128], [128][128] (transposed, padded)
  std::vector<void*> owned;
};

namespace {

#define CR_CHECK(expr)            \
  do {                            \
    int _st = (expr);             \
    if (_st != VG_OK) return _st; \
  } while (0)

template <typename T>
int cr_alloc(vg_corrector* c, T** p, size_t n, const char* what) {
  cudaError_t err = cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(n, 1) * sizeof(T));
  if (err != cudaSuccess) return cuda_status(err, what);
  c->owned.push_back(*p);
  return cuda_status(cudaMemset(*p, 0, std::max<size_t>(n, 1) * sizeof(T)), what);
}

constexpr int WGRAD_MAX_CHUNKS = 296;  // 2 x 152 SMs of row chunks, x 5 taps
constexpr int LOSS_BLOCKS = 1024;

int wgrad_chunks(int rows) { return std::min(div_up(rows, 16), WGRAD_MAX_CHUNKS); }

template <int CIN, int COUT, int MODE>
cudaError_t conv(const __nv_bfloat16* x, const __nv_bfloat16* w, const float* b, const __nv_bfloat16* mask, void* out,
                 int rows, cudaStream_t s) {
  const size_t smem = (size_t)5 * COUT * CIN * 2 + (size_t)CROWS * CIN * 2;
  cudaError_t err = ensure_smem((const void*)k_conv<CIN, COUT, MODE>, smem);
  if (err != cudaSuccess) return err;
  k_conv<CIN, COUT, MODE><<<div_up(rows, CORR_ROWS_PER_CTA), CORR_THREADS, smem, s>>>(x, w, b, mask, out, rows);
  return cudaGetLastError();
}

template <int CIN, int COUTP>
cudaError_t wgrad(vg_corrector* c, const __nv_bfloat16* x, const __nv_bfloat16* dy, int rows, int cout, float* dw,
                  float* db, cudaStream_t s) {
  const int chunks = wgrad_chunks(rows);
  const int per = div_up(rows, chunks);
  const size_t smem = (size_t)CP * COUTP * 2 + (size_t)CROWS * CIN * 2;
  cudaError_t err = ensure_smem((const void*)k_wgrad<CIN, COUTP>, smem);
  if (err != cudaSuccess) return err;
  k_wgrad<CIN, COUTP><<<dim3(chunks, 5), CORR_THREADS, smem, s>>>(x, dy, rows, per, c->part, c->bpart);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  k_wgrad_reduce<<<div_up(cout * CIN * 5 + cout, 256), 256, 0, s>>>(c->part, c->bpart, chunks, COUTP, CIN, cout, dw,
                                                                   db);
  return cudaGetLastError();
}

int pack_all(vg_corrector* c, cudaStream_t s) {
  struct L {
    int off, cout, cin, frows, bcols;
    __nv_bfloat16 *f, *b;
  } ls[4] = {{OFF_W1, HID, L1_IN, HID, 0, c->w1f, nullptr},
             {OFF_W2, HID, HID, HID, HID, c->w2f, c->w2b},
             {OFF_W3, HID, HID, HID, HID, c->w3f, c->w3b},
             {OFF_W4, 1, HID, L4_OUT, 16, c->w4f, c->w4b}};
  for (auto& l : ls) {
    const int P = l.frows > l.bcols ? l.frows : l.bcols;
    k_pack<<<div_up(5 * P * l.cin, 256), 256, 0, s>>>(c->params + l.off, l.cout, l.cin, l.frows, l.bcols, l.f, l.b);
    CR_CHECK(cuda_status(cudaGetLastError(), "corrector pack"));
  }
  return VG_OK;
}

// pred = net(features(batch)) for the batch's rows (FP32 [rows][128])
int forward(vg_corrector* c, const vg_corr_batch& b, cudaStream_t s) {
  const int rows = b.rows, group_rows = b.group_rows;
  if (group_rows > 0) {
    k_group_mean<<<rows / group_rows, CP, 0, s>>>(b.g, group_rows, c->gmean);
    CR_CHECK(cuda_status(cudaGetLastError(), "corrector group mean"));
    if (b.g_prev) {
      k_group_mean<<<rows / group_rows, CP, 0, s>>>(b.g_prev, group_rows, c->pmean);
      CR_CHECK(cuda_status(cudaGetLastError(), "corrector group mean"));
    }
  }
  k_features<<<rows, CP, 0, s>>>(b.g, c->gmean, b.g_prev, c->pmean, group_rows, b.row_feat, rows, c->vmax, c->x0,
                                 c->scale);
  CR_CHECK(cuda_status(cudaGetLastError(), "corrector features"));
  CR_CHECK(cuda_status(conv<L1_IN, HID, 0>(c->x0, c->w1f, c->params + OFF_B1, nullptr, c->a1, rows, s), "conv1"));
  CR_CHECK(cuda_status(conv<HID, HID, 0>(c->a1, c->w2f, c->params + OFF_B2, nullptr, c->a2, rows, s), "conv2"));
  CR_CHECK(cuda_status(conv<HID, HID, 0>(c->a2, c->w3f, c->params + OFF_B3, nullptr, c->a3, rows, s), "conv3"));
  CR_CHECK(cuda_status(conv<HID, L4_OUT, 1>(c->a3, c->w4f, c->params + OFF_B4, nullptr, c->pred, rows, s), "conv4"));
  return VG_OK;
}

int loss(vg_corrector* c, const vg_corr_batch& b, cudaStream_t s) {
  if (b.group_rows > 0) {
    k_group_mean<<<b.rows / b.group_rows, CP, 0, s>>>(b.target, b.group_rows, c->tmean);
    CR_CHECK(cuda_status(cudaGetLastError(), "corrector group mean"));
  }
  k_loss<<<LOSS_BLOCKS, CP, 0, s>>>(c->pred, b.g, b.target, c->gmean, c->tmean, b.group_rows, c->scale, c->tau,
                                    c->basis, c->basis_t, c->nq, b.rows, c->dy4, c->loss_part);
  return cuda_status(cudaGetLastError(), "corrector loss");
}

int read_loss(vg_corrector* c, int rows, double* loss_out, cudaStream_t s) {
  if (!loss_out) return VG_OK;
  float lp[LOSS_BLOCKS];
  CR_CHECK(cuda_status(cudaMemcpyAsync(lp, c->loss_part, sizeof(lp), cudaMemcpyDeviceToHost, s), "corrector loss"));
  CR_CHECK(cuda_status(cudaStreamSynchronize(s), "corrector loss"));
  double t = 0.0;
  for (float x : lp) t += x;
  *loss_out = t / ((double)rows * CP);
  return VG_OK;
}

// gradients of the loss into c->grads (after forward and loss)
int backward(vg_corrector* c, int rows, cudaStream_t s) {
  float* G = c->grads;
  CR_CHECK(cuda_status(wgrad<HID, 16>(c, c->a3, c->dy4, rows, 1, G + OFF_W4, G + OFF_B4, s), "wgrad4"));
  CR_CHECK(cuda_status(conv<16, HID, 2>(c->dy4, c->w4b, nullptr, c->a3, c->d3, rows, s), "dgrad4"));
  CR_CHECK(cuda_status(wgrad<HID, HID>(c, c->a2, c->d3, rows, HID, G + OFF_W3, G + OFF_B3, s), "wgrad3"));
  CR_CHECK(cuda_status(conv<HID, HID, 2>(c->d3, c->w3b, nullptr, c->a2, c->d2, rows, s), "dgrad3"));
  CR_CHECK(cuda_status(wgrad<HID, HID>(c, c->a1, c->d2, rows, HID, G + OFF_W2, G + OFF_B2, s), "wgrad2"));
  CR_CHECK(cuda_status(conv<HID, HID, 2>(c->d2, c->w2b, nullptr, c->a1, c->d1, rows, s), "dgrad2"));
  CR_CHECK(cuda_status(wgrad<L1_IN, HID>(c, c->x0, c->d1, rows, HID, G + OFF_W1, G + OFF_B1, s), "wgrad1"));
  return VG_OK;
}

int check_batch(const vg_corrector* c, const vg_corr_batch* b, bool need_target) {
  if (!c || !b || !b->g) {
    set_error("corrector: null corrector, batch or state");
    return VG_ERR_ARG;
  }
  if (b->rows <= 0 || b->rows > c->max_rows) {
    set_error("corrector: rows must be in [1, max_rows]");
    return VG_ERR_ARG;
  }
  if (b->group_rows < 0 || (b->group_rows > 0 && b->rows % b->group_rows != 0)) {
    set_error("corrector: group_rows must be 0 or divide rows");
    return VG_ERR_ARG;
  }
  if (need_target && !b->target) {
    set_error("corrector: this call needs a target");
    return VG_ERR_ARG;
  }
  return VG_OK;
}

}  // namespace

extern "C" {

int vg_corr_num_params(void) { return N_PARAMS; }

int vg_corr_create(int32_t max_rows, int32_t protect_modes, float vmax, float tau, const float* params_host,
                   vg_corrector** out) {
  if (!out || max_rows <= 0 || !params_host || protect_modes < 0 || protect_modes > CP / 2 || !(vmax > 0.f) ||
      !(tau > 0.f)) {
    set_error("corrector: bad arguments (max_rows > 0, 0 <= protect_modes <= 64, vmax > 0, tau > 0, parameters)");
    return VG_ERR_ARG;
  }
  *out = nullptr;
  vg_corrector* c = new vg_corrector();
  c->max_rows = max_rows;
  c->vmax = vmax;
  c->tau = tau;
  c->protect_modes = protect_modes;
  c->nq = protect_modes > 0 ? 2 * protect_modes - 1 : 0;
  c->step = 0;
  c->wg_chunks = wgrad_chunks(max_rows);
  const size_t pos = (size_t)max_rows * CP;
  int st = VG_OK;
#define CR_TRY(expr)                        \
  do {                                      \
    st = (expr);                            \
    if (st != VG_OK) {                      \
      for (void* p : c->owned) cudaFree(p); \
      delete c;                             \
      return st;                            \
    }                                       \
  } while (0)
  CR_TRY(cr_alloc(c, &c->params, N_PARAMS, "corrector params"));
  CR_TRY(cr_alloc(c, &c->grads, N_PARAMS, "corrector params"));
  CR_TRY(cr_alloc(c, &c->adam_m, N_PARAMS, "corrector params"));
  CR_TRY(cr_alloc(c, &c->adam_v, N_PARAMS, "corrector params"));
  CR_TRY(cr_alloc(c, &c->w1f, (size_t)5 * HID * L1_IN, "corrector weights"));
  CR_TRY(cr_alloc(c, &c->w2f, (size_t)5 * HID * HID, "corrector weights"));
  CR_TRY(cr_alloc(c, &c->w3f, (size_t)5 * HID * HID, "corrector weights"));
  CR_TRY(cr_alloc(c, &c->w4f, (size_t)5 * L4_OUT * HID, "corrector weights"));
  CR_TRY(cr_alloc(c, &c->w2b, (size_t)5 * HID * HID, "corrector weights"));
  CR_TRY(cr_alloc(c, &c->w3b, (size_t)5 * HID * HID, "corrector weights"));
  CR_TRY(cr_alloc(c, &c->w4b, (size_t)5 * HID * 16, "corrector weights"));
  CR_TRY(cr_alloc(c, &c->x0, pos * L1_IN, "corrector activations"));
  CR_TRY(cr_alloc(c, &c->a1, pos * HID, "corrector activations"));
  CR_TRY(cr_alloc(c, &c->a2, pos * HID, "corrector activations"));
  CR_TRY(cr_alloc(c, &c->a3, pos * HID, "corrector activations"));
  CR_TRY(cr_alloc(c, &c->dy4, pos * 16, "corrector gradients"));
  CR_TRY(cr_alloc(c, &c->d3, pos * HID, "corrector gradients"));
  CR_TRY(cr_alloc(c, &c->d2, pos * HID, "corrector gradients"));
  CR_TRY(cr_alloc(c, &c->d1, pos * HID, "corrector gradients"));
  CR_TRY(cr_alloc(c, &c->pred, pos, "corrector output"));
  CR_TRY(cr_alloc(c, &c->scale, (size_t)max_rows, "corrector output"));
  CR_TRY(cr_alloc(c, &c->part, (size_t)c->wg_chunks * 5 * HID * HID, "corrector partials"));
  CR_TRY(cr_alloc(c, &c->bpart, (size_t)c->wg_chunks * HID, "corrector partials"));
  CR_TRY(cr_alloc(c, &c->loss_part, LOSS_BLOCKS, "corrector loss"));
  CR_TRY(cr_alloc(c, &c->gmean, pos, "corrector group means"));
  CR_TRY(cr_alloc(c, &c->tmean, pos, "corrector group means"));
  CR_TRY(cr_alloc(c, &c->pmean, pos, "corrector group means"));
  {
    // orthonormal basis of the protected modes on the 128-point row
    std::vector<float> b((size_t)std::max(c->nq, 1) * CP, 0.f), bt((size_t)CP * CP, 0.f);
    const double pi = 3.14159265358979323846;
    for (int qq = 0; qq < c->nq; ++qq) {
      const int m = (qq + 1) / 2;
      for (int j = 0; j < CP; ++j) {
        double val;
        if (qq == 0) val = 1.0 / std::sqrt((double)CP);
        else if (qq & 1) val = std::cos(2.0 * pi * m * j / CP) * std::sqrt(2.0 / CP);
        else val = std::sin(2.0 * pi * m * j / CP) * std::sqrt(2.0 / CP);
        b[(size_t)qq * CP + j] = (float)val;
        bt[(size_t)j * CP + qq] = (float)val;
      }
    }
    CR_TRY(cr_alloc(c, &c->basis, b.size(), "corrector basis"));
    CR_TRY(cr_alloc(c, &c->basis_t, bt.size(), "corrector basis"));
    CR_TRY(cuda_status(cudaMemcpy(c->basis, b.data(), b.size() * sizeof(float), cudaMemcpyHostToDevice),
                       "corrector basis"));
    CR_TRY(cuda_status(cudaMemcpy(c->basis_t, bt.data(), bt.size() * sizeof(float), cudaMemcpyHostToDevice),
                       "corrector basis"));
  }
  CR_TRY(cuda_status(cudaMemcpy(c->params, params_host, N_PARAMS * sizeof(float), cudaMemcpyHostToDevice),
                     "corrector params"));
  CR_TRY(pack_all(c, 0));
  CR_TRY(cuda_status(cudaDeviceSynchronize(), "corrector setup"));
#undef CR_TRY
  *out = c;
  return VG_OK;
}

int vg_corr_destroy(vg_corrector* c) {
  if (!c) return VG_OK;
  cudaDeviceSynchronize();
  for (void* p : c->owned) cudaFree(p);
  delete c;
  return VG_OK;
}

int vg_corr_get_params(vg_corrector* c, float* host_out) {
  if (!c || !host_out) {
    set_error("corrector: null argument");
    return VG_ERR_ARG;
  }
  return cuda_status(cudaMemcpy(host_out, c->params, N_PARAMS * sizeof(float), cudaMemcpyDeviceToHost),
                     "corrector get params");
}

int vg_corr_set_params(vg_corrector* c, const float* host_in) {
  if (!c || !host_in) {
    set_error("corrector: null argument");
    return VG_ERR_ARG;
  }
  CR_CHECK(cuda_status(cudaMemcpy(c->params, host_in, N_PARAMS * sizeof(float), cudaMemcpyHostToDevice),
                       "corrector set params"));
  c->step = 0;
  CR_CHECK(cuda_status(cudaMemset(c->adam_m, 0, N_PARAMS * sizeof(float)), "corrector set params"));
  CR_CHECK(cuda_status(cudaMemset(c->adam_v, 0, N_PARAMS * sizeof(float)), "corrector set params"));
  CR_CHECK(pack_all(c, 0));
  return cuda_status(cudaDeviceSynchronize(), "corrector set params");
}

int vg_corr_set_tau(vg_corrector* c, float tau) {
  if (!c || !(tau > 0.f)) {
    set_error("corrector: tau must be positive");
    return VG_ERR_ARG;
  }
  c->tau = tau;
  return VG_OK;
}

int vg_corr_apply(vg_corrector* c, const vg_corr_batch* b, float* g_out, vg_stream stream) {
  CR_CHECK(check_batch(c, b, false));
  if (!g_out) {
    set_error("corrector: null output");
    return VG_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  CR_CHECK(forward(c, *b, s));
  k_apply<<<b->rows, CP, 0, s>>>(b->g, c->gmean, b->group_rows, c->pred, c->scale, c->tau, c->basis, c->basis_t,
                                 c->nq, g_out);
  return cuda_status(cudaGetLastError(), "corrector apply");
}

int vg_corr_loss(vg_corrector* c, const vg_corr_batch* b, double* loss_out, vg_stream stream) {
  CR_CHECK(check_batch(c, b, true));
  if (!loss_out) {
    set_error("corrector: null loss");
    return VG_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  CR_CHECK(forward(c, *b, s));
  CR_CHECK(loss(c, *b, s));
  return read_loss(c, b->rows, loss_out, s);
}

int vg_corr_gradients(vg_corrector* c, const vg_corr_batch* b, float* grad_host, double* loss_out,
                      vg_stream stream) {
  CR_CHECK(check_batch(c, b, true));
  cudaStream_t s = (cudaStream_t)stream;
  CR_CHECK(forward(c, *b, s));
  CR_CHECK(loss(c, *b, s));
  CR_CHECK(backward(c, b->rows, s));
  if (grad_host)
    CR_CHECK(cuda_status(cudaMemcpyAsync(grad_host, c->grads, N_PARAMS * sizeof(float), cudaMemcpyDeviceToHost, s),
                         "corrector gradients"));
  CR_CHECK(read_loss(c, b->rows, loss_out, s));
  if (grad_host) CR_CHECK(cuda_status(cudaStreamSynchronize(s), "corrector gradients"));
  return VG_OK;
}

int vg_corr_train_step(vg_corrector* c, const vg_corr_batch* b, float lr, double* loss_out, vg_stream stream) {
  CR_CHECK(check_batch(c, b, true));
  if (!(lr > 0.f)) {
    set_error("corrector: learning rate must be positive");
    return VG_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  CR_CHECK(forward(c, *b, s));
  CR_CHECK(loss(c, *b, s));
  CR_CHECK(backward(c, b->rows, s));
  c->step += 1;
  const double b1 = 0.9, b2 = 0.999;
  const float c1 = (float)(1.0 - std::pow(b1, (double)c->step));
  const float c2 = (float)(1.0 - std::pow(b2, (double)c->step));
  k_adam<<<div_up(N_PARAMS, 256), 256, 0, s>>>(c->params, c->grads, c->adam_m, c->adam_v, N_PARAMS, lr, (float)b1,
                                               (float)b2, 1e-8f, c1, c2);
  CR_CHECK(cuda_status(cudaGetLastError(), "corrector adam"));
  CR_CHECK(pack_all(c, s));
  return read_loss(c, b->rows, loss_out, s);
}

}  // extern "C"
