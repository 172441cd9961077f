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
__global__ void k_group_mean(const float* __restrict__ g, int group_rows, float2* __restrict__ out) {
  const int grp = blockIdx.x, p = threadIdx.x;  // blockDim = CP
  const float* src = g + (size_t)grp * group_rows * CP + p;
  // double-float (TwoSum) accumulation: FP64-grade, on the FP32 pipes
  float hi = 0.f, lo = 0.f;
  for (int r = 0; r < group_rows; ++r) {
    const float x = src[(size_t)r * CP];
    const float t = hi + x;
    const float bb = t - hi;
    lo += (hi - (t - bb)) + (x - bb);
    hi = t;
  }
  // the mean as a double-float pair (hi, lo), so that the kernels that take
  // it out of a row stay on the FP32 pipes
  const double m = ((double)hi + (double)lo) / (double)group_rows;
  const float mh = (float)m;
  out[(size_t)grp * CP + p] = make_float2(mh, (float)(m - (double)mh));
}

// deviation of g[q] (row `row`, position p) from its group mean, rounded once
// (g - hi is exact when g is within a factor 2 of the mean, the case where
// the mean dwarfs the deviation; then one rounding for lo)
__device__ __forceinline__ float deviation(float gq, const float2* __restrict__ gmean, int group_rows, int row,
                                           int p) {
  if (group_rows <= 0) return gq;
  const float2 m = gmean[(size_t)(row / group_rows) * CP + p];
  return __fsub_rn(__fsub_rn(gq, m.x), m.y);
}
// the group mean plus a deviation, rounded once more (inverse of deviation)
__device__ __forceinline__ float with_mean(float dn, const float2* __restrict__ gmean, int group_rows, int row,
                                           int p) {
  if (group_rows <= 0) return dn;
  const float2 m = gmean[(size_t)(row / group_rows) * CP + p];
  return __fadd_rn(m.x, __fadd_rn(m.y, dn));
}

// features [row][p][16]: d / s, v / vmax, the row's scalar feature (the
// collision-rate channel), d_prev / s, zeros; d = g minus its group mean
// (or g itself without groups), d_prev the same of the row before the
// coarse step (zero channel without it), s = RMS of d over the row
__global__ void k_features(const float* __restrict__ g, const float2* __restrict__ gmean,
                           const float* __restrict__ gp, const float2* __restrict__ pmean, int group_rows,
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

// high_pass for two rows' values at once (one pass over the basis)
__device__ __forceinline__ void high_pass2(float a, float b, const float* __restrict__ basis,
                                           const float* __restrict__ basis_t, int nq, float* sh, float* coef,
                                           float& ha, float& hb) {
  const int p = threadIdx.x;
  if (nq == 0) {
    ha = a;
    hb = b;
    return;
  }
  sh[p] = a;
  sh[CP + p] = b;
  __syncthreads();
  if (p < nq) {
    float ca0 = 0.f, ca1 = 0.f, cb0 = 0.f, cb1 = 0.f;
#pragma unroll 8
    for (int j = 0; j < CP; j += 2) {
      const float w0 = basis_t[j * CP + p], w1 = basis_t[(j + 1) * CP + p];
      ca0 = fmaf(sh[j], w0, ca0);
      cb0 = fmaf(sh[CP + j], w0, cb0);
      ca1 = fmaf(sh[j + 1], w1, ca1);
      cb1 = fmaf(sh[CP + j + 1], w1, cb1);
    }
    coef[p] = ca0 + ca1;
    coef[CP + p] = cb0 + cb1;
  }
  __syncthreads();
  float ra = a, rb = b;
#pragma unroll 4
  for (int q = 0; q < nq; ++q) {
    const float w = basis[q * CP + p];
    ra = fmaf(-coef[q], w, ra);
    rb = fmaf(-coef[CP + q], w, rb);
  }
  __syncthreads();
  ha = ra;
  hb = rb;
}

// loss = mean((P (pred - want))^2) over rows x positions, P the projection
// onto the corrected modes (|m| >= M) and want = ((target - tmean) - (g -
// gmean)) / (s tau) the correction in units of the row RMS s times a global
// scale tau (means only with groups); dy4 channel 0 = d loss / d pred =
// 2 P (pred - want) / n.  One row at a time per CTA, blockDim = CP.
__global__ void k_loss(const float* __restrict__ pred, const float* __restrict__ g, const float* __restrict__ target,
                       const float2* __restrict__ gmean, const float2* __restrict__ tmean, int group_rows,
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
constexpr int APPLY_ROWS = 8;  // rows per CTA of k_apply: 4 packed pairs of d and 4 of c

// The projection P off the protected modes |m| < M of the 128-point rows, by
// FFT: two real rows packed as one complex sequence z = a + i b, FFT, the
// bins k < M and k > 128 - M set to zero (which removes those modes from a
// and b alike), inverse FFT / 128.  Each of a CTA's 8 sequences (4 pairs of
// deviations d, 4 pairs of corrections c) is transformed by its own 16
// threads.  Then the cap: m + P'd + (Pd + c') * min(1, |Pd| / |Pd + c'|),
// c' = P c, per row.
__global__ void __launch_bounds__(CP) k_apply(const float* __restrict__ g, const float2* __restrict__ gmean,
                                               int group_rows, const float* __restrict__ pred,
                                               const float* __restrict__ scale, float tau, int protect_modes,
                                               const cx<float>* __restrict__ tw, int rows, float* __restrict__ out) {
  constexpr int SL = sp_len<float>(CP) + 1;  // padded length of one sequence
  __shared__ cx<float> seq[2 * (APPLY_ROWS / 2)][SL];
  __shared__ float wsum[2][APPLY_ROWS][CP / 32];
  const int p = threadIdx.x, row0 = blockIdx.x * APPLY_ROWS;
  float d[APPLY_ROWS], c[APPLY_ROWS];
#pragma unroll
  for (int r = 0; r < APPLY_ROWS; ++r) {
    const int row = row0 + r < rows ? row0 + r : rows - 1;  // a short last block repeats its last row
    const size_t q = (size_t)row * CP + p;
    d[r] = deviation(g[q], gmean, group_rows, row, p);
    c[r] = (scale[row] * tau) * pred[q];
  }
  float dh[APPLY_ROWS], ch[APPLY_ROWS];
  if (protect_modes > 0) {
#pragma unroll
    for (int h = 0; h < APPLY_ROWS / 2; ++h) {
      seq[h][sp<float>(p)] = {d[2 * h], d[2 * h + 1]};
      seq[APPLY_ROWS / 2 + h][sp<float>(p)] = {c[2 * h], c[2 * h + 1]};
    }
    __syncthreads();
    {
      constexpr int GT = CP / 8;  // 16 threads per radix-8 sequence of 128
      const int sq = p / GT, t = p - sq * GT;
      const GroupSync gs = GroupSync::of(sq, GT);
      cx<float>* z = seq[sq];
      block_fft<float, CP, false, 8>(z, t, tw, gs);
      for (int k = t; k < CP; k += GT)
        if (k < protect_modes || k > CP - protect_modes) z[sp<float>(k)] = {0.f, 0.f};
      gs();
      block_fft<float, CP, true, 8>(z, t, tw, gs);
    }
    __syncthreads();
    const float inv = 1.f / CP;
#pragma unroll
    for (int h = 0; h < APPLY_ROWS / 2; ++h) {
      const cx<float> zd = seq[h][sp<float>(p)], zc = seq[APPLY_ROWS / 2 + h][sp<float>(p)];
      dh[2 * h] = zd.x * inv;
      dh[2 * h + 1] = zd.y * inv;
      ch[2 * h] = zc.x * inv;
      ch[2 * h + 1] = zc.y * inv;
    }
  } else {
#pragma unroll
    for (int r = 0; r < APPLY_ROWS; ++r) {
      dh[r] = d[r];
      ch[r] = c[r];
    }
  }
  // hn = Pd + Pc; row sums of (Pd)^2 and hn^2 by warp shuffles, then the warps
  float hn[APPLY_ROWS];
#pragma unroll
  for (int r = 0; r < APPLY_ROWS; ++r) {
    hn[r] = dh[r] + ch[r];
    float so = dh[r] * dh[r], sn = hn[r] * hn[r];
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
      so += __shfl_xor_sync(0xffffffffu, so, m);
      sn += __shfl_xor_sync(0xffffffffu, sn, m);
    }
    if ((p & 31) == 0) {
      wsum[0][r][p >> 5] = so;
      wsum[1][r][p >> 5] = sn;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < APPLY_ROWS; ++r) {
    const int row = row0 + r;
    if (row >= rows) break;
    const float r_old = (wsum[0][r][0] + wsum[0][r][1]) + (wsum[0][r][2] + wsum[0][r][3]);
    const float r_new = (wsum[1][r][0] + wsum[1][r][1]) + (wsum[1][r][2] + wsum[1][r][3]);
    const float factor = r_new > r_old ? sqrtf(r_old / r_new) : 1.f;
    const float dn = (d[r] - dh[r]) + hn[r] * factor;
    out[(size_t)row * CP + p] = with_mean(dn, gmean, group_rows, row, p);
  }
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


// ---------------------------------------------------------------------------
// Fused forward pass on the 5th-generation tensor cores (tcgen05).
//
// One persistent CTA per SM (128 threads, 4 warps) keeps all four layers'
// BF16 weights (100 KB) and two activation tiles in shared memory and runs
// the network row by row: features -> 4 x (tcgen05.mma into a TMEM
// accumulator of 128 lanes (positions) x N columns (channels), then an
// epilogue that reads TMEM back with tcgen05.ld, adds the bias, applies the
// ReLU and writes the next layer's BF16 tile) -> the network output and the
// row scale.  No activation touches HBM.  The projected, capped correction
// runs after it in k_apply, whose many small CTAs hide the latency of its
// per-row projections (one CTA per SM here could not).
//
// Every tile is in the K-major, non-swizzled canonical layout: element
// (row r, channel c) at (c / 8) * LBO + r * 16 + (c % 8) * 2 bytes, so that an
// 8 x 16-byte core matrix is 128 contiguous bytes, core matrices along the
// rows are 128 B apart (SBO) and along K LBO = 16 * rows apart.  A tap t of
// the convolution is then the activation tile's descriptor moved by 16 t
// bytes (rows t .. t + 127 of the 132-row tile with its 2-row halos).
// ---------------------------------------------------------------------------

// rows in flight per CTA (build-time knob: each slot is 4 warps, 64 TMEM
// columns and one 132 x 64 tile; 7 slots fit 72 registers a thread and
// 229 KB of shared memory, and apply 3 % faster than 6)
#ifndef VG_TC_SLOTS
#define VG_TC_SLOTS 7
#endif
constexpr int TC_SLOTS = VG_TC_SLOTS;
constexpr int TC_THREADS = TC_SLOTS * 128;               // 4 warps per slot
constexpr int TC_TILE_ROWS = CROWS;                      // 132
constexpr int TC_LBO_ACT = 16 * TC_TILE_ROWS;            // 2112 B
constexpr int TC_ACT_BYTES = 8 * TC_LBO_ACT;             // 64 channels
// the first layer folds its taps into K (im2col): K = 5 taps x 4 real input
// channels = 20, padded to 32, so it is 2 MMAs where 5 taps x one 16-channel
// K-step were 5; its B operand is [64 outputs][32] with k = 4 t + c
constexpr int L1_REAL = 4, TC_K1 = 32;
constexpr int TC_W1_BYTES = HID * TC_K1 * 2, TC_W2_TAP = HID * HID * 2;
// the last layer (one output channel) puts its five taps in N instead: one
// 16 x 64 B operand whose row t is tap t (rows 5..15 zero), so that the
// layer is 4 MMAs (K = 64) of M = 128, N = 16, D4[p][t] = sum_c h3[p][c] w4[t][c],
// and the epilogue adds out[p] = sum_t D4[p + t - 2][t]; at N = 16 an MMA
// costs about as much as at N = 64, so this is 4 MMAs where 5 taps x 4
// K-steps were 20
constexpr int TC_W4_BYTES = 16 * HID * 2;
constexpr int TC_W_BYTES = TC_W1_BYTES + 2 * 5 * TC_W2_TAP + TC_W4_BYTES;  // 88064
constexpr int TC_OFF_W1 = 0;
constexpr int TC_OFF_W2 = TC_OFF_W1 + TC_W1_BYTES;
constexpr int TC_OFF_W3 = TC_OFF_W2 + 5 * TC_W2_TAP;
constexpr int TC_OFF_W4 = TC_OFF_W3 + 5 * TC_W2_TAP;
// per slot one tile of 64 channels, updated in place: a layer's epilogue
// overwrites the layer's own input, which its MMAs have finished reading
// (their completion is what the epilogue waits for); the 16-channel input
// of the first layer is the tile's first two channel groups
constexpr int TC_OFF_SLOT = TC_W_BYTES;
constexpr int TC_SLOT_BYTES = TC_ACT_BYTES;
// floats: bias[256], red[slots][128], the last layer's tap sums xch[slots][5][128]
constexpr int TC_OFF_F = TC_OFF_SLOT + TC_SLOTS * TC_SLOT_BYTES;
constexpr int TC_NF = 256 + TC_SLOTS * 128 + TC_SLOTS * 5 * CP;
constexpr int TC_OFF_BAR = TC_OFF_F + TC_NF * 4;         // done[slots] mbarriers, TMEM address
constexpr int TC_SMEM = TC_OFF_BAR + 8 * TC_SLOTS + 16;
constexpr int TC_TMEM_COLS = 512;                        // 64 per slot, rounded up to a power of two
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;  // 2 s: a wait that long has failed
static_assert(TC_SMEM <= 227 * 1024, "fused corrector tiles exceed shared memory");
static_assert(TC_SLOTS * 64 <= TC_TMEM_COLS, "TMEM columns");
static_assert(TC_OFF_SLOT % 16 == 0 && TC_SLOT_BYTES % 16 == 0 && TC_OFF_BAR % 8 == 0,
              "tile offsets must be 16-byte aligned");

// byte offset of (row, channel) in a canonical K-major tile whose K-adjacent
// core matrices are lbo bytes apart
__host__ __device__ constexpr int tc_off(int r, int c, int lbo) { return (c >> 3) * lbo + r * 16 + (c & 7) * 2; }

// shared-memory matrix descriptor: start address, LBO and SBO in 16-byte
// units, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M x N
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// bounded wait for the phase `parity` of an mbarrier: false once TC_WAIT_NS
// of the global timer have passed without the phase completing
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = global_ns();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > TC_WAIT_NS) return false;
  }
}

// 16 consecutive TMEM columns of this warp's 32 lanes, as FP32
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// the same without the wait: several loads in flight, then one tc_wait_ld()
__device__ __forceinline__ void tc_ld16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// issue one layer: 5 taps x (CIN / 16) K-steps of M = 128, N = NOUT, reading
// the activation tile at act (lbo = TC_LBO_ACT) and the weight taps at w
template <int CIN, int NOUT>
__device__ __forceinline__ void tc_layer_issue(uint32_t tmem, uint32_t act, uint32_t w) {
  constexpr uint32_t idesc = tc_idesc(128, NOUT);
  constexpr int WTAP = NOUT * CIN * 2;
  // the descriptors of tap t, K-step kc are the tile's and the weights' base
  // descriptors with the start address moved by a compile-time offset (the
  // 14-bit address field holds any shared-memory address, so adding the
  // offset in 16-byte units cannot carry out of it)
  const uint64_t a0 = tc_desc(act, TC_LBO_ACT, 128);
  const uint64_t b0 = tc_desc(w, 16 * NOUT, 128);
  int first = 1;
#pragma unroll
  for (int t = 0; t < 5; ++t) {
#pragma unroll
    for (int kc = 0; kc < CIN / 16; ++kc) {
      const uint64_t a = a0 + (uint64_t)((16 * t + 2 * kc * TC_LBO_ACT) >> 4);
      const uint64_t b = b0 + (uint64_t)((t * WTAP + 2 * kc * (16 * NOUT)) >> 4);
      tc_mma(tmem, a, b, idesc, first ? 0 : 1);
      first = 0;
    }
  }
}

// issue the first layer: 2 K-steps of M = 128, N = 64 over the im2col rows
// (position p at tile row p + 2, K = 32) against the folded weights at w
__device__ __forceinline__ void tc_first_issue(uint32_t tmem, uint32_t act, uint32_t w) {
  constexpr uint32_t idesc = tc_idesc(128, HID);
  const uint64_t a0 = tc_desc(act, TC_LBO_ACT, 128);
  const uint64_t b0 = tc_desc(w, 16 * HID, 128);
#pragma unroll
  for (int kc = 0; kc < TC_K1 / 16; ++kc) {
    const uint64_t a = a0 + (uint64_t)((16 * CHALO + 2 * kc * TC_LBO_ACT) >> 4);
    const uint64_t b = b0 + (uint64_t)((2 * kc * (16 * HID)) >> 4);
    tc_mma(tmem, a, b, idesc, kc > 0 ? 1 : 0);
  }
}

// issue the last layer: 4 K-steps of M = 128, N = 16 over the tile's own
// rows (positions 0..127 at tile rows 2..129: the tap-2 start) against the
// taps-as-rows weight operand at w
__device__ __forceinline__ void tc_last_issue(uint32_t tmem, uint32_t act, uint32_t w) {
  constexpr uint32_t idesc = tc_idesc(128, 16);
  const uint64_t a0 = tc_desc(act, TC_LBO_ACT, 128);
  const uint64_t b0 = tc_desc(w, 16 * 16, 128);
#pragma unroll
  for (int kc = 0; kc < HID / 16; ++kc) {
    const uint64_t a = a0 + (uint64_t)((16 * CHALO + 2 * kc * TC_LBO_ACT) >> 4);
    const uint64_t b = b0 + (uint64_t)((2 * kc * (16 * 16)) >> 4);
    tc_mma(tmem, a, b, idesc, kc > 0 ? 1 : 0);
  }
}

// epilogue of a hidden layer: TMEM (this thread's position, 64 channels) +
// bias, ReLU, BF16 into row p + 2 of the next tile; two halves of 32
// columns, each with its two 16-column loads in flight together (the
// register budget of TC_SLOTS slots per CTA)
__device__ __forceinline__ void tc_hidden_epilogue(uint32_t tmem, int quarter, int p, const float* bias,
                                                   unsigned char* out_tile) {
  const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    uint32_t r[2][16];
    tc_ld16_nowait(tmem + lane_base + 32 * half, r[0]);
    tc_ld16_nowait(tmem + lane_base + 32 * half + 16, r[1]);
    tc_wait_ld();
#pragma unroll
    for (int q = 0; q < 2; ++q) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int c = 32 * half + 16 * q + 8 * h + 2 * j;
          const __nv_bfloat162 pr =
              __floats2bfloat162_rn(fmaxf(__uint_as_float(r[q][8 * h + 2 * j]) + bias[c], 0.f),
                                    fmaxf(__uint_as_float(r[q][8 * h + 2 * j + 1]) + bias[c + 1], 0.f));
          w[j] = *reinterpret_cast<const uint32_t*>(&pr);
        }
        *reinterpret_cast<uint4*>(out_tile + tc_off(p + CHALO, 32 * half + 16 * q + 8 * h, TC_LBO_ACT)) =
            make_uint4(w[0], w[1], w[2], w[3]);
      }
    }
  }
}

__device__ __forceinline__ void slot_sync(int slot) {
  asm volatile("bar.sync %0, 128;\n" ::"r"(1 + slot) : "memory");
}
// true on every thread of the slot if v is true on any (a named-barrier vote)
__device__ __forceinline__ bool slot_any(int slot, bool v) {
  uint32_t r;
  asm volatile(
      "{\n.reg .pred pi, po;\nsetp.ne.u32 pi, %1, 0;\nbar.red.or.pred po, %2, 128, pi;\nselp.u32 %0, 1, 0, po;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(1 + slot)
      : "memory");
  return r != 0;
}

// TC_SLOTS slots of 4 warps; each slot carries its own row through the
// four layers with its own TMEM columns and tile, and one elected thread of
// the slot issues the slot's MMAs, so that one slot's epilogue overlaps the
// others' MMAs.  Per slot one mbarrier, done, armed by tcgen05.commit when
// the layer's MMAs are complete.  Row k of slot s is blockIdx.x + gridDim.x *
// (k * TC_SLOTS + s).  Every wait is bounded: a wait that gives up sets err,
// and the slot leaves together after a barrier vote.
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_corr_forward_tc(const float* __restrict__ g, const float* __restrict__ gp, const float2* __restrict__ gmean,
                      const float2* __restrict__ pmean, int group_rows, const float* __restrict__ row_feat, int rows,
                      float vmax, const uint4* __restrict__ wtc, const float* __restrict__ params,
                      float* __restrict__ pred_out, float* __restrict__ scale_out, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  float* bias = reinterpret_cast<float*>(smem + TC_OFF_F);  // b1, b2, b3 [64] each, b4
  const uint32_t s_base = (uint32_t)__cvta_generic_to_shared(smem);
  const uint32_t bar_done = s_base + TC_OFF_BAR;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + TC_OFF_BAR + 8 * TC_SLOTS);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     s_base + TC_OFF_BAR + 8 * TC_SLOTS),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (threadIdx.x == 0) {
    for (int q = 0; q < TC_SLOTS; ++q)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar_done + 8 * q) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  for (int i = threadIdx.x; i < TC_W_BYTES / 16; i += TC_THREADS) reinterpret_cast<uint4*>(smem)[i] = wtc[i];
  for (int i = threadIdx.x; i < 3 * HID; i += TC_THREADS)
    bias[i] = params[i < HID ? OFF_B1 + i : (i < 2 * HID ? OFF_B2 + i - HID : OFF_B3 + i - 2 * HID)];
  if (threadIdx.x == 0) bias[3 * HID] = params[OFF_B4];
  // zero the halo rows (0, 1, 130, 131) of every tile
  for (int i = threadIdx.x; i < TC_SLOTS * 4 * 8; i += TC_THREADS) {
    const int grp = i & 7, hr = (i >> 3) & 3, tile = i >> 5;  // tile = slot
    const int hrow = hr < 2 ? hr : CROWS - 4 + hr;
    *reinterpret_cast<uint4*>(smem + TC_OFF_SLOT + tile * TC_ACT_BYTES + tc_off(hrow, 8 * grp, TC_LBO_ACT)) =
        make_uint4(0, 0, 0, 0);
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const int slot = warp >> 2;
  const int quarter = warp & 3;          // the TMEM lanes this warp may read
  const int p = 32 * quarter + lane;     // position = TMEM lane
  const bool issuer = (p == 0);          // the slot's MMA issuer
  float* red = bias + 256 + 128 * slot;
  float* xch = bias + 256 + 128 * TC_SLOTS + 5 * CP * slot;  // [5][128]
  unsigned char* tile = smem + TC_OFF_SLOT + slot * TC_SLOT_BYTES;
  const uint32_t tile_s = s_base + TC_OFF_SLOT + slot * TC_SLOT_BYTES;
  const uint32_t td = tmem + 64 * slot, lane_base = (uint32_t)(quarter * 32) << 16;
  const uint32_t bar = bar_done + 8 * slot;
  const float dvv = 2.f * vmax / CP;
  const float vfeat = __fadd_rn(-vmax, __fmul_rn(dvv, (float)p + 0.5f)) / vmax;
  uint32_t phase = 0;
  int commits = 0;
  bool ok = true;
  // this thread's inputs of a row, loaded one row ahead so that their
  // latency hides behind the current row's layers
  float in_g = 0.f, in_gp = 0.f, in_f = 0.f;
  float2 in_m = make_float2(0.f, 0.f), in_pm = make_float2(0.f, 0.f);
  auto fetch = [&](int r) {
    const size_t qq = (size_t)r * CP + p;
    in_g = g[qq];
    in_gp = gp ? gp[qq] : 0.f;
    in_f = row_feat ? row_feat[r] : 0.f;
    if (group_rows > 0) {
      const size_t mi = (size_t)(r / group_rows) * CP + p;
      in_m = gmean[mi];
      in_pm = gp ? pmean[mi] : make_float2(0.f, 0.f);
    }
  };
  // the slot's tile is complete: make it visible to the tensor core, then
  // its issuer starts layer L
  auto issue = [&](int L) {
    fence_async_smem();
    tc_fence_before();
    slot_sync(slot);
    if (issuer) {
      tc_fence_after();
      switch (L) {
        case 0: tc_first_issue(td, tile_s, s_base + TC_OFF_W1); break;
        case 1: tc_layer_issue<HID, HID>(td, tile_s, s_base + TC_OFF_W2); break;
        case 2: tc_layer_issue<HID, HID>(td, tile_s, s_base + TC_OFF_W3); break;
        default: tc_last_issue(td, tile_s, s_base + TC_OFF_W4); break;
      }
      tc_commit(bar);
    }
    ++commits;
  };
  int row = blockIdx.x + gridDim.x * slot;
  if (row < rows) fetch(row);
  while (ok && row < rows) {
    const size_t q = (size_t)row * CP + p;
    const float d = group_rows > 0 ? __fsub_rn(__fsub_rn(in_g, in_m.x), in_m.y) : in_g;
    const float dp = gp ? (group_rows > 0 ? __fsub_rn(__fsub_rn(in_gp, in_pm.x), in_pm.y) : in_gp) : 0.f;
    const float feat = in_f;
    const int next = row + gridDim.x * TC_SLOTS;
    if (next < rows) fetch(next);
    // row RMS: the same pairwise tree as k_features (partners 64, 32, ...,
    // 1 apart), the last five levels by shuffles within a warp
    red[p] = d * d;
    slot_sync(slot);
    if (p < 64) red[p] += red[p + 64];
    slot_sync(slot);
    if (p < 32) {
      float ss = red[p] + red[p + 32];
#pragma unroll
      for (int m = 16; m > 0; m >>= 1) ss += __shfl_down_sync(0xffffffffu, ss, m);
      if (p == 0) red[CP - 1] = ss;  // red[127] is no longer read
    }
    slot_sync(slot);
    const float s = sqrtf(red[CP - 1] / CP) + 1e-30f;
    {
      // im2col of the first layer: this position's 4 features go to channels
      // 4t..4t+3 of the output position q = p - t + 2 that reads it at tap t;
      // the owner of each row zeroes the taps that fall outside the row and
      // channels 20..31 (rows 2..129 only: the halo rows stay zero)
      const __nv_bfloat162 c01 = __floats2bfloat162_rn(d / s, vfeat);
      const __nv_bfloat162 c23 = __floats2bfloat162_rn(feat, dp / s);
      const uint2 fv = make_uint2(*reinterpret_cast<const uint32_t*>(&c01), *reinterpret_cast<const uint32_t*>(&c23));
#pragma unroll
      for (int t = 0; t < 5; ++t) {
        const int q = p - t + CHALO;
        if (q >= 0 && q < CP) *reinterpret_cast<uint2*>(tile + tc_off(q + CHALO, 4 * t, TC_LBO_ACT)) = fv;
        const int src = p + t - CHALO;
        if (src < 0 || src >= CP)
          *reinterpret_cast<uint2*>(tile + tc_off(p + CHALO, 4 * t, TC_LBO_ACT)) = make_uint2(0u, 0u);
      }
      *reinterpret_cast<uint2*>(tile + tc_off(p + CHALO, 20, TC_LBO_ACT)) = make_uint2(0u, 0u);
      *reinterpret_cast<uint4*>(tile + tc_off(p + CHALO, 24, TC_LBO_ACT)) = make_uint4(0u, 0u, 0u, 0u);
    }
    issue(0);
    float pred = 0.f;
    for (int L = 0; L < 4; ++L) {
      const bool done = mbar_wait(bar, phase);
      phase ^= 1u;
      if (slot_any(slot, !done)) {  // the slot leaves together, never half of it
        ok = false;
        break;
      }
      tc_fence_after();
      if (L < 3) {
        tc_hidden_epilogue(td, quarter, p, bias + HID * L, tile);
        issue(L + 1);
      } else {
        // D4[p][t] (t < 5) of this position; out[p] = sum_t D4[p + t - 2][t]
        // over the positions inside the row (the halo rows are zero)
        float v[16];
        tc_ld16(td + lane_base, v);
#pragma unroll
        for (int t = 0; t < 5; ++t) xch[t * CP + p] = v[t];
        slot_sync(slot);
        pred = bias[3 * HID];
#pragma unroll
        for (int t = 0; t < 5; ++t) {
          const int q = p + t - CHALO;
          if (q >= 0 && q < CP) pred += xch[t * CP + q];
        }
      }
    }
    if (!ok) break;
    pred_out[q] = pred;
    if (p == 0) scale_out[row] = s;
    row = next;
  }
  if (!ok) {
    if (p == 0) atomicOr(err, 1);
    // no MMA of this slot may still write TMEM when it is freed
    if (commits > 0) mbar_wait(bar, (uint32_t)((commits - 1) & 1));
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

// the four layers' BF16 weights in the fused kernel's shared-memory image
__global__ void k_pack_tc(const float* __restrict__ w, __nv_bfloat16* __restrict__ img) {
  // layers 2 and 3: (offset in params, cout, cin, N, byte offset in the image);
  // layers 1 and 4 have their own folded layouts below
  const int n_total = HID * TC_K1 + 2 * 5 * HID * HID + 16 * HID;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n_total; q += gridDim.x * blockDim.x) {
    int r = q, off, cout, cin, np, base;
    if (r < HID * TC_K1) {
      // first layer, taps folded into K: k = 4 t + c (c < 4 real channels;
      // channels 4..15 of the first layer only ever meet zero inputs)
      const int o = r / TC_K1, k = r % TC_K1;
      const float val = k < 5 * L1_REAL ? w[OFF_W1 + ((size_t)o * L1_IN + k % L1_REAL) * 5 + k / L1_REAL] : 0.f;
      img[(TC_OFF_W1 + tc_off(o, k, 16 * HID)) / 2] = __float2bfloat16(val);
      continue;
    } else if ((r -= HID * TC_K1) < 5 * HID * HID) {
      off = OFF_W2; cout = HID; cin = HID; np = HID; base = TC_OFF_W2;
    } else if ((r -= 5 * HID * HID) < 5 * HID * HID) {
      off = OFF_W3; cout = HID; cin = HID; np = HID; base = TC_OFF_W3;
    } else {
      // last layer: row t of the 16 x 64 operand is tap t of the one output
      r -= 5 * HID * HID;
      const int t = r / HID, c = r % HID;
      const float val = t < 5 ? w[OFF_W4 + (size_t)c * 5 + t] : 0.f;
      img[(TC_OFF_W4 + tc_off(t, c, 16 * 16)) / 2] = __float2bfloat16(val);
      continue;
    }
    const int t = r / (np * cin), o = (r / cin) % np, c = r % cin;
    const float val = o < cout ? w[off + ((size_t)o * cin + c) * 5 + t] : 0.f;
    const int byte = base + t * np * cin * 2 + tc_off(o, c, 16 * np);
    img[byte / 2] = __float2bfloat16(val);
  }
}

// ---------------------------------------------------------------------------
// Training layers on the tensor cores (tcgen05).
//
// The training forward keeps every activation in HBM for the backward pass,
// so it runs one layer per launch, and so do the data gradients (the same
// convolution with the transposed, tap-flipped weights and the ReLU mask of
// the forward activation).  k_conv_tc: persistent CTAs of TRN_SLOTS slots of
// 4 warps; a slot takes one row at a time into its tile (the fused forward's
// K-major layout with 2-row halos), its elected thread issues the layer's
// MMAs (M = 128 positions, N = COUT, K = 5 taps x CIN; a tap is the tile
// descriptor moved by 16 t bytes) into the slot's TMEM columns, and the
// slot's epilogue writes the row channels-last to HBM.
//
// The weight gradients reduce over positions:
// dW[o][c][t] = sum_rows sum_p dy[p][o] x[p + t - 2][c].  k_wgrad_tc makes
// the position the MMA's K and keeps both operands in the MN-major layout,
// which is the channels-last tile itself: 8 channels in 16 bytes, one
// position per 16-byte row, so a tap shift along K is again the descriptor
// moved by 16 t bytes.  M = 128 stacks copies of the input tile, copy q
// shifted by q rows, so that one MMA covers taps (g NCOPY + q); N is the
// output channels of dy.  Each CTA accumulates a chunk of rows in TMEM and
// writes its partial sums; k_wgrad_reduce adds the chunks in a fixed order.
// ---------------------------------------------------------------------------

// descriptor of an MN-major operand (no swizzle): core matrices of 8 K rows
// (positions) x 16 bytes (8 MN elements: channels); the leading-dimension
// offset is the stride between 8-position groups along K and the stride
// offset the one between 8-channel groups along MN (the gradient tests
// against the CPU oracle hold this assignment; the swapped one fails them)
__device__ __forceinline__ uint64_t tc_desc_mn(uint32_t addr, uint32_t mn_stride, uint32_t k_stride) {
  return tc_desc(addr, k_stride, mn_stride);
}

constexpr int TRN_SLOTS = 4;
constexpr int TRN_THREADS = 128 * TRN_SLOTS;

// 16-byte global -> shared copies that complete asynchronously (L2 only):
// the next row's tiles load while the current row's MMAs run
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

__host__ __device__ constexpr int tmem_cols_for(int n) { return n <= 32 ? 32 : (n <= 64 ? 64 : (n <= 128 ? 128 : (n <= 256 ? 256 : 512))); }

template <int CIN, int COUT>
__host__ __device__ constexpr int trn_conv_wbytes() { return 5 * COUT * CIN * 2; }
template <int CIN, int COUT>
__host__ __device__ constexpr int trn_conv_smem() {
  return trn_conv_wbytes<CIN, COUT>() + 2 * TRN_SLOTS * (CIN / 8) * TC_LBO_ACT + 8 * TRN_SLOTS + 16;
}

// MODE 0: out = relu(conv + b) (bf16); MODE 1: out[p] = conv + b, channel 0
// only (fp32); MODE 2: out = conv * (mask > 0) (bf16, no bias).
// w: bf16 [5][WROWS][CIN] (rows WROWS..COUT - 1 are zero)
template <int CIN, int COUT, int WROWS, int MODE>
__global__ void __launch_bounds__(TRN_THREADS, 1)
    k_conv_tc(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ w,
              const float* __restrict__ bias, const __nv_bfloat16* __restrict__ mask, void* out, int rows,
              int* __restrict__ err) {
  static_assert(CIN % 16 == 0 && COUT % 16 == 0 && WROWS <= COUT, "layer shape");
  constexpr int WTAP = COUT * CIN * 2;
  constexpr int W_BYTES = trn_conv_wbytes<CIN, COUT>();
  constexpr int TILE = (CIN / 8) * TC_LBO_ACT;
  constexpr int TILES = 2 * TRN_SLOTS;  // two per slot: the current row's and the next one's
  constexpr int TMEM_COLS = tmem_cols_for(TRN_SLOTS * COUT);
  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t s_base = (uint32_t)__cvta_generic_to_shared(smem);
  const uint32_t bar0 = s_base + W_BYTES + TILES * TILE;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + W_BYTES + TILES * TILE + 8 * TRN_SLOTS);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     bar0 + 8 * TRN_SLOTS),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (threadIdx.x == 0) {
    for (int q = 0; q < TRN_SLOTS; ++q)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0 + 8 * q) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  // weights: tap t, output row n, input chunk j -> t WTAP + tc_off(n, 8 j, 16 COUT)
  for (int i = threadIdx.x; i < 5 * COUT * (CIN / 8); i += TRN_THREADS) {
    const int j = i % (CIN / 8), n = (i / (CIN / 8)) % COUT, t = i / ((CIN / 8) * COUT);
    const uint4 v = n < WROWS ? reinterpret_cast<const uint4*>(w + ((size_t)t * WROWS + n) * CIN)[j]
                              : make_uint4(0u, 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(smem + t * WTAP + tc_off(n, 8 * j, 16 * COUT)) = v;
  }
  // halo rows (0, 1, 130, 131) of every tile stay zero
  for (int i = threadIdx.x; i < TILES * 4 * (CIN / 8); i += TRN_THREADS) {
    const int j = i % (CIN / 8), hr = (i / (CIN / 8)) % 4, sl = i / (4 * (CIN / 8));
    const int hrow = hr < 2 ? hr : CROWS - 4 + hr;
    *reinterpret_cast<uint4*>(smem + W_BYTES + sl * TILE + tc_off(hrow, 8 * j, TC_LBO_ACT)) =
        make_uint4(0u, 0u, 0u, 0u);
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const int slot = warp >> 2, quarter = warp & 3;
  const int p = 32 * quarter + lane;
  const bool issuer = (p == 0);
  const uint32_t td = tmem + COUT * slot, lane_base = (uint32_t)(quarter * 32) << 16;
  const uint32_t bar = bar0 + 8 * slot;
  uint32_t phase = 0;
  int commits = 0;
  bool ok = true;
  // this thread's position of a row into row p + 2 of tile b, asynchronously
  auto fetch = [&](int row, int b) {
    const uint4* src = reinterpret_cast<const uint4*>(x + ((size_t)row * CP + p) * CIN);
    unsigned char* tile = smem + W_BYTES + (2 * slot + b) * TILE;
#pragma unroll
    for (int j = 0; j < CIN / 8; ++j) cp_async16(tile + tc_off(p + CHALO, 8 * j, TC_LBO_ACT), src + j);
    cp_async_commit();
  };
  const int stride = gridDim.x * TRN_SLOTS;
  int b = 0;
  if (blockIdx.x * TRN_SLOTS + slot < rows) fetch(blockIdx.x * TRN_SLOTS + slot, 0);
  for (int row = blockIdx.x * TRN_SLOTS + slot; row < rows; row += stride, b ^= 1) {
    const size_t q = (size_t)row * CP + p;
    cp_async_wait_all();
    fence_async_smem();
    tc_fence_before();
    slot_sync(slot);
    if (issuer) {
      tc_fence_after();
      tc_layer_issue<CIN, COUT>(td, s_base + W_BYTES + (2 * slot + b) * TILE, s_base);
      tc_commit(bar);
    }
    ++commits;
    // the next row into the other tile (its last reader, the previous row's
    // MMAs, completed before that row's epilogue)
    if (row + stride < rows) fetch(row + stride, b ^ 1);
    const bool done = mbar_wait(bar, phase);
    phase ^= 1u;
    if (slot_any(slot, !done)) {
      ok = false;
      break;
    }
    tc_fence_after();
#pragma unroll
    for (int c0 = 0; c0 < (MODE == 1 ? 16 : COUT); c0 += 16) {
      float v[16];
      tc_ld16(td + lane_base + c0, v);
      if (MODE == 1) {
        static_cast<float*>(out)[q] = v[0] + bias[0];
      } else {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint32_t wv[4];
          uint4 mk = make_uint4(0u, 0u, 0u, 0u);
          if (MODE == 2) mk = reinterpret_cast<const uint4*>(mask + q * COUT + c0 + 8 * h)[0];
          const __nv_bfloat162* m2 = reinterpret_cast<const __nv_bfloat162*>(&mk);
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int c = c0 + 8 * h + 2 * j;
            float a = v[8 * h + 2 * j], b = v[8 * h + 2 * j + 1];
            if (MODE == 0) {
              a = fmaxf(a + bias[c], 0.f);
              b = fmaxf(b + bias[c + 1], 0.f);
            } else {
              if (!(__bfloat162float(m2[j].x) > 0.f)) a = 0.f;
              if (!(__bfloat162float(m2[j].y) > 0.f)) b = 0.f;
            }
            const __nv_bfloat162 pr = __floats2bfloat162_rn(a, b);
            wv[j] = *reinterpret_cast<const uint32_t*>(&pr);
          }
          reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(out) + q * COUT + c0 + 8 * h)[0] =
              make_uint4(wv[0], wv[1], wv[2], wv[3]);
        }
      }
    }
    // every thread of the slot has read its TMEM lanes before the next row's
    // MMAs overwrite them
    tc_fence_before();
    slot_sync(slot);
  }
  cp_async_wait_all();  // no copy may land after the CTA is gone
  if (!ok) {
    if (p == 0) atomicOr(err, 1);
    // no MMA of this slot may still write TMEM when it is freed
    if (commits > 0) mbar_wait(bar, (uint32_t)((commits - 1) & 1));
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// weight-gradient shapes: NCOPY taps per MMA group (copies of the input tile
// in M = 128), NGROUP groups for the five taps, R rows per copy
template <int CIN>
struct WgradShape {
  static constexpr int NCOPY = CIN == 64 ? 2 : 5;
  static constexpr int COPIES = 128 / CIN;  // copies in M (those >= NCOPY stay zero)
  static constexpr int NGROUP = (5 + NCOPY - 1) / NCOPY;
  static constexpr int R = CP + (NGROUP - 1) * NCOPY;
  static constexpr int A_BYTES = 16 * R * 16;  // 16 chunks of 8 (copy, channel) rows
};
template <int CIN, int COUTP>
__host__ __device__ constexpr int trn_wgrad_stage() {
  return WgradShape<CIN>::A_BYTES + (COUTP / 8) * CP * 16;
}
template <int CIN, int COUTP>
__host__ __device__ constexpr int trn_wgrad_smem() {
  return 2 * trn_wgrad_stage<CIN, COUTP>() + 16 + 16;
}

// one CTA of 128 threads (thread p: position p of a row, then TMEM lane p)
// per chunk of rows; two row stages, so that the tiles of a row are written
// while the previous row's MMAs run.  part[chunk][t][o][c], bpart[chunk][o].
template <int CIN, int COUTP>
__global__ void __launch_bounds__(128, 1)
    k_wgrad_tc(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ dy, int rows,
               int rows_per_chunk, float* __restrict__ part, float* __restrict__ bpart, int* __restrict__ err) {
  using S = WgradShape<CIN>;
  static_assert(CIN == 64 || CIN == 16, "input channels");
  static_assert(COUTP % 16 == 0 && COUTP <= 64, "output channels");
  constexpr int STAGE = trn_wgrad_stage<CIN, COUTP>();
  constexpr int TMEM_COLS = tmem_cols_for(S::NGROUP * COUTP);
  constexpr uint32_t MN_A = (uint32_t)S::R * 16, MN_B = (uint32_t)CP * 16;
  constexpr uint32_t idesc = tc_idesc(128, COUTP) | (1u << 15) | (1u << 16);  // A and B MN-major
  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t s_base = (uint32_t)__cvta_generic_to_shared(smem);
  const uint32_t bar0 = s_base + 2 * STAGE;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 2 * STAGE + 16);
  const int warp = threadIdx.x >> 5, p = threadIdx.x;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(bar0 + 16),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar0 + 8) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  // both stages zero: the rows a shifted copy never receives, and the copies
  // beyond NCOPY, stay zero
  for (int i = threadIdx.x; i < 2 * STAGE / 16; i += 128) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const int r_begin = blockIdx.x * rows_per_chunk;
  const int r_end = min(rows, r_begin + rows_per_chunk);
  float bsum = 0.f;
  uint32_t phase[2] = {0u, 0u};
  bool pending[2] = {false, false};
  bool ok = true;
  int n = 0;
  // row `row`'s input copies and dy into stage st, asynchronously (copy c
  // holds x[r + c - 2] at row r)
  auto fetch = [&](int row, int st) {
    unsigned char* A = smem + st * STAGE;
    unsigned char* B = A + S::A_BYTES;
    const size_t q = (size_t)row * CP + p;
    const uint4* xs = reinterpret_cast<const uint4*>(x + q * CIN);
    const uint4* ys = reinterpret_cast<const uint4*>(dy + q * COUTP);
#pragma unroll
    for (int j = 0; j < CIN / 8; ++j)
#pragma unroll
      for (int c = 0; c < S::NCOPY; ++c) {
        const int r = p + CHALO - c;
        if (r >= 0 && r < S::R) cp_async16(A + (c * (CIN / 8) + j) * MN_A + r * 16, xs + j);
      }
#pragma unroll
    for (int j = 0; j < COUTP / 8; ++j) cp_async16(B + j * MN_B + p * 16, ys + j);
    cp_async_commit();
  };
  if (r_begin < r_end) fetch(r_begin, 0);
  for (int row = r_begin; row < r_end; ++row, ++n) {
    const int st = n & 1;
    unsigned char* B = smem + st * STAGE + S::A_BYTES;
    cp_async_wait_all();
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      const uint32_t a_s = s_base + st * STAGE, b_s = a_s + S::A_BYTES;
#pragma unroll
      for (int g = 0; g < S::NGROUP; ++g) {
#pragma unroll
        for (int ks = 0; ks < CP / 16; ++ks) {
          const uint64_t a = tc_desc_mn(a_s + 16 * (g * S::NCOPY) + 256 * ks, MN_A, 128);
          const uint64_t b = tc_desc_mn(b_s + 256 * ks, MN_B, 128);
          tc_mma(tmem + g * COUTP, a, b, idesc, (row > r_begin || ks > 0) ? 1 : 0);
        }
      }
      tc_commit(bar0 + 8 * st);
    }
    pending[st] = true;
    // the next row into the other stage, once the MMAs that read it are done
    if (row + 1 < r_end) {
      const int so = st ^ 1;
      if (pending[so]) {
        const bool done = mbar_wait(bar0 + 8 * so, phase[so]);
        phase[so] ^= 1u;
        pending[so] = false;
        if (__syncthreads_or(!done)) {
          ok = false;
          break;
        }
      }
      fetch(row + 1, so);
    }
    // bias gradient: column sums of dy over the row's positions
    if (threadIdx.x < COUTP) {
      const int o = threadIdx.x;
      const unsigned char* col = B + (o >> 3) * MN_B + (o & 7) * 2;
      float rs = 0.f;
      for (int pp = 0; pp < CP; ++pp) rs += __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(col + pp * 16));
      bsum += rs;
    }
  }
  cp_async_wait_all();
  // the outstanding commits of both stages
  for (int st = 0; st < 2; ++st)
    if (pending[st]) {
      const bool done = mbar_wait(bar0 + 8 * st, phase[st]);
      if (!done) ok = false;
    }
  ok = !__syncthreads_or(!ok);
  tc_fence_after();
  if (ok && r_end > r_begin) {
    const int c = p % CIN, cp = p / CIN;  // TMEM lane p = (copy, channel)
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll
    for (int g = 0; g < S::NGROUP; ++g) {
#pragma unroll
      for (int c0 = 0; c0 < COUTP; c0 += 16) {
        float v[16];
        tc_ld16(tmem + lane_base + g * COUTP + c0, v);
        const int t = g * S::NCOPY + cp;
        if (cp < S::NCOPY && t < 5) {
          float* dst = part + (((size_t)blockIdx.x * 5 + t) * COUTP + c0) * CIN + c;
#pragma unroll
          for (int j = 0; j < 16; ++j) dst[(size_t)j * CIN] = v[j];
        }
      }
    }
    if (threadIdx.x < COUTP) bpart[(size_t)blockIdx.x * COUTP + threadIdx.x] = bsum;
  } else if (r_end > r_begin) {
    if (threadIdx.x == 0) atomicOr(err, 1);
  } else {
    // an empty chunk contributes zeros
    for (int i = threadIdx.x; i < 5 * COUTP * CIN; i += 128) part[(size_t)blockIdx.x * 5 * COUTP * CIN + i] = 0.f;
    if (threadIdx.x < COUTP) bpart[(size_t)blockIdx.x * COUTP + threadIdx.x] = 0.f;
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
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
  float2 *gmean, *tmean, *pmean;  // group means [groups][128] as double-float pairs
  float vmax, tau;
  int engine;               // 0: tcgen05 (fused inference, per-layer training), 1: mma.sync kernels
  int n_sm;
  __nv_bfloat16* wtc;       // the fused kernel's weight image [TC_W_BYTES / 2]
  cx<double>* tw64;         // FFT twiddles of the projection
  cx<float>* tw32;
  int* err;                 // device error word of the fused kernel
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

// the training layers on the tensor cores (engine 0)
template <int CIN, int COUT, int WROWS, int MODE>
cudaError_t conv_tc(vg_corrector* c, const __nv_bfloat16* x, const __nv_bfloat16* w, const float* b,
                    const __nv_bfloat16* mask, void* out, int rows, cudaStream_t s) {
  constexpr int smem = trn_conv_smem<CIN, COUT>();
  cudaError_t err = ensure_smem((const void*)k_conv_tc<CIN, COUT, WROWS, MODE>, smem);
  if (err != cudaSuccess) return err;
  const int grid = std::max(1, std::min(c->n_sm, div_up(rows, TRN_SLOTS)));
  k_conv_tc<CIN, COUT, WROWS, MODE><<<grid, TRN_THREADS, smem, s>>>(x, w, b, mask, out, rows, c->err);
  return cudaGetLastError();
}

template <int CIN, int COUTP>
cudaError_t wgrad_tc(vg_corrector* c, const __nv_bfloat16* x, const __nv_bfloat16* dy, int rows, int cout, float* dw,
                     float* db, cudaStream_t s) {
  const int chunks = wgrad_chunks(rows);
  const int per = div_up(rows, chunks);
  constexpr int smem = trn_wgrad_smem<CIN, COUTP>();
  cudaError_t err = ensure_smem((const void*)k_wgrad_tc<CIN, COUTP>, smem);
  if (err != cudaSuccess) return err;
  k_wgrad_tc<CIN, COUTP><<<chunks, 128, smem, s>>>(x, dy, rows, per, c->part, c->bpart, c->err);
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
  k_pack_tc<<<div_up(TC_W_BYTES / 2, 256), 256, 0, s>>>(c->params, c->wtc);
  return cuda_status(cudaGetLastError(), "corrector pack");
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
  const float* P = c->params;
  if (c->engine == 0) {
    CR_CHECK(cuda_status(conv_tc<L1_IN, HID, HID, 0>(c, c->x0, c->w1f, P + OFF_B1, nullptr, c->a1, rows, s), "conv1"));
    CR_CHECK(cuda_status(conv_tc<HID, HID, HID, 0>(c, c->a1, c->w2f, P + OFF_B2, nullptr, c->a2, rows, s), "conv2"));
    CR_CHECK(cuda_status(conv_tc<HID, HID, HID, 0>(c, c->a2, c->w3f, P + OFF_B3, nullptr, c->a3, rows, s), "conv3"));
    CR_CHECK(cuda_status(conv_tc<HID, 16, L4_OUT, 1>(c, c->a3, c->w4f, P + OFF_B4, nullptr, c->pred, rows, s), "conv4"));
    return VG_OK;
  }
  CR_CHECK(cuda_status(conv<L1_IN, HID, 0>(c->x0, c->w1f, P + OFF_B1, nullptr, c->a1, rows, s), "conv1"));
  CR_CHECK(cuda_status(conv<HID, HID, 0>(c->a1, c->w2f, P + OFF_B2, nullptr, c->a2, rows, s), "conv2"));
  CR_CHECK(cuda_status(conv<HID, HID, 0>(c->a2, c->w3f, P + OFF_B3, nullptr, c->a3, rows, s), "conv3"));
  CR_CHECK(cuda_status(conv<HID, L4_OUT, 1>(c->a3, c->w4f, P + OFF_B4, nullptr, c->pred, rows, s), "conv4"));
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
  if (c->engine == 0) {
    CR_CHECK(cuda_status(wgrad_tc<HID, 16>(c, c->a3, c->dy4, rows, 1, G + OFF_W4, G + OFF_B4, s), "wgrad4"));
    CR_CHECK(cuda_status(conv_tc<16, HID, HID, 2>(c, c->dy4, c->w4b, nullptr, c->a3, c->d3, rows, s), "dgrad4"));
    CR_CHECK(cuda_status(wgrad_tc<HID, HID>(c, c->a2, c->d3, rows, HID, G + OFF_W3, G + OFF_B3, s), "wgrad3"));
    CR_CHECK(cuda_status(conv_tc<HID, HID, HID, 2>(c, c->d3, c->w3b, nullptr, c->a2, c->d2, rows, s), "dgrad3"));
    CR_CHECK(cuda_status(wgrad_tc<HID, HID>(c, c->a1, c->d2, rows, HID, G + OFF_W2, G + OFF_B2, s), "wgrad2"));
    CR_CHECK(cuda_status(conv_tc<HID, HID, HID, 2>(c, c->d2, c->w2b, nullptr, c->a1, c->d1, rows, s), "dgrad2"));
    CR_CHECK(cuda_status(wgrad_tc<L1_IN, HID>(c, c->x0, c->d1, rows, HID, G + OFF_W1, G + OFF_B1, s), "wgrad1"));
    return VG_OK;
  }
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
  CR_TRY(cr_alloc(c, &c->wtc, (size_t)TC_W_BYTES / 2, "corrector weights"));
  CR_TRY(cr_alloc(c, &c->tw64, (size_t)FFT_NMAX, "corrector twiddles"));
  CR_TRY(cr_alloc(c, &c->tw32, (size_t)FFT_NMAX, "corrector twiddles"));
  {
    vg_plan tmp;
    std::memset(&tmp, 0, sizeof(tmp));
    tmp.tw64 = c->tw64;
    tmp.tw32 = c->tw32;
    CR_TRY(cuda_status(launch_twiddles(tmp, 0), "corrector twiddles"));
  }
  CR_TRY(cr_alloc(c, &c->err, 1, "corrector status"));
  {
    int dev = 0;
    cudaGetDevice(&dev);
    c->n_sm = 1;
    cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, dev);
  }
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
  if (c->engine == 0) {
    if (b->group_rows > 0) {
      k_group_mean<<<b->rows / b->group_rows, CP, 0, s>>>(b->g, b->group_rows, c->gmean);
      CR_CHECK(cuda_status(cudaGetLastError(), "corrector group mean"));
      if (b->g_prev) {
        k_group_mean<<<b->rows / b->group_rows, CP, 0, s>>>(b->g_prev, b->group_rows, c->pmean);
        CR_CHECK(cuda_status(cudaGetLastError(), "corrector group mean"));
      }
    }
    CR_CHECK(cuda_status(ensure_smem((const void*)k_corr_forward_tc, TC_SMEM), "corrector fused kernel"));
    const int grid = std::min(b->rows, c->n_sm);
    k_corr_forward_tc<<<grid, TC_THREADS, TC_SMEM, s>>>(b->g, b->g_prev, c->gmean, c->pmean, b->group_rows,
                                                        b->row_feat, b->rows, c->vmax,
                                                        reinterpret_cast<const uint4*>(c->wtc), c->params, c->pred,
                                                        c->scale, c->err);
    CR_CHECK(cuda_status(cudaGetLastError(), "corrector forward"));
  } else {
    CR_CHECK(forward(c, *b, s));
  }
  k_apply<<<div_up(b->rows, APPLY_ROWS), CP, 0, s>>>(b->g, c->gmean, b->group_rows, c->pred, c->scale, c->tau,
                                                     c->protect_modes, c->tw32, b->rows, g_out);
  return cuda_status(cudaGetLastError(), "corrector apply");
}

int vg_corr_set_engine(vg_corrector* c, int32_t engine) {
  if (!c || engine < 0 || engine > 1) {
    set_error("corrector: engine must be 0 (tcgen05) or 1 (per-layer mma.sync)");
    return VG_ERR_ARG;
  }
  c->engine = engine;
  return VG_OK;
}

int vg_corr_status(vg_corrector* c, int32_t* flags) {
  if (!c || !flags) {
    set_error("corrector: null argument");
    return VG_ERR_ARG;
  }
  int h = 0;
  CR_CHECK(cuda_status(cudaMemcpy(&h, c->err, sizeof(int), cudaMemcpyDeviceToHost), "corrector status"));
  *flags = h;
  if (h) {
    set_error("corrector: a bounded wait of the fused kernel ran out (its output is invalid)");
    return VG_ERR_TIMEOUT;
  }
  return VG_OK;
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
