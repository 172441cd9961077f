// Plan state and launch shapes of the FP32 delta-f path.
#pragma once

#include "vg_common.cuh"
#include "vg_fft.cuh"

namespace vg {

// Per-run constants of the delta-f row pass (all device pointers, FP32 copies
// of FP64 host values; the moments of f0 stay FP64).
struct RowConsts {
  const float* v;   // [nv]
  const float* f0;  // [nv] background
  const float* S;   // [nv] (f0[j-1] - 2 f0[j] + f0[j+1]) / dv^2, truncated at the ends
  const float* Mv;  // [nv] (v[j-1] f0[j-1] - v[j+1] f0[j+1]) / (2 dv)
  const float* D;   // [nv] (f0[j-1] - f0[j+1]) / (2 dv)
  const float2* vhl;  // [nv] v split into FP32 (hi, lo) for exact phase products
  double dv, dv_sq, dkv;
  double f0m[7];    // trapz(f0 v^p), p = 0..5, and trapz(f0^2)
  float i2dv;       // 1 / (2 dv)
  float v0f, dvf;   // v[0] and dv in FP32 (the grid is uniform)
  // the same in double-float, for the per-row collision scalars (the FP64
  // pipe of this part is 1/64 of FP32, so a row's scalars stay off it)
  float2 dv2f, idv2f;  // dv and 1 / dv^2 split (hi, lo)
  float2 f0m2f[3];     // f0m[0..2] split
};

struct RowArgs {
  float* g;
  int nx;
  const float* e32;  // field of the kicks, FP32 copy
  double dt1, dt2;   // leading / trailing half-kick steps (0: skip)
  float hk1, hk2;    // -dkv dt / 2 of each kick: half angle per kv index and unit field
  int fp, dougherty;
  float2 nudt2;   // nu dt split (hi, lo)
  float nudt_f;
  int want_mom;     // storage moments + x modes of the post-collision state
  double* mom;      // [nx][8] slots, each the raw double-float sum (df32) of one moment
  int n_modes;
  cx<float>* mpart; // [grid][n_modes][nv] per-CTA partial x modes
  int macc_global;  // the CTA accumulates its x modes in its mpart slice (else in shared memory)
  const cx<float>* F0;  // [nv/2+1] unnormalised FFT_v(f0)
  const cx<float>* tw;
  // the row constants in device memory: a kernel that built a RowConsts
  // copy of its own would keep it on the stack (~150 B of local memory)
  const RowConsts* rc;
};

struct F32Plan {
  double dkx, dkv, c0;  // kx[1], kv[1], trapz(f0) - 1
  cx<float>* F0;
  float* v32;
  float* f0_32;
  float* S;
  float* Mv;
  float* D;
  RowConsts rc;
  RowConsts* rc_dev;   // device copy of rc (for RowArgs)
  float2* vhl;         // [nv] v as FP32 (hi, lo)
  float* e32;          // [nx] FP32 copy of the field
  float2* dpart;       // [max col grid][nx] density partials (hi, lo)
  int npart;
  cx<float>* mpart;    // [max row grid][4][nv]
  float2* spart;       // [F32_STORE_MAX_CTAS][7] per-CTA series partials (hi, lo) of the store
  int mgrid;
  int col_grid_max, row_grid_max, col_grid, row_grid;
  int n_sm;
};

// launch shapes of the single-run kernels (shared by their __launch_bounds__
// and the launchers; the batched sweep chooses its own)
// column tiles: radix 8 up to nx = 1024, radix 16 above; S column pairs per
// CTA, at least 4 (32-byte row segments) but at most 512 threads, so that a
// thread keeps up to 128 registers
__host__ __device__ constexpr int col32_radix(int nx) { return nx <= 8 ? nx : (nx <= 1024 ? 8 : 16); }
__host__ __device__ constexpr int col32_seqs_raw(int g) { return (256 / g) > 4 ? (256 / g) : 4; }
__host__ __device__ constexpr int col32_seqs(int nx, int r) {
  return (nx / r) * col32_seqs_raw(nx / r) <= 512 ? col32_seqs_raw(nx / r)
                                                   : (512 / (nx / r) > 1 ? 512 / (nx / r) : 1);
}
// row radix of the single-run kernels: radix 8 up to 4096; radix 32 above
// (8192 = 32 x 32 x 8: three passes, and a 256-thread row-pair group that
// leaves room for a second CTA on the SM to hide the passes' barriers)
__host__ __device__ constexpr int row32_radix(int n) { return n <= 8 ? n : (n <= 4096 ? 8 : 32); }
__host__ __device__ constexpr int row32_block(int n, int r) { return (n / r) >= 256 ? (n / r) : 256; }
// per row-pair group, each part 16-byte aligned: padded sequence (sp_len,
// the layout the row kernels index), boundary-solve scratch of 8G floats
// (2 x G float4), double-float reduction slots
__host__ __device__ constexpr size_t round16(size_t b) { return (b + 15) & ~(size_t)15; }
__host__ __device__ constexpr size_t row32_seq_bytes(int n, int r) {
  return round16((size_t)(n + (n >> row_pad_shift(r))) * 8 + 16);
}
__host__ __device__ constexpr size_t row32_group_bytes(int n, int r) {
  return row32_seq_bytes(n, r) + (size_t)8 * (n / r) * 4 + round16((size_t)((n / r) / 32 + 1) * 9 * 8);
}

constexpr int F32_MAX_MODES = 4;
constexpr int F32_STORE_MAX_CTAS = 64;  // CTAs of the per-step fields/series pass

// (hi, lo) FP32 split of an FP64 value
inline float2 split_f2(double a) {
  const float h = (float)a;
  return make_float2(h, (float)(a - (double)h));
}

}  // namespace vg
