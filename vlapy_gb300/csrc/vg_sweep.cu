// Batched sweep: many independent FP32 delta-f runs of uneven shape advanced
// together, every launch covering all runs.
//
// Layout in HBM: one FP32 buffer holds every run's g[nx][nv] back to back
// (runs in their input order); fields e, 1 - n and the row moments are
// packed the same way along x.  Runs share per-nv constants (v grid, the
// Maxwellian background f0, its stencils and spectrum); per run only k, nu
// and the offsets differ.  A step is four launches -- x-drift over (run,
// tile) items, field solve over groups of runs of one nx, the fused row pass
// over (run, row-pair group) items, and the storage of e and the series --
// preceded once per call by the first half kick.  Kernels dispatch on the
// item's shape to the same device bodies as the single-run path.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include <cuda.h>

#include "vg_f32_body.cuh"
#include "vg_internal.cuh"

namespace vg {

struct SweepRunDev {
  int nx, nv, cls;     // cls: index of the run's nv class
  int ntiles, W;       // column tiles of the x-drift
  int fp;              // collide this run
  long long g_off;     // cells before this run
  int x_off;           // x points before this run
  long long dp_off;    // density-partial elements (float2) before this run
  double k, nudt;
  float2 nudt2;  // nudt split (hi, lo)
  float2 kdt;          // -k dt split into FP32 (hi, lo): the x-drift angle per unit m and v
  float nudt_f;
};

constexpr int SWEEP_BLOCK = 256;
// threads per CTA of the row kernels (build-time knob; the radix-16 kernels
// are register-bound, so smaller CTAs give finer occupancy steps)
#ifndef VG_SWEEP_ROW_BLOCK
#define VG_SWEEP_ROW_BLOCK 256
#endif
constexpr int SWEEP_ROW_BLOCK = VG_SWEEP_ROW_BLOCK;
// resident CTAs per SM the row and column kernels are compiled for (the
// register budget per thread follows); build-time tuning knobs
#ifndef VG_ROW_MIN_BLOCKS
#define VG_ROW_MIN_BLOCKS 4
#endif
// nv classes (bit log2 nv) whose row kernel runs radix-16 FFT passes (16
// elements per thread: one pass fewer for nv = 256 and 1024, and for nv = 512
// a row pair per warp); build-time knob.  On the 4096-run sweep, radix 16 for
// nv = 256, 512 and 1024 gives the fastest row pass (1.76 ms, against 1.92 ms
// with nv = 512 on radix 8 and 2.29 ms with nv = 1024 on radix 8)
#ifndef VG_SWEEP_R16_MASK
#define VG_SWEEP_R16_MASK 0x700
#endif
// CTAs per SM of the x-drift kernels (64 registers a thread at 4; the
// radix-16 ones hold 16 elements a thread)
#ifndef VG_COL_MIN_BLOCKS
#define VG_COL_MIN_BLOCKS 4
#endif
// (3: a small spill, but on the 4096-run sweep the nx = 128 x-drift takes
// 0.43 ms against 0.46 ms at 2 CTAs and at radix 8)
#ifndef VG_COL_MIN_BLOCKS_R16
#define VG_COL_MIN_BLOCKS_R16 3
#endif
constexpr int SWEEP_FIELD_BLOCK = 128;
constexpr int SWEEP_MAX_CLASSES = 6;  // nv in {64, ..., 2048}

// FFT radix of the sweep's x-drift: radix 16 for the nx in the build-time
// mask (bit log2 nx): nx = 128 (16 x 8 instead of 8 x 8 x 2), nx = 64 (16 x 4)
// and nx = 32 (16 x 2): fewer threads a column pair, the autotuner's choice
// on a GB300 (1.748 ms per 4096-run step, against 1.787 with nx = 128 alone)
#ifndef VG_SWEEP_COL_R16_MASK
#define VG_SWEEP_COL_R16_MASK 0xE0
#endif
// radix 32 for the nx (>= 64) in this mask, ahead of the radix-16 one
// (32 elements a thread; build-time knob, none by default), and the CTAs per
// SM of those x-drift kernels
#ifndef VG_SWEEP_COL_R32_MASK
#define VG_SWEEP_COL_R32_MASK 0x0
#endif
#ifndef VG_COL_MIN_BLOCKS_R32
#define VG_COL_MIN_BLOCKS_R32 2
#endif
__host__ __device__ constexpr int sweep_col_radix(int nx) {
  return (nx >= 64 && nx <= 256 && ((VG_SWEEP_COL_R32_MASK >> ilog2(nx)) & 1))   ? 32
         : (nx >= 32 && nx <= 256 && ((VG_SWEEP_COL_R16_MASK >> ilog2(nx)) & 1)) ? 16
                                                                                 : col32_radix(nx);
}
__host__ __device__ constexpr int sweep_col_min_blocks(int nx) {
  return sweep_col_radix(nx) == 32   ? VG_COL_MIN_BLOCKS_R32
         : sweep_col_radix(nx) == 16 ? VG_COL_MIN_BLOCKS_R16
                                     : VG_COL_MIN_BLOCKS;
}
__host__ __device__ constexpr int sweep_col_w(int nx) { return 2 * (SWEEP_BLOCK / (nx / sweep_col_radix(nx))); }
// nv classes (bit log2 nv) on radix-32 passes (32 elements a thread; a row
// pair per warp at nv = 1024, per half warp at 512; build-time knob).
// nv = 1024 (two passes instead of 16 x 16 x 4): row pass 1.333 ms against
// 1.365 ms on radix 16; nv = 512 as well (32 x 16): 1.787 against 1.818 ms
// per 4096-run step, the autotuner's choice on a GB300
#ifndef VG_SWEEP_R32_MASK
#define VG_SWEEP_R32_MASK 0x600
#endif
#ifndef VG_ROW_MIN_BLOCKS_R32
#define VG_ROW_MIN_BLOCKS_R32 2
#endif
__host__ __device__ constexpr int sweep_row_radix(int nv) {
  return (nv >= 256 && nv <= 4096 && ((VG_SWEEP_R32_MASK >> ilog2(nv)) & 1))   ? 32
         : (nv >= 64 && nv <= 4096 && ((VG_SWEEP_R16_MASK >> ilog2(nv)) & 1)) ? 16
                                                                               : row32_radix(nv);
}
// threads per CTA of the nv-class row kernel: SWEEP_ROW_BLOCK, or one group
// where a group (nv / radix threads) is larger
__host__ __device__ constexpr int sweep_row_block(int nv) {
  return nv / sweep_row_radix(nv) > SWEEP_ROW_BLOCK ? nv / sweep_row_radix(nv) : SWEEP_ROW_BLOCK;
}
// CTAs per SM of the radix-16 row kernels (16 elements a thread): 3, at 80
// registers with a small spill, runs the 4096-run row pass in 1.37 ms against
// 1.47 ms at 2 CTAs (128 registers)
#ifndef VG_ROW_MIN_BLOCKS_R16
#define VG_ROW_MIN_BLOCKS_R16 3
#endif
__host__ __device__ constexpr int sweep_row_min_blocks(int nv) {
  return sweep_row_radix(nv) == 32   ? VG_ROW_MIN_BLOCKS_R32
         : sweep_row_radix(nv) == 16 ? VG_ROW_MIN_BLOCKS_R16
                                     : VG_ROW_MIN_BLOCKS;
}

struct SweepConsts {
  RowConsts rc[SWEEP_MAX_CLASSES];
  const cx<float>* F0[SWEEP_MAX_CLASSES];
  const double* v64[SWEEP_MAX_CLASSES];
  double c0[SWEEP_MAX_CLASSES];
};

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// x-drift of one (run, tile) item per CTA; one kernel per nx class keeps
// each instantiation's code and registers small.  The tile is nx x W columns
// (W = 2 SWEEP_BLOCK / G, always whole: nv is a multiple of W); each group of
// G = nx/R threads transforms one column pair packed as a complex sequence.
// The lanes of a warp are L different column pairs at the same x (L = 32, or
// fewer when the tile has fewer pairs), so every global access of the tile
// is a contiguous row segment; a group's G threads sit in G/(32/L) warps and
// synchronise by a named barrier of those warps.  The first forward pass
// reads its elements x = t + i G straight from global memory and the last
// inverse pass leaves them in registers, which go straight back, so shared
// memory holds only the passes in between.
__host__ __device__ constexpr int sweep_col_lanes(int nx) {
  return (SWEEP_BLOCK / (nx / sweep_col_radix(nx))) < 32 ? SWEEP_BLOCK / (nx / sweep_col_radix(nx)) : 32;
}
// stride of the groups' sequences in complex elements: odd, so the L lanes
// of a pass access (same index, consecutive groups) fall in distinct bank
// pairs; for nx = 256 (8 lanes of 4 rows) sp_len + 2.  Chosen by counting
// the wavefronts of every pass and of the rotation.
__host__ __device__ constexpr int sweep_col_ld(int nx) {
  return nx == 256 ? sp_len<float>(nx) + 2 : (sp_len<float>(nx) | 1);
}
// shared memory of one x-drift item: the groups' padded sequences, then the
// density-partial scratch (floats)
template <int NX>
__host__ __device__ constexpr size_t sweep_col_work_bytes() {
  return (size_t)(SWEEP_BLOCK / (NX / sweep_col_radix(NX))) * sweep_col_ld(NX) * sizeof(cx<float>) +
         (size_t)(SWEEP_BLOCK / ((NX / sweep_col_radix(NX)) * sweep_col_lanes(NX))) * NX * sizeof(float);
}

// One (run, tile) item of the x-drift.  load(io, x0, stride, c) fills this
// thread's R elements: io[i] = the column pair (c, c + 1) of the tile at
// x = x0 + i stride.
template <int NX, typename LoadFn>
__device__ __forceinline__ void sweep_col_item(const SweepRunDev& r, int tile, float* g,
                                               const SweepConsts* __restrict__ scp,
                                               const cx<float>* __restrict__ tw, float2* dpart,
                                               unsigned char* smem, LoadFn load) {
  constexpr int R = sweep_col_radix(NX);
  constexpr int G = NX / R;
  constexpr int W = sweep_col_w(NX);
  constexpr int L = sweep_col_lanes(NX);
  constexpr int SET = G * L;  // threads of the groups that synchronise together
  constexpr int NSET = SWEEP_BLOCK / SET;
  constexpr int LDG = sweep_col_ld(NX);
  static_assert(W == 2 * (SWEEP_BLOCK / G) && SET % 32 == 0 && NSET <= 15, "tile shape");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int vr = warp * (32 / L) + lane / L;  // this lane's row slot
  const int t = vr & (G - 1), set = vr / G;
  const int grp = (lane & (L - 1)) + L * set;
  cx<float>* sg = reinterpret_cast<cx<float>*>(smem) + (size_t)grp * LDG;
  float* red = reinterpret_cast<float*>(smem + (size_t)(SWEEP_BLOCK / G) * LDG * sizeof(cx<float>));
  const GroupSync sync = {1u + (unsigned)set, (unsigned)SET, 0xffffffffu};
  const int nv = r.nv;
  const int c = tile * W + 2 * grp;  // this group's column pair (c, c + 1)
  float* gc = g + r.g_off + c;
  cx<float> io[R];
  load(io, t, G, 2 * grp);
  block_fft_io<float, NX, false, R, 1>(sg, t, tw, sync, io);
  // theta(m) = m * (-dkx dt) v_col (kx = m dkx on the bins m <= NX/2); the angle
  // per unit m is the double-float product of kdt = -dkx dt and v (both split)
  const float2* vhl = scp->rc[r.cls].vhl;
  const Ang aa = mul_angle(r.kdt, vhl[c]);
  const Ang ab = mul_angle(r.kdt, vhl[c + 1]);
  {
    // phases exp(i m a) for this thread's bins m = t, t+G, ...: one sincos for
    // the start, one for the step, complex products in between
    const float scale = 1.f / NX;
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
  sync();
  block_fft_io<float, NX, true, R, 2>(sg, t, tw, sync, io);
#pragma unroll
  for (int i = 0; i < R; ++i)
    *reinterpret_cast<float2*>(gc + (size_t)(t + i * G) * nv) = make_float2(io[i].x, io[i].y);
  // density partials of the tile: trapz weights (1/2 at the two v end
  // points), summed in FP32 over the L column pairs of a warp row (lanes of
  // equal row slot, by transposition), then over the sets in double-float
  const float wa = (c == 0) ? 0.5f : 1.f, wb = (c + 1 == nv - 1) ? 0.5f : 1.f;
  float d[R];
#pragma unroll
  for (int i = 0; i < R; ++i) d[i] = fmaf(wa, io[i].x, wb * io[i].y);
  int idx;
  bool writer;
  lane_transpose_sum<R, L>(d, lane, idx, writer);
  constexpr int CNT = R > L ? R / L : 1;
  if (writer)
#pragma unroll
    for (int q = 0; q < CNT; ++q) red[set * NX + t + (idx + q) * G] = d[q];
  __syncthreads();
  float2* out = dpart + r.dp_off + (size_t)tile * NX;
  for (int x = threadIdx.x; x < NX; x += SWEEP_BLOCK) {
    df32 acc = {0.f, 0.f};
#pragma unroll
    for (int q = 0; q < NSET; ++q) acc = df_add(acc, {red[q * NX + x], 0.f});
    out[x] = make_float2(acc.hi, acc.lo);
  }
}

template <int NX>
__global__ void __launch_bounds__(SWEEP_BLOCK, sweep_col_min_blocks(NX)) k_sweep_col(const SweepRunDev* __restrict__ runs,
                                                              const int2* __restrict__ items, float* g,
                                                              const SweepConsts* __restrict__ scp,
                                                              const cx<float>* __restrict__ tw, float2* dpart) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int2 it = items[blockIdx.x];
  const SweepRunDev r = runs[it.x];
  constexpr int W = sweep_col_w(NX);
  // the first FFT pass reads its elements straight from global memory
  const float* gt = g + r.g_off + (size_t)it.y * W;
  const int nv = r.nv;
  sweep_col_item<NX>(r, it.y, g, scp, tw, dpart, smem_raw, [&](auto& io, int x0, int stride, int col) {
#pragma unroll
    for (int i = 0; i < (int)(sizeof(io) / sizeof(io[0])); ++i) {
      const float2 q = *reinterpret_cast<const float2*>(gt + (size_t)(x0 + i * stride) * nv + col);
      io[i].x = q.x;
      io[i].y = q.y;
    }
  });
}

// ---- the x-drift fed by the tensor-memory accelerator ----------------------
// For each x class, one tensor map per nv class views the whole state as
// rows of nv floats (every run starts on a row: its cell offset is a multiple
// of its nv), with a box of NX rows x W columns: one (run, tile) item.
// Persistent CTAs walk their items with one tile stage in shared memory: the
// load of a CTA's next item is issued (one thread, cp.async.bulk.tensor,
// completion counted on the stage's mbarrier) as soon as every thread has
// taken the current item's elements into registers, so it overlaps the
// current item's transforms; one stage keeps the kernel at the plain
// kernel's CTAs per SM.  Every wait is bounded: after TMA_WAIT_NS of the
// global timer without the stage's bytes the CTA records the event in *err,
// waits (again bounded) for its copy in flight and stops.
struct SweepTmaps {
  CUtensorMap m[SWEEP_MAX_CLASSES];
};
constexpr unsigned long long TMA_WAIT_NS = 2000000000ull;  // 2 s of the global timer

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// bounded wait for phase `parity` of an mbarrier; false when it ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

template <int NX>
__host__ __device__ constexpr size_t sweep_col_tile_bytes() {
  return (size_t)NX * sweep_col_w(NX) * sizeof(float);
}
// dynamic shared memory of the TMA kernel: the tile stage (128-byte
// aligned), the item work area, the mbarrier
template <int NX>
__host__ __device__ constexpr size_t sweep_col_tma_smem() {
  return 128 + sweep_col_tile_bytes<NX>() + sweep_col_work_bytes<NX>() + 16;
}

template <int NX>
__global__ void __launch_bounds__(SWEEP_BLOCK, sweep_col_min_blocks(NX)) k_sweep_col_tma(
    const SweepRunDev* __restrict__ runs, const int2* __restrict__ items, int n_items, float* g,
    const SweepConsts* __restrict__ scp, const cx<float>* __restrict__ tw, float2* dpart,
    const __grid_constant__ SweepTmaps maps, int* err, unsigned long long wait_ns, int no_loads) {
  constexpr int W = sweep_col_w(NX);
  constexpr uint32_t TILE = (uint32_t)sweep_col_tile_bytes<NX>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((128 - (reinterpret_cast<uintptr_t>(smem_raw) & 127)) & 127);
  const float* tile = reinterpret_cast<const float*>(base);
  unsigned char* work = base + TILE;
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(work + sweep_col_work_bytes<NX>());
  const uint32_t tile0 = (uint32_t)__cvta_generic_to_shared(base);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  // one thread: expect the stage's bytes, then load item idx's box into it
  auto issue = [&](int idx) {
    const int2 it = items[idx];
    const SweepRunDev r = runs[it.x];
    const int cx0 = it.y * W, row0 = (int)(r.g_off / r.nv);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(TILE) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
            tile0),
        "l"(reinterpret_cast<uint64_t>(&maps.m[r.cls])), "r"(cx0), "r"(row0), "r"(bar)
        : "memory");
  };
  const int stride = gridDim.x;
  // (no_loads: a test hook, no tile is ever requested, so every wait runs out)
  if (threadIdx.x == 0 && (int)blockIdx.x < n_items && !no_loads) issue(blockIdx.x);
  uint32_t parity = 0;
  for (int idx = blockIdx.x; idx < n_items; idx += stride, parity ^= 1u) {
    const bool ok = mbar_wait_bounded(bar, parity, wait_ns);
    if (__syncthreads_or(!ok)) {
      // the stage did not fill in time: record it, let the copy in flight
      // land (waiting up to the default limit), stop
      if (threadIdx.x == 0) {
        atomicOr(err, VG_FLAG_TIMEOUT);
        if (!no_loads) mbar_wait_bounded(bar, parity, TMA_WAIT_NS);
      }
      __syncthreads();
      return;
    }
    const int2 it = items[idx];
    const SweepRunDev r = runs[it.x];
    sweep_col_item<NX>(r, it.y, g, scp, tw, dpart, work, [&](auto& io, int x0, int xs, int col) {
#pragma unroll
      for (int i = 0; i < (int)(sizeof(io) / sizeof(io[0])); ++i) {
        const float2 q = *reinterpret_cast<const float2*>(tile + (size_t)(x0 + i * xs) * W + col);
        io[i].x = q.x;
        io[i].y = q.y;
      }
      // every thread has its elements: the stage is free for the next item
      __syncthreads();
      if (threadIdx.x == 0 && idx + stride < n_items && !no_loads) issue(idx + stride);
    });
  }
}

// field solve of up to SWEEP_FIELD_BLOCK/G runs of one nx per CTA
template <int NX>
__device__ __forceinline__ void sweep_field_runs(const SweepRunDev* __restrict__ runs, int first, int count,
                                                 const SweepConsts& sc, const float2* __restrict__ dpart,
                                                 const cx<float>* __restrict__ tw, double* __restrict__ e,
                                                 float* __restrict__ e32, unsigned char* smem, int* flags) {
  constexpr int G = fft_threads<float>(NX);
  const int grp = threadIdx.x / G, t = threadIdx.x - grp * G;
  cx<float>* s = reinterpret_cast<cx<float>*>(smem) + (size_t)grp * sp_len<float>(NX);
  const bool valid = grp < count;
  const SweepRunDev r = runs[valid ? first + grp : first];
  const double dv = sc.rc[r.cls].dv, c0 = sc.c0[r.cls];
  for (int x = t; x < NX; x += G) {
    df32 acc = {0.f, 0.f};
    if (valid)
      for (int p = 0; p < r.ntiles; ++p) {
        const float2 q = dpart[r.dp_off + (size_t)p * NX + x];
        acc = df_add(acc, {q.x, q.y});
      }
    s[sp<float>(x)] = {valid ? (float)(-(dv * df_to_double(acc)) - c0) : 0.f, 0.f};
  }
  __syncthreads();
  block_fft<float, NX, false>(s, t, tw);
  const float scale = 1.f / NX;
  for (int m = t; m < NX; m += G) {
    // 1 / kx with kx = 2 pi fftfreq(nx, dx) = m' k, the zero mode removed
    const int mm = (m < NX / 2) ? m : m - NX;
    const float ik = (m == 0) ? 0.f : (float)(1.0 / ((double)mm * r.k)) * scale;
    const cx<float> z = s[sp<float>(m)];
    s[sp<float>(m)] = {-ik * z.y, ik * z.x};
  }
  __syncthreads();
  block_fft<float, NX, true>(s, t, tw);
  if (valid)
    for (int x = t; x < NX; x += G) {
      const float ex = s[sp<float>(x)].x;
      e[r.x_off + x] = (double)ex;
      e32[r.x_off + x] = ex;
      if (!isfinite(ex)) atomicOr(flags, VG_FLAG_NONFINITE);
    }
}

__global__ void __launch_bounds__(SWEEP_FIELD_BLOCK) k_sweep_field(const SweepRunDev* __restrict__ runs,
                                                                   const int4* __restrict__ items,
                                                                   const SweepConsts* __restrict__ scp,
                                                                   const float2* __restrict__ dpart,
                                                                   const cx<float>* __restrict__ tw,
                                                                   double* __restrict__ e, float* __restrict__ e32,
                                                                   int* flags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int4 it = items[blockIdx.x];  // (nx, first run, count, -)
  const SweepConsts& sc = *scp;
  switch (it.x) {
    case 8: sweep_field_runs<8>(runs, it.y, it.z, sc, dpart, tw, e, e32, smem_raw, flags); break;
    case 16: sweep_field_runs<16>(runs, it.y, it.z, sc, dpart, tw, e, e32, smem_raw, flags); break;
    case 32: sweep_field_runs<32>(runs, it.y, it.z, sc, dpart, tw, e, e32, smem_raw, flags); break;
    case 64: sweep_field_runs<64>(runs, it.y, it.z, sc, dpart, tw, e, e32, smem_raw, flags); break;
    case 128: sweep_field_runs<128>(runs, it.y, it.z, sc, dpart, tw, e, e32, smem_raw, flags); break;
    default: sweep_field_runs<256>(runs, it.y, it.z, sc, dpart, tw, e, e32, smem_raw, flags); break;
  }
}

struct SweepRowArgs {
  float* g;
  const float* e32;
  double* mom;
  double dt1, dt2;
  // -dkv dt / 2 of this launch's nv class: scalars, since indexing a kernel
  // parameter array by the run's class would copy the arguments to the stack
  float hk1, hk2;
  int fp, want_mom, dougherty;
  const cx<float>* tw;
};

// CTAs per SM of the kick-only row kernel (the leading half kick of a call;
// 2 for the radix-32 classes, whose 32 elements a thread need the registers)
#ifndef VG_KICK_MIN_BLOCKS
#define VG_KICK_MIN_BLOCKS 4
#endif
// one (run, row-pair group) item per CTA; one kernel per nv class (KICK:
// the leading half kick alone, a lighter instantiation)
template <int N, bool KICK = false>
__global__ void __launch_bounds__(sweep_row_block(N), KICK ? (sweep_row_radix(N) == 32 ? 2 : VG_KICK_MIN_BLOCKS)
                                                           : sweep_row_min_blocks(N)) k_sweep_row(const SweepRunDev* __restrict__ runs,
                                                              const int2* __restrict__ items, SweepRowArgs sa,
                                                              const SweepConsts* __restrict__ scp) {
  constexpr int R = sweep_row_radix(N);
  constexpr int G = N / R;
  constexpr int P = sweep_row_block(N) / G;
  // whole groups; a group of more than a warp takes named barrier 1 + grp
  static_assert(P * G == sweep_row_block(N) && (G <= 32 || P <= 15), "row-pair groups per CTA");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int2 it = items[blockIdx.x];
  const SweepRunDev r = runs[it.x];
  const int grp = threadIdx.x / G, t = threadIdx.x - grp * G;
  RowArgs a;
  a.g = sa.g + r.g_off;
  a.nx = r.nx;
  a.e32 = sa.e32 + r.x_off;
  a.dt1 = sa.dt1;
  a.dt2 = sa.dt2;
  a.hk1 = sa.hk1;
  a.hk2 = sa.hk2;
  a.fp = sa.fp && r.fp;
  a.dougherty = sa.dougherty;
  a.nudt2 = r.nudt2;
  a.nudt_f = r.nudt_f;
  a.want_mom = sa.want_mom;
  a.mom = sa.mom + (size_t)r.x_off * MOM_STRIDE;
  a.n_modes = 0;
  a.mpart = nullptr;
  a.macc_global = 0;
  a.F0 = scp->F0[r.cls];
  a.tw = sa.tw;
  a.rc = &scp->rc[r.cls];
  // the row-pair groups of a CTA are independent: each synchronises alone
  // the sweep's series use the power moments p = 0, 1, 2 only
  row_pair<N, R, GroupSync, 3, KICK>(a, it.y * P + grp, smem_raw + (size_t)grp * row32_group_bytes(N, R), nullptr,
                                     P, grp, t, GroupSync::of(grp, G));
}

// e history row and the seven series of every run (one CTA per run, one
// row per thread): each warp adds its rows' double-float sums by
// transposition, then seven threads add the four warps' totals in order
__global__ void __launch_bounds__(128) k_sweep_store(const SweepRunDev* __restrict__ runs, int n_runs,
                                                     const SweepConsts* __restrict__ scp,
                                                     const double* __restrict__ mom, const double* __restrict__ e,
                                                     double* __restrict__ e_row, double* __restrict__ s_row) {
  __shared__ df32 red[4][8];
  const SweepRunDev r = runs[blockIdx.x];
  const RowConsts& rc = scp->rc[r.cls];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  df32 acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = {0.f, 0.f};
  for (int x = threadIdx.x; x < r.nx; x += blockDim.x) {
    const double ex = e[r.x_off + x];
    if (e_row) e_row[r.x_off + x] = ex;
    const double* slots = mom + (size_t)(r.x_off + x) * MOM_STRIDE;
    const double src[7] = {row_moment(slots, 0, rc), row_moment(slots, 1, rc), row_moment(slots, 2, rc), ex * ex,
                           0.0, row_moment(slots, 6, rc), row_moment(slots, 7, rc)};
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      const float hi = (float)src[q];
      acc[q] = df_add(acc[q], {hi, (float)(src[q] - (double)hi)});
    }
  }
  int idx;
  bool writer;
  warp_transpose_sum_df<8>(acc, lane, idx, writer);
  if (writer) red[warp][idx] = acc[0];
  __syncthreads();
  if (s_row && threadIdx.x < 7) {
    df32 t = red[0][threadIdx.x];
    for (int w = 1; w < 4; ++w) t = df_add(t, red[w][threadIdx.x]);
    s_row[(size_t)blockIdx.x * 7 + threadIdx.x] = df_to_double(t) / r.nx;
  }
}

// initial state g = A cos(k x_j) M(v) (the x-mean of f = M (1 + A cos k x) is M)
__global__ void k_sweep_init(const SweepRunDev* __restrict__ runs, const double* __restrict__ amp,
                             const SweepConsts* __restrict__ scp, float* __restrict__ g, double* __restrict__ e,
                             float* __restrict__ e32) {
  __shared__ double cx_s[256];  // cos(k x_j) of the run's x points (nx <= 256)
  const SweepRunDev r = runs[blockIdx.x];
  const double A = amp[blockIdx.x];
  const float* f0 = scp->rc[r.cls].f0;
  const size_t n = (size_t)r.nx * r.nv;
  // k x_j = pi (2 j + 1) / nx on the cell-centred grid of [0, 2 pi / k)
  for (int x = threadIdx.x; x < r.nx; x += blockDim.x) cx_s[x] = cospi((2.0 * x + 1.0) / (double)r.nx);
  __syncthreads();
  for (size_t q = threadIdx.x; q < n; q += blockDim.x) {
    const int x = (int)(q / r.nv), vj = (int)(q % r.nv);
    g[r.g_off + q] = (float)(A * cx_s[x] * (double)f0[vj]);
  }
  // the first half-kick of a batch reads the FP32 copy of the field
  for (int x = threadIdx.x; x < r.nx; x += blockDim.x) {
    e[r.x_off + x] = 0.0;
    e32[r.x_off + x] = 0.f;
  }
}

__global__ void k_sweep_e_to_f32(const double* __restrict__ e, int n, float* __restrict__ e32) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) e32[i] = (float)e[i];
}

// Damping rate and frequency of every run from its field history, on the
// device: the amplitude of the first x-Fourier mode per step,
// a_t = |sum_x e_t(x) exp(-2 pi i x / nx)|, its peaks inside [t_min, t_max]
// (interior samples above the previous one and not below the next), each
// refined by a parabola through log a at its three samples, then the
// least-squares slope of log peak height against peak time (the rate) and
// pi over the mean peak spacing (the frequency of a standing wave, whose |E_1|
// peaks twice a period).  Fewer than three peaks give NaN.  One CTA per run;
// dynamic shared memory holds the amplitudes (rows doubles) and the mode's
// twiddles (2 nx doubles).
__global__ void k_sweep_damping(const SweepRunDev* __restrict__ runs, const double* __restrict__ e_hist, int x_points,
                                int rows, double t0, double dt, double t_min, double t_max,
                                double* __restrict__ rate, double* __restrict__ freq) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* amp = reinterpret_cast<double*>(smem_raw);
  double* cw = amp + rows;
  const SweepRunDev r = runs[blockIdx.x];
  double* sw = cw + r.nx;
  for (int x = threadIdx.x; x < r.nx; x += blockDim.x) sincospi(2.0 * x / (double)r.nx, &sw[x], &cw[x]);
  __syncthreads();
  for (int t = threadIdx.x; t < rows; t += blockDim.x) {
    const double* e = e_hist + (size_t)t * x_points + r.x_off;
    double re = 0.0, im = 0.0;
    for (int x = 0; x < r.nx; ++x) {
      re = fma(e[x], cw[x], re);
      im = fma(-e[x], sw[x], im);
    }
    amp[t] = sqrt(re * re + im * im);
  }
  __syncthreads();
  // the window [i0, i1] of samples with t_min <= t <= t_max
  int i0 = (int)ceil((t_min - t0) / dt - 1e-9), i1 = (int)floor((t_max - t0) / dt + 1e-9);
  if (i0 < 0) i0 = 0;
  if (i1 > rows - 1) i1 = rows - 1;
  double n = 0.0, st = 0.0, sl = 0.0, stt = 0.0, stl = 0.0, first = 1e300, last = -1e300;
  for (int j = i0 + 1 + threadIdx.x; j <= i1 - 1; j += blockDim.x) {
    const double a0 = amp[j - 1], a1 = amp[j], a2 = amp[j + 1];
    if (!(a1 > a0 && a1 >= a2) || !(a0 > 0.0) || !(a2 > 0.0)) continue;
    const double y0 = log(a0), y1 = log(a1), y2 = log(a2);
    const double den = y0 - 2.0 * y1 + y2;
    const double off = den != 0.0 ? 0.5 * (y0 - y2) / den : 0.0;
    const double tp = t0 + j * dt + off * dt, lp = y1 - 0.25 * (y0 - y2) * off;
    n += 1.0;
    st += tp;
    sl += lp;
    stt += tp * tp;
    stl += tp * lp;
    first = fmin(first, tp);
    last = fmax(last, tp);
  }
  __shared__ double red[7][32];
  double v[7] = {n, st, sl, stt, stl, first, last};
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    for (int m = 16; m > 0; m >>= 1) {
      const double o = __shfl_xor_sync(0xffffffffu, v[k], m);
      v[k] = k == 5 ? fmin(v[k], o) : (k == 6 ? fmax(v[k], o) : v[k] + o);
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0)
    for (int k = 0; k < 7; ++k) red[k][wid] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    double a[7] = {0, 0, 0, 0, 0, 1e300, -1e300};
    for (int w = 0; w < nw; ++w) {
      for (int k = 0; k < 5; ++k) a[k] += red[k][w];
      a[5] = fmin(a[5], red[5][w]);
      a[6] = fmax(a[6], red[6][w]);
    }
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    if (a[0] < 3.0) {
      rate[blockIdx.x] = nan;
      freq[blockIdx.x] = nan;
    } else {
      const double mt = a[1] / a[0], ml = a[2] / a[0];
      rate[blockIdx.x] = (a[4] - a[0] * mt * ml) / (a[3] - a[0] * mt * mt);
      freq[blockIdx.x] = 3.14159265358979323846 * (a[0] - 1.0) / (a[6] - a[5]);
    }
  }
}

__global__ void k_sweep_read(const SweepRunDev* __restrict__ runs, int run, const SweepConsts* __restrict__ scp,
                             const float* __restrict__ g, const double* __restrict__ f0d, const double* __restrict__ e,
                             double* __restrict__ f_out, double* __restrict__ e_out) {
  const SweepRunDev r = runs[run];
  const size_t n = (size_t)r.nx * r.nv;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    if (f_out) f_out[q] = (double)g[r.g_off + q] + f0d[q % r.nv];
  if (e_out && blockIdx.x == 0)
    for (int x = threadIdx.x; x < r.nx; x += blockDim.x) e_out[x] = e[r.x_off + x];
}

}  // namespace vg

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

using namespace vg;

struct vg_sweep {
  int n_runs, collision;
  double vmax, dt;
  long long cells;
  int x_points;
  std::vector<SweepRunDev> runs_h;
  std::vector<double> amp_h;
  std::vector<int> nv_of_class;
  std::vector<void*> owned;  // device allocations freed at destroy
  // device
  SweepRunDev* runs;
  SweepRunDev* field_runs;  // runs ordered as the field items address them
  double* amp;
  SweepConsts consts_h;
  SweepConsts* consts;
  float* g;
  double* e;
  double* mom;
  float* e32;
  float2* dpart;
  cx<float>* tw32;
  cx<double>* tw64;
  std::vector<double*> f0d;  // per nv class: FP64 background
  // work lists, one per shape class (items of one class are contiguous)
  int2* col_items;
  std::vector<int> col_nx, col_first, col_count;
  int4* field_items;
  int n_field;
  int2* row_items;
  std::vector<int> row_nv, row_first, row_count;
  size_t field_smem;
  std::map<std::tuple<int, const void*, const void*, int, int, cudaStream_t, unsigned>, cudaGraphExec_t> graphs;
  // caller events recorded after each step of a vg_sweep_run_steps call
  // (step k of the call records step_events[k]); events_gen tells the graphs
  // captured with one set of events from those of another
  std::vector<cudaEvent_t> step_events;
  unsigned events_gen = 0;
  ProfState prof;
  // x-drift through the tensor-memory accelerator, per x class
  bool use_tma = false;           // some x class loads its tiles through the TMA
  std::vector<char> tma_x;        // per x class (col_nx order): this class does
  std::vector<SweepTmaps> tmaps;  // per x class, one map per nv class
  int* err = nullptr;             // status bits (VG_FLAG_*): TMA waits that ran out, non-finite fields
  unsigned long long wait_ns = 2000000000ull;  // limit of the TMA x-drift's tile waits
  int lost_tiles = 0;             // test hook: the TMA x-drift requests no tiles
  int n_sm = 0;
  // the size classes of a phase run side by side: side streams that branch
  // from the caller's stream and join it again, and the events that do it
  // ([0] the branch point, [q] the end of side stream q - 1)
  bool concurrent = false;
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> ev;
};

namespace {

#define SW_CHECK(expr)            \
  do {                            \
    int _st = (expr);             \
    if (_st != VG_OK) return _st; \
  } while (0)

template <typename T>
int sw_alloc(vg_sweep* s, T** dst, size_t n, const void* src, const char* what) {
  *dst = nullptr;
  cudaError_t err = cudaMalloc(reinterpret_cast<void**>(dst), std::max<size_t>(n, 1) * sizeof(T));
  if (err != cudaSuccess) return cuda_status(err, what);
  s->owned.push_back(*dst);
  if (src) err = cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
  else err = cudaMemset(*dst, 0, std::max<size_t>(n, 1) * sizeof(T));
  return cuda_status(err, what);
}

void host_fft_sw(std::vector<double>& re, std::vector<double>& im) {
  const size_t n = re.size();
  for (size_t i = 1, j = 0; i < n; ++i) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      std::swap(re[i], re[j]);
      std::swap(im[i], im[j]);
    }
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    const double ang = -2.0 * M_PI / (double)len;
    for (size_t i = 0; i < n; i += len)
      for (size_t k = 0; k < len / 2; ++k) {
        const double c = std::cos(ang * k), sn = std::sin(ang * k);
        const double ur = re[i + k], ui = im[i + k];
        const double vr = re[i + k + len / 2] * c - im[i + k + len / 2] * sn;
        const double vi = re[i + k + len / 2] * sn + im[i + k + len / 2] * c;
        re[i + k] = ur + vr;
        im[i + k] = ui + vi;
        re[i + k + len / 2] = ur - vr;
        im[i + k + len / 2] = ui - vi;
      }
  }
}

// Per-nv constants: the reference's cell-centred grid (linspace of
// vlapy/initializers.py:66), the trapz-normalised Maxwellian background, its
// collision stencils, spectrum and moments.
int sweep_class(vg_sweep* s, int cls, int nv) {
  const double vmax = s->vmax;
  const double dv = 2.0 * vmax / nv;
  std::vector<double> v(nv), f0(nv);
  const double lo = -vmax + dv / 2.0, hi = vmax - dv / 2.0, step = (hi - lo) / (nv - 1);
  for (int j = 0; j < nv; ++j) v[j] = lo + j * step;
  v[nv - 1] = hi;
  double norm = 0.0;
  for (int j = 0; j < nv; ++j) {
    f0[j] = std::exp(-(v[j] * v[j]) / 2.0);
    norm += ((j == 0 || j == nv - 1) ? 0.5 : 1.0) * f0[j];
  }
  norm *= dv;
  for (int j = 0; j < nv; ++j) f0[j] /= norm;
  const double dv2 = dv * dv;
  std::vector<float> v32(nv), f32v(nv), S(nv), Mv(nv), D(nv);
  std::vector<float2> vhl(nv);
  double mom[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int j = 0; j < nv; ++j) {
    vhl[j] = split_f2(v[j]);
    const double fm = j > 0 ? f0[j - 1] : 0.0, fp = j < nv - 1 ? f0[j + 1] : 0.0;
    const double vm = j > 0 ? v[j - 1] : 0.0, vp = j < nv - 1 ? v[j + 1] : 0.0;
    S[j] = (float)((fm - 2.0 * f0[j] + fp) / dv2);
    Mv[j] = (float)((vm * fm - vp * fp) / (2.0 * dv));
    D[j] = (float)((fm - fp) / (2.0 * dv));
    v32[j] = (float)v[j];
    f32v[j] = (float)f0[j];
    const double w = (j == 0 || j == nv - 1) ? 0.5 : 1.0;
    double p = 1.0;
    for (int k = 0; k < 6; ++k) {
      mom[k] += w * f0[j] * p;
      p *= v[j];
    }
    mom[6] += w * f0[j] * f0[j];
  }
  for (int k = 0; k < 7; ++k) mom[k] *= dv;
  std::vector<double> re(f0), im(nv, 0.0);
  host_fft_sw(re, im);
  std::vector<cx<float>> F0(nv / 2 + 1);
  for (int k = 0; k <= nv / 2; ++k) F0[k] = {(float)re[k], (float)im[k]};
  float *dv32, *df0, *dS, *dM, *dD;
  float2* dvhl;
  cx<float>* dF0;
  double *dv64, *df064;
  SW_CHECK(sw_alloc(s, &dv32, nv, v32.data(), "sweep constants"));
  SW_CHECK(sw_alloc(s, &df0, nv, f32v.data(), "sweep constants"));
  SW_CHECK(sw_alloc(s, &dS, nv, S.data(), "sweep constants"));
  SW_CHECK(sw_alloc(s, &dM, nv, Mv.data(), "sweep constants"));
  SW_CHECK(sw_alloc(s, &dD, nv, D.data(), "sweep constants"));
  SW_CHECK(sw_alloc(s, &dF0, F0.size(), F0.data(), "sweep constants"));
  SW_CHECK(sw_alloc(s, &dvhl, vhl.size(), vhl.data(), "sweep constants"));
  SW_CHECK(sw_alloc(s, &dv64, nv, v.data(), "sweep constants"));
  SW_CHECK(sw_alloc(s, &df064, nv, f0.data(), "sweep constants"));
  RowConsts& rc = s->consts_h.rc[cls];
  rc.v = dv32;
  rc.f0 = df0;
  rc.S = dS;
  rc.Mv = dM;
  rc.D = dD;
  rc.vhl = dvhl;
  rc.i2dv = (float)(0.5 / dv);
  rc.v0f = (float)v[0];
  rc.dvf = (float)dv;
  rc.dv = dv;
  rc.dv_sq = dv2;
  rc.dkv = 2.0 * M_PI / (nv * dv);
  for (int k = 0; k < 7; ++k) rc.f0m[k] = mom[k];
  rc.dv2f = split_f2(dv);
  rc.idv2f = split_f2(1.0 / dv2);
  for (int k = 0; k < 3; ++k) rc.f0m2f[k] = split_f2(mom[k]);
  s->consts_h.F0[cls] = dF0;
  s->consts_h.v64[cls] = dv64;
  s->consts_h.c0[cls] = mom[0] - 1.0;
  s->f0d[cls] = df064;
  return VG_OK;
}

void free_sweep(vg_sweep* s) {
  if (!s) return;
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  for (cudaStream_t q : s->side) cudaStreamDestroy(q);
  for (cudaEvent_t e : s->ev) cudaEventDestroy(e);
  for (void* p : s->owned)
    if (p) cudaFree(p);
  delete s;
}

// SK_ROW: a step's row pass with the next step's leading half kick;
// SK_ROW_LAST: the last step's of a call, which ends without it
enum SweepProfKind { SK_KICK = 0, SK_X_DRIFT, SK_FIELD, SK_ROW, SK_STORE, SK_ROW_LAST, SK_COUNT };
const char* const kSweepNames[SK_COUNT] = {"sweep_kick", "sweep_x_drift", "sweep_field", "sweep_row_pass",
                                          "sweep_store", "sweep_row_pass_last"};

template <int NX>
cudaError_t sweep_col_launch(vg_sweep* s, int c, cudaStream_t st) {
  if (s->use_tma && s->tma_x[c]) {
    const size_t smem = sweep_col_tma_smem<NX>();
    cudaError_t err = ensure_smem((const void*)k_sweep_col_tma<NX>, smem);
    if (err != cudaSuccess) return err;
    int per_sm = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_col_tma<NX>, SWEEP_BLOCK, smem);
    if (err != cudaSuccess) return err;
    const int grid = std::max(1, std::min(s->col_count[c], std::max(1, per_sm) * s->n_sm));
    k_sweep_col_tma<NX><<<grid, SWEEP_BLOCK, smem, st>>>(s->runs, s->col_items + s->col_first[c], s->col_count[c],
                                                         s->g, s->consts, s->tw32, s->dpart, s->tmaps[c], s->err,
                                                         s->wait_ns, s->lost_tiles);
    return cudaGetLastError();
  }
  const size_t smem = sweep_col_work_bytes<NX>();
  cudaError_t err = ensure_smem((const void*)k_sweep_col<NX>, smem);
  if (err != cudaSuccess) return err;
  k_sweep_col<NX><<<s->col_count[c], SWEEP_BLOCK, smem, st>>>(s->runs, s->col_items + s->col_first[c], s->g,
                                                              s->consts, s->tw32, s->dpart);
  return cudaGetLastError();
}

template <int N, bool KICK = false>
cudaError_t sweep_row_launch(vg_sweep* s, int c, const SweepRowArgs& a, cudaStream_t st) {
  constexpr int R = sweep_row_radix(N);
  const size_t smem = (size_t)(sweep_row_block(N) / (N / R)) * row32_group_bytes(N, R);
  cudaError_t err = ensure_smem((const void*)k_sweep_row<N, KICK>, smem);
  if (err != cudaSuccess) return err;
  k_sweep_row<N, KICK><<<s->row_count[c], sweep_row_block(N), smem, st>>>(s->runs, s->row_items + s->row_first[c],
                                                                         a, s->consts);
  return cudaGetLastError();
}

// launch(c, stream) for each of the n size classes of one phase (classes in
// ascending size).  With side streams the classes run side by side: the
// largest on st, each other on a side stream that first waits for st's work
// so far, and st waits for every side stream before the next phase (inside a
// stream capture the classes become parallel branches of the graph).  The
// largest class goes first, so its CTAs take the SMs and the smaller classes
// fill what its last wave leaves idle.  The classes touch disjoint runs, so
// the results do not depend on how their kernels overlap.
template <typename Fn>
cudaError_t over_classes(vg_sweep* s, int n, cudaStream_t st, Fn launch) {
  if (!s->concurrent || n <= 1 || n > (int)s->ev.size()) {
    for (int c = 0; c < n; ++c) {
      const cudaError_t err = launch(c, st);
      if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
  }
  cudaError_t err = cudaEventRecord(s->ev[0], st);
  for (int q = 0; q < n && err == cudaSuccess; ++q) {
    cudaStream_t sq = q == 0 ? st : s->side[q - 1];
    if (q > 0) err = cudaStreamWaitEvent(sq, s->ev[0], 0);
    if (err == cudaSuccess) err = launch(n - 1 - q, sq);
    if (err == cudaSuccess && q > 0) err = cudaEventRecord(s->ev[q], sq);
  }
  // join every side stream that branched, also after an error
  for (int q = 1; q < n; ++q) {
    const cudaError_t j = cudaStreamWaitEvent(st, s->ev[q], 0);
    if (err == cudaSuccess) err = j;
  }
  return err;
}

int sweep_setup_streams(vg_sweep* s) {
  const char* off = std::getenv("VG_SWEEP_SERIAL");
  const int n = (int)std::max(s->row_nv.size(), s->col_nx.size());
  if ((off && *off && std::strcmp(off, "0") != 0) || n <= 1) return VG_OK;
  for (int q = 1; q < n; ++q) {
    cudaStream_t side = nullptr;
    SW_CHECK(cuda_status(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking), "sweep streams"));
    s->side.push_back(side);
  }
  for (int q = 0; q < n; ++q) {
    cudaEvent_t e = nullptr;
    SW_CHECK(cuda_status(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "sweep events"));
    s->ev.push_back(e);
  }
  s->concurrent = true;
  return VG_OK;
}

int sweep_sequence(vg_sweep* s, int nsteps, double* e_hist, double* s_hist, int rows, int row0,
                   cudaStream_t st) {
  const double dt = s->dt;
  const int dg = s->collision == VG_COLL_DG;
  auto row = [&](double dt1, double dt2, int fp, int mom, int kind) {
    SweepRowArgs a;
    a.g = s->g;
    a.e32 = s->e32;
    a.mom = s->mom;
    a.dt1 = dt1;
    a.dt2 = dt2;
    a.fp = fp;
    a.want_mom = mom;
    a.dougherty = dg;
    a.tw = s->tw32;
    return cuda_status(prof_call(&s->prof, kind, st, [&] {
                         return over_classes(s, (int)s->row_nv.size(), st, [&](int c, cudaStream_t cs) {
                           cudaError_t err = cudaSuccess;
                           SweepRowArgs ac = a;
                           const int cls = (int)(std::find(s->nv_of_class.begin(), s->nv_of_class.end(),
                                                           s->row_nv[c]) - s->nv_of_class.begin());
                           const double dkv = s->consts_h.rc[cls].dkv;
                           ac.hk1 = (float)(-0.5 * dkv * dt1);
                           ac.hk2 = (float)(-0.5 * dkv * dt2);
                           const bool kick = kind == SK_KICK;
#define VG_ROW_CASE(NV)                                                                       \
  case NV:                                                                                    \
    err = kick ? sweep_row_launch<NV, true>(s, c, ac, cs) : sweep_row_launch<NV>(s, c, ac, cs); \
    break;
                           switch (s->row_nv[c]) {
                             VG_ROW_CASE(64)
                             VG_ROW_CASE(128)
                             VG_ROW_CASE(256)
                             VG_ROW_CASE(512)
                             VG_ROW_CASE(1024)
                             default: err = kick ? sweep_row_launch<2048, true>(s, c, ac, cs)
                                                 : sweep_row_launch<2048>(s, c, ac, cs);
                                      break;
                           }
#undef VG_ROW_CASE
                           return err;
                         });
                       }),
                       "sweep row pass");
  };
  SW_CHECK(row(0.5 * dt, 0.0, 0, 0, SK_KICK));
  for (int k = 0; k < nsteps; ++k) {
    SW_CHECK(cuda_status(prof_call(&s->prof, SK_X_DRIFT, st, [&] {
                           return over_classes(s, (int)s->col_nx.size(), st, [&](int c, cudaStream_t cs) {
                             switch (s->col_nx[c]) {
                               case 8: return sweep_col_launch<8>(s, c, cs);
                               case 16: return sweep_col_launch<16>(s, c, cs);
                               case 32: return sweep_col_launch<32>(s, c, cs);
                               case 64: return sweep_col_launch<64>(s, c, cs);
                               case 128: return sweep_col_launch<128>(s, c, cs);
                               default: return sweep_col_launch<256>(s, c, cs);
                             }
                           });
                         }),
                         "sweep x drift"));
    SW_CHECK(cuda_status(prof_call(&s->prof, SK_FIELD, st, [&] {
                           k_sweep_field<<<s->n_field, SWEEP_FIELD_BLOCK, s->field_smem, st>>>(
                               s->field_runs, s->field_items, s->consts, s->dpart, s->tw32, s->e, s->e32, s->err);
                           return cudaGetLastError();
                         }),
                         "sweep field"));
    const int r = row0 + k;
    const bool store = (e_hist || s_hist) && r >= 0 && r < rows;
    const bool last = k + 1 == nsteps;
    SW_CHECK(row(0.5 * dt, last ? 0.0 : 0.5 * dt, 1, store ? 1 : 0, last ? SK_ROW_LAST : SK_ROW));
    if (store) {
      double* er = e_hist ? e_hist + (size_t)r * s->x_points : nullptr;
      double* sr = s_hist ? s_hist + (size_t)r * s->n_runs * 7 : nullptr;
      SW_CHECK(cuda_status(prof_call(&s->prof, SK_STORE, st, [&] {
                             k_sweep_store<<<s->n_runs, 128, 0, st>>>(s->runs, s->n_runs, s->consts, s->mom, s->e, er, sr);
                             return cudaGetLastError();
                           }),
                           "sweep store"));
    }
    if (k < (int)s->step_events.size() && s->step_events[k]) {
      // under stream capture a plain record only orders the captured work;
      // an external record puts the record itself into the graph, so that
      // every replay records the caller's event
      cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
      SW_CHECK(cuda_status(cudaStreamIsCapturing(st, &cap), "sweep step event"));
      SW_CHECK(cuda_status(cudaEventRecordWithFlags(s->step_events[k], st,
                                                    cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal
                                                                                         : cudaEventRecordDefault),
                           "sweep step event"));
    }
  }
  return VG_OK;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Tensor maps of the TMA x-drift: per x class and nv class, the state as rows
// of nv floats, boxes of nx rows x W columns.  The TMA path is taken when
// every run's cell offset is a multiple of its nv (so that it starts on a
// row), the tile is at most 256 elements along each axis (the box limit), the
// driver exposes cuTensorMapEncodeTiled and VG_SWEEP_NO_TMA is unset or "0";
// otherwise the x-drift loads its tiles with ordinary loads.
int sweep_setup_tma(vg_sweep* s) {
  s->use_tma = false;
  const char* off = std::getenv("VG_SWEEP_NO_TMA");
  if (off && *off && std::strcmp(off, "0") != 0) return VG_OK;
  for (const SweepRunDev& r : s->runs_h)
    if (r.g_off % r.nv != 0 || r.W % 4 != 0) return VG_OK;
  int dev = 0;
  SW_CHECK(cuda_status(cudaGetDevice(&dev), "device"));
  SW_CHECK(cuda_status(cudaDeviceGetAttribute(&s->n_sm, cudaDevAttrMultiProcessorCount, dev), "device"));
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn) {
    cudaGetLastError();
    return VG_OK;
  }
  EncodeTiledFn encode = reinterpret_cast<EncodeTiledFn>(fn);
  s->tmaps.assign(s->col_nx.size(), SweepTmaps{});
  s->tma_x.assign(s->col_nx.size(), 0);
  for (size_t xc = 0; xc < s->col_nx.size(); ++xc) {
    const int nx = s->col_nx[xc];
    std::memset(&s->tmaps[xc], 0, sizeof(SweepTmaps));
    if (sweep_col_w(nx) > 256 || nx > 256) continue;  // a TMA box is at most 256 along each axis
    for (size_t c = 0; c < s->nv_of_class.size(); ++c) {
      const int nv = s->nv_of_class[c];
      if (sweep_col_w(nx) > nv) continue;  // no run of this nx has this nv (nv >= W for every run)
      const cuuint64_t dims[2] = {(cuuint64_t)nv, (cuuint64_t)(s->cells / nv)};
      const cuuint64_t strides[1] = {(cuuint64_t)nv * sizeof(float)};
      const cuuint32_t box[2] = {(cuuint32_t)sweep_col_w(nx), (cuuint32_t)nx};
      const cuuint32_t estr[2] = {1, 1};
      const CUresult rc = encode(&s->tmaps[xc].m[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, s->g, dims, strides, box,
                                 estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (rc != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)rc) + ") for the x-drift tile of nx=" +
                  std::to_string(nx) + ", nv=" + std::to_string(nv));
        return VG_ERR_CUDA;
      }
    }
    s->tma_x[xc] = 1;
    s->use_tma = true;
  }
  return VG_OK;
}

}  // namespace

extern "C" {

int vg_sweep_create(const vg_sweep_desc* d, vg_sweep** out) {
  if (!d || !out || d->n_runs <= 0 || !d->runs || !(d->vmax > 0.0)) {
    set_error("bad sweep descriptor");
    return VG_ERR_ARG;
  }
  if (d->collision != VG_COLL_DG && d->collision != VG_COLL_LB) {
    set_error("sweep collision operator must be VG_COLL_DG or VG_COLL_LB");
    return VG_ERR_ARG;
  }
  *out = nullptr;
  vg_sweep* s = new vg_sweep();
  s->n_runs = d->n_runs;
  s->collision = d->collision;
  s->vmax = d->vmax;
  s->dt = d->dt;
  std::memset(&s->consts_h, 0, sizeof(SweepConsts));
  std::map<int, int> cls_of;
  long long cells = 0, dp = 0;
  int xoff = 0;
  for (int i = 0; i < d->n_runs; ++i) {
    const vg_sweep_run& q = d->runs[i];
    if (!is_pow2(q.nx) || !is_pow2(q.nv) || q.nx < 8 || q.nx > 256 || q.nv < 64 || q.nv > 2048 ||
        q.nv < sweep_col_w(q.nx) || !(q.k > 0.0) || !(q.nu >= 0.0)) {
      set_error("sweep run " + std::to_string(i) + ": needs power-of-two nx in [8, 256], nv in [64, 2048], " +
                "nv >= the column tile width 4096/nx, k > 0 and nu >= 0");
      free_sweep(s);
      return VG_ERR_UNSUPPORTED;
    }
    if (!cls_of.count(q.nv)) {
      if ((int)cls_of.size() == SWEEP_MAX_CLASSES) {
        set_error("too many distinct nv in one sweep");
        free_sweep(s);
        return VG_ERR_UNSUPPORTED;
      }
      const int c = (int)cls_of.size();
      cls_of[q.nv] = c;
      s->nv_of_class.push_back(q.nv);
    }
    SweepRunDev r;
    r.nx = q.nx;
    r.nv = q.nv;
    r.cls = cls_of[q.nv];
    r.W = sweep_col_w(q.nx);
    r.ntiles = q.nv / r.W;
    r.fp = q.nu > 0.0;
    r.g_off = cells;
    r.x_off = xoff;
    r.dp_off = dp;
    r.k = q.k;
    r.nudt = q.nu * d->dt;
    r.kdt = split_f2(-q.k * d->dt);
    r.nudt_f = (float)r.nudt;
    r.nudt2 = split_f2(r.nudt);
    cells += (long long)q.nx * q.nv;
    xoff += q.nx;
    dp += (long long)r.ntiles * q.nx;
    s->runs_h.push_back(r);
    s->amp_h.push_back(q.amplitude);
  }
  s->cells = cells;
  s->x_points = xoff;
  s->f0d.resize(s->nv_of_class.size());
  int st = VG_OK;
#define SW_TRY(expr)   \
  do {                 \
    st = (expr);       \
    if (st != VG_OK) { \
      free_sweep(s);   \
      return st;       \
    }                  \
  } while (0)
  for (size_t c = 0; c < s->nv_of_class.size(); ++c) SW_TRY(sweep_class(s, (int)c, s->nv_of_class[c]));
  SW_TRY(sw_alloc(s, &s->runs, s->runs_h.size(), s->runs_h.data(), "sweep runs"));
  SW_TRY(sw_alloc(s, &s->amp, s->amp_h.size(), s->amp_h.data(), "sweep runs"));
  SW_TRY(sw_alloc(s, &s->consts, 1, &s->consts_h, "sweep constants"));
  SW_TRY(sw_alloc<float>(s, &s->g, (size_t)cells, nullptr, "sweep state"));
  SW_TRY(sw_alloc<double>(s, &s->e, (size_t)xoff, nullptr, "sweep fields"));
  SW_TRY(sw_alloc<double>(s, &s->mom, (size_t)xoff * MOM_STRIDE, nullptr, "sweep moments"));
  SW_TRY(sw_alloc<float>(s, &s->e32, (size_t)xoff, nullptr, "sweep fields"));
  SW_TRY(sw_alloc<float2>(s, &s->dpart, (size_t)dp, nullptr, "sweep density partials"));
  SW_TRY(sw_alloc<cx<double>>(s, &s->tw64, FFT_NMAX, nullptr, "twiddles"));
  SW_TRY(sw_alloc<cx<float>>(s, &s->tw32, FFT_NMAX, nullptr, "twiddles"));
  {
    vg_plan tmp;
    std::memset(&tmp, 0, sizeof(tmp));
    tmp.tw64 = s->tw64;
    tmp.tw32 = s->tw32;
    SW_TRY(cuda_status(launch_twiddles(tmp, 0), "twiddles"));
  }
  // work lists and shared-memory sizes: (run, tile) items grouped by nx,
  // (run, row-pair group) items grouped by nv, field items by nx
  std::map<int, std::vector<int2>> col_by, row_by;
  std::vector<int4> field;
  std::vector<SweepRunDev> field_runs;
  size_t field_smem = 0;
  std::map<int, std::vector<int>> by_nx;
  for (int i = 0; i < s->n_runs; ++i) {
    const SweepRunDev& r = s->runs_h[i];
    for (int t = 0; t < r.ntiles; ++t) col_by[r.nx].push_back(make_int2(i, t));
    const int G = r.nv / sweep_row_radix(r.nv);
    const int P = sweep_row_block(r.nv) / G;
    for (int pg = 0; pg * P < r.nx / 2; ++pg) row_by[r.nv].push_back(make_int2(i, pg));
    by_nx[r.nx].push_back(i);
  }
  std::vector<int2> col, row;
  for (auto& kv : col_by) {
    s->col_nx.push_back(kv.first);
    s->col_first.push_back((int)col.size());
    s->col_count.push_back((int)kv.second.size());
    col.insert(col.end(), kv.second.begin(), kv.second.end());
  }
  for (auto& kv : row_by) {
    s->row_nv.push_back(kv.first);
    s->row_first.push_back((int)row.size());
    s->row_count.push_back((int)kv.second.size());
    row.insert(row.end(), kv.second.begin(), kv.second.end());
  }
  for (auto& kv : by_nx) {
    const int nx = kv.first;
    const int per = SWEEP_FIELD_BLOCK / fft_threads<float>(nx);
    field_smem = std::max(field_smem, (size_t)per * sp_len<float>(nx) * sizeof(cx<float>));
    const auto& ids = kv.second;
    for (size_t b = 0; b < ids.size(); b += per) {
      const int cnt = (int)std::min<size_t>(per, ids.size() - b);
      field.push_back(make_int4(nx, (int)field_runs.size(), cnt, 0));
      for (int q = 0; q < cnt; ++q) field_runs.push_back(s->runs_h[ids[b + q]]);
    }
  }
  SW_TRY(sw_alloc(s, &s->col_items, col.size(), col.data(), "sweep work list"));
  SW_TRY(sw_alloc(s, &s->row_items, row.size(), row.data(), "sweep work list"));
  SW_TRY(sw_alloc(s, &s->field_items, field.size(), field.data(), "sweep work list"));
  SW_TRY(sw_alloc(s, &s->field_runs, field_runs.size(), field_runs.data(), "sweep work list"));
  s->n_field = (int)field.size();
  s->field_smem = field_smem;
  SW_TRY(cuda_status(ensure_smem((const void*)k_sweep_field, field_smem), "sweep smem"));
  SW_TRY(sw_alloc<int>(s, &s->err, 1, nullptr, "sweep status"));
  SW_TRY(sweep_setup_tma(s));
  SW_TRY(sweep_setup_streams(s));
  SW_TRY(cuda_status(cudaDeviceSynchronize(), "sweep setup"));
#undef SW_TRY
  *out = s;
  return VG_OK;
}

int vg_sweep_destroy(vg_sweep* s) {
  if (!s) return VG_OK;
  cudaDeviceSynchronize();
  free_sweep(s);
  return VG_OK;
}

int vg_sweep_sizes(const vg_sweep* s, int64_t* cells, int64_t* x_points) {
  if (!s) {
    set_error("null sweep");
    return VG_ERR_ARG;
  }
  if (cells) *cells = s->cells;
  if (x_points) *x_points = s->x_points;
  return VG_OK;
}

int vg_sweep_x_offsets(const vg_sweep* s, int64_t* out) {
  if (!s || !out) {
    set_error("null sweep or output");
    return VG_ERR_ARG;
  }
  for (int i = 0; i < s->n_runs; ++i) out[i] = s->runs_h[i].x_off;
  return VG_OK;
}

int vg_sweep_reset(vg_sweep* s, vg_stream stream) {
  if (!s) {
    set_error("null sweep");
    return VG_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  k_sweep_init<<<s->n_runs, 256, 0, st>>>(s->runs, s->amp, s->consts, s->g, s->e, s->e32);
  return cuda_status(cudaGetLastError(), "sweep reset");
}

int vg_sweep_run_steps(vg_sweep* s, int32_t nsteps, double* e_hist, double* series_hist, int32_t hist_rows,
                       int32_t hist_row0, int32_t use_graph, vg_stream stream) {
  if (!s || nsteps < 0 || hist_rows < 0) {
    set_error("null sweep or negative counts");
    return VG_ERR_ARG;
  }
  if (nsteps == 0) return VG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (s->prof.enabled || !use_graph) return sweep_sequence(s, nsteps, e_hist, series_hist, hist_rows, hist_row0, st);
  if (st == 0) {
    set_error("graph mode needs a non-default stream");
    return VG_ERR_ARG;
  }
  const auto key =
      std::make_tuple(nsteps, (const void*)e_hist, (const void*)series_hist, hist_rows, hist_row0, st, s->events_gen);
  auto it = s->graphs.find(key);
  if (it == s->graphs.end()) {
    SW_CHECK(cuda_status(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed), "begin capture"));
    const int rc = sweep_sequence(s, nsteps, e_hist, series_hist, hist_rows, hist_row0, st);
    cudaGraph_t graph = nullptr;
    cudaError_t err = cudaStreamEndCapture(st, &graph);
    if (rc != VG_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    SW_CHECK(cuda_status(err, "end capture"));
    cudaGraphExec_t exec = nullptr;
    err = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    SW_CHECK(cuda_status(err, "graph instantiate"));
    it = s->graphs.emplace(key, exec).first;
  }
  return cuda_status(cudaGraphLaunch(it->second, st), "graph launch");
}

int vg_sweep_set_step_events(vg_sweep* s, void* const* events, int32_t n) {
  if (!s || n < 0 || (n > 0 && !events)) {
    set_error("null sweep, negative count or null event array");
    return VG_ERR_ARG;
  }
  s->step_events.assign(n, nullptr);
  for (int k = 0; k < n; ++k) s->step_events[k] = (cudaEvent_t)events[k];
  ++s->events_gen;
  // graphs captured before record the previous events (or none) and are
  // never replayed again: free them (one still in flight is freed when it
  // completes)
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  return VG_OK;
}

int vg_sweep_read_run(vg_sweep* s, int32_t run, double* f_out, double* e_out, vg_stream stream) {
  if (!s || run < 0 || run >= s->n_runs) {
    set_error("null sweep or run index out of range");
    return VG_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const SweepRunDev& r = s->runs_h[run];
  k_sweep_read<<<64, 256, 0, st>>>(s->runs, run, s->consts, s->g, s->f0d[r.cls], s->e, f_out, e_out);
  return cuda_status(cudaGetLastError(), "sweep read");
}

int vg_sweep_get_state(vg_sweep* s, float* g_out, double* e_out, vg_stream stream) {
  if (!s) {
    set_error("null sweep");
    return VG_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (g_out)
    SW_CHECK(cuda_status(cudaMemcpyAsync(g_out, s->g, (size_t)s->cells * sizeof(float), cudaMemcpyDeviceToDevice, st),
                         "sweep get state"));
  if (e_out)
    SW_CHECK(cuda_status(cudaMemcpyAsync(e_out, s->e, (size_t)s->x_points * sizeof(double),
                                         cudaMemcpyDeviceToDevice, st),
                         "sweep get state"));
  return VG_OK;
}

int vg_sweep_set_state(vg_sweep* s, const float* g_in, const double* e_in, vg_stream stream) {
  if (!s) {
    set_error("null sweep");
    return VG_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (g_in)
    SW_CHECK(cuda_status(cudaMemcpyAsync(s->g, g_in, (size_t)s->cells * sizeof(float), cudaMemcpyDeviceToDevice, st),
                         "sweep set state"));
  if (e_in) {
    SW_CHECK(cuda_status(cudaMemcpyAsync(s->e, e_in, (size_t)s->x_points * sizeof(double),
                                         cudaMemcpyDeviceToDevice, st),
                         "sweep set state"));
    k_sweep_e_to_f32<<<div_up((int)s->x_points, 256), 256, 0, st>>>(s->e, (int)s->x_points, s->e32);
    SW_CHECK(cuda_status(cudaGetLastError(), "sweep set state"));
  }
  return VG_OK;
}

int vg_sweep_damping(vg_sweep* s, const double* e_hist, int32_t rows, double t0, double t_min, double t_max,
                     double* rate_out, double* freq_out, vg_stream stream) {
  if (!s || !e_hist || !rate_out || !freq_out || rows < 3 || rows > 16384 || !(t_max > t_min)) {
    set_error("sweep damping: needs a history of 3..16384 rows, outputs and t_min < t_max");
    return VG_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const size_t smem = (size_t)rows * sizeof(double) + 2 * 256 * sizeof(double);
  SW_CHECK(cuda_status(ensure_smem((const void*)k_sweep_damping, smem), "sweep damping"));
  k_sweep_damping<<<s->n_runs, 256, smem, st>>>(s->runs, e_hist, (int)s->x_points, rows, t0, s->dt, t_min, t_max,
                                                 rate_out, freq_out);
  return cuda_status(cudaGetLastError(), "sweep damping");
}

int vg_sweep_status(vg_sweep* s, int32_t* flags, int32_t* uses_tma) {
  if (!s) {
    set_error("null sweep");
    return VG_ERR_ARG;
  }
  int h = 0;
  SW_CHECK(cuda_status(cudaDeviceSynchronize(), "sweep status"));
  SW_CHECK(cuda_status(cudaMemcpy(&h, s->err, sizeof(int), cudaMemcpyDeviceToHost), "sweep status"));
  if (flags) *flags = h;
  if (uses_tma) *uses_tma = s->use_tma ? 1 : 0;
  if (h & VG_FLAG_TIMEOUT) {
    set_error("a bounded wait of the TMA x-drift ran out (the steps it ended are not valid)");
    return VG_ERR_TIMEOUT;
  }
  if (h & VG_FLAG_NONFINITE) {
    set_error("a field solve produced NaN or Inf (the steps from it on are not valid)");
    return VG_ERR_NUMERIC;
  }
  return VG_OK;
}

int vg_sweep_set_wait_limit(vg_sweep* s, int64_t ns) {
  if (!s || ns < 0) {
    set_error("null sweep or negative wait limit");
    return VG_ERR_ARG;
  }
  s->wait_ns = (unsigned long long)ns;
  // graphs captured before hold the old limit as a kernel argument
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  return VG_OK;
}

int vg_sweep_inject_lost_tiles(vg_sweep* s, int32_t on) {
  if (!s) {
    set_error("null sweep");
    return VG_ERR_ARG;
  }
  s->lost_tiles = on ? 1 : 0;
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  return VG_OK;
}

int vg_sweep_state_ptr(vg_sweep* s, float** g, double** e) {
  if (!s) {
    set_error("null sweep");
    return VG_ERR_ARG;
  }
  if (g) *g = s->g;
  if (e) *e = s->e;
  return VG_OK;
}

int vg_sweep_profile_enable(vg_sweep* s, int32_t enable) {
  if (!s) {
    set_error("null sweep");
    return VG_ERR_ARG;
  }
  s->prof.enabled = enable != 0;
  return VG_OK;
}

int vg_sweep_profile_read(vg_sweep* s, vg_prof_entry* out, int32_t max, int32_t* n_out) {
  if (!s || !n_out || (max > 0 && !out)) {
    set_error("null sweep or output");
    return VG_ERR_ARG;
  }
  const double cells = (double)s->cells;
  const double bytes[SK_COUNT] = {8.0 * cells, 8.0 * cells, 8.0 * 2.0 * s->x_points, 8.0 * cells,
                                  8.0 * 9.0 * s->x_points, 8.0 * cells};
  int n = 0;
  SW_CHECK(prof_collect(&s->prof, SK_COUNT, kSweepNames, bytes, out, max, &n));
  *n_out = n;
  return VG_OK;
}

}  // extern "C"
