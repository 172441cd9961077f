// Shared-memory Stockham FFT for one CTA-cooperative complex sequence.
//
// A length-N sequence (N a power of two, 2..16384) lives in shared memory.
// N/R threads cooperate on it: every pass each thread loads R (or fewer, on
// the last, shorter-radix pass) elements with stride N/r, applies the
// twiddles exp(-+2 pi i m k / (Ns r)), does a radix-r DFT in registers and
// writes the results back in Stockham autosort order, so the output is in
// natural order with no bit reversal.  All sequences of a CTA run the same
// passes in lockstep and synchronise with __syncthreads, so every thread of
// the CTA must call the transform.
//
// Twiddles come from one table built once per plan (sincospi in FP64),
// ordered by span: for every power of two L = 2..FFT_NMAX it holds
// exp(-2 pi i k / L), k = 0..L/2-1, at index L/2 - 1 + k (tw_index).  The
// twiddle w^(m k) of span Ns r is entry k of span Ns r / m, so the threads of
// a pass (consecutive k) load consecutive entries: one coalesced load per m.
//
// The passes synchronise through a policy object: CtaSync (__syncthreads,
// every thread of the CTA calls the transform) or GroupSync (only the
// threads that share the sequence: a named barrier for groups of whole
// warps, __syncwarp for a group inside one warp), which lets the sequences of
// a CTA run their passes independently.
#pragma once

#include "vg_common.cuh"

namespace vg {

struct CtaSync {
  static constexpr bool cta_wide = true;
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct GroupSync {
  static constexpr bool cta_wide = false;
  unsigned id;     // named barrier (1..15) of a group of count > 32 threads
  unsigned count;  // threads in the group: a multiple of 32, or a divisor of 32
  unsigned mask;   // the group's lanes when count <= 32
  __device__ __forceinline__ void operator()() const {
    if (count > 32) asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(count) : "memory");
    else __syncwarp(mask);
  }
  // the sync of group grp of g threads, groups laid out back to back
  static __device__ __forceinline__ GroupSync of(int grp, int g) {
    GroupSync s;
    s.id = 1u + (unsigned)grp;
    s.count = (unsigned)g;
    s.mask = g >= 32 ? 0xffffffffu : (((1u << g) - 1u) << ((grp * g) & 31));
    return s;
  }
};

constexpr int FFT_LOG_NMAX = 14;
constexpr int FFT_NMAX = 1 << FFT_LOG_NMAX;

// Radix used per pass for a length-N transform of element type T: the whole
// sequence in one thread for N <= 8, otherwise radix 8, or radix 16 where
// radix 8 would need more than 256 (FP64) / 1024 (FP32) threads per sequence
// and so cap the registers per thread.
template <typename T>
__host__ __device__ constexpr int fft_radix(int n) {
  return n <= 8 ? n : (sizeof(T) == 8 ? (n <= 2048 ? 8 : 16) : (n <= 8192 ? 8 : 16));
}
template <typename T>
__host__ __device__ constexpr int fft_threads(int n) { return n / fft_radix<T>(n); }
// CTA sizes of the row (pairs of rows) and column (tiles of columns) kernels
template <typename T>
__host__ __device__ constexpr int row_block(int n) {
  return fft_threads<T>(n) >= 256 ? fft_threads<T>(n) : 256;
}
template <typename T>
__host__ __device__ constexpr int col_seqs(int nx) {
  return (256 / fft_threads<T>(nx) >= 2) ? 256 / fft_threads<T>(nx)
       : (2 * fft_threads<T>(nx) <= 512 ? 2 : 1);
}

// Shared-memory layout of a sequence: one padding element after every 8
// (complex double) or 16 (complex float) elements, so that the stride-r
// Stockham writes and the contiguous per-thread chunks of the tridiagonal
// solver fall in distinct banks.
// one pad element per 2^shift elements (FP32 value: build-time knob)
#ifndef VG_PAD_SHIFT_F32
#define VG_PAD_SHIFT_F32 4
#endif
template <typename T>
__host__ __device__ constexpr int pad_shift() { return sizeof(T) == 8 ? 3 : VG_PAD_SHIFT_F32; }
template <typename T, int PS = pad_shift<T>()>
__device__ __forceinline__ int sp(int i) { return i + (i >> PS); }
template <typename T, int PS = pad_shift<T>()>
__host__ __device__ constexpr int sp_len(int n) { return n + (n >> PS); }
// The FP32 row kernels on radix-32 passes pad one element per 32 instead:
// their stride-32 accesses (the first pass's stores, the solve's 32-element
// chunks) then step 33 elements, an odd count, and fall in distinct bank pairs,
// where the one-per-16 layout makes them step 34 (a 4-way bank conflict).
__host__ __device__ constexpr int row_pad_shift(int r) { return r == 32 ? 5 : pad_shift<float>(); }
// Padded offset of element base + m * S, m = 0..r-1, as sp(base) plus a
// compile-time constant per m wherever the pad pattern allows (CASE):
//  1: S a multiple of the pad period P: sp(base) + m (S + S/P);
//  2: base mod P < S (with S | P), or S = 1 and base a multiple of r (r | P):
//     no pad boundary falls between base and base + m S other than those
//     of m S itself, so sp(base) + m S + (m S) / P;
//  0: otherwise the element's own sp().
template <typename T, int S, int CASE, int PS = pad_shift<T>()>
__device__ __forceinline__ int sp_step(int spbase, int base, int m) {
  constexpr int P = 1 << PS;
  if constexpr (CASE == 1) return spbase + m * (S + S / P);
  else if constexpr (CASE == 2) return spbase + m * S + ((m * S) >> PS);
  else return sp<T, PS>(base + m * S);
}

// multiply by exp(-+2 pi i k / R), forward sign '-' unless INV
template <typename T, int R, bool INV>
__device__ __forceinline__ cx<T> rot_const(int k, cx<T> a) {
  static_assert(R >= 1 && 32 % R == 0, "the rotation table covers radices dividing 32");
  if (k == 0) return a;
  if (4 * k == R) return INV ? cx<T>{-a.y, a.x} : cx<T>{a.y, -a.x};
  const int j = (32 / R) * k;
  const T c = (T)cos32(j), s = (T)sin32(j);
  if (INV) return {a.x * c - a.y * s, a.x * s + a.y * c};
  return {a.x * c + a.y * s, a.y * c - a.x * s};
}

template <typename T, int R, bool INV>
struct Dft {
  static __device__ __forceinline__ void run(cx<T>* a) {
    cx<T> e[R / 2], o[R / 2];
#pragma unroll
    for (int i = 0; i < R / 2; ++i) {
      e[i] = a[2 * i];
      o[i] = a[2 * i + 1];
    }
    Dft<T, R / 2, INV>::run(e);
    Dft<T, R / 2, INV>::run(o);
#pragma unroll
    for (int k = 0; k < R / 2; ++k) {
      const cx<T> t = rot_const<T, R, INV>(k, o[k]);
      a[k] = e[k] + t;
      a[k + R / 2] = e[k] - t;
    }
  }
};
template <typename T, bool INV>
struct Dft<T, 2, INV> {
  static __device__ __forceinline__ void run(cx<T>* a) {
    const cx<T> t = a[0];
    a[0] = t + a[1];
    a[1] = t - a[1];
  }
};
template <typename T, bool INV>
struct Dft<T, 1, INV> {
  static __device__ __forceinline__ void run(cx<T>*) {}
};

// index of exp(-2 pi i k / L) in the span-ordered table (L a power of two,
// 0 <= k < L/2)
__host__ __device__ constexpr int tw_index(int L, int k) { return L / 2 - 1 + k; }

// the table entry q: its span L = 2h (h the largest power of two <= q + 1)
// and k = q + 1 - h, so the entry is exp(-2 pi i k / L) = exp(-i pi k / h)
__host__ __device__ inline void tw_entry(int q, int& k, int& h) {
  h = 1;
  while (2 * h <= q + 1) h *= 2;
  k = q + 1 - h;
}

template <typename T>
__device__ __forceinline__ cx<T> twiddle(const cx<T>* __restrict__ tw, int q, bool inv) {
  cx<T> w = tw[q];
  if (inv) w.y = -w.y;
  return w;
}

// One Stockham pass and the ones after it.  IO bit 0: the first pass takes
// its inputs from the caller's registers io (thread t's elements t + i N/R,
// exactly what that pass reads) instead of shared memory; bit 1: the last
// pass leaves its outputs in io (again elements t + i N/R) instead of
// writing them back.  Either saves one round trip through shared memory.
template <typename T, int N, int R, bool INV, int NS, int IO = 0, int PS = pad_shift<T>()>
struct StockhamPass {
  template <typename Sync>
  static __device__ __forceinline__ void run(cx<T>* s, int t, const cx<T>* __restrict__ tw, const Sync& sync,
                                             cx<T> (&io)[R]) {
    constexpr int r = (N / NS < R) ? (N / NS) : R;
    constexpr int NB = N / r;      // butterflies in this pass
    constexpr int G = N / R;       // threads per sequence
    constexpr int BPT = NB / G;    // butterflies per thread
    constexpr bool from_regs = (IO & 1) && NS == 1;
    constexpr bool to_regs = (IO & 2) && NS * r == N;
    static_assert(!from_regs || (BPT == 1 && r == R), "the first pass reads one radix-R butterfly per thread");
    constexpr int PP = 1 << PS;
    // loads: element j + m NB; NB a multiple of the pad period makes the
    // offsets constant past sp(j)
    constexpr int LCASE = (NB % PP == 0) ? 1 : 0;
    // stores: element base + m NS with base = (j - k) r + k: for NS = 1 base
    // is a multiple of r; for NS r >= P, base mod P = k < NS
    constexpr int SCASE = (NS % PP == 0) ? 1 : ((NS == 1 && PP % r == 0) || (PP % NS == 0 && NS * r >= PP)) ? 2 : 0;
    cx<T> a[BPT][r];
#pragma unroll
    for (int b = 0; b < BPT; ++b) {
      const int j = t + b * G;
      const int k = j & (NS - 1);
      const int spj = sp<T, PS>(j);
#pragma unroll
      for (int m = 0; m < r; ++m) {
        if constexpr (from_regs) a[b][m] = io[m];
        else a[b][m] = s[sp_step<T, NB, LCASE, PS>(spj, j, m)];
      }
      if (NS > 1) {
        // twiddles w^m: the power-of-two m from the table, the others as
        // products of those (one extra rounding), halving the table loads
        cx<T> w[r];
#pragma unroll
        for (int m = 1; m < r; m <<= 1) w[m] = twiddle(tw, tw_index(NS * r / m, k), INV);
#pragma unroll
        for (int m = 3; m < r; ++m)
          if (m & (m - 1)) w[m] = cmul(w[m & (m - 1)], w[m & -m]);
#pragma unroll
        for (int m = 1; m < r; ++m) a[b][m] = cmul(a[b][m], w[m]);
      }
      Dft<T, r, INV>::run(a[b]);
    }
    if constexpr (to_regs) {
      // outputs base + m NS with base = j = t + b G, i.e. elements t + G (b + m BPT)
#pragma unroll
      for (int b = 0; b < BPT; ++b)
#pragma unroll
        for (int m = 0; m < r; ++m) io[b + m * BPT] = a[b][m];
    } else {
      sync();
#pragma unroll
      for (int b = 0; b < BPT; ++b) {
        const int j = t + b * G;
        const int k = j & (NS - 1);
        const int base = (j - k) * r + k;
        const int spb = sp<T, PS>(base);
#pragma unroll
        for (int m = 0; m < r; ++m) s[sp_step<T, NS, SCASE, PS>(spb, base, m)] = a[b][m];
      }
      sync();
      StockhamPass<T, N, R, INV, NS * r, IO, PS>::run(s, t, tw, sync, io);
    }
  }
};
template <typename T, int N, int R, bool INV, int IO, int PS>
struct StockhamPass<T, N, R, INV, N, IO, PS> {
  template <typename Sync>
  static __device__ __forceinline__ void run(cx<T>*, int, const cx<T>* __restrict__, const Sync&, cx<T> (&)[R]) {}
};

// In-place unnormalised transform of s[0..N) by the N/R threads t = 0..N/R-1
// (R defaults to fft_radix<T>(N)).  Caller must have synchronised after
// writing s; the result is visible to the synchronised threads on return.
template <typename T, int N, bool INV, int R = fft_radix<T>(N), typename Sync = CtaSync>
__device__ __forceinline__ void block_fft(cx<T>* s, int t, const cx<T>* __restrict__ tw, const Sync& sync = Sync()) {
  constexpr int RR = R < N ? R : N;
  cx<T> unused[RR];
  StockhamPass<T, N, RR, INV, 1, 0>::run(s, t, tw, sync, unused);
}
// The same with register input (IO = 1: io holds elements t + i N/R, s need
// not hold the sequence) or register output (IO = 2: the result's elements
// t + i N/R end in io and s is left as scratch).
template <typename T, int N, bool INV, int R, int IO, typename Sync, int PS = pad_shift<T>()>
__device__ __forceinline__ void block_fft_io(cx<T>* s, int t, const cx<T>* __restrict__ tw, const Sync& sync,
                                             cx<T> (&io)[R]) {
  static_assert(R <= N, "radix larger than the sequence");
  StockhamPass<T, N, R, INV, 1, IO, PS>::run(s, t, tw, sync, io);
}

// Two real sequences a, b packed as z = a + i b; s holds Z = FFT(z).  Replace
// it by FFT(a' + i b') where a' = Re IFFT(Pa . FFT(a)), b' likewise, and
// P(k) = cos(th(k)) + i sin(th(k)).  At the Nyquist bin only Re(P) acts,
// which is what taking the real part of the inverse transform does to the
// reference's full complex product.  phase(k, &ca, &sa, &cb, &sb) returns the
// two rotations for bin k.
template <typename T, typename PhaseFn>
__device__ __forceinline__ void two_real_rotate(cx<T>* s, int N, int t, int G, PhaseFn phase) {
  for (int k = t; k <= N / 2; k += G) {
    T ca, sa, cb, sb;
    // one phase() call per visited bin, in increasing k (callers may step a
    // recurrence inside it)
    phase(k, ca, sa, cb, sb);
    if (k == 0) {
      const cx<T> z = s[0];
      // DC bins of both real sequences are real: only Re(P) survives
      s[0] = {z.x * ca, z.y * cb};
      continue;
    }
    if (2 * k == N) {
      const cx<T> z = s[sp<T>(k)];
      s[sp<T>(k)] = {z.x * ca, z.y * cb};
      continue;
    }
    const cx<T> zk = s[sp<T>(k)], zm = s[sp<T>(N - k)];
    const cx<T> fa = {(zk.x + zm.x) * T(0.5), (zk.y - zm.y) * T(0.5)};
    const cx<T> fb = {(zk.y + zm.y) * T(0.5), (zm.x - zk.x) * T(0.5)};
    const cx<T> ga = {ca * fa.x - sa * fa.y, ca * fa.y + sa * fa.x};
    const cx<T> gb = {cb * fb.x - sb * fb.y, cb * fb.y + sb * fb.x};
    s[sp<T>(k)] = {ga.x - gb.y, ga.y + gb.x};
    s[sp<T>(N - k)] = {ga.x + gb.y, gb.x - ga.y};
  }
}

}  // namespace vg
