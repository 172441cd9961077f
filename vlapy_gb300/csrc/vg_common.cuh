// Common device/host helpers for the VlaPy GB300 kernels: complex type, error
// plumbing and small math helpers.  Everything here is header-only.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vg {

template <typename T>
struct __align__(2 * sizeof(T)) cx {
  T x, y;
};

template <typename T>
__device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return {a.x + b.x, a.y + b.y}; }
template <typename T>
__device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return {a.x - b.x, a.y - b.y}; }
template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename T>
__device__ __forceinline__ cx<T> cscale(cx<T> a, T s) { return {a.x * s, a.y * s}; }

// cos(2*pi*j/16), exact to double precision; folded at compile time when j is.
__host__ __device__ constexpr double cos16(int j) {
  return (j & 15) == 0 ? 1.0
       : (j & 15) == 1 ? 0.92387953251128675613
       : (j & 15) == 2 ? 0.70710678118654752440
       : (j & 15) == 3 ? 0.38268343236508977173
       : (j & 15) == 4 ? 0.0
       : (j & 15) == 5 ? -0.38268343236508977173
       : (j & 15) == 6 ? -0.70710678118654752440
       : (j & 15) == 7 ? -0.92387953251128675613
       : (j & 15) == 8 ? -1.0
       : (j & 15) == 9 ? -0.92387953251128675613
       : (j & 15) == 10 ? -0.70710678118654752440
       : (j & 15) == 11 ? -0.38268343236508977173
       : (j & 15) == 12 ? 0.0
       : (j & 15) == 13 ? 0.38268343236508977173
       : (j & 15) == 14 ? 0.70710678118654752440
       : 0.92387953251128675613;
}
__host__ __device__ constexpr double sin16(int j) { return cos16(j + 12); }

// Exactly-rounded FP64 products and sums that nvcc may not contract into FMAs.
// Used where the FP64 mode must reproduce NumPy's rounding bit for bit.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

constexpr int div_up(int a, int b) { return (a + b - 1) / b; }

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }
__host__ __device__ constexpr bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

}  // namespace vg
