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

// cos(2*pi*j/32), exact to double precision; folded at compile time when j is.
// The first quadrant holds cos(pi q/16), q = 0..8; the others follow by symmetry.
__host__ __device__ constexpr double cos32_q(int q) {
  return q == 0 ? 1.0
       : q == 1 ? 0.98078528040323044913
       : q == 2 ? 0.92387953251128675613
       : q == 3 ? 0.83146961230254523708
       : q == 4 ? 0.70710678118654752440
       : q == 5 ? 0.55557023301960222474
       : q == 6 ? 0.38268343236508977173
       : q == 7 ? 0.19509032201612826785
       : 0.0;
}
__host__ __device__ constexpr double cos32(int j) {
  return (j & 31) <= 8 ? cos32_q(j & 31)
       : (j & 31) <= 16 ? -cos32_q(16 - (j & 31))
       : (j & 31) <= 24 ? -cos32_q((j & 31) - 16)
       : cos32_q(32 - (j & 31));
}
__host__ __device__ constexpr double sin32(int j) { return cos32(j + 24); }
// the 16-point values are the even entries (identical doubles)
__host__ __device__ constexpr double cos16(int j) { return cos32(2 * j); }
__host__ __device__ constexpr double sin16(int j) { return sin32(2 * j); }

// Exactly-rounded FP64 products and sums that nvcc may not contract into FMAs.
// Used where the FP64 mode must reproduce NumPy's rounding bit for bit.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

constexpr int div_up(int a, int b) { return (a + b - 1) / b; }

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }
__host__ __device__ constexpr bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

}  // namespace vg
