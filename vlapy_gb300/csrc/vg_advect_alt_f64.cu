// The alternative FP64 advection operators of vlapy/core/vlasov.py: the
// backward semi-Lagrangian steps in x and in v (get_vdfdx_sl :42-80,
// get_edfdv_sl :168-210) and the centred-difference v step
// (get_edfdv_center_differenced :143-165).  All three are out of place, as
// the reference's closures return a new array.
//
// Semi-Lagrangian.  The reference fits a bicubic interpolating spline
// (scipy's RectBivariateSpline: FITPACK, s = 0) over the grid extended by one
// periodic cell at each end of the advected axis, and evaluates it at the
// departure points of the grid nodes.  Along the other axis every departure
// point is a grid node, and there a tensor-product interpolating spline is
// the 1-D interpolating spline of that line.  With s = 0 and cubic order
// FITPACK places its interior knots at the data points except the second and
// the second-last: the not-a-knot cubic spline.  Each line (a v column for
// the x step, an x row for the v step) of N points, padded to n = N + 2, is
// therefore:
//   1. solved for the spline's second derivatives M_k.  The not-a-knot
//      conditions (M_0 - 2 M_1 + M_2 = 0 and its mirror) turn the first and
//      last interior equations into 6 M_1 = r_1 and 6 M_{n-2} = r_{n-2};
//      M_2 .. M_{n-3} solve the (1, 4, 1) system left between them, by Thomas
//      elimination with a pivot table shared by all lines;
//   2. evaluated on the cubic piece that holds each departure point, clamped
//      to the padded range as FITPACK's evaluator (fpbisp) clamps it.
// Step 1 runs one thread per v column for the x step (a serial recurrence over
// nx; the columns are many) and one warp per x row for the v step (the rows are
// few and long: a warp-parallel scan of the recurrence).  Step 2 runs one thread
// per cell, coalesced along v.  FITPACK solves for B-spline coefficients by Givens
// rotations instead, so the two agree to rounding, not bit for bit.
//
// Centred difference.  f - (e * df/dv) * dt with numpy.gradient's uniform
// second-order stencils: (f[j+1] - f[j-1]) / (2 dv) inside, the one-sided
// three-point forms at the two ends, each product and sum rounded separately
// (no FMA contraction), so the result is NumPy's bit for bit.
#include "vg_internal.cuh"

namespace vg {

namespace {

// padded node k of a line of N points -> index of its value in the line
__device__ __forceinline__ int pad_src(int k, int N) { return k == 0 ? N - 1 : (k == N + 1 ? 0 : k - 1); }

// Thomas elimination along one line.  Line values at f[lb + idx * es], second
// derivatives at M[mb + k * ms] for the padded node k = 0 .. N + 1.
__device__ void sl_solve_line(const double* __restrict__ f, size_t lb, size_t es, double* __restrict__ M,
                              size_t mb, size_t ms, int N, double h, const double* __restrict__ w) {
  auto y = [&](int k) { return f[lb + (size_t)pad_src(k, N) * es]; };
  auto sd = [&](int k) { return (y(k - 1) + y(k + 1)) - 2.0 * y(k); };
  const double inv_h2 = 1.0 / (h * h);
  const double c6 = 6.0 * inv_h2;
  const double m1 = sd(1) * inv_h2;   // M_1
  const double mn = sd(N) * inv_h2;   // M_{n-2}
  const int m = N - 2;                // unknowns M_2 .. M_{N-1}
  // forward elimination; a sliding window of three line values
  double ym = y(1), y0 = y(2);
  double d = 0.0;
  // unrolled so that the loads of several iterations (independent of the
  // recurrence) are in flight together
#pragma unroll 8
  for (int q = 0; q < m; ++q) {
    const int k = q + 2;
    const double yp = y(k + 1);
    double rhs = ((ym + yp) - 2.0 * y0) * c6;
    if (q == 0) rhs -= m1;
    if (q == m - 1) rhs -= mn;
    d = (rhs - d) * w[q];
    M[mb + (size_t)k * ms] = d;
    ym = y0;
    y0 = yp;
  }
  // back substitution: M_{N-1} = d'_{m-1}, M_k = d'_k - w_k M_{k+1}
  // The loads of M come in batches of eight ahead of the recurrence: a load
  // after a store to the same array at a run-time stride is not reordered by
  // the compiler, and each would otherwise wait on L2.
  double next = d;
  int k = N - 2;
  for (; k >= 2 + 7; k -= 8) {
    double dd[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) dd[u] = M[mb + (size_t)(k - u) * ms];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      next = dd[u] - w[k - u - 2] * next;
      M[mb + (size_t)(k - u) * ms] = next;
    }
  }
  for (; k >= 2; --k) {
    const size_t at = mb + (size_t)k * ms;
    next = M[at] - w[k - 2] * next;
    M[at] = next;
  }
  M[mb + 1 * ms] = m1;
  M[mb + (size_t)N * ms] = mn;
  M[mb] = 2.0 * m1 - M[mb + 2 * ms];
  M[mb + (size_t)(N + 1) * ms] = 2.0 * mn - M[mb + (size_t)(N - 1) * ms];
}

// x step: one thread per v column; M[k][nv]
__global__ void k_sl_solve_x(const double* __restrict__ f, double* __restrict__ M, int nx, int nv,
                             const double* __restrict__ x, const double* __restrict__ w) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nv) return;
  sl_solve_line(f, (size_t)j, (size_t)nv, M, (size_t)j, (size_t)nv, nx, x[2] - x[1], w);
}

// v step: one WARP per x row; M[nx][nv + 2].  The rows are few (nx) and long
// (nv), so the serial recurrences are split: lane l owns the unknowns
// q in [l L, (l + 1) L), L = ceil(m / 32).  Each Thomas sweep is a chain of
// affine maps (forward d_q = -w_q d_{q-1} + w_q r_q; backward
// x_q = -w_q x_{q+1} + d_q), so a lane composes its chunk's map, a 5-step
// shuffle scan composes the maps of the lanes before it (after it, for the
// backward sweep), and the lane replays its chunk from the value that gives.
// The maps contract (|w_q| < 0.27), so the reassociation changes only rounding.
__global__ void k_sl_solve_v(const double* __restrict__ f, double* __restrict__ M, int nx, int nv,
                             const double* __restrict__ v, const double* __restrict__ w) {
  constexpr unsigned FULL = 0xffffffffu;
  const int row = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= nx) return;  // uniform per warp
  const int N = nv, m = N - 2;
  const double* y = f + (size_t)row * nv;   // y(k) = y[pad_src(k, N)]
  double* Mr = M + (size_t)row * (nv + 2);
  const double h = v[2] - v[1];
  const double inv_h2 = 1.0 / (h * h);
  const double c6 = 6.0 * inv_h2;
  const double m1 = ((y[N - 1] + y[1]) - 2.0 * y[0]) * inv_h2;            // M_1
  const double mn = ((y[N - 2] + y[0]) - 2.0 * y[N - 1]) * inv_h2;        // M_{n-2}
  const int L = (m + 31) >> 5;
  const int q0 = min(lane * L, m), q1 = min(q0 + L, m);
  // right-hand side of unknown q (padded node k = q + 2, line values k - 2 .. k)
  auto rhs = [&](int q) {
    double r = ((y[q] + y[q + 2]) - 2.0 * y[q + 1]) * c6;
    if (q == 0) r -= m1;
    if (q == m - 1) r -= mn;
    return r;
  };
  // forward sweep
  double A = 1.0, B = 0.0;
  for (int q = q0; q < q1; ++q) {
    const double wq = w[q];
    A = -wq * A;
    B = (rhs(q) - B) * wq;
  }
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double Ap = __shfl_up_sync(FULL, A, off), Bp = __shfl_up_sync(FULL, B, off);
    if (lane >= off) {
      B = A * Bp + B;
      A = A * Ap;
    }
  }
  double d = __shfl_up_sync(FULL, B, 1);
  if (lane == 0) d = 0.0;
  for (int q = q0; q < q1; ++q) {
    d = (rhs(q) - d) * w[q];
    Mr[q + 2] = d;
  }
  // backward sweep, from x_m = 0; each lane reads back only its own chunk
  A = 1.0;
  B = 0.0;
  for (int q = q1 - 1; q >= q0; --q) {
    const double wq = w[q];
    A = -wq * A;
    B = Mr[q + 2] - wq * B;
  }
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double Ap = __shfl_down_sync(FULL, A, off), Bp = __shfl_down_sync(FULL, B, off);
    if (lane + off < 32) {
      B = A * Bp + B;
      A = A * Ap;
    }
  }
  double x = __shfl_down_sync(FULL, B, 1);
  if (lane == 31) x = 0.0;
  for (int q = q1 - 1; q >= q0; --q) {
    x = Mr[q + 2] - w[q] * x;
    Mr[q + 2] = x;
  }
  __syncwarp();  // M_2 and M_{N-1} come from other lanes' chunks
  if (lane == 0) {
    Mr[1] = m1;
    Mr[N] = mn;
    Mr[0] = 2.0 * m1 - Mr[2];
    Mr[N + 1] = 2.0 * mn - Mr[N - 1];
  }
}

// Evaluation at the departure points: x_i - v_j dt (ALONG_X) or v_j - e_i dt.
template <bool ALONG_X>
__global__ void k_sl_eval(const double* __restrict__ fin, double* __restrict__ fout,
                          const double* __restrict__ M, int nx, int nv, const double* __restrict__ x,
                          const double* __restrict__ v, const double* __restrict__ e, double dt) {
  const double* g = ALONG_X ? x : v;
  const int N = ALONG_X ? nx : nv;
  // the padded grid of the reference: one node of spacing g[2] - g[1] added at each end
  const double h = g[2] - g[1];
  const double p0 = g[0] - h, pend = g[N - 1] + h;
  const double inv_h = 1.0 / h;
  const size_t cells = (size_t)nx * nv;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < cells; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q / (size_t)nv);
    const int j = (int)(q - (size_t)i * nv);
    double X = ALONG_X ? __dsub_rn(x[i], __dmul_rn(v[j], dt)) : __dsub_rn(v[j], __dmul_rn(e[i], dt));
    X = fmin(fmax(X, p0), pend);
    const double u = (X - p0) * inv_h;
    int k = (int)floor(u);
    k = min(max(k, 0), N);
    const double t = u - (double)k;
    const double s = 1.0 - t;
    size_t lb, es, mb, ms;
    if (ALONG_X) {
      lb = (size_t)j; es = (size_t)nv; mb = (size_t)j; ms = (size_t)nv;
    } else {
      lb = (size_t)i * nv; es = 1; mb = (size_t)i * (nv + 2); ms = 1;
    }
    const double ya = fin[lb + (size_t)pad_src(k, N) * es];
    const double yb = fin[lb + (size_t)pad_src(k + 1, N) * es];
    const double ma = M[mb + (size_t)k * ms];
    const double mb1 = M[mb + (size_t)(k + 1) * ms];
    // s y_k + t y_{k+1} + h^2/6 [(s^3 - s) M_k + (t^3 - t) M_{k+1}],
    // with s^3 - s = -t s (2 - t) and t^3 - t = -t s (1 + t)
    fout[q] = (s * ya + t * yb) - (h * h / 6.0) * (t * s) * ((2.0 - t) * ma + (1.0 + t) * mb1);
  }
}

__global__ void k_edfdv_cd2(const double* __restrict__ fin, double* __restrict__ fout,
                            const double* __restrict__ e, int nx, int nv, double dv, double dt) {
  const size_t cells = (size_t)nx * nv;
  const double two_dv = 2.0 * dv;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < cells; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q / (size_t)nv);
    const int j = (int)(q - (size_t)i * nv);
    const double* r = fin + (size_t)i * nv;
    double g;
    if (j == 0) {
      g = __dadd_rn(__dadd_rn(__dmul_rn(-1.5 / dv, r[0]), __dmul_rn(2.0 / dv, r[1])), __dmul_rn(-0.5 / dv, r[2]));
    } else if (j == nv - 1) {
      g = __dadd_rn(__dadd_rn(__dmul_rn(0.5 / dv, r[nv - 3]), __dmul_rn(-2.0 / dv, r[nv - 2])),
                    __dmul_rn(1.5 / dv, r[nv - 1]));
    } else {
      g = __dsub_rn(r[j + 1], r[j - 1]) / two_dv;
    }
    fout[q] = __dsub_rn(r[j], __dmul_rn(__dmul_rn(e[i], g), dt));
  }
}

int cell_blocks(size_t cells) {
  const size_t b = (cells + 255) / 256;
  return (int)(b < 152 * 16 ? (b ? b : 1) : 152 * 16);
}

}  // namespace

cudaError_t ensure_sl_scratch(vg_plan& p) {
  if (p.sl_m) return cudaSuccess;
  const int nmax = p.nx > p.nv ? p.nx : p.nv;
  // pivots of the (1, 4, 1) Thomas elimination: w_0 = 1/4, w_q = 1 / (4 - w_{q-1})
  std::vector<double> w((size_t)nmax);
  double c = 0.0;
  for (int q = 0; q < nmax; ++q) {
    c = 1.0 / (4.0 - c);
    w[q] = c;
  }
  double* m = nullptr;
  double* wd = nullptr;
  cudaError_t err = cudaMalloc(&m, sizeof(double) * (size_t)(p.nx + 2) * (size_t)(p.nv + 2));
  if (err == cudaSuccess) err = cudaMalloc(&wd, sizeof(double) * (size_t)nmax);
  if (err == cudaSuccess) err = cudaMemcpy(wd, w.data(), sizeof(double) * (size_t)nmax, cudaMemcpyHostToDevice);
  if (err != cudaSuccess) {
    if (m) cudaFree(m);
    if (wd) cudaFree(wd);
    return err;
  }
  p.sl_m = m;
  p.sl_w = wd;
  return cudaSuccess;
}

cudaError_t launch_vdfdx_sl_f64(const vg_plan& p, const double* fin, double* fout, double dt, cudaStream_t s) {
  // one-warp CTAs (each column's chain is bound by its warp's FP64 issue, not by the CTA shape)
  k_sl_solve_x<<<div_up(p.nv, 32), 32, 0, s>>>(fin, p.sl_m, p.nx, p.nv, p.x, p.sl_w);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  k_sl_eval<true><<<cell_blocks((size_t)p.nx * p.nv), 256, 0, s>>>(fin, fout, p.sl_m, p.nx, p.nv, p.x, p.v,
                                                                    nullptr, dt);
  return cudaGetLastError();
}

cudaError_t launch_edfdv_sl_f64(const vg_plan& p, const double* fin, const double* e, double* fout, double dt,
                                cudaStream_t s) {
  k_sl_solve_v<<<div_up(p.nx, 4), 128, 0, s>>>(fin, p.sl_m, p.nx, p.nv, p.v, p.sl_w);  // a warp per row
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  k_sl_eval<false><<<cell_blocks((size_t)p.nx * p.nv), 256, 0, s>>>(fin, fout, p.sl_m, p.nx, p.nv, p.x, p.v,
                                                                     e, dt);
  return cudaGetLastError();
}

cudaError_t launch_edfdv_cd2_f64(const vg_plan& p, const double* fin, const double* e, double* fout, double dt,
                                 cudaStream_t s) {
  k_edfdv_cd2<<<cell_blocks((size_t)p.nx * p.nv), 256, 0, s>>>(fin, fout, e, p.nx, p.nv, p.dv, dt);
  return cudaGetLastError();
}

}  // namespace vg
