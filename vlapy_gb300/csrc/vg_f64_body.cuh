// FP64 device bodies shared by the single-run kernels (vg_reduce_f64.cu,
// vg_advect_f64.cu) and the batched FP64 sweep (vg_sweep_f64.cu): NumPy's
// pairwise summation, the driver pulses, the spectral Poisson solve of one
// run, the Thomas solve of one row and the x-drift of one column tile.  A run
// of the batch goes through the same code as a single run.
#pragma once

#include "vg_internal.cuh"

namespace vg {

// ---------------------------------------------------------------------------
// pairwise-sum helpers
// ---------------------------------------------------------------------------

// Sum of leaf (start, len) of terms term(j), NumPy order.
template <typename TermFn>
__device__ __forceinline__ double leaf_sum(int start, int len, TermFn term) {
  if (len < 8) {
    double r = 0.0;
    for (int i = 0; i < len; ++i) r = add_rn(r, term(start + i));
    return r;
  }
  double a0 = term(start), a1 = term(start + 1), a2 = term(start + 2), a3 = term(start + 3);
  double a4 = term(start + 4), a5 = term(start + 5), a6 = term(start + 6), a7 = term(start + 7);
  int i = 8;
  const int stop = len - (len % 8);
  for (; i < stop; i += 8) {
    a0 = add_rn(a0, term(start + i));
    a1 = add_rn(a1, term(start + i + 1));
    a2 = add_rn(a2, term(start + i + 2));
    a3 = add_rn(a3, term(start + i + 3));
    a4 = add_rn(a4, term(start + i + 4));
    a5 = add_rn(a5, term(start + i + 5));
    a6 = add_rn(a6, term(start + i + 6));
    a7 = add_rn(a7, term(start + i + 7));
  }
  double res = add_rn(add_rn(add_rn(a0, a1), add_rn(a2, a3)), add_rn(add_rn(a4, a5), add_rn(a6, a7)));
  for (; i < len; ++i) res = add_rn(res, term(start + i));
  return res;
}

// Replay the combine program over leaf sums leaf[0..n_leaves).
__device__ __forceinline__ double combine_leaves(const int* __restrict__ table, const double* leaf) {
  const int nl = table[0], np = table[1];
  const int* prog = table + 2 + 2 * nl;
  double stk[24];
  int sp = 0;
  for (int i = 0; i < np; ++i) {
    const int op = prog[i];
    if (op >= 0) {
      stk[sp++] = leaf[op];
    } else {
      const double r = stk[--sp];
      const double l = stk[--sp];
      stk[sp++] = add_rn(l, r);
    }
  }
  return sp ? stk[0] : 0.0;
}

// ---------------------------------------------------------------------------
// row moments: out[row][q] = trapz_v p_q(f[row]) with NumPy's rounding
// ---------------------------------------------------------------------------

__device__ __forceinline__ double mom_product(int kind, int arg, double fj, int j,
                                              const double* __restrict__ v,
                                              const double* __restrict__ v_pow, int nv,
                                              double vbar) {
  switch (kind) {
    case MOM_ONE: return fj;
    case MOM_V: return mul_rn(fj, v[j]);
    case MOM_W: return mul_rn(fj, v_pow[(size_t)arg * nv + j]);
    case MOM_SQ: return mul_rn(fj, fj);
    case MOM_FLOGF: return mul_rn(fj, log(fj));
    default: {  // MOM_DG2: f * (v - vbar) ** 2.0
      const double d = sub_rn(v[j], vbar);
      return mul_rn(fj, mul_rn(d, d));
    }
  }
}

// ---------------------------------------------------------------------------
// driver pulses, vlapy/field_driver.py:24-50 (+ the sin^2 envelope)
// ---------------------------------------------------------------------------

__device__ __forceinline__ double pulse_sum(const vg_pulse* __restrict__ P, int np, double t, double x) {
  double total = 0.0;
  for (int i = 0; i < np; ++i) {
    const vg_pulse q = P[i];
    const double arg = sub_rn(mul_rn(q.k0, x), mul_rn(q.w0, t));
    double term;
    if (q.envelope == VG_ENV_SIN2) {
      if (t < 0.0 || t > q.t_R) {
        term = 0.0;
      } else {
        const double sn = sin(__ddiv_rn(mul_rn(3.141592653589793, t), q.t_R));
        term = mul_rn(mul_rn(q.a0, mul_rn(sn, sn)), sin(arg));
      }
    } else {
      const double env = 0.5 * sub_rn(tanh((t - q.t_L) / q.t_wL), tanh((t - q.t_R) / q.t_wR));
      term = mul_rn(mul_rn(mul_rn(env, q.k0), q.a0), sin(arg));
    }
    total = add_rn(total, term);
  }
  return total;
}

struct FieldTimeDev {
  const double* t_ptr;
  double t_host;
  int nadd;
  double add[6];
};

__device__ __forceinline__ double field_time(const FieldTimeDev& ft) {
  double t = ft.t_ptr ? *ft.t_ptr : ft.t_host;
  for (int i = 0; i < ft.nadd; ++i) t = add_rn(t, ft.add[i]);
  return t;
}

__device__ __forceinline__ double driver_value(const double* __restrict__ driver, int use_pulses,
                                               const vg_pulse* __restrict__ P, int np, double t,
                                               const double* __restrict__ x, int n) {
  if (driver) return driver[n];
  if (use_pulses) return pulse_sum(P, np, t, x[n]);
  return 0.0;
}

// spectral Poisson of one run (vlapy/core/field.py:39-88): e = driver +
// Re IFFT(i/kx FFT(rho)), rho = 1 - dens (is_density) or dens; the G = NX/R
// threads t of a group share the padded sequence s
template <int NX>
__device__ __forceinline__ void poisson_fft_body(const double* __restrict__ dens, int is_density,
                                                 const double* __restrict__ inv_kx,
                                                 const double* __restrict__ driver, int use_pulses,
                                                 const vg_pulse* __restrict__ P, int np,
                                                 const double* __restrict__ x, const FieldTimeDev& ft,
                                                 const cx<double>* __restrict__ tw, double* __restrict__ e,
                                                 cx<double>* s, int t, int* flags) {
  constexpr int R = fft_radix<double>(NX);
  constexpr int G = NX / R;
  for (int n = t; n < NX; n += G) s[sp<double>(n)] = {is_density ? sub_rn(1.0, dens[n]) : dens[n], 0.0};
  __syncthreads();
  block_fft<double, NX, false>(s, t, tw);
  // (1j * inv_kx) * Z = (0 + i k)(zr + i zi) = (0*zr - k*zi) + i (0*zi + k*zr)
  for (int k = t; k < NX; k += G) {
    const cx<double> z = s[sp<double>(k)];
    const double ik = inv_kx[k];
    s[sp<double>(k)] = {sub_rn(mul_rn(0.0, z.x), mul_rn(ik, z.y)), add_rn(mul_rn(0.0, z.y), mul_rn(ik, z.x))};
  }
  __syncthreads();
  block_fft<double, NX, true>(s, t, tw);
  const double tt = field_time(ft);
  const double sc = 1.0 / NX;
  for (int n = t; n < NX; n += G) {
    const double self = s[sp<double>(n)].x * sc;
    const double en = add_rn(driver_value(driver, use_pulses, P, np, tt, x, n), self);
    e[n] = en;
    if (flags && !isfinite(en)) atomicOr(flags, VG_FLAG_NONFINITE);
  }
}

// Implicit Fokker-Planck step of one row, operation for operation as
// vlapy/core/collisions.py:86-160 (Dougherty; Lenard-Bernstein with vbar = 0
// and no drift shift, :26-83) builds the diagonals and :222-265 eliminates:
//   A = -vth / dv^2, b = 1 + nudt (2 vth / dv^2),
//   drift(j) = (v_j - vbar) * 0.5 / dv,
//   a_j = nudt (A + drift(j)), c_j = nudt (A - drift(j + 1)),
// then Thomas in place on fr with scratch sr[2 nv] (pivots b_j, then c_j).
// Each drift(j) is divided once and each c_j kept for the back substitution,
// which gives the same roundings as forming every diagonal entry anew.
__device__ __forceinline__ void thomas_row_f64(double* __restrict__ fr, double* __restrict__ sr, int nv,
                                               const double* __restrict__ v, double vbar, double vth,
                                               int dougherty, double nudt, double dv, double dv_sq) {
  const double A = __ddiv_rn(-vth, dv_sq);
  const double b = add_rn(1.0, mul_rn(nudt, __ddiv_rn(mul_rn(2.0, vth), dv_sq)));
  auto drift = [&](int j) {
    const double num = dougherty ? sub_rn(v[j], vbar) : v[j];
    return __ddiv_rn(num * 0.5, dv);
  };
  double* br = sr;
  double* cr = sr + nv;
  double bprev = b, dprev = fr[0];
  double dr_prev = drift(0);
  br[0] = b;
  for (int j = 1; j < nv; ++j) {
    const double dr = drift(j);
    const double a = mul_rn(nudt, add_rn(A, dr_prev));  // a[j - 1]
    const double c = mul_rn(nudt, sub_rn(A, dr));       // c[j - 1]
    cr[j - 1] = c;
    const double m = __ddiv_rn(a, bprev);
    const double bj = sub_rn(b, mul_rn(m, c));
    const double dj = sub_rn(fr[j], mul_rn(m, dprev));
    br[j] = bj;
    fr[j] = dj;
    bprev = bj;
    dprev = dj;
    dr_prev = dr;
  }
  double xj = __ddiv_rn(dprev, bprev);
  fr[nv - 1] = xj;
  for (int j = nv - 2; j >= 0; --j) {
    xj = __ddiv_rn(sub_rn(fr[j], mul_rn(cr[j], xj)), br[j]);
    fr[j] = xj;
  }
}

// x-drift of one tile of W columns (c0 ..) of f[NX][nv] (vlapy/core/vlasov.py:106-108):
// pairs of columns packed as complex sequences, FFT along x, phase
// exp(i ((-kx) dt) v_col), inverse FFT.  smem: W/2 sequences of LD elements.
constexpr int COL_PAD = 1;
template <int NX>
__device__ __forceinline__ void vdfdx_tile_body(double* __restrict__ f, int nv, int c0, int W,
                                                const double* __restrict__ kx, const double* __restrict__ v,
                                                double dt, const cx<double>* __restrict__ tw,
                                                unsigned char* smem) {
  constexpr int R = fft_radix<double>(NX);
  constexpr int G = NX / R;
  constexpr int LD = sp_len<double>(NX) + COL_PAD;
  cx<double>* s = reinterpret_cast<cx<double>*>(smem);
  double* sd = reinterpret_cast<double*>(smem);
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

}  // namespace vg
