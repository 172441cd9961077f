// FP64 reductions, field solve, tridiagonal solve and storage step.
//
// Every trapz over v and every mean over x is evaluated with NumPy's pairwise
// summation tree (a table built at plan creation): leaves of <= 128 terms are
// summed with eight interleaved accumulators, one leaf per thread, and one
// thread per moment replays the post-order combine program.  Products use
// explicitly rounded intrinsics so nvcc cannot contract them into FMAs.  With
// f equal, densities and moments are then bit-identical to the reference's
// np.trapz (vlapy/core/field.py:36, vlapy/core/step.py:164-223).
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

__global__ void k_row_moments_f64(const double* __restrict__ f, int nv, const double* __restrict__ v,
                                  const double* __restrict__ v_pow, MomSpec spec,
                                  const int* __restrict__ table, double dv,
                                  double* __restrict__ out, int ostride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* row = reinterpret_cast<double*>(smem_raw);
  const int nl = table[0];
  double* leaf = row + nv;               // [nm][nl]
  __shared__ double res[MOM_STRIDE];
  const size_t r = blockIdx.x;
  for (int j = threadIdx.x; j < nv; j += blockDim.x) row[j] = f[r * nv + j];
  __syncthreads();
  const int* leaves = table + 2;
  for (int phase = 0; phase < 2; ++phase) {
    for (int idx = threadIdx.x; idx < spec.nm * nl; idx += blockDim.x) {
      const int q = idx / nl, L = idx - q * nl;
      const int kind = spec.kind[q];
      if ((kind == MOM_DG2) != (phase == 1)) continue;
      const int arg = spec.arg[q];
      const double vbar = kind == MOM_DG2 ? res[arg] : 0.0;
      auto term = [&](int j) {
        const double p0 = mom_product(kind, arg, row[j], j, v, v_pow, nv, vbar);
        const double p1 = mom_product(kind, arg, row[j + 1], j + 1, v, v_pow, nv, vbar);
        return mul_rn(dv, add_rn(p1, p0)) * 0.5;
      };
      leaf[q * nl + L] = leaf_sum(leaves[2 * L], leaves[2 * L + 1], term);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < spec.nm; q += blockDim.x) {
      if ((spec.kind[q] == MOM_DG2) != (phase == 1)) continue;
      const double val = nv > 1 ? combine_leaves(table, leaf + q * nl) : 0.0;
      res[q] = val;
      out[r * ostride + q] = val;
    }
    __syncthreads();
  }
}

cudaError_t launch_row_moments_f64(const vg_plan& p, const double* f, const MomSpec& spec,
                                   double* out, int out_stride, cudaStream_t s) {
  const size_t smem = ((size_t)p.nv + (size_t)spec.nm * p.pw_v_leaves) * sizeof(double);
  cudaError_t err = ensure_smem((const void*)k_row_moments_f64, smem);
  if (err != cudaSuccess) return err;
  k_row_moments_f64<<<p.nx, 256, smem, s>>>(f, p.nv, p.v, p.v_pow, spec, p.pw_v, p.dv, out, out_stride);
  return cudaGetLastError();
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

__global__ void k_driver(const vg_pulse* __restrict__ P, int np, const double* __restrict__ x, int nx,
                         FieldTimeDev ft, double* __restrict__ out) {
  const double t = field_time(ft);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nx; i += gridDim.x * blockDim.x)
    out[i] = pulse_sum(P, np, t, x[i]);
}

static FieldTimeDev to_dev(const FieldTime& ft) {
  FieldTimeDev d;
  d.t_ptr = ft.t_ptr;
  d.t_host = ft.t_host;
  d.nadd = ft.nadd;
  for (int i = 0; i < 6; ++i) d.add[i] = ft.add[i];
  return d;
}

cudaError_t launch_driver(const vg_plan& p, const FieldTime& ft, double* out, cudaStream_t s) {
  k_driver<<<div_up(p.nx, 256), 256, 0, s>>>(p.pulses, p.n_pulses, p.x, p.nx, to_dev(ft), out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// spectral Poisson, vlapy/core/field.py:39-88
// ---------------------------------------------------------------------------

__device__ __forceinline__ double driver_value(const double* __restrict__ driver, int use_pulses,
                                               const vg_pulse* __restrict__ P, int np, double t,
                                               const double* __restrict__ x, int n) {
  if (driver) return driver[n];
  if (use_pulses) return pulse_sum(P, np, t, x[n]);
  return 0.0;
}

template <int NX>
__global__ void __launch_bounds__(fft_threads<double>(NX)) k_poisson_fft_f64(
    const double* __restrict__ dens, int is_density, const double* __restrict__ inv_kx,
    const double* __restrict__ driver, int use_pulses, const vg_pulse* __restrict__ P, int np,
    const double* __restrict__ x, FieldTimeDev ft, const cx<double>* __restrict__ tw,
    double* __restrict__ e) {
  constexpr int R = fft_radix<double>(NX);
  constexpr int G = NX / R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<double>* s = reinterpret_cast<cx<double>*>(smem_raw);
  const int t = threadIdx.x;
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
    e[n] = add_rn(driver_value(driver, use_pulses, P, np, tt, x, n), self);
  }
}

// Direct DFT for lengths that are not powers of two (O(nx^2), one CTA).
__global__ void k_poisson_dft_f64(const double* __restrict__ dens, int is_density, int nx,
                                  const double* __restrict__ inv_kx, const double* __restrict__ driver,
                                  int use_pulses, const vg_pulse* __restrict__ P, int np,
                                  const double* __restrict__ x, FieldTimeDev ft,
                                  double* __restrict__ work, double* __restrict__ e) {
  // work: [nx] rho, then [2*nx] spectrum
  double* rho = work;
  cx<double>* Y = reinterpret_cast<cx<double>*>(work + nx + (nx & 1));
  for (int n = threadIdx.x; n < nx; n += blockDim.x) rho[n] = is_density ? sub_rn(1.0, dens[n]) : dens[n];
  __syncthreads();
  for (int k = threadIdx.x; k < nx; k += blockDim.x) {
    double zr = 0.0, zi = 0.0;
    for (int n = 0; n < nx; ++n) {
      const long long q = ((long long)n * k) % nx;
      double sn, cs;
      sincospi(2.0 * (double)q / (double)nx, &sn, &cs);
      zr += rho[n] * cs;
      zi -= rho[n] * sn;
    }
    const double ik = inv_kx[k];
    Y[k] = {-ik * zi, ik * zr};
  }
  __syncthreads();
  const double tt = field_time(ft);
  for (int n = threadIdx.x; n < nx; n += blockDim.x) {
    double acc = 0.0;
    for (int k = 0; k < nx; ++k) {
      const long long q = ((long long)n * k) % nx;
      double sn, cs;
      sincospi(2.0 * (double)q / (double)nx, &sn, &cs);
      acc += Y[k].x * cs - Y[k].y * sn;
    }
    e[n] = driver_value(driver, use_pulses, P, np, tt, x, n) + acc / nx;
  }
}

namespace {
template <int NX>
cudaError_t poisson_n(const vg_plan& p, const double* dens, int is_density, const double* driver,
                      const FieldTime& ft, double* e, cudaStream_t s) {
  constexpr int G = fft_threads<double>(NX);
  const size_t smem = (size_t)sp_len<double>(NX) * sizeof(cx<double>);
  cudaError_t err = ensure_smem((const void*)k_poisson_fft_f64<NX>, smem);
  if (err != cudaSuccess) return err;
  k_poisson_fft_f64<NX><<<1, G, smem, s>>>(dens, is_density, p.inv_kx, driver, ft.use_pulses, p.pulses,
                                           p.n_pulses, p.x, to_dev(ft), p.tw64, e);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_poisson_f64(const vg_plan& p, const double* dens, int is_density, const double* driver,
                               const FieldTime& ft, double* e, cudaStream_t s) {
  if (p.nx_pow2 && p.nx <= 8192) {
    switch (ilog2(p.nx)) {
      case 1: return poisson_n<2>(p, dens, is_density, driver, ft, e, s);
      case 2: return poisson_n<4>(p, dens, is_density, driver, ft, e, s);
      case 3: return poisson_n<8>(p, dens, is_density, driver, ft, e, s);
      case 4: return poisson_n<16>(p, dens, is_density, driver, ft, e, s);
      case 5: return poisson_n<32>(p, dens, is_density, driver, ft, e, s);
      case 6: return poisson_n<64>(p, dens, is_density, driver, ft, e, s);
      case 7: return poisson_n<128>(p, dens, is_density, driver, ft, e, s);
      case 8: return poisson_n<256>(p, dens, is_density, driver, ft, e, s);
      case 9: return poisson_n<512>(p, dens, is_density, driver, ft, e, s);
      case 10: return poisson_n<1024>(p, dens, is_density, driver, ft, e, s);
      case 11: return poisson_n<2048>(p, dens, is_density, driver, ft, e, s);
      case 12: return poisson_n<4096>(p, dens, is_density, driver, ft, e, s);
      case 13: return poisson_n<8192>(p, dens, is_density, driver, ft, e, s);
      default: break;
    }
  }
  k_poisson_dft_f64<<<1, 256, 0, s>>>(dens, is_density, p.nx, p.inv_kx, driver, ft.use_pulses, p.pulses,
                                      p.n_pulses, p.x, to_dev(ft), p.etmp, e);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// implicit Fokker-Planck: vlapy/core/collisions.py:26-160 (diagonals) and
// :222-265 (Thomas), one thread per x row, operation for operation
// ---------------------------------------------------------------------------

__global__ void k_thomas_f64(double* __restrict__ f, int nrows, int nv, const double* __restrict__ v,
                             const double* __restrict__ mom, int mstride, int vbar_col, int vth_col,
                             int dougherty, double nudt, double dv, double dv_sq,
                             double* __restrict__ bb) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nrows) return;
  const double vbar = dougherty ? mom[(size_t)row * mstride + vbar_col] : 0.0;
  const double vth = mom[(size_t)row * mstride + vth_col];
  const double A = __ddiv_rn(-vth, dv_sq);
  const double b = add_rn(1.0, mul_rn(nudt, __ddiv_rn(mul_rn(2.0, vth), dv_sq)));
  auto drift = [&](int j) {
    const double num = dougherty ? sub_rn(v[j], vbar) : v[j];
    return __ddiv_rn(num * 0.5, dv);
  };
  auto sub_diag = [&](int j) { return mul_rn(nudt, add_rn(A, drift(j))); };      // a[j], j < nv-1
  auto sup_diag = [&](int j) { return mul_rn(nudt, sub_rn(A, drift(j + 1))); };  // c[j], j < nv-1
  double* fr = f + (size_t)row * nv;
  double* br = bb + (size_t)row * nv;
  double bprev = b, dprev = fr[0];
  br[0] = b;
  for (int j = 1; j < nv; ++j) {
    const double m = __ddiv_rn(sub_diag(j - 1), bprev);
    const double bj = sub_rn(b, mul_rn(m, sup_diag(j - 1)));
    const double dj = sub_rn(fr[j], mul_rn(m, dprev));
    br[j] = bj;
    fr[j] = dj;
    bprev = bj;
    dprev = dj;
  }
  double xj = __ddiv_rn(dprev, bprev);
  fr[nv - 1] = xj;
  for (int j = nv - 2; j >= 0; --j) {
    xj = __ddiv_rn(sub_rn(fr[j], mul_rn(sup_diag(j), xj)), br[j]);
    fr[j] = xj;
  }
}

cudaError_t launch_thomas_f64(const vg_plan& p, double* f, const double* mom, int vbar_col, int vth_col,
                              cudaStream_t s) {
  k_thomas_f64<<<div_up(p.nx, 64), 64, 0, s>>>(f, p.nx, p.nv, p.v, mom, MOM_STRIDE, vbar_col, vth_col,
                                               p.collision == VG_COLL_DG, p.nudt, p.dv, p.dv_sq, p.bb);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// storage step, vlapy/core/step.py:116-283
// ---------------------------------------------------------------------------

// fields[.][i] and the seven x-means; mom holds n, j, T, q, fv4, vN, f^2, f log f per row
__global__ void k_fields_series_f64(const double* __restrict__ mom, const double* __restrict__ e,
                                    const double* __restrict__ de, int nx, int i, vg_history h,
                                    const int* __restrict__ table) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* leaf = reinterpret_cast<double*>(smem_raw);  // [7][nl]
  const int nl = table[0];
  const int* leaves = table + 2;
  const size_t off = (size_t)i * nx;
  for (int n = threadIdx.x; n < nx; n += blockDim.x) {
    if (h.fields[0]) h.fields[0][off + n] = e[n];
    if (h.fields[1]) h.fields[1][off + n] = de ? de[n] : 0.0;
    for (int q = 0; q < 6; ++q)
      if (h.fields[2 + q]) h.fields[2 + q][off + n] = mom[(size_t)n * MOM_STRIDE + q];
  }
  // series sources: n, j, T, e^2, de^2, f^2, flogf
  for (int idx = threadIdx.x; idx < 7 * nl; idx += blockDim.x) {
    const int q = idx / nl, L = idx - q * nl;
    auto term = [&](int n) -> double {
      switch (q) {
        case 0: return mom[(size_t)n * MOM_STRIDE + 0];
        case 1: return mom[(size_t)n * MOM_STRIDE + 1];
        case 2: return mom[(size_t)n * MOM_STRIDE + 2];
        case 3: return mul_rn(e[n], e[n]);
        case 4: return de ? mul_rn(de[n], de[n]) : 0.0;
        case 5: return mom[(size_t)n * MOM_STRIDE + 6];
        default: return mom[(size_t)n * MOM_STRIDE + 7];
      }
    };
    leaf[q * nl + L] = leaf_sum(leaves[2 * L], leaves[2 * L + 1], term);
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    const int q = threadIdx.x;
    const double m = __ddiv_rn(combine_leaves(table, leaf + q * nl), (double)nx);
    if (h.series[q]) h.series[q][i] = m;
  }
}

// stored_f[i][slot][v] = complex64(sum_x f[x][v] exp(-2 pi i m x / nx))
__global__ void k_store_modes_f64(const double* __restrict__ f, int nx, int nv, int n_modes, int n_slots,
                                  int nx_pow2, const cx<double>* __restrict__ tw, int i,
                                  cx<float>* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nv) return;
  cx<float>* dst = out + (size_t)i * n_slots * nv;
  for (int m = 0; m < n_modes && m < n_slots; ++m) {
    double zr = 0.0, zi = 0.0;
    for (int xx = 0; xx < nx; ++xx) {
      const long long q = ((long long)m * xx) % nx;
      double cs, sn;
      if (q == 0) {
        cs = 1.0;
        sn = 0.0;
      } else if (nx_pow2) {
        // exp(-2 pi i q / nx) from the span-ordered table; q >= nx/2 is the
        // negated entry q - nx/2
        const bool hi = 2 * q >= nx;
        const cx<double> w = tw[tw_index(nx, hi ? (int)(q - nx / 2) : (int)q)];
        cs = hi ? -w.x : w.x;
        sn = hi ? w.y : -w.y;
      } else {
        sincospi(2.0 * (double)q / (double)nx, &sn, &cs);
      }
      const double fv = f[(size_t)xx * nv + j];
      zr += fv * cs;
      zi -= fv * sn;
    }
    const cx<float> z = {__double2float_rn(zr), __double2float_rn(zi)};
    if (n_modes == 1) {
      for (int sl = 0; sl < n_slots; ++sl) dst[(size_t)sl * nv + j] = z;
    } else {
      dst[(size_t)m * nv + j] = z;
    }
  }
}

cudaError_t launch_storage_f64(const vg_plan& p, const double* f, const double* e, const double* de,
                               const vg_history& h, int i, cudaStream_t s) {
  MomSpec spec;
  spec.nm = 8;
  const int kinds[8] = {MOM_ONE, MOM_V, MOM_W, MOM_W, MOM_W, MOM_W, MOM_SQ, MOM_FLOGF};
  const int args[8] = {0, 0, 1, 2, 3, 4, 0, 0};
  for (int q = 0; q < 8; ++q) {
    spec.kind[q] = kinds[q];
    spec.arg[q] = args[q];
  }
  cudaError_t err = launch_row_moments_f64(p, f, spec, p.mom, MOM_STRIDE, s);
  if (err != cudaSuccess) return err;
  const size_t smem = (size_t)7 * p.pw_x_leaves * sizeof(double);
  k_fields_series_f64<<<1, 256, smem, s>>>(p.mom, e, de, p.nx, i, h, p.pw_x);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  if (h.stored_f) {
    if (h.store_all) {
      err = cudaMemcpyAsync(static_cast<double*>(h.stored_f) + (size_t)i * p.nx * p.nv, f,
                            (size_t)p.nx * p.nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
    } else {
      k_store_modes_f64<<<div_up(p.nv, 128), 128, 0, s>>>(f, p.nx, p.nv, h.n_modes, h.n_slots,
                                                          p.nx_pow2 && p.nx <= FFT_NMAX,
                                                          p.tw64, i, static_cast<cx<float>*>(h.stored_f));
      err = cudaGetLastError();
    }
  }
  return err;
}

// ---------------------------------------------------------------------------
// twiddle tables
// ---------------------------------------------------------------------------

__global__ void k_twiddles(cx<double>* __restrict__ t64, cx<float>* __restrict__ t32) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= FFT_NMAX) return;
  int k, h;
  tw_entry(q, k, h);
  double sn, cs;
  sincospi((double)k / (double)h, &sn, &cs);
  t64[q] = {cs, -sn};
  t32[q] = {(float)cs, (float)-sn};
}

cudaError_t launch_twiddles(vg_plan& p, cudaStream_t s) {
  k_twiddles<<<div_up(FFT_NMAX, 256), 256, 0, s>>>(p.tw64, p.tw32);
  return cudaGetLastError();
}

}  // namespace vg
