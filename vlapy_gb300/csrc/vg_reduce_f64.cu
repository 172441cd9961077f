// FP64 reductions, field solve, tridiagonal solve and storage step.
//
// Every trapz over v and every mean over x is evaluated with NumPy's pairwise
// summation tree (a table built at plan creation): leaves of <= 128 terms are
// summed with eight interleaved accumulators (one thread per accumulator chain
// in the row moments), and one thread per moment replays the post-order
// combine program.  Products use
// explicitly rounded intrinsics so nvcc cannot contract them into FMAs.  With
// f equal, densities and moments are then bit-identical to the reference's
// np.trapz (vlapy/core/field.py:36, vlapy/core/step.py:164-223).
#include "vg_internal.cuh"
#include "vg_f64_body.cuh"

namespace vg {


// One CTA per row.  The work of a NumPy pairwise sum is spread over the
// threads without changing a single rounding: (A) the integrand products of a
// group of qg moments are formed once per element into shared memory; (B)
// every leaf of <= 128 terms is NumPy's eight interleaved accumulators, each
// a serial chain that one thread runs; (C) one thread per leaf adds the eight
// in NumPy's order plus the tail terms; then one thread per moment replays
// the combine program over the leaves.  Moments of the second phase
// (MOM_DG2) use the vbar the first phase produced.
__global__ void k_row_moments_f64(const double* __restrict__ f, int nv, const double* __restrict__ v,
                                  const double* __restrict__ v_pow, MomSpec spec,
                                  const int* __restrict__ table, double dv,
                                  double* __restrict__ out, int ostride, int qg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nl = table[0];
  double* prod = reinterpret_cast<double*>(smem_raw);  // [qg][nv]
  double* acc = prod + (size_t)qg * nv;               // [qg][nl][8]
  double* leaf = acc + (size_t)qg * nl * 8;           // [nm][nl]
  __shared__ double res[MOM_STRIDE];
  const size_t r = blockIdx.x;
  const double* fr = f + r * nv;
  const int* leaves = table + 2;
  const int nm = spec.nm;
  for (int phase = 0; phase < 2; ++phase) {
    for (int q0 = 0; q0 < nm; q0 += qg) {
      auto active = [&](int q) { return q < nm && (spec.kind[q] == MOM_DG2) == (phase == 1); };
      // (A) products p_q(j)
      for (int idx = threadIdx.x; idx < qg * nv; idx += blockDim.x) {
        const int qq = idx / nv, j = idx - qq * nv, q = q0 + qq;
        if (!active(q)) continue;
        const int kind = spec.kind[q], arg = spec.arg[q];
        const double vbar = kind == MOM_DG2 ? res[arg] : 0.0;
        prod[idx] = mom_product(kind, arg, fr[j], j, v, v_pow, nv, vbar);
      }
      __syncthreads();
      // trapz term j: (dv * (p(j + 1) + p(j))) / 2
      auto term = [&](const double* pq, int j) { return mul_rn(dv, add_rn(pq[j + 1], pq[j])) * 0.5; };
      // (B) the accumulator chains
      for (int idx = threadIdx.x; idx < qg * nl * 8; idx += blockDim.x) {
        const int qq = idx / (nl * 8), rem = idx - qq * nl * 8, L = rem >> 3, a = rem & 7;
        if (!active(q0 + qq) || nv < 2) continue;
        const double* pq = prod + (size_t)qq * nv;
        const int st = leaves[2 * L], len = leaves[2 * L + 1];
        if (len < 8) {
          if (a == 0) {
            double x = 0.0;
            for (int i = 0; i < len; ++i) x = add_rn(x, term(pq, st + i));
            acc[(size_t)qq * nl * 8 + L * 8] = x;
          }
          continue;
        }
        const int stop = len - (len % 8);
        double x = term(pq, st + a);
        for (int i = 8 + a; i < stop; i += 8) x = add_rn(x, term(pq, st + i));
        acc[(size_t)qq * nl * 8 + L * 8 + a] = x;
      }
      __syncthreads();
      // (C) the leaves
      for (int idx = threadIdx.x; idx < qg * nl; idx += blockDim.x) {
        const int qq = idx / nl, L = idx - qq * nl, q = q0 + qq;
        if (!active(q) || nv < 2) continue;
        const double* pq = prod + (size_t)qq * nv;
        const double* ac = acc + (size_t)qq * nl * 8 + L * 8;
        const int st = leaves[2 * L], len = leaves[2 * L + 1];
        double x;
        if (len < 8) {
          x = ac[0];
        } else {
          x = add_rn(add_rn(add_rn(ac[0], ac[1]), add_rn(ac[2], ac[3])), add_rn(add_rn(ac[4], ac[5]), add_rn(ac[6], ac[7])));
          for (int i = len - (len % 8); i < len; ++i) x = add_rn(x, term(pq, st + i));
        }
        leaf[(size_t)q * nl + L] = x;
      }
      __syncthreads();
    }
    for (int q = threadIdx.x; q < nm; q += blockDim.x) {
      if ((spec.kind[q] == MOM_DG2) != (phase == 1)) continue;
      const double val = nv > 1 ? combine_leaves(table, leaf + (size_t)q * nl) : 0.0;
      res[q] = val;
      out[r * ostride + q] = val;
    }
    __syncthreads();
  }
}

cudaError_t launch_row_moments_f64(const vg_plan& p, const double* f, const MomSpec& spec,
                                   double* out, int out_stride, cudaStream_t s) {
  // products of as many moments at once as fit in 64 KB (at least one)
  const int nm = spec.nm;
  int qg = (int)(65536 / ((size_t)p.nv * sizeof(double)));
  qg = qg < 1 ? 1 : (qg > nm ? nm : qg);
  const size_t nl = (size_t)p.pw_v_leaves;
  const size_t smem = ((size_t)qg * p.nv + (size_t)qg * nl * 8 + (size_t)nm * nl) * sizeof(double);
  cudaError_t err = ensure_smem((const void*)k_row_moments_f64, smem);
  if (err != cudaSuccess) return err;
  k_row_moments_f64<<<p.nx, 256, smem, s>>>(f, p.nv, p.v, p.v_pow, spec, p.pw_v, p.dv, out, out_stride, qg);
  return cudaGetLastError();
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


template <int NX>
__global__ void __launch_bounds__(fft_threads<double>(NX)) k_poisson_fft_f64(
    const double* __restrict__ dens, int is_density, const double* __restrict__ inv_kx,
    const double* __restrict__ driver, int use_pulses, const vg_pulse* __restrict__ P, int np,
    const double* __restrict__ x, FieldTimeDev ft, const cx<double>* __restrict__ tw,
    double* __restrict__ e, int* flags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  poisson_fft_body<NX>(dens, is_density, inv_kx, driver, use_pulses, P, np, x, ft, tw, e,
                       reinterpret_cast<cx<double>*>(smem_raw), threadIdx.x, flags);
}

// Direct DFT for lengths that are not powers of two (O(nx^2), one CTA).
__global__ void k_poisson_dft_f64(const double* __restrict__ dens, int is_density, int nx,
                                  const double* __restrict__ inv_kx, const double* __restrict__ driver,
                                  int use_pulses, const vg_pulse* __restrict__ P, int np,
                                  const double* __restrict__ x, FieldTimeDev ft,
                                  double* __restrict__ work, double* __restrict__ e, int* flags) {
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
    const double en = driver_value(driver, use_pulses, P, np, tt, x, n) + acc / nx;
    e[n] = en;
    if (flags && !isfinite(en)) atomicOr(flags, VG_FLAG_NONFINITE);
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
                                           p.n_pulses, p.x, to_dev(ft), p.tw64, e, p.flags);
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
                                      p.n_pulses, p.x, to_dev(ft), p.etmp, e, p.flags);
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
  thomas_row_f64(f + (size_t)row * nv, bb + (size_t)row * 2 * nv, nv, v, vbar, vth, dougherty, nudt, dv, dv_sq);
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
