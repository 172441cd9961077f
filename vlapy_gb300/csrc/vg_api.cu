// C ABI of libvlagpu.so: plan lifetime, sub-operators and the time step.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "vg_internal.cuh"

namespace vg {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

int cuda_status(cudaError_t err, const char* what) {
  if (err == cudaSuccess) return VG_OK;
  set_error(std::string(what) + ": " + cudaGetErrorName(err) + " (" + cudaGetErrorString(err) + ")");
  return VG_ERR_CUDA;
}

int prof_collect(ProfState* ps, int n_kinds, const char* const* names, const double* bytes_per_launch,
                 vg_prof_entry* out, int max, int* n_out) {
  std::vector<double> ms(n_kinds, 0.0);
  std::vector<long long> cnt(n_kinds, 0);
  for (auto& r : ps->recs) {
    cudaError_t err = cudaEventSynchronize(r.e);
    if (err != cudaSuccess) return cuda_status(err, "profile sync");
    float t = 0.f;
    err = cudaEventElapsedTime(&t, r.b, r.e);
    if (err != cudaSuccess) return cuda_status(err, "profile elapsed");
    ms[r.kind] += t;
    cnt[r.kind] += 1;
  }
  ps->recs.clear();
  ps->used = 0;
  int n = 0;
  for (int k = 0; k < n_kinds; ++k) {
    if (!cnt[k] || n >= max) continue;
    std::memset(&out[n], 0, sizeof(vg_prof_entry));
    std::snprintf(out[n].name, sizeof(out[n].name), "%s", names[k]);
    out[n].launches = cnt[k];
    out[n].total_ms = ms[k];
    out[n].bytes_per_launch = bytes_per_launch[k];
    ++n;
  }
  *n_out = n;
  return VG_OK;
}

cudaError_t ensure_smem(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_pair(kernel, dev);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return cudaSuccess;
  cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err == cudaSuccess) done[key] = bytes;
  return err;
}

// NumPy pairwise-sum tree (numpy/_core/src/umath/loops_utils.h.src,
// pairwise_sum): blocks of <= 128 terms summed with 8 accumulators, larger
// ranges split at n/2 rounded down to a multiple of 8.
static void pairwise_tree(int start, int len, std::vector<int>& leaves, std::vector<int>& prog) {
  if (len <= 128) {
    prog.push_back((int)(leaves.size() / 2));
    leaves.push_back(start);
    leaves.push_back(len);
    return;
  }
  int half = len / 2;
  half -= half % 8;
  pairwise_tree(start, half, leaves, prog);
  pairwise_tree(start + half, len - half, leaves, prog);
  prog.push_back(-1);
}

std::vector<int> pairwise_table(int n) {
  std::vector<int> leaves, prog;
  pairwise_tree(0, n, leaves, prog);
  std::vector<int> out;
  out.push_back((int)(leaves.size() / 2));
  out.push_back((int)prog.size());
  out.insert(out.end(), leaves.begin(), leaves.end());
  out.insert(out.end(), prog.begin(), prog.end());
  return out;
}

struct GraphKey {
  const void* f;
  const void* e;
  const void* tb;
  const void* db;
  vg_history h;
  int i0, n;
  cudaStream_t s;
  bool operator<(const GraphKey& o) const { return std::memcmp(this, &o, sizeof(GraphKey)) < 0; }
};
struct GraphCache {
  std::map<GraphKey, cudaGraphExec_t> execs;
};

// Kernel kinds of the step sequence, for vg_profile_*.  PK_ROW32: a leapfrog
// step's row pass with the next step's leading half kick (and the kick-free
// row pass of the composed integrators); PK_ROW32_LAST: the last leapfrog
// step's of a call, which ends without it.
enum ProfKind {
  PK_EDFDV = 0, PK_VDFDX, PK_DENSITY, PK_POISSON, PK_FP_MOMENTS, PK_FP_SOLVE, PK_STORAGE,
  PK_X_DRIFT32, PK_FIELD32, PK_ROW32, PK_KICK32, PK_STORE32, PK_ROW32_LAST, PK_COUNT
};
static const char* kProfNames[PK_COUNT] = {"edfdv", "vdfdx", "density", "poisson", "fp_moments", "fp_solve",
                                            "storage", "x_drift_f32", "field_f32", "row_pass_f32", "kick_f32",
                                            "store_f32", "row_pass_last_f32"};

// algorithmic DRAM bytes of one launch of each kind: the f traffic the
// operation cannot avoid (read + write of f for in-place transforms, one
// read for reductions), FP64 elements
static double prof_bytes(const vg_plan* p, int kind) {
  const double cells = (double)p->nx * (double)p->nv;
  const double es = p->precision == VG_F64 ? 8.0 : 4.0;
  switch (kind) {
    case PK_EDFDV:
    case PK_VDFDX:
    case PK_FP_SOLVE: return 2.0 * es * cells;
    case PK_DENSITY:
    case PK_FP_MOMENTS:
    case PK_STORAGE: return es * cells;
    case PK_X_DRIFT32:
    case PK_ROW32:
    case PK_ROW32_LAST:
    case PK_KICK32: return 2.0 * 4.0 * cells;
    case PK_STORE32: return 8.0 * 8.0 * p->nx;
    default: return 3.0 * 8.0 * p->nx;
  }
}

}  // namespace vg

using namespace vg;

namespace {

template <typename T>
int dev_copy(T** dst, const T* src, size_t n, const char* what) {
  *dst = nullptr;
  if (n == 0) return VG_OK;
  cudaError_t err = cudaMalloc(reinterpret_cast<void**>(dst), n * sizeof(T));
  if (err != cudaSuccess) return cuda_status(err, what);
  if (src) {
    err = cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
    if (err != cudaSuccess) return cuda_status(err, what);
  } else {
    err = cudaMemset(*dst, 0, n * sizeof(T));
    if (err != cudaSuccess) return cuda_status(err, what);
  }
  return VG_OK;
}

void free_plan(vg_plan* p) {
  if (!p) return;
  void* ptrs[] = {p->x, p->v, p->kx, p->kv, p->inv_kx, p->v_pow, p->f_bg, p->pulses, p->tw64, p->tw32,
                  p->pw_v, p->pw_x, p->dens, p->mom, p->bb, p->rho, p->etmp, p->sl_m, p->sl_w, p->flags};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (p->graph_cache) {
    auto* gc = static_cast<GraphCache*>(p->graph_cache);
    for (auto& kv : gc->execs) cudaGraphExecDestroy(kv.second);
    delete gc;
  }
  delete static_cast<ProfState*>(p->prof);
  if (p->f32) {
    F32Plan* q = p->f32;
    void* qp[] = {q->F0, q->v32, q->f0_32, q->S, q->Mv, q->D, q->dpart, q->mpart, q->spart, q->vhl, q->e32, q->rc_dev};
    for (void* x : qp)
      if (x) cudaFree(x);
    delete q;
  }
  delete p;
}

#define VG_CHECK(expr)            \
  do {                            \
    int _st = (expr);             \
    if (_st != VG_OK) return _st; \
  } while (0)

int require_plan(const vg_plan* p) {
  if (!p) {
    set_error("null plan");
    return VG_ERR_ARG;
  }
  return VG_OK;
}

// exponential advection sizes: powers of two by shared-memory FFTs, other
// lengths by direct DFTs (shared memory holds 5 N doubles of a line)
int require_fft_v(const vg_plan* p) {
  if (p->nv_pow2 ? p->nv > 8192 : p->nv > DFT_ADVECT_NMAX) {
    set_error("v-advection needs nv a power of two <= 8192 or any nv <= " + std::to_string(DFT_ADVECT_NMAX) +
              ", got " + std::to_string(p->nv));
    return VG_ERR_UNSUPPORTED;
  }
  return VG_OK;
}

int require_fft_x(const vg_plan* p) {
  if (p->nx_pow2 ? p->nx > 8192 : p->nx > DFT_ADVECT_NMAX) {
    set_error("x-advection needs nx a power of two <= 8192 or any nx <= " + std::to_string(DFT_ADVECT_NMAX) +
              ", got " + std::to_string(p->nx));
    return VG_ERR_UNSUPPORTED;
  }
  return VG_OK;
}

template <typename Fn>
cudaError_t prof_run(vg_plan* p, int kind, cudaStream_t s, Fn fn) {
  return prof_call(static_cast<ProfState*>(p->prof), kind, s, fn);
}

// One FP step: moments of the operator, then the tridiagonal solve.
int collision_f64(vg_plan* p, double* f, cudaStream_t s) {
  if (p->collision == VG_COLL_NONE) return VG_OK;
  MomSpec spec;
  if (p->collision == VG_COLL_DG) {
    spec.nm = 2;
    spec.kind[0] = MOM_V;   // vbar = trapz(f v)
    spec.arg[0] = 0;
    spec.kind[1] = MOM_DG2; // v0t^2 = trapz(f (v - vbar)^2)
    spec.arg[1] = 0;
  } else {
    spec.nm = 2;
    spec.kind[0] = MOM_ONE;  // unused slot, keeps the column layout of the DG case
    spec.arg[0] = 0;
    spec.kind[1] = MOM_W;    // v0t^2 = trapz(f v**2.0)
    spec.arg[1] = 0;
  }
  VG_CHECK(cuda_status(prof_run(p, PK_FP_MOMENTS, s, [&] { return launch_row_moments_f64(*p, f, spec, p->mom, MOM_STRIDE, s); }),
                       "collision moments"));
  return cuda_status(prof_run(p, PK_FP_SOLVE, s, [&] { return launch_thomas_f64(*p, f, p->mom, 0, 1, s); }),
                     "tridiagonal solve");
}

int field_f64(vg_plan* p, const double* f, const double* driver, const FieldTime& ft, double* e,
              cudaStream_t s) {
  MomSpec spec;
  spec.nm = 1;
  spec.kind[0] = MOM_ONE;
  spec.arg[0] = 0;
  VG_CHECK(cuda_status(prof_run(p, PK_DENSITY, s, [&] { return launch_row_moments_f64(*p, f, spec, p->dens, 1, s); }),
                       "charge density"));
  return cuda_status(prof_run(p, PK_POISSON, s, [&] { return launch_poisson_f64(*p, p->dens, 1, driver, ft, e, s); }),
                     "poisson");
}

// The launch sequence of nsteps steps (vlapy/core/step.py:302-326).
int step_sequence_f64(vg_plan* p, double* f, double* e, const vg_history* h, const double* tb,
                      const double* db, int i0, int nsteps, cudaStream_t s) {
  const double dt = p->dt;
  for (int k = 0; k < nsteps; ++k) {
    const int i = i0 + k;
    FieldTime ft;
    ft.t_ptr = tb + i;
    ft.t_host = 0.0;
    ft.use_pulses = p->n_pulses > 0;
    auto field_at = [&](std::initializer_list<double> adds) {
      ft.nadd = 0;
      for (double a : adds) ft.add[ft.nadd++] = a;
      return field_f64(p, f, nullptr, ft, e, s);
    };
    auto E = [&](double d) {
      return cuda_status(prof_run(p, PK_EDFDV, s, [&] { return launch_edfdv_f64(*p, f, e, d, s); }), "edfdv");
    };
    auto X = [&](double d) {
      return cuda_status(prof_run(p, PK_VDFDX, s, [&] { return launch_vdfdx_f64(*p, f, d, s); }), "vdfdx");
    };
    if (p->integrator == VG_LEAPFROG) {
      // vlapy/core/vlasov_poisson.py:36-58
      VG_CHECK(E(0.5 * dt));
      VG_CHECK(X(dt));
      VG_CHECK(field_at({dt}));
      VG_CHECK(E(0.5 * dt));
    } else if (p->integrator == VG_PEFRL) {
      // vlapy/core/vlasov_poisson.py:82-152
      const double xsi = 0.1786178958448091, lambd = -0.2123418310626054, chi = -0.6626458266981849e-1;
      const double d1 = xsi * dt, d2 = chi * dt, d3 = (1.0 - 2.0 * (chi + xsi)) * dt, d4 = d2, d5 = d1;
      const double k1 = 0.5 * (1.0 - 2.0 * lambd) * dt, k2 = lambd * dt, k3 = k2, k4 = k1;
      VG_CHECK(X(d1));
      VG_CHECK(field_at({d1}));
      VG_CHECK(E(k1));
      VG_CHECK(X(d2));
      VG_CHECK(field_at({d1, d2}));
      VG_CHECK(E(k2));
      VG_CHECK(X(d3));
      VG_CHECK(field_at({d1, d2, d3}));
      VG_CHECK(E(k3));
      VG_CHECK(X(d4));
      VG_CHECK(field_at({d1, d2, d3, d4}));
      VG_CHECK(E(k4));
      VG_CHECK(X(d5));
      VG_CHECK(field_at({d1, d2, d3, d4, d5}));
    } else {
      // vlapy/core/vlasov_poisson.py:157-232
      const double a1 = 0.168735950563437422448196, a2 = 0.377851589220928303880766,
                   a3 = -0.093175079568731452657924, b1 = 0.049086460976116245491441,
                   b2 = 0.264177609888976700200146, b3 = 0.186735929134907054308413,
                   c1 = -0.000069728715055305084099, c2 = -0.000625704827430047189169,
                   c3 = -0.002213085124045325561636, d2c = -2.916600457689847816445691e-6,
                   d3c = 3.048480261700038788680723e-5, e3 = 4.985549387875068121593988e-7;
      const double D1 = b1 + 2.0 * c1 * std::pow(dt, 2.0);
      const double D2 = b2 + 2.0 * c2 * std::pow(dt, 2.0) + 4.0 * d2c * std::pow(dt, 4.0);
      const double D3 = b3 + 2.0 * c3 * std::pow(dt, 2.0) + 4.0 * d3c * std::pow(dt, 4.0) -
                        8.0 * e3 * std::pow(dt, 6.0);
      const double xs[5] = {a1, a2, a3, a2, a1};
      const double ks[5] = {D2, D3, D3, D2, D1};
      VG_CHECK(E(D1 * dt));
      for (int q = 0; q < 5; ++q) {
        VG_CHECK(X(xs[q] * dt));
        VG_CHECK(field_at({xs[q] * dt}));
        VG_CHECK(E(ks[q] * dt));
      }
    }
    VG_CHECK(collision_f64(p, f, s));
    if (h) {
      const double* de = db ? db + (size_t)i * p->nx : nullptr;
      VG_CHECK(cuda_status(prof_run(p, PK_STORAGE, s, [&] { return launch_storage_f64(*p, f, e, de, *h, i, s); }),
                           "storage step"));
    }
  }
  return VG_OK;
}

// forward FFT (sign -1) of a power-of-two length, host double precision
void host_fft(std::vector<double>& re, std::vector<double>& im) {
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
    for (size_t i = 0; i < n; i += len) {
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
}

template <typename T>
int upload(T** dst, const std::vector<T>& src, const char* what) {
  return dev_copy(dst, src.data(), src.size(), what);
}

// Constants of the delta-f path: the background f0 in FP32, its collision
// stencils and spectrum, and its moments in FP64.
int setup_f32(vg_plan* p, const vg_run_desc* d) {
  if (!p->nv_pow2 || !p->nx_pow2 || p->nv > 16384 || p->nx > 8192) {
    set_error("the FP32 delta-f mode needs power-of-two nx <= 8192 and nv <= 16384");
    return VG_ERR_UNSUPPORTED;
  }
  F32Plan* q = new F32Plan();
  std::memset(q, 0, sizeof(F32Plan));
  p->f32 = q;
  const int nv = d->nv, nx = d->nx;
  const double dv = d->dv, dv2 = d->dv_sq;
  const double* f0 = d->f_background;
  const double* v = d->v;
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
    double vp_ = 1.0;
    for (int k = 0; k < 6; ++k) {
      mom[k] += w * f0[j] * vp_;
      vp_ *= v[j];
    }
    mom[6] += w * f0[j] * f0[j];
  }
  for (int k = 0; k < 7; ++k) mom[k] *= dv;
  std::vector<double> re(f0, f0 + nv), im(nv, 0.0);
  host_fft(re, im);
  std::vector<cx<float>> F0(nv / 2 + 1);
  for (int k = 0; k <= nv / 2; ++k) F0[k] = {(float)re[k], (float)im[k]};
  VG_CHECK(upload(&q->v32, v32, "f32 constants"));
  VG_CHECK(upload(&q->f0_32, f32v, "f32 constants"));
  VG_CHECK(upload(&q->S, S, "f32 constants"));
  VG_CHECK(upload(&q->Mv, Mv, "f32 constants"));
  VG_CHECK(upload(&q->D, D, "f32 constants"));
  VG_CHECK(upload(&q->F0, F0, "f32 constants"));
  VG_CHECK(upload(&q->vhl, vhl, "f32 constants"));
  VG_CHECK(dev_copy<float>(&q->e32, nullptr, (size_t)nx, "f32 field"));
  q->dkx = nx > 1 ? d->kx[1] : 0.0;
  q->dkv = d->kv[1];
  q->c0 = mom[0] - 1.0;
  q->rc.v = q->v32;
  q->rc.f0 = q->f0_32;
  q->rc.S = q->S;
  q->rc.Mv = q->Mv;
  q->rc.D = q->D;
  q->rc.vhl = q->vhl;
  q->rc.i2dv = (float)(0.5 / dv);
  q->rc.v0f = (float)v[0];
  q->rc.dvf = (float)dv;
  q->rc.dv = dv;
  q->rc.dv_sq = dv2;
  q->rc.dkv = q->dkv;
  for (int k = 0; k < 7; ++k) q->rc.f0m[k] = mom[k];
  q->rc.dv2f = split_f2(dv);
  q->rc.idv2f = split_f2(1.0 / dv2);
  for (int k = 0; k < 3; ++k) q->rc.f0m2f[k] = split_f2(mom[k]);
  VG_CHECK(upload(&q->rc_dev, std::vector<RowConsts>(1, q->rc), "f32 constants"));
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  q->n_sm = nsm;
  q->col_grid_max = 8 * nsm;
  q->row_grid_max = 8 * nsm;
  VG_CHECK(dev_copy<float2>(&q->dpart, nullptr, (size_t)q->col_grid_max * nx, "density partials"));
  VG_CHECK(dev_copy<cx<float>>(&q->mpart, nullptr, (size_t)q->row_grid_max * F32_MAX_MODES * nv, "mode partials"));
  VG_CHECK(dev_copy<float2>(&q->spart, nullptr, (size_t)F32_STORE_MAX_CTAS * 7, "series partials"));
  return VG_OK;
}

int modes_of(const vg_history* h) {
  return (h && h->stored_f && !h->store_all) ? h->n_modes : 0;
}

// The FP32 delta-f launch sequence of nsteps steps.  For leapfrog the second
// half kick of step n and the first of step n+1 use the same field and run in
// the same row pass, around the collision step and the storage moments.
int step_sequence_f32(vg_plan* p, float* g, double* e, const vg_history* h, const double* tb, const double* db,
                      int i0, int nsteps, cudaStream_t s) {
  const double dt = p->dt;
  const int nm = modes_of(h);
  auto X = [&](double d) {
    return cuda_status(prof_run(p, PK_X_DRIFT32, s, [&] { return launch_col_f32(*p, g, d, s); }), "x drift");
  };
  auto K = [&](double d) {
    return cuda_status(prof_run(p, PK_KICK32, s, [&] { return launch_row_f32(*p, g, e, d, 0.0, 0, 0, 0, s); }),
                       "kick");
  };
  FieldTime ft;
  ft.t_host = 0.0;
  ft.use_pulses = p->n_pulses > 0;
  auto F = [&](int i, std::initializer_list<double> adds) {
    ft.t_ptr = tb + i;
    ft.nadd = 0;
    for (double a : adds) ft.add[ft.nadd++] = a;
    return cuda_status(prof_run(p, PK_FIELD32, s, [&] { return launch_field_f32(*p, nullptr, ft, e, s); }),
                       "field");
  };
  auto STORE = [&](int i) -> int {
    if (!h) return VG_OK;
    const double* de = db ? db + (size_t)i * p->nx : nullptr;
    return cuda_status(prof_run(p, PK_STORE32, s, [&] { return launch_store_f32(*p, g, e, de, *h, i, nm, s); }),
                       "store");
  };
  VG_CHECK(cuda_status(launch_e_to_f32(*p, e, s), "field copy"));
  if (p->integrator == VG_LEAPFROG) {
    VG_CHECK(K(0.5 * dt));
    for (int k = 0; k < nsteps; ++k) {
      const int i = i0 + k;
      VG_CHECK(X(dt));
      VG_CHECK(F(i, {dt}));
      const bool last = k + 1 == nsteps;
      const double trail = last ? 0.0 : 0.5 * dt;
      VG_CHECK(cuda_status(prof_run(p, last ? PK_ROW32_LAST : PK_ROW32, s, [&] {
                             return launch_row_f32(*p, g, e, 0.5 * dt, trail, 1, h != nullptr, nm, s);
                           }),
                           "row pass"));
      VG_CHECK(STORE(i));
    }
    return VG_OK;
  }
  for (int k = 0; k < nsteps; ++k) {
    const int i = i0 + k;
    if (p->integrator == VG_PEFRL) {
      const double xsi = 0.1786178958448091, lambd = -0.2123418310626054, chi = -0.6626458266981849e-1;
      const double d1 = xsi * dt, d2 = chi * dt, d3 = (1.0 - 2.0 * (chi + xsi)) * dt, d4 = d2, d5 = d1;
      const double k1 = 0.5 * (1.0 - 2.0 * lambd) * dt, k2 = lambd * dt, k3 = k2, k4 = k1;
      VG_CHECK(X(d1));
      VG_CHECK(F(i, {d1}));
      VG_CHECK(K(k1));
      VG_CHECK(X(d2));
      VG_CHECK(F(i, {d1, d2}));
      VG_CHECK(K(k2));
      VG_CHECK(X(d3));
      VG_CHECK(F(i, {d1, d2, d3}));
      VG_CHECK(K(k3));
      VG_CHECK(X(d4));
      VG_CHECK(F(i, {d1, d2, d3, d4}));
      VG_CHECK(K(k4));
      VG_CHECK(X(d5));
      VG_CHECK(F(i, {d1, d2, d3, d4, d5}));
    } else {
      const double a1 = 0.168735950563437422448196, a2 = 0.377851589220928303880766,
                   a3 = -0.093175079568731452657924, b1 = 0.049086460976116245491441,
                   b2 = 0.264177609888976700200146, b3 = 0.186735929134907054308413,
                   c1 = -0.000069728715055305084099, c2 = -0.000625704827430047189169,
                   c3 = -0.002213085124045325561636, d2c = -2.916600457689847816445691e-6,
                   d3c = 3.048480261700038788680723e-5, e3 = 4.985549387875068121593988e-7;
      const double D1 = b1 + 2.0 * c1 * std::pow(dt, 2.0);
      const double D2 = b2 + 2.0 * c2 * std::pow(dt, 2.0) + 4.0 * d2c * std::pow(dt, 4.0);
      const double D3 = b3 + 2.0 * c3 * std::pow(dt, 2.0) + 4.0 * d3c * std::pow(dt, 4.0) -
                        8.0 * e3 * std::pow(dt, 6.0);
      const double xs[5] = {a1, a2, a3, a2, a1};
      const double ks[5] = {D2, D3, D3, D2, D1};
      VG_CHECK(K(D1 * dt));
      for (int q = 0; q < 5; ++q) {
        VG_CHECK(X(xs[q] * dt));
        VG_CHECK(F(i, {xs[q] * dt}));
        VG_CHECK(K(ks[q] * dt));
      }
    }
    VG_CHECK(cuda_status(prof_run(p, PK_ROW32, s, [&] {
                           return launch_row_f32(*p, g, e, 0.0, 0.0, 1, h != nullptr, nm, s);
                         }),
                         "row pass"));
    VG_CHECK(STORE(i));
  }
  return VG_OK;
}

}  // namespace

extern "C" {

int vg_version(void) { return 1; }

const char* vg_last_error(void) { return g_err.c_str(); }

int vg_plan_create(const vg_run_desc* d, vg_plan** out) {
  if (!d || !out) {
    set_error("null descriptor or output pointer");
    return VG_ERR_ARG;
  }
  *out = nullptr;
  if (d->nx < 2 || d->nv < 2) {
    set_error("nx and nv must be >= 2");
    return VG_ERR_ARG;
  }
  if (!d->x || !d->v || !d->kx || !d->kv || !d->one_over_kx || !d->v_pow) {
    set_error("descriptor arrays x, v, kx, kv, one_over_kx, v_pow are required");
    return VG_ERR_ARG;
  }
  if (d->precision != VG_F64 && d->precision != VG_F32_DELTA_F) {
    set_error("unknown precision mode");
    return VG_ERR_ARG;
  }
  if (d->precision == VG_F32_DELTA_F && !d->f_background) {
    set_error("VG_F32_DELTA_F needs f_background");
    return VG_ERR_ARG;
  }
  if (d->collision < VG_COLL_NONE || d->collision > VG_COLL_DG || d->integrator < VG_LEAPFROG ||
      d->integrator > VG_H_SIXTH || d->n_pulses < 0 || (d->n_pulses > 0 && !d->pulses)) {
    set_error("bad collision, integrator or pulse fields");
    return VG_ERR_ARG;
  }
  vg_plan* p = new vg_plan();
  std::memset(p, 0, sizeof(vg_plan));
  p->nx = d->nx;
  p->nv = d->nv;
  p->precision = d->precision;
  p->collision = d->collision;
  p->integrator = d->integrator;
  p->n_pulses = d->n_pulses;
  p->dt = d->dt;
  p->nu = d->nu;
  p->dx = d->dx;
  p->dv = d->dv;
  p->dv_sq = d->dv_sq;
  p->nudt = d->nu * d->dt;
  p->nx_pow2 = is_pow2(d->nx);
  p->nv_pow2 = is_pow2(d->nv);
  const size_t nx = d->nx, nv = d->nv;
  int st = VG_OK;
#define TRY(expr)                         \
  do {                                    \
    st = (expr);                          \
    if (st != VG_OK) {                    \
      free_plan(p);                       \
      return st;                          \
    }                                     \
  } while (0)
  TRY(dev_copy(&p->x, d->x, nx, "x"));
  TRY(dev_copy(&p->v, d->v, nv, "v"));
  TRY(dev_copy(&p->kx, d->kx, nx, "kx"));
  TRY(dev_copy(&p->kv, d->kv, nv, "kv"));
  TRY(dev_copy(&p->inv_kx, d->one_over_kx, nx, "one_over_kx"));
  TRY(dev_copy(&p->v_pow, d->v_pow, 5 * nv, "v_pow"));
  if (d->f_background) TRY(dev_copy(&p->f_bg, d->f_background, nv, "f_background"));
  if (d->n_pulses > 0) TRY(dev_copy(&p->pulses, d->pulses, (size_t)d->n_pulses, "pulses"));
  TRY(dev_copy<cx<double>>(&p->tw64, nullptr, FFT_NMAX, "twiddles"));
  TRY(dev_copy<cx<float>>(&p->tw32, nullptr, FFT_NMAX, "twiddles"));
  std::vector<int> tv = pairwise_table(d->nv - 1), tx = pairwise_table(d->nx);
  p->pw_v_leaves = tv[0];
  p->pw_x_leaves = tx[0];
  p->pw_v_words = (int)tv.size();
  p->pw_x_words = (int)tx.size();
  TRY(dev_copy(&p->pw_v, tv.data(), tv.size(), "pairwise table"));
  TRY(dev_copy(&p->pw_x, tx.data(), tx.size(), "pairwise table"));
  TRY(dev_copy<double>(&p->dens, nullptr, nx, "scratch"));
  TRY(dev_copy<double>(&p->mom, nullptr, nx * MOM_STRIDE, "scratch"));
  TRY(dev_copy<double>(&p->rho, nullptr, nx, "scratch"));
  TRY(dev_copy<double>(&p->etmp, nullptr, 4 * nx + 4, "scratch"));
  TRY(dev_copy<int>(&p->flags, nullptr, 1, "status"));
  if (d->precision == VG_F64 && d->collision != VG_COLL_NONE)
    TRY(dev_copy<double>(&p->bb, nullptr, 2 * nx * nv, "thomas scratch"));
  if (d->precision == VG_F32_DELTA_F) TRY(setup_f32(p, d));
  TRY(cuda_status(launch_twiddles(*p, 0), "twiddles"));
  TRY(cuda_status(cudaDeviceSynchronize(), "plan setup"));
  p->graph_cache = new GraphCache();
  p->prof = new ProfState();
#undef TRY
  *out = p;
  return VG_OK;
}

int vg_plan_destroy(vg_plan* p) {
  if (!p) return VG_OK;
  cudaDeviceSynchronize();
  free_plan(p);
  return VG_OK;
}

int vg_plan_status(vg_plan* p, int32_t* flags) {
  VG_CHECK(require_plan(p));
  if (!flags) {
    set_error("null flags");
    return VG_ERR_ARG;
  }
  int h = 0;
  VG_CHECK(cuda_status(cudaMemcpy(&h, p->flags, sizeof(int), cudaMemcpyDeviceToHost), "plan status"));
  *flags = h;
  if (h & VG_FLAG_NONFINITE) {
    set_error("a field solve produced NaN or Inf (the steps from it on are not valid)");
    return VG_ERR_NUMERIC;
  }
  return VG_OK;
}

int vg_edfdv(vg_plan* p, void* f, const double* e, double dt, vg_stream stream) {
  VG_CHECK(require_plan(p));
  if (!f || !e) {
    set_error("null f or e");
    return VG_ERR_ARG;
  }
  if (p->f32) {
    cudaStream_t s = (cudaStream_t)stream;
    VG_CHECK(cuda_status(launch_e_to_f32(*p, e, s), "field copy"));
    return cuda_status(launch_row_f32(*p, static_cast<float*>(f), e, dt, 0.0, 0, 0, 0, s), "edfdv");
  }
  VG_CHECK(require_fft_v(p));
  return cuda_status(launch_edfdv_f64(*p, static_cast<double*>(f), e, dt, (cudaStream_t)stream), "edfdv");
}

int vg_vdfdx(vg_plan* p, void* f, double dt, vg_stream stream) {
  VG_CHECK(require_plan(p));
  if (!f) {
    set_error("null f");
    return VG_ERR_ARG;
  }
  if (p->f32) return cuda_status(launch_col_f32(*p, static_cast<float*>(f), dt, (cudaStream_t)stream), "vdfdx");
  VG_CHECK(require_fft_x(p));
  return cuda_status(launch_vdfdx_f64(*p, static_cast<double*>(f), dt, (cudaStream_t)stream), "vdfdx");
}

namespace {

// checks shared by the out-of-place FP64 alternatives: an FP64 plan, distinct
// non-null buffers, and the grid sizes the reference's own routine accepts
int require_alt(const vg_plan* p, const void* fin, const void* fout, int min_nx, int min_nv, const char* what) {
  VG_CHECK(require_plan(p));
  if (p->f32) {
    set_error(std::string(what) + " is implemented in the FP64 mode only");
    return VG_ERR_UNSUPPORTED;
  }
  if (!fin || !fout) {
    set_error(std::string(what) + ": null f_in or f_out");
    return VG_ERR_ARG;
  }
  if (fin == fout) {
    set_error(std::string(what) + " is out of place: f_out must not be f_in");
    return VG_ERR_ARG;
  }
  if (p->nx < min_nx || p->nv < min_nv) {
    set_error(std::string(what) + " needs nx >= " + std::to_string(min_nx) + " and nv >= " +
              std::to_string(min_nv) + ", got " + std::to_string(p->nx) + " x " + std::to_string(p->nv));
    return VG_ERR_ARG;
  }
  return VG_OK;
}

}  // namespace

int vg_vdfdx_sl(vg_plan* p, const double* f_in, double* f_out, double dt, vg_stream stream) {
  // x_pad needs x[2] (nx >= 3); the cubic spline along v needs nv >= 4
  VG_CHECK(require_alt(p, f_in, f_out, 3, 4, "vdfdx sl"));
  VG_CHECK(cuda_status(ensure_sl_scratch(*p), "sl scratch"));
  return cuda_status(launch_vdfdx_sl_f64(*p, f_in, f_out, dt, (cudaStream_t)stream), "vdfdx sl");
}

int vg_edfdv_sl(vg_plan* p, const double* f_in, const double* e, double* f_out, double dt, vg_stream stream) {
  // the cubic spline along x (and the cubic fit of e) needs nx >= 4; v_pad needs v[2]
  VG_CHECK(require_alt(p, f_in, f_out, 4, 3, "edfdv sl"));
  if (!e) {
    set_error("edfdv sl: null e");
    return VG_ERR_ARG;
  }
  VG_CHECK(cuda_status(ensure_sl_scratch(*p), "sl scratch"));
  return cuda_status(launch_edfdv_sl_f64(*p, f_in, e, f_out, dt, (cudaStream_t)stream), "edfdv sl");
}

int vg_edfdv_cd2(vg_plan* p, const double* f_in, const double* e, double* f_out, double dt, vg_stream stream) {
  // numpy.gradient with edge_order=2 needs three points along v
  VG_CHECK(require_alt(p, f_in, f_out, 1, 3, "edfdv cd2"));
  if (!e) {
    set_error("edfdv cd2: null e");
    return VG_ERR_ARG;
  }
  return cuda_status(launch_edfdv_cd2_f64(*p, f_in, e, f_out, dt, (cudaStream_t)stream), "edfdv cd2");
}

int vg_charge_density(vg_plan* p, const void* f, double* n, vg_stream stream) {
  VG_CHECK(require_plan(p));
  if (!f || !n) {
    set_error("null f or n");
    return VG_ERR_ARG;
  }
  if (p->f32)
    return cuda_status(launch_dens_rows_f32(*p, static_cast<const float*>(f), n, 1, (cudaStream_t)stream),
                       "charge density");
  MomSpec spec;
  spec.nm = 1;
  spec.kind[0] = MOM_ONE;
  spec.arg[0] = 0;
  return cuda_status(launch_row_moments_f64(*p, static_cast<const double*>(f), spec, n, 1, (cudaStream_t)stream),
                     "charge density");
}

int vg_poisson(vg_plan* p, const double* rho, double* e, vg_stream stream) {
  VG_CHECK(require_plan(p));
  if (!rho || !e) {
    set_error("null rho or e");
    return VG_ERR_ARG;
  }
  FieldTime ft{};
  ft.use_pulses = 0;
  return cuda_status(launch_poisson_f64(*p, rho, 0, nullptr, ft, e, (cudaStream_t)stream), "poisson");
}

int vg_field_solve(vg_plan* p, const void* f, const double* driver, double* e, vg_stream stream) {
  VG_CHECK(require_plan(p));
  if (!f || !e) {
    set_error("null f or e");
    return VG_ERR_ARG;
  }
  FieldTime ft{};
  ft.use_pulses = 0;
  if (p->f32) {
    cudaStream_t s = (cudaStream_t)stream;
    VG_CHECK(cuda_status(launch_dens_rows_f32(*p, static_cast<const float*>(f), p->rho, 0, s), "density"));
    return cuda_status(launch_poisson_only_f32(*p, p->rho, driver, ft, e, s), "poisson");
  }
  return field_f64(p, static_cast<const double*>(f), driver, ft, e, (cudaStream_t)stream);
}

int vg_collision_step(vg_plan* p, void* f, vg_stream stream) {
  VG_CHECK(require_plan(p));
  if (!f) {
    set_error("null f");
    return VG_ERR_ARG;
  }
  if (p->f32) {
    if (p->collision == VG_COLL_NONE) return VG_OK;
    return cuda_status(launch_row_f32(*p, static_cast<float*>(f), nullptr, 0.0, 0.0, 1, 0, 0, (cudaStream_t)stream),
                       "collision step");
  }
  return collision_f64(p, static_cast<double*>(f), (cudaStream_t)stream);
}

static int check_history(const vg_plan* p, const vg_history* h, int i_last) {
  if (!h) return VG_OK;
  if (i_last >= h->nt) {
    set_error("storage index beyond the history length");
    return VG_ERR_STATE;
  }
  if (h->stored_f && !h->store_all) {
    if (h->n_slots < 1 || h->n_modes < 1 || (h->n_modes != 1 && h->n_modes != h->n_slots) ||
        h->n_modes > p->nx) {
      set_error("stored_f: n_modes must be 1 or equal n_slots, and <= nx");
      return VG_ERR_ARG;
    }
  }
  return VG_OK;
}

int vg_storage_step(vg_plan* p, const void* f, const double* e, const double* de, const vg_history* h,
                    int32_t i, vg_stream stream) {
  VG_CHECK(require_plan(p));
  if (!f || !e || !h || i < 0) {
    set_error("null f, e or history, or negative index");
    return VG_ERR_ARG;
  }
  VG_CHECK(check_history(p, h, i));
  if (p->f32) {
    cudaStream_t s = (cudaStream_t)stream;
    const int nm = modes_of(h);
    float* g = const_cast<float*>(static_cast<const float*>(f));
    VG_CHECK(cuda_status(launch_row_f32(*p, g, e, 0.0, 0.0, 0, 1, nm, s), "storage moments"));
    return cuda_status(launch_store_f32(*p, g, e, de, *h, i, nm, s), "storage step");
  }
  return cuda_status(launch_storage_f64(*p, static_cast<const double*>(f), e, de, *h, i, (cudaStream_t)stream),
                     "storage step");
}

int vg_driver(vg_plan* p, double t, double* out, vg_stream stream) {
  VG_CHECK(require_plan(p));
  if (!out) {
    set_error("null output");
    return VG_ERR_ARG;
  }
  FieldTime ft{};
  ft.t_ptr = nullptr;
  ft.t_host = t;
  ft.nadd = 0;
  ft.use_pulses = 1;
  return cuda_status(launch_driver(*p, ft, out, (cudaStream_t)stream), "driver");
}

int vg_run_steps(vg_plan* p, void* f, double* e, const vg_history* h, const double* time_batch,
                 const double* driver_batch, int32_t i0, int32_t nsteps, int32_t use_graph, vg_stream stream) {
  VG_CHECK(require_plan(p));
  if (!p->f32) {
    VG_CHECK(require_fft_v(p));
    VG_CHECK(require_fft_x(p));
  }
  if (!f || !e || !time_batch || i0 < 0 || nsteps < 0) {
    set_error("null f, e or time_batch, or negative step range");
    return VG_ERR_ARG;
  }
  if (nsteps == 0) return VG_OK;
  VG_CHECK(check_history(p, h, i0 + nsteps - 1));
  if (p->f32 && modes_of(h) > F32_MAX_MODES) {
    set_error("the FP32 delta-f mode stores at most 4 x-Fourier modes per step");
    return VG_ERR_UNSUPPORTED;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* fd = static_cast<double*>(f);
  if (static_cast<ProfState*>(p->prof)->enabled) use_graph = 0;
  auto seq = [&]() {
    return p->f32 ? step_sequence_f32(p, static_cast<float*>(f), e, h, time_batch, driver_batch, i0, nsteps, s)
                  : step_sequence_f64(p, fd, e, h, time_batch, driver_batch, i0, nsteps, s);
  };
  if (!use_graph) return seq();
  auto* gc = static_cast<GraphCache*>(p->graph_cache);
  GraphKey key;
  std::memset(&key, 0, sizeof(key));
  key.f = f;
  key.e = e;
  key.tb = time_batch;
  key.db = driver_batch;
  if (h) key.h = *h;
  key.i0 = i0;
  key.n = nsteps;
  key.s = s;
  auto it = gc->execs.find(key);
  if (it == gc->execs.end()) {
    if (s == 0) {
      set_error("graph mode needs a non-default stream");
      return VG_ERR_ARG;
    }
    VG_CHECK(cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed), "begin capture"));
    int st = seq();
    cudaGraph_t graph = nullptr;
    cudaError_t cerr = cudaStreamEndCapture(s, &graph);
    if (st != VG_OK) {
      if (graph) cudaGraphDestroy(graph);
      return st;
    }
    VG_CHECK(cuda_status(cerr, "end capture"));
    cudaGraphExec_t exec = nullptr;
    cerr = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    VG_CHECK(cuda_status(cerr, "graph instantiate"));
    it = gc->execs.emplace(key, exec).first;
  }
  return cuda_status(cudaGraphLaunch(it->second, s), "graph launch");
}

int vg_profile_enable(vg_plan* p, int32_t enable) {
  VG_CHECK(require_plan(p));
  auto* ps = static_cast<ProfState*>(p->prof);
  ps->enabled = enable != 0;
  return VG_OK;
}

int vg_profile_read(vg_plan* p, vg_prof_entry* out, int32_t max, int32_t* n_out) {
  VG_CHECK(require_plan(p));
  if (!n_out || (max > 0 && !out)) {
    set_error("null output");
    return VG_ERR_ARG;
  }
  double bytes[PK_COUNT];
  for (int k = 0; k < PK_COUNT; ++k) bytes[k] = prof_bytes(p, k);
  int n = 0;
  VG_CHECK(prof_collect(static_cast<ProfState*>(p->prof), PK_COUNT, kProfNames, bytes, out, max, &n));
  *n_out = n;
  return VG_OK;
}

}  // extern "C"
