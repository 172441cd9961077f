// Batched FP64 step: many independent runs of the reference's FP64 time
// step (vlapy/core/step.py:286-328: leapfrog with exponential advection,
// spectral Poisson, the implicit collision step and the per-step moments)
// advanced together, every launch covering all runs of one shape class.
//
// Each run is described as for vg_plan_create (host grids computed by NumPy,
// so a run of the batch sees the same bits as a single plan) and goes
// through the same device bodies as a single plan: a batch of one run gives
// the plan's result bit for bit.  Runs are laid out back to back in the
// caller's buffers (f[nx][nv] per run, e[nx] per run) with the runs of one
// nv contiguous, so the row operators (v-advection, moments, tridiagonal
// solve) treat a class as one tall array of rows; the column operator
// (x-advection) and the Poisson solve take (run, tile) and run items.
//
// A step per class: half kick, x-drift, density and field, half kick,
// collision moments and solve (rows of collisionless runs are left as they
// are, as the reference's collision step returns f unchanged for nu = 0),
// then the run's e and its seven series (means over x by NumPy's pairwise
// tree) into the caller's history rows.
#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "vg_internal.cuh"
#include "vg_f64_body.cuh"

namespace vg {

struct BatchRunDev {
  int nx, nv;
  long long f_off;  // cells before this run
  int x_off;        // x points before this run
  int run;          // index in the caller's order (series row)
  const double* kx;
  const double* inv_kx;
  const double* v;  // the v grid of the run's nv class
  const int* pw_x;  // pairwise table over nx (x-means)
};

constexpr int BATCH_MOMS = 5;  // n, j, T, f^2, f log f per row (the series' sources)

// x-drift of one (run, tile) item per CTA (one kernel per nx class)
template <int NX>
__global__ void __launch_bounds__(col_seqs<double>(NX) * fft_threads<double>(NX))
    k_batch_vdfdx(const BatchRunDev* __restrict__ runs, const int2* __restrict__ items, double* f, int W,
                  double dt, const cx<double>* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int2 it = items[blockIdx.x];
  const BatchRunDev r = runs[it.x];
  vdfdx_tile_body<NX>(f + r.f_off, r.nv, it.y * W, W, r.kx, r.v, dt, tw, smem_raw);
}

// spectral Poisson of one run per CTA (one kernel per nx class); no driver
template <int NX>
__global__ void __launch_bounds__(fft_threads<double>(NX))
    k_batch_poisson(const BatchRunDev* __restrict__ runs, const int* __restrict__ ids,
                    const double* __restrict__ dens, const cx<double>* __restrict__ tw, double* e,
                    int* flags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const BatchRunDev r = runs[ids[blockIdx.x]];
  FieldTimeDev ft;
  ft.t_ptr = nullptr;
  ft.t_host = 0.0;
  ft.nadd = 0;
  poisson_fft_body<NX>(dens + r.x_off, 1, r.inv_kx, nullptr, 0, nullptr, 0, nullptr, ft, tw, e + r.x_off,
                       reinterpret_cast<cx<double>*>(smem_raw), threadIdx.x, flags);
}

// tridiagonal collision solve, one thread per row of a class; rows of
// collisionless runs (nudt == 0) are left as they are
__global__ void k_batch_thomas(double* f, int nrows, int nv, const double* __restrict__ v,
                               const double* __restrict__ mom, const double* __restrict__ nudt_row,
                               int dougherty, double dv, double dv_sq, double* __restrict__ bb) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nrows) return;
  const double nudt = nudt_row[row];
  if (nudt == 0.0) return;
  const double vbar = dougherty ? mom[(size_t)row * 2 + 0] : 0.0;
  const double vth = mom[(size_t)row * 2 + 1];
  thomas_row_f64(f + (size_t)row * nv, bb + (size_t)row * 2 * nv, nv, v, vbar, vth, dougherty, nudt, dv, dv_sq);
}

// e history row and the seven series of one run per CTA: the x-means of n,
// j, T, e^2, driver^2 (no driver: 0), f^2 and f log f by NumPy's pairwise
// tree over nx, divided by nx (vlapy/core/step.py:174-229)
__global__ void k_batch_store(const BatchRunDev* __restrict__ runs, const double* __restrict__ mom,
                              const double* __restrict__ e, int n_runs, double* __restrict__ e_row,
                              double* __restrict__ s_row) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* leaf = reinterpret_cast<double*>(smem_raw);  // [7][nl]
  const BatchRunDev r = runs[blockIdx.x];
  const int* table = r.pw_x;
  const int nl = table[0];
  const int* leaves = table + 2;
  const double* er = e + r.x_off;
  const double* mr = mom + (size_t)r.x_off * BATCH_MOMS;
  if (e_row)
    for (int n = threadIdx.x; n < r.nx; n += blockDim.x) e_row[r.x_off + n] = er[n];
  for (int idx = threadIdx.x; idx < 7 * nl; idx += blockDim.x) {
    const int q = idx / nl, L = idx - q * nl;
    auto term = [&](int n) -> double {
      switch (q) {
        case 0: return mr[(size_t)n * BATCH_MOMS + 0];
        case 1: return mr[(size_t)n * BATCH_MOMS + 1];
        case 2: return mr[(size_t)n * BATCH_MOMS + 2];
        case 3: return mul_rn(er[n], er[n]);
        case 4: return 0.0;
        case 5: return mr[(size_t)n * BATCH_MOMS + 3];
        default: return mr[(size_t)n * BATCH_MOMS + 4];
      }
    };
    leaf[q * nl + L] = leaf_sum(leaves[2 * L], leaves[2 * L + 1], term);
  }
  __syncthreads();
  if (s_row && threadIdx.x < 7) {
    const int q = threadIdx.x;
    s_row[(size_t)r.run * 7 + q] = __ddiv_rn(combine_leaves(table, leaf + q * nl), (double)r.nx);
  }
}

}  // namespace vg

using namespace vg;

struct vg_batch {
  int n_runs, collision;
  double dt;
  long long cells;
  int x_points;
  std::vector<void*> owned;
  BatchRunDev* runs = nullptr;
  cx<double>* tw64 = nullptr;
  cx<float>* tw32 = nullptr;
  double* dens = nullptr;      // [x_points]
  double* mom = nullptr;       // [x_points][BATCH_MOMS]
  double* fpmom = nullptr;     // [x_points][2]
  double* nudt_row = nullptr;  // [x_points]
  double* bb = nullptr;        // [max class rows][2][nv]
  int* flags = nullptr;        // status bits raised on the device (VG_FLAG_*)
  int max_pw_x_leaves = 0;
  // nv classes: a contiguous block of runs each
  struct Cls {
    int nv;
    long long f_off;
    int x_off, rows;
    int pw_v_leaves;
    double dv, dv_sq;
    double *v, *kv, *v_pow;
    int* pw_v;
  };
  std::vector<Cls> cls;
  // nx classes: x-drift items and Poisson run lists
  struct XCls {
    int nx, W;
    int2* items;
    int n_items;
    int* ids;
    int n_ids;
  };
  std::vector<XCls> xcls;
  std::map<std::tuple<const void*, const void*, int, const void*, const void*, int, int, cudaStream_t>,
           cudaGraphExec_t>
      graphs;
  ProfState prof;
};

namespace {

#define B_CHECK(expr)             \
  do {                            \
    int _st = (expr);             \
    if (_st != VG_OK) return _st; \
  } while (0)

template <typename T>
int b_alloc(vg_batch* b, T** dst, size_t n, const void* src, const char* what) {
  *dst = nullptr;
  cudaError_t err = cudaMalloc(reinterpret_cast<void**>(dst), std::max<size_t>(n, 1) * sizeof(T));
  if (err != cudaSuccess) return cuda_status(err, what);
  b->owned.push_back(*dst);
  if (src) err = cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
  else err = cudaMemset(*dst, 0, std::max<size_t>(n, 1) * sizeof(T));
  return cuda_status(err, what);
}

void free_batch(vg_batch* b) {
  if (!b) return;
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  for (void* p : b->owned)
    if (p) cudaFree(p);
  delete b;
}

enum BatchProfKind { BK_EDFDV = 0, BK_VDFDX, BK_DENSITY, BK_POISSON, BK_FP_MOMENTS, BK_FP_SOLVE, BK_STORE, BK_COUNT };
const char* const kBatchNames[BK_COUNT] = {"batch_edfdv", "batch_vdfdx", "batch_density", "batch_poisson",
                                          "batch_fp_moments", "batch_fp_solve", "batch_store"};

// a plan-shaped view of one nv class for the row launchers
vg_plan class_view(const vg_batch* b, const vg_batch::Cls& c) {
  vg_plan v;
  std::memset(&v, 0, sizeof(v));
  v.nx = c.rows;
  v.nv = c.nv;
  v.precision = VG_F64;
  v.collision = b->collision;
  v.dv = c.dv;
  v.dv_sq = c.dv_sq;
  v.nv_pow2 = is_pow2(c.nv);
  v.nx_pow2 = 1;
  v.v = c.v;
  v.kv = c.kv;
  v.v_pow = c.v_pow;
  v.pw_v = c.pw_v;
  v.pw_v_leaves = c.pw_v_leaves;
  v.tw64 = b->tw64;
  v.tw32 = b->tw32;
  return v;
}

template <int NX>
cudaError_t batch_vdfdx_launch(const vg_batch* b, const vg_batch::XCls& xc, double* f, double dt, cudaStream_t s) {
  constexpr int G = fft_threads<double>(NX);
  const int S = xc.W / 2;
  const size_t smem = (size_t)S * (sp_len<double>(NX) + COL_PAD) * sizeof(cx<double>);
  cudaError_t err = ensure_smem((const void*)k_batch_vdfdx<NX>, smem);
  if (err != cudaSuccess) return err;
  k_batch_vdfdx<NX><<<xc.n_items, S * G, smem, s>>>(b->runs, xc.items, f, xc.W, dt, b->tw64);
  return cudaGetLastError();
}

template <int NX>
cudaError_t batch_poisson_launch(const vg_batch* b, const vg_batch::XCls& xc, double* e, cudaStream_t s) {
  constexpr int G = fft_threads<double>(NX);
  const size_t smem = (size_t)sp_len<double>(NX) * sizeof(cx<double>);
  cudaError_t err = ensure_smem((const void*)k_batch_poisson<NX>, smem);
  if (err != cudaSuccess) return err;
  k_batch_poisson<NX><<<xc.n_ids, G, smem, s>>>(b->runs, xc.ids, b->dens, b->tw64, e, b->flags);
  return cudaGetLastError();
}

#define VG_BATCH_NX_CASES(M, ...) \
  M(2, __VA_ARGS__) M(4, __VA_ARGS__) M(8, __VA_ARGS__) M(16, __VA_ARGS__) M(32, __VA_ARGS__) \
  M(64, __VA_ARGS__) M(128, __VA_ARGS__) M(256, __VA_ARGS__) M(512, __VA_ARGS__) M(1024, __VA_ARGS__)

cudaError_t batch_vdfdx_all(const vg_batch* b, double* f, double dt, cudaStream_t s) {
  for (const auto& xc : b->xcls) {
    cudaError_t err = cudaErrorInvalidValue;
    switch (xc.nx) {
#define CASE(NX, ...) \
  case NX: err = batch_vdfdx_launch<NX>(b, xc, f, dt, s); break;
      VG_BATCH_NX_CASES(CASE, 0)
#undef CASE
      default: break;
    }
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

cudaError_t batch_poisson_all(const vg_batch* b, double* e, cudaStream_t s) {
  for (const auto& xc : b->xcls) {
    cudaError_t err = cudaErrorInvalidValue;
    switch (xc.nx) {
#define CASE(NX, ...) \
  case NX: err = batch_poisson_launch<NX>(b, xc, e, s); break;
      VG_BATCH_NX_CASES(CASE, 0)
#undef CASE
      default: break;
    }
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

int batch_sequence(vg_batch* b, double* f, double* e, int nsteps, double* e_hist, double* s_hist, int rows,
                   int row0, cudaStream_t s) {
  const double dt = b->dt;
  auto edfdv = [&](double d) {
    return cuda_status(prof_call(&b->prof, BK_EDFDV, s, [&] {
                         for (const auto& c : b->cls) {
                           const vg_plan view = class_view(b, c);
                           cudaError_t err = launch_edfdv_f64(view, f + c.f_off, e + c.x_off, d, s);
                           if (err != cudaSuccess) return err;
                         }
                         return cudaSuccess;
                       }),
                       "batch edfdv");
  };
  auto moments = [&](int kind, const MomSpec& spec, double* out, int stride) {
    return cuda_status(prof_call(&b->prof, kind, s, [&] {
                         for (const auto& c : b->cls) {
                           const vg_plan view = class_view(b, c);
                           cudaError_t err =
                               launch_row_moments_f64(view, f + c.f_off, spec, out + (size_t)c.x_off * stride, stride, s);
                           if (err != cudaSuccess) return err;
                         }
                         return cudaSuccess;
                       }),
                       "batch moments");
  };
  MomSpec dens_spec;
  dens_spec.nm = 1;
  dens_spec.kind[0] = MOM_ONE;
  dens_spec.arg[0] = 0;
  MomSpec fp_spec;
  fp_spec.nm = 2;
  if (b->collision == VG_COLL_DG) {
    fp_spec.kind[0] = MOM_V;  // vbar = trapz(f v)
    fp_spec.arg[0] = 0;
    fp_spec.kind[1] = MOM_DG2;  // v0t^2 = trapz(f (v - vbar)^2)
    fp_spec.arg[1] = 0;
  } else {
    fp_spec.kind[0] = MOM_ONE;  // unused slot (LB has no drift)
    fp_spec.arg[0] = 0;
    fp_spec.kind[1] = MOM_W;  // v0t^2 = trapz(f v**2.0)
    fp_spec.arg[1] = 0;
  }
  MomSpec st_spec;
  st_spec.nm = BATCH_MOMS;
  const int kinds[BATCH_MOMS] = {MOM_ONE, MOM_V, MOM_W, MOM_SQ, MOM_FLOGF};
  const int args[BATCH_MOMS] = {0, 0, 1, 0, 0};
  for (int q = 0; q < BATCH_MOMS; ++q) {
    st_spec.kind[q] = kinds[q];
    st_spec.arg[q] = args[q];
  }
  for (int k = 0; k < nsteps; ++k) {
    // vlapy/core/vlasov_poisson.py:36-58, then the collision step and storage
    B_CHECK(edfdv(0.5 * dt));
    B_CHECK(cuda_status(prof_call(&b->prof, BK_VDFDX, s, [&] { return batch_vdfdx_all(b, f, dt, s); }),
                        "batch vdfdx"));
    B_CHECK(moments(BK_DENSITY, dens_spec, b->dens, 1));
    B_CHECK(cuda_status(prof_call(&b->prof, BK_POISSON, s, [&] { return batch_poisson_all(b, e, s); }),
                        "batch poisson"));
    B_CHECK(edfdv(0.5 * dt));
    B_CHECK(moments(BK_FP_MOMENTS, fp_spec, b->fpmom, 2));
    B_CHECK(cuda_status(prof_call(&b->prof, BK_FP_SOLVE, s, [&] {
                          for (const auto& c : b->cls) {
                            k_batch_thomas<<<div_up(c.rows, 64), 64, 0, s>>>(
                                f + c.f_off, c.rows, c.nv, c.v, b->fpmom + (size_t)c.x_off * 2, b->nudt_row + c.x_off,
                                b->collision == VG_COLL_DG, c.dv, c.dv_sq, b->bb);
                            cudaError_t err = cudaGetLastError();
                            if (err != cudaSuccess) return err;
                          }
                          return cudaSuccess;
                        }),
                        "batch collision solve"));
    const int r = row0 + k;
    if ((e_hist || s_hist) && r >= 0 && r < rows) {
      B_CHECK(moments(BK_STORE, st_spec, b->mom, BATCH_MOMS));
      double* er = e_hist ? e_hist + (size_t)r * b->x_points : nullptr;
      double* sr = s_hist ? s_hist + (size_t)r * b->n_runs * 7 : nullptr;
      B_CHECK(cuda_status(prof_call(&b->prof, BK_STORE, s, [&] {
                            const size_t smem = (size_t)7 * b->max_pw_x_leaves * sizeof(double);
                            k_batch_store<<<b->n_runs, 128, smem, s>>>(b->runs, b->mom, e, b->n_runs, er, sr);
                            return cudaGetLastError();
                          }),
                          "batch store"));
    }
  }
  return VG_OK;
}

}  // namespace

extern "C" {

int vg_batch_create(const vg_run_desc* runs, int32_t n_runs, vg_batch** out) {
  if (!runs || !out || n_runs <= 0) {
    set_error("batch: null runs or output, or no runs");
    return VG_ERR_ARG;
  }
  *out = nullptr;
  const vg_run_desc& r0 = runs[0];
  int coll_op = VG_COLL_NONE;
  for (int i = 0; i < n_runs; ++i) {
    const vg_run_desc& d = runs[i];
    const std::string where = "batch run " + std::to_string(i) + ": ";
    if (d.precision != VG_F64 || d.integrator != VG_LEAPFROG || d.n_pulses != 0 || d.f_background) {
      set_error(where + "the batch takes FP64 leapfrog runs without driver pulses");
      return VG_ERR_UNSUPPORTED;
    }
    if (!is_pow2(d.nx) || d.nx < 2 || d.nx > 1024 || d.nv < 2 ||
        (is_pow2(d.nv) ? d.nv > 8192 : d.nv > DFT_ADVECT_NMAX)) {
      set_error(where + "needs a power-of-two nx in [2, 1024] and nv a power of two <= 8192 or any nv <= " +
                std::to_string(DFT_ADVECT_NMAX));
      return VG_ERR_UNSUPPORTED;
    }
    if (!d.x || !d.v || !d.kx || !d.kv || !d.one_over_kx || !d.v_pow || d.dt != r0.dt || !(d.nu >= 0.0)) {
      set_error(where + "missing grids, a different dt or a negative nu");
      return VG_ERR_ARG;
    }
    if (d.collision != VG_COLL_NONE && d.nu > 0.0) {
      if (coll_op != VG_COLL_NONE && d.collision != coll_op) {
        set_error(where + "all collisional runs of a batch use one operator");
        return VG_ERR_UNSUPPORTED;
      }
      coll_op = d.collision;
    }
    // runs of one nv are contiguous and share the velocity grid bit for bit
    if (i > 0 && d.nv != runs[i - 1].nv) {
      for (int j = 0; j < i - 1; ++j)
        if (runs[j].nv == d.nv) {
          set_error(where + "runs of equal nv must be contiguous in the batch");
          return VG_ERR_ARG;
        }
    }
    if (i > 0 && d.nv == runs[i - 1].nv) {
      const vg_run_desc& p = runs[i - 1];
      if (d.dv != p.dv || d.dv_sq != p.dv_sq || std::memcmp(d.v, p.v, sizeof(double) * d.nv) ||
          std::memcmp(d.kv, p.kv, sizeof(double) * d.nv) || std::memcmp(d.v_pow, p.v_pow, sizeof(double) * 5 * d.nv)) {
        set_error(where + "runs of equal nv must share the velocity grid");
        return VG_ERR_ARG;
      }
    }
  }
  vg_batch* b = new vg_batch();
  b->n_runs = n_runs;
  b->collision = coll_op == VG_COLL_NONE ? VG_COLL_DG : coll_op;
  b->dt = r0.dt;
  int st = VG_OK;
#define B_TRY(expr)    \
  do {                 \
    st = (expr);       \
    if (st != VG_OK) { \
      free_batch(b);   \
      return st;       \
    }                  \
  } while (0)
  std::vector<BatchRunDev> rd(n_runs);
  std::vector<double> kx_all, inv_all, nudt_row;
  std::map<int, int*> pw_x_of;
  long long cells = 0;
  int xoff = 0;
  size_t bb_need = 0;
  for (int i = 0; i < n_runs; ++i) {
    const vg_run_desc& d = runs[i];
    if (i == 0 || d.nv != runs[i - 1].nv) {
      vg_batch::Cls c;
      std::memset(&c, 0, sizeof(c));
      c.nv = d.nv;
      c.f_off = cells;
      c.x_off = xoff;
      c.dv = d.dv;
      c.dv_sq = d.dv_sq;
      B_TRY(b_alloc(b, &c.v, d.nv, d.v, "batch grids"));
      B_TRY(b_alloc(b, &c.kv, d.nv, d.kv, "batch grids"));
      B_TRY(b_alloc(b, &c.v_pow, 5 * (size_t)d.nv, d.v_pow, "batch grids"));
      const std::vector<int> tv = pairwise_table(d.nv - 1);
      c.pw_v_leaves = tv[0];
      B_TRY(b_alloc(b, &c.pw_v, tv.size(), tv.data(), "batch tables"));
      b->cls.push_back(c);
    }
    vg_batch::Cls& c = b->cls.back();
    c.rows += d.nx;
    bb_need = std::max(bb_need, (size_t)c.rows * 2 * (size_t)c.nv);
    if (!pw_x_of.count(d.nx)) {
      const std::vector<int> tx = pairwise_table(d.nx);
      int* p = nullptr;
      B_TRY(b_alloc(b, &p, tx.size(), tx.data(), "batch tables"));
      pw_x_of[d.nx] = p;
      b->max_pw_x_leaves = std::max(b->max_pw_x_leaves, tx[0]);
    }
    BatchRunDev& r = rd[i];
    r.nx = d.nx;
    r.nv = d.nv;
    r.f_off = cells;
    r.x_off = xoff;
    r.run = i;
    r.v = c.v;
    r.pw_x = pw_x_of[d.nx];
    kx_all.insert(kx_all.end(), d.kx, d.kx + d.nx);
    inv_all.insert(inv_all.end(), d.one_over_kx, d.one_over_kx + d.nx);
    // nu * dt as vg_plan_create forms it; 0 leaves the run's rows as they are
    const double nudt = (d.collision != VG_COLL_NONE && d.nu > 0.0) ? d.nu * d.dt : 0.0;
    nudt_row.insert(nudt_row.end(), (size_t)d.nx, nudt);
    cells += (long long)d.nx * d.nv;
    xoff += d.nx;
  }
  b->cells = cells;
  b->x_points = xoff;
  double *kx_d = nullptr, *inv_d = nullptr;
  B_TRY(b_alloc(b, &kx_d, kx_all.size(), kx_all.data(), "batch grids"));
  B_TRY(b_alloc(b, &inv_d, inv_all.size(), inv_all.data(), "batch grids"));
  for (int i = 0; i < n_runs; ++i) {
    rd[i].kx = kx_d + rd[i].x_off;
    rd[i].inv_kx = inv_d + rd[i].x_off;
  }
  B_TRY(b_alloc(b, &b->runs, rd.size(), rd.data(), "batch runs"));
  B_TRY(b_alloc(b, &b->nudt_row, nudt_row.size(), nudt_row.data(), "batch runs"));
  B_TRY(b_alloc<double>(b, &b->dens, (size_t)xoff, nullptr, "batch scratch"));
  B_TRY(b_alloc<int>(b, &b->flags, 1, nullptr, "batch status"));
  B_TRY(b_alloc<double>(b, &b->mom, (size_t)xoff * BATCH_MOMS, nullptr, "batch scratch"));
  B_TRY(b_alloc<double>(b, &b->fpmom, (size_t)xoff * 2, nullptr, "batch scratch"));
  B_TRY(b_alloc<double>(b, &b->bb, bb_need, nullptr, "batch thomas scratch"));
  B_TRY(b_alloc<cx<double>>(b, &b->tw64, FFT_NMAX, nullptr, "twiddles"));
  B_TRY(b_alloc<cx<float>>(b, &b->tw32, FFT_NMAX, nullptr, "twiddles"));
  {
    vg_plan tmp;
    std::memset(&tmp, 0, sizeof(tmp));
    tmp.tw64 = b->tw64;
    tmp.tw32 = b->tw32;
    B_TRY(cuda_status(launch_twiddles(tmp, 0), "twiddles"));
  }
  // x classes: (run, column tile) items of the x-drift and the Poisson run lists
  std::map<int, std::pair<std::vector<int2>, std::vector<int>>> by_nx;
  for (int i = 0; i < n_runs; ++i) {
    const int nx = rd[i].nx;
    const int W = 2 * col_seqs<double>(nx);
    auto& e = by_nx[nx];
    for (int t = 0; t * W < rd[i].nv; ++t) e.first.push_back(make_int2(i, t));
    e.second.push_back(i);
  }
  for (auto& kv : by_nx) {
    vg_batch::XCls xc;
    xc.nx = kv.first;
    xc.W = 2 * col_seqs<double>(kv.first);
    xc.n_items = (int)kv.second.first.size();
    xc.n_ids = (int)kv.second.second.size();
    B_TRY(b_alloc(b, &xc.items, kv.second.first.size(), kv.second.first.data(), "batch work list"));
    B_TRY(b_alloc(b, &xc.ids, kv.second.second.size(), kv.second.second.data(), "batch work list"));
    b->xcls.push_back(xc);
  }
  B_TRY(cuda_status(cudaDeviceSynchronize(), "batch setup"));
#undef B_TRY
  *out = b;
  return VG_OK;
}

int vg_batch_destroy(vg_batch* b) {
  if (!b) return VG_OK;
  cudaDeviceSynchronize();
  free_batch(b);
  return VG_OK;
}

int vg_batch_status(vg_batch* b, int32_t* flags) {
  if (!b || !flags) {
    set_error("null batch or flags");
    return VG_ERR_ARG;
  }
  int h = 0;
  B_CHECK(cuda_status(cudaMemcpy(&h, b->flags, sizeof(int), cudaMemcpyDeviceToHost), "batch status"));
  *flags = h;
  if (h & VG_FLAG_NONFINITE) {
    set_error("a field solve produced NaN or Inf (the steps from it on are not valid)");
    return VG_ERR_NUMERIC;
  }
  return VG_OK;
}

int vg_batch_sizes(const vg_batch* b, int64_t* cells, int64_t* x_points) {
  if (!b) {
    set_error("null batch");
    return VG_ERR_ARG;
  }
  if (cells) *cells = b->cells;
  if (x_points) *x_points = b->x_points;
  return VG_OK;
}

int vg_batch_run_steps(vg_batch* b, double* f, double* e, int32_t nsteps, double* e_hist, double* series_hist,
                       int32_t hist_rows, int32_t hist_row0, int32_t use_graph, vg_stream stream) {
  if (!b || !f || !e || nsteps < 0 || hist_rows < 0) {
    set_error("batch: null batch, f or e, or negative counts");
    return VG_ERR_ARG;
  }
  if (nsteps == 0) return VG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (b->prof.enabled || !use_graph) return batch_sequence(b, f, e, nsteps, e_hist, series_hist, hist_rows, hist_row0, st);
  if (st == 0) {
    set_error("graph mode needs a non-default stream");
    return VG_ERR_ARG;
  }
  const auto key = std::make_tuple((const void*)f, (const void*)e, nsteps, (const void*)e_hist,
                                   (const void*)series_hist, hist_rows, hist_row0, st);
  auto it = b->graphs.find(key);
  if (it == b->graphs.end()) {
    B_CHECK(cuda_status(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed), "begin capture"));
    const int rc = batch_sequence(b, f, e, nsteps, e_hist, series_hist, hist_rows, hist_row0, st);
    cudaGraph_t graph = nullptr;
    cudaError_t err = cudaStreamEndCapture(st, &graph);
    if (rc != VG_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    B_CHECK(cuda_status(err, "end capture"));
    cudaGraphExec_t exec = nullptr;
    err = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    B_CHECK(cuda_status(err, "graph instantiate"));
    it = b->graphs.emplace(key, exec).first;
  }
  return cuda_status(cudaGraphLaunch(it->second, st), "graph launch");
}

int vg_batch_profile_enable(vg_batch* b, int32_t enable) {
  if (!b) {
    set_error("null batch");
    return VG_ERR_ARG;
  }
  b->prof.enabled = enable != 0;
  return VG_OK;
}

int vg_batch_profile_read(vg_batch* b, vg_prof_entry* out, int32_t max, int32_t* n_out) {
  if (!b || !n_out || (max > 0 && !out)) {
    set_error("null batch or output");
    return VG_ERR_ARG;
  }
  // algorithmic bytes per launch group: read + write of f for the in-place
  // transforms and the solve, one read for the moment passes
  const double cells = (double)b->cells;
  const double bytes[BK_COUNT] = {16.0 * cells, 16.0 * cells, 8.0 * cells, 16.0 * b->x_points,
                                  8.0 * cells,  16.0 * cells, 8.0 * cells};
  int n = 0;
  B_CHECK(prof_collect(&b->prof, BK_COUNT, kBatchNames, bytes, out, max, &n));
  *n_out = n;
  return VG_OK;
}

}  // extern "C"
