// Internal plan layout and kernel launchers shared by the translation units.
#pragma once

#include <string>
#include <vector>

#include "vg_common.cuh"
#include "vg_f32_plan.cuh"
#include "vg_fft.cuh"
#include "vlagpu.h"

struct vg_plan {
  // scalars of the run
  int nx, nv, precision, collision, integrator, n_pulses;
  double dt, nu, dx, dv, dv_sq, nudt;
  int nx_pow2, nv_pow2;
  // device constants
  double* x;
  double* v;
  double* kx;
  double* kv;
  double* inv_kx;
  double* v_pow;     // [5][nv]
  double* f_bg;      // [nv] (delta-f background) or null
  vg_pulse* pulses;  // [n_pulses]
  vg::cx<double>* tw64;  // [FFT_NMAX]
  vg::cx<float>* tw32;   // [FFT_NMAX]
  int* pw_v;   // NumPy pairwise tree over nv-1 trapz terms
  int* pw_x;   // NumPy pairwise tree over nx values (x-means)
  int pw_v_leaves, pw_x_leaves, pw_v_words, pw_x_words;
  // scratch
  double* dens;   // [nx]
  double* mom;    // [nx][MOM_STRIDE]
  double* bb;     // [nx][2][nv] Thomas elimination scratch (pivots, upper diagonal; FP64 mode)
  double* rho;    // [nx]
  double* etmp;   // [nx]
  int* flags;     // status bits raised on the device (VG_FLAG_*; null: none kept)
  // semi-Lagrangian steps (allocated by their first call): spline second
  // derivatives [(nx + 2) * (nv + 2)] and the Thomas pivot table [max(nx, nv)]
  double* sl_m;
  double* sl_w;
  // graph cache and per-kernel profiling state
  void* graph_cache;
  void* prof;
  // FP32 delta-f state (null in FP64 mode)
  vg::F32Plan* f32;
};

namespace vg {

constexpr int MOM_STRIDE = 8;

// moment kinds for the pairwise-trapz row kernel
enum MomKind : int { MOM_ONE = 0, MOM_W = 1, MOM_SQ = 2, MOM_FLOGF = 3, MOM_DG2 = 4, MOM_V = 5 };
struct MomSpec {
  int nm;
  int kind[MOM_STRIDE];
  int arg[MOM_STRIDE];  // MOM_W: row of v_pow; MOM_DG2: index of the vbar moment
};

// Per-kernel event timing shared by plans and sweeps: while enabled, each
// launcher call is bracketed by two events on its stream.
struct ProfState {
  bool enabled = false;
  std::vector<cudaEvent_t> pool;
  size_t used = 0;
  struct Rec {
    int kind;
    cudaEvent_t b, e;
  };
  std::vector<Rec> recs;
  ~ProfState() {
    for (cudaEvent_t ev : pool) cudaEventDestroy(ev);
  }
  cudaEvent_t next() {
    if (used == pool.size()) {
      cudaEvent_t ev;
      if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
      pool.push_back(ev);
    }
    return pool[used++];
  }
};

template <typename Fn>
cudaError_t prof_call(ProfState* ps, int kind, cudaStream_t s, Fn fn) {
  if (!ps || !ps->enabled) return fn();
  cudaEvent_t b = ps->next(), e = ps->next();
  if (!b || !e) return cudaErrorMemoryAllocation;
  cudaError_t err = cudaEventRecord(b, s);
  if (err != cudaSuccess) return err;
  err = fn();
  if (err != cudaSuccess) return err;
  err = cudaEventRecord(e, s);
  ps->recs.push_back({kind, b, e});
  return err;
}

// Sum the recorded launches per kind into vg_prof_entry lines (clears the record).
int prof_collect(ProfState* ps, int n_kinds, const char* const* names, const double* bytes_per_launch,
                 vg_prof_entry* out, int max, int* n_out);

void set_error(const std::string& msg);
// NumPy's pairwise summation tree over n terms as [n_leaves, n_prog,
// (start, len) per leaf, post-order program] (leaf index, -1 = combine)
std::vector<int> pairwise_table(int n);
int cuda_status(cudaError_t err, const char* what);
// raise a kernel's dynamic shared-memory limit once (not a stream operation,
// so it is legal while a stream is being captured)
cudaError_t ensure_smem(const void* kernel, size_t bytes);

// longest line the direct-DFT advection takes (lengths that are not powers of
// two; its shared memory holds 5 N doubles)
constexpr int DFT_ADVECT_NMAX = 4096;

// launchers (return cudaError_t of the launch)
cudaError_t launch_edfdv_f64(const vg_plan& p, double* f, const double* e, double dt, cudaStream_t s);
cudaError_t launch_vdfdx_f64(const vg_plan& p, double* f, double dt, cudaStream_t s);
// alternative FP64 operators (vg_advect_alt_f64.cu); out of place
cudaError_t ensure_sl_scratch(vg_plan& p);
cudaError_t launch_vdfdx_sl_f64(const vg_plan& p, const double* fin, double* fout, double dt, cudaStream_t s);
cudaError_t launch_edfdv_sl_f64(const vg_plan& p, const double* fin, const double* e, double* fout, double dt,
                                cudaStream_t s);
cudaError_t launch_edfdv_cd2_f64(const vg_plan& p, const double* fin, const double* e, double* fout, double dt,
                                 cudaStream_t s);
cudaError_t launch_row_moments_f64(const vg_plan& p, const double* f, const MomSpec& spec,
                                   double* out, int out_stride, cudaStream_t s);
// e = [driver or pulses(t)] + Re IFFT(i/kx FFT(rho)), rho = 1 - dens (dens_is_density) or dens
struct FieldTime {
  const double* t_ptr;  // device time value (time_batch + i) or null -> t_host
  double t_host;
  int nadd;
  double add[6];        // sub-step offsets added left to right
  int use_pulses;
};
cudaError_t launch_poisson_f64(const vg_plan& p, const double* dens, int dens_is_density,
                               const double* driver, const FieldTime& ft, double* e, cudaStream_t s);
cudaError_t launch_thomas_f64(const vg_plan& p, double* f, const double* mom, int vbar_col,
                              int vth_col, cudaStream_t s);
cudaError_t launch_storage_f64(const vg_plan& p, const double* f, const double* e, const double* de,
                               const vg_history& h, int i, cudaStream_t s);
cudaError_t launch_driver(const vg_plan& p, const FieldTime& ft, double* out, cudaStream_t s);
cudaError_t launch_twiddles(vg_plan& p, cudaStream_t s);

// FP32 delta-f path (vg_step_f32.cu)
cudaError_t launch_col_f32(const vg_plan& p, float* g, double dt, cudaStream_t s);
cudaError_t launch_field_f32(const vg_plan& p, const double* driver, const FieldTime& ft, double* e,
                             cudaStream_t s);
cudaError_t launch_dens_rows_f32(const vg_plan& p, const float* g, double* rho_out, int as_density,
                                 cudaStream_t s);
cudaError_t launch_poisson_only_f32(const vg_plan& p, const double* rho, const double* driver,
                                    const FieldTime& ft, double* e, cudaStream_t s);
cudaError_t launch_row_f32(const vg_plan& p, float* g, const double* e, double dt1, double dt2, int fp, int mom,
                           int n_modes, cudaStream_t s);
// FP32 copy of a caller-provided field for the kicks
cudaError_t launch_e_to_f32(const vg_plan& p, const double* e, cudaStream_t s);
cudaError_t launch_store_f32(const vg_plan& p, const float* g, const double* e, const double* de,
                             const vg_history& h, int i, int n_modes, cudaStream_t s);

}  // namespace vg
