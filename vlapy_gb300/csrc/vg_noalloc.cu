// Field solve without any device allocation.
//
// vg_field_solve needs a plan, and a plan cudaMallocs its constants and its
// scratch.  Some callers cannot allocate: their device memory belongs to
// another allocator (a framework's caching allocator or a fixed pool that a
// cudaMalloc of ours would fragment or exhaust), or they cannot afford the
// device-wide synchronisation that cudaMalloc/cudaFree may imply.  For them
// vg_field_solve_noalloc computes the same e = driver + field(1 - trapz_v f)
// with the same FP64 kernels, but every piece of scratch it needs -- the
// density n(x), the FFT twiddle table, NumPy's summation-tree table and the
// work area of the direct DFT -- lives in one file-scope __device__ array of
// fixed size, which each GPU that loads this library holds until exit.
//
// The first call on a device resolves the array's device address with
// cudaGetSymbolAddress (with that device current) and fills the twiddle
// table; make that first call before any stream capture.  Every call shares
// the array and keeps the last call's contents; nothing in it has to start
// at zero (each call overwrites the density, the table and the DFT work area
// before reading them).  Calls whose executions overlap on the GPU (on
// different streams, or from different threads) race on the array and must
// be ordered by the caller.
#include <cstring>
#include <mutex>
#include <vector>

#include "vg_internal.cuh"

namespace vg {

// limits of the no-allocation entry point
constexpr int NOALLOC_MAX_NX = 8192;
constexpr int NOALLOC_MAX_NV = 16384;
constexpr size_t NA_DENS_OFF = 0;                                             // double [NOALLOC_MAX_NX]
constexpr size_t NA_TW_OFF = NA_DENS_OFF + sizeof(double) * NOALLOC_MAX_NX;   // cx<double>[FFT_NMAX]
constexpr size_t NA_ETMP_OFF = NA_TW_OFF + sizeof(cx<double>) * FFT_NMAX;     // double [4 nx + 4]
constexpr size_t NA_PW_OFF = NA_ETMP_OFF + sizeof(double) * (4 * NOALLOC_MAX_NX + 4);  // int [table]
// leaves hold 64..128 terms: at most (nv - 1) / 64 + 1 = 257 of them; the table is
// 2 + 2 leaves + (2 leaves - 1) words
constexpr size_t NA_PW_WORDS = 2 + 4 * 257;
constexpr size_t NA_BYTES = NA_PW_OFF + sizeof(int) * NA_PW_WORDS;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

__global__ void k_noalloc_twiddles(cx<double>* __restrict__ t64) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= FFT_NMAX) return;
  int k, h;
  tw_entry(q, k, h);
  double sn, cs;
  sincospi((double)k / (double)h, &sn, &cs);
  t64[q] = {cs, -sn};
}

namespace {

struct DeviceScratch {
  bool ready = false;
  unsigned char* ptr = nullptr;
};
std::mutex g_na_mu;
DeviceScratch g_na_dev[64];

// NumPy's pairwise tree over n terms, packed as [n_leaves, n_prog, (start, len)..., prog...]
void na_tree(int start, int len, std::vector<int>& leaves, std::vector<int>& prog) {
  if (len <= 128) {
    prog.push_back((int)(leaves.size() / 2));
    leaves.push_back(start);
    leaves.push_back(len);
    return;
  }
  int half = len / 2;
  half -= half % 8;
  na_tree(start, half, leaves, prog);
  na_tree(start + half, len - half, leaves, prog);
  prog.push_back(-1);
}

int na_setup(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_na_mu);
  DeviceScratch& d = g_na_dev[dev];
  if (!d.ready) {
    void* p = nullptr;
    int st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch), "no-alloc scratch address");
    if (st != VG_OK) return st;
    d.ptr = static_cast<unsigned char*>(p);
    k_noalloc_twiddles<<<div_up(FFT_NMAX, 256), 256>>>(reinterpret_cast<cx<double>*>(d.ptr + NA_TW_OFF));
    st = cuda_status(cudaGetLastError(), "no-alloc twiddles");
    if (st != VG_OK) return st;
    st = cuda_status(cudaDeviceSynchronize(), "no-alloc set-up");
    if (st != VG_OK) return st;
    d.ready = true;
  }
  *out = d.ptr;
  return VG_OK;
}

}  // namespace
}  // namespace vg

using namespace vg;

extern "C" int vg_field_solve_noalloc(const double* f, int32_t nx, int32_t nv, double dv, const double* one_over_kx,
                                      const double* driver, double* e, vg_stream stream) {
  if (!f || !one_over_kx || !e) {
    set_error("null f, one_over_kx or e");
    return VG_ERR_ARG;
  }
  if (nx < 2 || nv < 2 || nx > NOALLOC_MAX_NX || nv > NOALLOC_MAX_NV) {
    set_error("vg_field_solve_noalloc: needs 2 <= nx <= " + std::to_string(NOALLOC_MAX_NX) + " and 2 <= nv <= " +
              std::to_string(NOALLOC_MAX_NV) + ", got nx=" + std::to_string(nx) + ", nv=" + std::to_string(nv));
    return VG_ERR_ARG;
  }
  int dev = 0;
  int st = cuda_status(cudaGetDevice(&dev), "current device");
  if (st != VG_OK) return st;
  if (dev < 0 || dev >= 64) {
    set_error("device index out of range for the no-alloc scratch table");
    return VG_ERR_ARG;
  }
  unsigned char* base = nullptr;
  st = na_setup(dev, &base);
  if (st != VG_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  // summation-tree table of the nv - 1 trapz terms, copied into the scratch
  std::vector<int> leaves, prog;
  na_tree(0, nv - 1, leaves, prog);
  std::vector<int> table;
  table.push_back((int)(leaves.size() / 2));
  table.push_back((int)prog.size());
  table.insert(table.end(), leaves.begin(), leaves.end());
  table.insert(table.end(), prog.begin(), prog.end());
  if (table.size() > NA_PW_WORDS) {
    set_error("summation table exceeds the no-alloc scratch");
    return VG_ERR_ARG;
  }
  int* d_table = reinterpret_cast<int*>(base + NA_PW_OFF);
  st = cuda_status(cudaMemcpyAsync(d_table, table.data(), table.size() * sizeof(int), cudaMemcpyHostToDevice, s),
                   "no-alloc table upload");
  if (st != VG_OK) return st;
  // a plan-shaped view over the caller's arrays and the static scratch (nothing allocated)
  vg_plan view;
  std::memset(&view, 0, sizeof(view));
  view.nx = nx;
  view.nv = nv;
  view.precision = VG_F64;
  view.dv = dv;
  view.nx_pow2 = is_pow2(nx);
  view.nv_pow2 = is_pow2(nv);
  view.inv_kx = const_cast<double*>(one_over_kx);
  view.tw64 = reinterpret_cast<cx<double>*>(base + NA_TW_OFF);
  view.pw_v = d_table;
  view.pw_v_leaves = table[0];
  view.dens = reinterpret_cast<double*>(base + NA_DENS_OFF);
  view.etmp = reinterpret_cast<double*>(base + NA_ETMP_OFF);
  MomSpec spec;
  spec.nm = 1;
  spec.kind[0] = MOM_ONE;
  spec.arg[0] = 0;
  st = cuda_status(launch_row_moments_f64(view, f, spec, view.dens, 1, s), "no-alloc density");
  if (st != VG_OK) return st;
  FieldTime ft{};
  ft.use_pulses = 0;
  return cuda_status(launch_poisson_f64(view, view.dens, 1, driver, ft, e, s), "no-alloc poisson");
}
