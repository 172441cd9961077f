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
// Host code cannot use the array's name as a device address, so each call
// asks cudaGetSymbolAddress for it (with the calling device current).  The
// first call on a device, and the first after the address changes (a new
// context after cudaDeviceReset), fills the twiddle table with a kernel on
// the caller's stream and waits for that stream; make that first call during
// set-up, before any stream capture.  Later calls only launch kernels on the
// caller's stream: the summation table for the call's nv is written on the
// device by a one-thread kernel, so no call copies from host memory.  Every
// call shares the array and keeps the last call's contents; nothing in it has
// to start at zero (each call overwrites the density, the table and the DFT
// work area before reading them).  Calls whose executions overlap on the GPU
// (on different streams, or from different threads) race on the array and
// must be ordered by the caller.
#include <cstring>
#include <mutex>

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

// NumPy's pairwise summation tree over n terms (a node of more than 128 terms
// splits at half = n/2 rounded down to a multiple of 8; smaller ones are
// leaves), laid out as [n_leaves, n_prog, (start, len) per leaf, prog...]
// with prog the post-order walk: a leaf's index when it is reached, -1 after
// both children of a node.  One thread, an explicit stack (the tree is at
// most 8 levels deep for n < 16384).
__global__ void k_noalloc_tree(int n, int n_leaves, int* __restrict__ table) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int st_start[48], st_len[48], st_open[48];
  int sp = 0, nl = 0, np = 0;
  int* leaves = table + 2;
  int* prog = table + 2 + 2 * n_leaves;
  st_start[0] = 0;
  st_len[0] = n;
  st_open[0] = 0;
  sp = 1;
  while (sp > 0) {
    --sp;
    const int start = st_start[sp], len = st_len[sp];
    if (len <= 128) {
      leaves[2 * nl] = start;
      leaves[2 * nl + 1] = len;
      prog[np++] = nl++;
    } else if (st_open[sp]) {
      prog[np++] = -1;
    } else {
      int half = len / 2;
      half -= half % 8;
      // the node again (closed after its children), then right, then left on top
      st_open[sp] = 1;
      ++sp;
      st_start[sp] = start + half;
      st_len[sp] = len - half;
      st_open[sp] = 0;
      ++sp;
      st_start[sp] = start;
      st_len[sp] = half;
      st_open[sp] = 0;
      ++sp;
    }
  }
  table[0] = nl;
  table[1] = np;
}

namespace {

struct DeviceScratch {
  bool ready = false;
  unsigned char* ptr = nullptr;
};
std::mutex g_na_mu;
DeviceScratch g_na_dev[64];

// leaves of NumPy's pairwise tree over n terms (the shape k_noalloc_tree walks)
int na_leaves(int len) {
  if (len <= 128) return 1;
  int half = len / 2;
  half -= half % 8;
  return na_leaves(half) + na_leaves(len - half);
}

// the scratch array's device address on the current device; fills the
// twiddles (on stream s, then waits for s) when the device has not been set up
// or the address has changed since
int na_setup(int dev, cudaStream_t s, unsigned char** out) {
  void* p = nullptr;
  int st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch), "no-alloc scratch address");
  if (st != VG_OK) return st;
  std::lock_guard<std::mutex> lk(g_na_mu);
  DeviceScratch& d = g_na_dev[dev];
  if (!d.ready || d.ptr != p) {
    d.ready = false;
    d.ptr = static_cast<unsigned char*>(p);
    k_noalloc_twiddles<<<div_up(FFT_NMAX, 256), 256, 0, s>>>(reinterpret_cast<cx<double>*>(d.ptr + NA_TW_OFF));
    st = cuda_status(cudaGetLastError(), "no-alloc twiddles");
    if (st != VG_OK) return st;
    st = cuda_status(cudaStreamSynchronize(s), "no-alloc set-up");
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
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* base = nullptr;
  st = na_setup(dev, s, &base);
  if (st != VG_OK) return st;
  // summation-tree table of the nv - 1 trapz terms, written on the device
  const int leaves = na_leaves(nv - 1);
  if ((size_t)(2 + 2 * leaves + (2 * leaves - 1)) > NA_PW_WORDS) {
    set_error("summation table exceeds the no-alloc scratch");
    return VG_ERR_ARG;
  }
  int* d_table = reinterpret_cast<int*>(base + NA_PW_OFF);
  k_noalloc_tree<<<1, 32, 0, s>>>(nv - 1, leaves, d_table);
  st = cuda_status(cudaGetLastError(), "no-alloc summation table");
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
  view.pw_v_leaves = leaves;
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
