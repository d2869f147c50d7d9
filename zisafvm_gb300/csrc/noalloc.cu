// zfvm_rate_of_change_noalloc: the rate of change of a solver's current state
// without any device allocation in the call.
//
// Who needs it.  zfvm_rate_of_change allocates and frees a small device buffer
// on every call, and cudaFree waits for all work on the device to finish.  Some
// callers cannot allow either: a host application whose own pool allocator has
// already reserved the device memory it may use (a further cudaMalloc can fail
// or break its accounting), or a time-critical loop in which a device-wide wait
// is not acceptable.  Those callers create the solver once at set-up, when
// allocation is still allowed, and call this entry point inside the loop.
//
// How.  The scratch of one stage -- the reconstructed values at the face
// points, the face fluxes, the per-cell source and equilibrium, the tendency
// and its cell-major copy for the host -- lives in one fixed array compiled
// into the library (ZFVM_NOALLOC_SCRATCH_BYTES on every device that loads the
// library, held until the process exits).  The three stage kernels are the
// same ones the solver's other entry points run; only their scratch pointers
// point into this array.  The call only reads the solver's state and writes
// its device clock (status flags), like zfvm_rate_of_change; with an
// equilibrium refresh schedule (steps_per_recompute > 1) it also advances the
// schedule and keeps the equilibrium in the solver's own buffers, as every
// reconstruction does.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "solver_obj.hpp"

// In host code this name is a host-side stand-in for the array, not a device
// address: the address handed to kernels comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char zfvm_noalloc_scratch[ZFVM_NOALLOC_SCRATCH_BYTES];

using namespace zfvm;
using namespace zfvm::dev;

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
unsigned char *g_scratch_address[kMaxDevices] = {};

// Device address of the array on device `dev`, which must be the current
// device.  The first call on a device looks it up (cudaGetSymbolAddress, which
// also loads this file's code on that device); later calls reuse it.
unsigned char *scratch_address(int dev) {
  if (dev < 0 || dev >= kMaxDevices) throw CudaError{cudaErrorInvalidDevice, "device ordinal beyond 64"};
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_address[dev]) {
    void *p = nullptr;
    CK(cudaGetSymbolAddress(&p, zfvm_noalloc_scratch));
    g_scratch_address[dev] = static_cast<unsigned char *>(p);
  }
  return g_scratch_address[dev];
}

// Hands out 256-byte aligned pieces of the array; with base == nullptr it only
// counts the bytes a layout needs.
struct Carve {
  unsigned char *base;
  size_t used = 0;
  template <class T>
  T *take(size_t count) {
    used = (used + 255) & ~size_t(255);
    T *p = base ? reinterpret_cast<T *>(base + used) : nullptr;
    used += count * sizeof(T);
    return p;
  }
};

struct Layout {
  // must be zero when the stage kernels start: the update kernel sums the
  // fluxes of faces the face kernel skips (inactive faces), and rows of the
  // tendency that belong to ghost cells are never written
  double *tend = nullptr, *nf = nullptr;
  float *g32 = nullptr, *mL32 = nullptr, *mR32 = nullptr;
  size_t zero_bytes = 0;
  // written by the kernels before they are read in the same call
  double *fv = nullptr, *dev0 = nullptr, *src = nullptr, *eqth = nullptr, *aos = nullptr;
  float *fv32 = nullptr, *src32 = nullptr, *dev032 = nullptr;
  float2 *eq32 = nullptr;
  size_t bytes = 0;
};

Layout plan(const zfvm_solver *s, unsigned char *base) {
  const size_t ld = s->ld, lde = s->lde, nv = s->nv, nd = s->nd;
  const size_t fpts = (size_t)s->nf * s->nqf * nv * ld;
  Layout L;
  Carve c{base};
  L.tend = c.take<double>(nv * ld);
  if (s->mixed) {
    L.g32 = c.take<float>(nv * lde);
    L.mL32 = c.take<float>(nd * lde);
    L.mR32 = c.take<float>(nd * lde);
  } else {
    L.nf = c.take<double>(nv * lde);
  }
  L.zero_bytes = c.used;
  if (s->mixed) {
    L.fv32 = c.take<float>(fpts);
    L.dev0 = c.take<double>(nv * ld);
    L.dev032 = c.take<float>(nv * ld);
    if (s->has_eq) L.eq32 = c.take<float2>(3 * ld);
    if (s->has_src) L.src32 = c.take<float>(nv * ld);
  } else {
    L.fv = c.take<double>(fpts);
    if (s->has_src) L.src = c.take<double>(nv * ld);
  }
  // with an equilibrium schedule the equilibrium outlives the call: the
  // solver's own buffer holds it
  if (s->has_eq && !s->sched_count.p) L.eqth = c.take<double>(4 * ld);
  L.aos = c.take<double>((size_t)5 * s->n_cells);
  L.bytes = c.used;
  return L;
}

// solver layout [nv][ld] -> the reference's cell-major rows (rho, m1, m2, m3, E)
__global__ void k_tendency_rows(const double *soa, double *aos, int n, int ld, int nv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double r[5] = {0, 0, 0, 0, 0};
  for (int v = 0; v < nv - 1; ++v) r[v] = soa[(size_t)v * ld + i];
  r[4] = soa[(size_t)(nv - 1) * ld + i];
  for (int v = 0; v < 5; ++v) aos[(size_t)i * 5 + v] = r[v];
}

}  // namespace

extern "C" int zfvm_rate_of_change_noalloc(zfvm_solver *s, double *tendency) {
  if (!s || !tendency) return fail(ZFVM_EINVAL, "null argument");
  SOLVER_GUARD_BEGIN
  const Layout need = plan(s, nullptr);
  if (need.bytes > (size_t)ZFVM_NOALLOC_SCRATCH_BYTES)
    return fail(ZFVM_EINVAL, "zfvm_rate_of_change_noalloc: this solver needs " + std::to_string(need.bytes) +
                                 " bytes of stage scratch (" + std::to_string(s->n_cells) +
                                 " cells), more than the fixed " + std::to_string(ZFVM_NOALLOC_SCRATCH_BYTES) +
                                 " bytes; use zfvm_rate_of_change");
  // the array handed to the kernels must be the one on the solver's device
  int current = -1;
  CK(cudaGetDevice(&current));
  if (current != s->device)
    return fail(ZFVM_EINVAL, "zfvm_rate_of_change_noalloc: the solver lives on device " + std::to_string(s->device) +
                                 " but device " + std::to_string(current) + " is current");
  const Layout L = plan(s, scratch_address(s->device));
  Clock c = read_clock(s);
  c.done = 0;
  c.status = 0;
  write_clock(s, c);
  CK(cudaMemsetAsync(L.tend, 0, L.zero_bytes, s->stream));
  StageArgs a = stage_args(s, 0, L.tend);
  a.fv = L.fv;
  a.fv32 = L.fv32;
  a.dev0 = L.dev0;
  a.dev032 = L.dev032;
  a.eq32 = L.eq32;
  a.nf = L.nf;
  a.src = L.src;
  if (L.eqth) a.eqth = L.eqth;
  a.g32 = L.g32;
  a.mL32 = L.mL32;
  a.mR32 = L.mR32;
  a.src32 = L.src32;
  for (int k = 0; k < 4; ++k) a.k[k] = nullptr, a.k32[k] = nullptr;
  solver_dispatch_stage(s, a);
  const int n = s->n_cells;
  k_tendency_rows<<<(n + 127) / 128, 128, 0, s->stream>>>(L.tend, L.aos, n, s->ld, s->nv);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(tendency, L.aos, (size_t)n * 5 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  const Clock c2 = read_clock(s);
  std::string msg;
  const int code = status_to_code(c2.status, msg);
  if (code) return fail(code, msg);
  return ZFVM_OK;
  SOLVER_GUARD_END
}
