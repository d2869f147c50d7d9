// Host-side solver object behind the C ABI: device buffers, the kernels'
// argument structs and the captured step graph.  Shared by the single-solver
// entry points (solver.cu) and the batch engine (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <new>
#include <string>
#include <vector>

#include "gravity.hpp"
#include "mesh_obj.hpp"
#include "solver_kernels.cuh"

namespace zfvm {

struct CudaError {
  cudaError_t err;
  std::string where;
};

#define CK(x)                                                            \
  do {                                                                   \
    cudaError_t e_ = (x);                                                \
    if (e_ != cudaSuccess) throw CudaError{e_, #x};                      \
  } while (0)

template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr, o.n = 0; }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) {
      release();
      p = o.p, n = o.n;
      o.p = nullptr, o.n = 0;
    }
    return *this;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    release();
    n = count;
    if (count) CK(cudaMalloc((void **)&p, count * sizeof(T)));
  }
  void upload(const std::vector<T> &h) {
    alloc(h.size());
    if (n) CK(cudaMemcpy(p, h.data(), n * sizeof(T), cudaMemcpyHostToDevice));
  }
  void zero(cudaStream_t s) {
    if (n) CK(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
  ~DBuf() { release(); }
};

}  // namespace zfvm

struct zfvm_solver {
  zfvm_mesh *mesh = nullptr;
  zfvm_scheme_desc scheme{};
  int nd = 2, nv = 4, nf = 3, nqf = 2, nqc = 3, ld = 0, lde = 0;
  int n_cells = 0, n_edges = 0;
  int shape_id = -1;
  int device = -1;  // the device current at creation, which owns every buffer and the stream
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_in = nullptr;    // recorded after a host upload
  cudaEvent_t ev_sync = nullptr;  // recorded by a batch before it uses the solver
  zfvm::RadialPotential pot;  // the gravity potential (its table copied from the scheme)
  zfvm::dev::Params P{};
  zfvm::dev::DevData D{};
  // device buffers
  zfvm::DBuf<uint8_t> flags, bloc, fkL, fkR, factive;
  zfvm::DBuf<int> l2g, cface, fL, fR, src_map;
  zfvm::DBuf<double> pinv, center, inv_len, mom, inv_vol, r_eff, fqx, fqw, frame, farea;
  zfvm::DBuf<float> pinv32, fv32, frame32, xfq32, xcq32, mom32, wg32, g32, mL32, mR32, src32, kbuf32, fqw32;
  zfvm::DBuf<double> gphi_w;
  zfvm::DBuf<double> phi_cq, phi_m1, phi_var, gphi_cq, cqx, cqw, phi_fq;
  zfvm::DBuf<double> u0, ux, kbuf, fv, nfb, srcb, eqth, tend, aos, dev0;
  zfvm::DBuf<float2> qsplit, m1s, vars;  // mixed: FP32 (hi, lo) pairs of u0, ux; <phi>, var(phi)
  zfvm::DBuf<float2> eq32, phi_fq2;       // mixed + equilibrium: (h_r, f, K) pairs; phi at face points
  zfvm::DBuf<float> dev032;               // mixed: FP32 copy of the cell deviation
  zfvm::DBuf<double> poly;                // exported reconstruction records (zfvm_reconstruct)
  zfvm::DBuf<double> uprev;               // step rejection: start state of the running step
  zfvm::DBuf<double> heat_w;              // heating: w_q * rate(x_q) at the cell quadrature points
  zfvm::DBuf<int> sched_count;            // equilibrium schedule: reconstructions since the last refresh
  zfvm::DBuf<double> sched;               // equilibrium schedule: scale and own average of the last refresh [4][ld]
  // advected variables (n_avars > 0): state, next stage, stage tendencies,
  // face-point values, face fluxes, tendency output, step-rejection save
  int na = 0;
  zfvm::DBuf<double> tq0, tqx, tk, tfv, tnf, ttend, tprev;
  std::vector<int> src_host;              // periodic source of every cell (host copy of src_map)
  std::vector<double> poly_host;
  zfvm::DBuf<zfvm::dev::Clock> clock;
  bool has_src = false, has_eq = false, mixed = false;
  // captured step loops: `graph` replays graph_steps steps, `graph_tail` the
  // remainder of a timed step count that is not a multiple of it
  cudaGraphExec_t graph = nullptr, graph_tail = nullptr;
  int graph_steps = 0, graph_tail_steps = 0;
  int64_t device_bytes = 0;
  zfvm_solver() = default;
  zfvm_solver(const zfvm_solver &) = delete;
  zfvm_solver &operator=(const zfvm_solver &) = delete;
  // Also runs when zfvm_solver_create fails part-way: the work on the stream
  // ends before the buffers (members, freed after this body) go away.
  ~zfvm_solver() {
    if (graph) cudaGraphExecDestroy(graph);
    if (graph_tail) cudaGraphExecDestroy(graph_tail);
    if (stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_sync) cudaEventDestroy(ev_sync);
  }
};


// helpers shared with the batch engine (solver.cu)
zfvm::dev::StageArgs stage_args(zfvm_solver *s, int stage, double *tend_out);
// the three kernels of one stage on the solver's stream, with the solver's
// launch configuration (the entry point without allocation swaps the scratch
// pointers of `a` and launches through this)
void solver_dispatch_stage(zfvm_solver *s, zfvm::dev::StageArgs &a);
zfvm::dev::TracerArgs tracer_args(zfvm_solver *s, int stage, double *tend_out);
// per-solver launches the batch engine adds on its own stream: the restore of
// a rejected step (after the clock), the advected variables' kernels of a
// stage (after the stage), and the close of a solver's last step
void solver_restore_on(zfvm_solver *s, cudaStream_t stream);
void solver_tracers_on(zfvm_solver *s, int stage, cudaStream_t stream);
void solver_close_step(zfvm_solver *s);
zfvm::dev::Clock read_clock(zfvm_solver *s);
zfvm::dev::Clock fresh_clock(const zfvm_solver *s, double t);
void write_clock(zfvm_solver *s, const zfvm::dev::Clock &c);
void reset_clock_for_run(zfvm_solver *s, int64_t n_steps, double t_end, double fixed_dt);
// ZFVM_* status and message for the device status bits of a Clock
int status_to_code(int st, std::string &msg);
// device bytes zfvm_solver_create allocates for this mesh and scheme (-1: no stencils)
int64_t solver_footprint(const zfvm_mesh *m, const zfvm_scheme_desc &sc);

// The C ABI's error guard: every failure inside an entry point becomes a status
// code and a zfvm_last_error message, nothing escapes the extern "C" boundary.
inline int cuda_fail(const zfvm::CudaError &e) {
  return zfvm::fail(ZFVM_ECUDA, e.where + ": " + cudaGetErrorString(e.err));
}
#define SOLVER_GUARD_BEGIN try {
#define SOLVER_GUARD_END                                  \
  }                                                       \
  catch (const zfvm::CudaError &e) {                      \
    return cuda_fail(e);                                  \
  }                                                       \
  catch (const zfvm::SetupError &e) {                     \
    return zfvm::fail(ZFVM_ESETUP, e.what());             \
  }                                                       \
  catch (const std::bad_alloc &) {                        \
    return zfvm::fail(ZFVM_ENOMEM, "host allocation failed"); \
  }
