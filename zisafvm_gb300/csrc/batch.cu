// Batch engine: many independent solves stepped together.
//
// Solvers are added to slots; slots of one kernel configuration form a group.
// Every RK stage launches one persistent reconstruction, one face and one
// update kernel per group; each walks the group's tile list (64, 128 or 256
// cells or faces per tile as the autotuner picked, one instance per tile), so
// meshes of any size share the launches.  Each slot keeps its own device clock: its own CFL time step, step
// count and end time; a slot that is done stops doing work.  The step loop is
// captured in a CUDA graph and replayed; adding or removing a slot only
// rebuilds the small device tables and re-captures the graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "solver_obj.hpp"

using namespace zfvm;
using namespace zfvm::dev;

namespace {

// mode 0: open a step for every slot; mode 1: close the last step only
__global__ void k_clock_multi(Clock *const *clocks, const double *cfl, int n, int mode) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) clock_step(clocks[k], cfl[k], mode);
}

// Host states of a batch round trip (zfvm_batch_step_host): per group
// instance, the staging rows and the buffers the layout kernels fill.
struct SlotIO {
  double *aos;       // n_cells x 5 rows (the solver's staging buffer)
  float2 *pairs;     // mixed form: FP32 pairs of the step and the stage state, else null
  const int *src;    // periodic source of every cell (ghost rows report their source)
  int slot, nv;
};

// Close every slot's open step (clock_step mode 1) and, for slots whose state
// is about to be replaced, restart the CFL minimum.  clock_slot maps clock
// index -> batch slot; mask[slot] bit 0: a new state comes in.
__global__ void k_clock_close_multi(Clock *const *clocks, const double *cfl, const int *clock_slot,
                                    const int *mask, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  clock_step(clocks[k], cfl[k], 1);
  if (mask[clock_slot[k]] & 1) clocks[k]->cfl_min = 0x7ff0000000000000ull;
}

// New states in, one block per cell tile of the slots that take one: AoS rows
// -> the step and stage states (SoA) and, in the mixed form, their FP32 pairs
// (as k_state_in); the CFL candidates of the new state go to the slot's clock
// (as k_cfl).
template <int NV>
__global__ void km_io_state_in(const BatchInst *__restrict__ inst, const SlotIO *__restrict__ io,
                               const Tile *__restrict__ tiles, const int *mask, int mixed) {
  const Tile tl = tiles[blockIdx.x];
  const SlotIO &o = io[tl.slot];
  if (!(mask[o.slot] & 1)) return;  // block-uniform: a tile belongs to one slot
  const BatchInst &I = inst[tl.slot];
  const DevData &d = I.d;
  const int i = tl.begin + threadIdx.x, ld = d.ld;
  double cand = INFINITY;
  if (i < d.n_cells) {
    double w[NV];
    float w32[NV];
    const size_t half = (size_t)NV * ld;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const double x = o.aos[(size_t)i * 5 + (v == NV - 1 ? 4 : v)];
      w[v] = x;
      w32[v] = __double2float_rn(x);
      I.a[0].u0[(size_t)v * ld + i] = x;
      I.a[0].ux[(size_t)v * ld + i] = x;
      if (o.pairs) {
        const float2 pr = make_float2(w32[v], __double2float_rn(x - (double)w32[v]));
        o.pairs[(size_t)v * ld + i] = pr;
        o.pairs[half + (size_t)v * ld + i] = pr;
      }
    }
    if (d.flags[i] & (kInterior | kFrozen))
      cand = mixed ? double(cfl_candidate_f32<NV>(w32, I.P.gamma32, float(d.r_eff[i])))
                   : cfl_candidate<NV>(w, I.P.gamma, d.r_eff[i]);
  }
  block_min_to_clock(cand, d.clock);
}

// States out, one block per cell tile of the slots read back: the step state
// (SoA) -> AoS rows, ghost rows from their periodic source (as k_soa_to_aos).
template <int NV>
__global__ void km_io_state_out(const BatchInst *__restrict__ inst, const SlotIO *__restrict__ io,
                                const Tile *__restrict__ tiles, const int *mask) {
  const Tile tl = tiles[blockIdx.x];
  const SlotIO &o = io[tl.slot];
  if (!(mask[o.slot] & 2)) return;
  const BatchInst &I = inst[tl.slot];
  const int i = tl.begin + threadIdx.x, ld = I.d.ld;
  if (i >= I.d.n_cells) return;
  const int j = o.src[i];
  double r[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int v = 0; v < NV - 1; ++v) r[v] = I.a[0].u0[(size_t)v * ld + j];
  r[4] = I.a[0].u0[(size_t)(NV - 1) * ld + j];
#pragma unroll
  for (int v = 0; v < 5; ++v) o.aos[(size_t)i * 5 + v] = r[v];
}

// number of slots still running
__global__ void k_count_running(Clock *const *clocks, int n, int *running) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n && !clocks[k]->done) atomicAdd(running, 1);
}

struct GroupKey {
  int shape, eq, src, mixed, flux, stages;
  bool operator<(const GroupKey &o) const {
    return std::tie(shape, eq, src, mixed, flux, stages) < std::tie(o.shape, o.eq, o.src, o.mixed, o.flux, o.stages);
  }
};

struct Group {
  GroupKey key;
  std::vector<int> slots;
  DBuf<BatchInst> inst;
  DBuf<SlotIO> io;
  DBuf<Tile> cell_tiles, face_tiles;
  int n_ct = 0, n_ft = 0;
  int block = 128;          // threads per block = cells or faces per tile
  int grid[3] = {0, 0, 0};  // persistent grid of the three kernels (0: one block per tile)
  bool tuned = false;
  // host round trips run the batch in parts (consecutive slot ranges):
  // part p's cell and face tiles are [part_ct[p], part_ct[p + 1]) and
  // [part_ft[p], part_ft[p + 1])
  std::vector<int> part_ct, part_ft;
};

// One part of a pipelined host round trip: its slot and clock ranges, stream,
// completion event and step graphs.
struct Part {
  int slot_lo = 0, slot_hi = 0, clk_lo = 0, clk_hi = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  cudaGraphExec_t graph = nullptr, graph_tail = nullptr;
  int graph_steps = 0, graph_tail_steps = 0;
};
// parts of a pipelined host round trip: the copies of one part overlap the
// steps of the others
constexpr int kIoParts = 4;

}  // namespace

struct zfvm_batch {
  int max_slots = 0;
  cudaStream_t stream = nullptr;
  std::vector<zfvm_solver *> slots;
  std::map<GroupKey, std::unique_ptr<Group>> groups;
  DBuf<Clock *> clock_ptrs;
  DBuf<double> cfls;
  DBuf<int> clock_slot;    // clock index -> slot
  DBuf<int> io_mask;       // per slot, for a host round trip: bit 0 state in, bit 1 state out
  std::vector<int> io_mask_host;
  DBuf<int> running;
  int n_clock = 0;
  // captured step loops: `graph` replays graph_steps steps, `graph_tail` the
  // remainder of a step count that is not a multiple of it
  cudaGraphExec_t graph = nullptr, graph_tail = nullptr;
  int graph_steps = 0, graph_tail_steps = 0;
  std::vector<Part> parts;  // slot ranges of a pipelined host round trip (rebuild)
  std::vector<cudaStream_t> part_streams;
  std::vector<cudaEvent_t> part_events;
  cudaEvent_t ev_fork = nullptr;
  bool dirty = true;
  int sms = 0;
};

namespace {

// One RK stage of group g over its tiles of part `part` (all tiles when part < 0).
void launch_group_stage(zfvm_batch *b, Group &g, int stage, cudaEvent_t *ev = nullptr, int part = -1,
                        cudaStream_t stream = nullptr) {
  const int c0 = part < 0 ? 0 : g.part_ct[part], c1 = part < 0 ? g.n_ct : g.part_ct[part + 1];
  const int f0 = part < 0 ? 0 : g.part_ft[part], f1 = part < 0 ? g.n_ft : g.part_ft[part + 1];
  if (c1 <= c0) return;
  BatchCfg c;
  c.ev = ev;
  c.eq = g.key.eq;
  c.src = g.key.src;
  c.mixed = g.key.mixed;
  c.flux = g.key.flux;
  c.block = g.block;
  c.grid_recon = g.grid[0];
  c.grid_face = g.grid[1];
  c.grid_update = g.grid[2];
  c.stream = stream ? stream : b->stream;
  const Tile *ct = g.cell_tiles.p + c0, *ft = g.face_tiles.p + f0;
  const int nc = c1 - c0, nf = f1 - f0;
  switch (g.key.shape) {
    case 0: launch_batch_stage_s2o3(g.inst.p, ct, nc, ft, nf, stage, c); break;
    case 1: launch_batch_stage_s2o2(g.inst.p, ct, nc, ft, nf, stage, c); break;
    case 2: launch_batch_stage_s3o3(g.inst.p, ct, nc, ft, nf, stage, c); break;
    case 3: launch_batch_stage_s3o2(g.inst.p, ct, nc, ft, nf, stage, c); break;
  }
  CK(cudaGetLastError());
}

// One batched step of every slot, or of the slots of part `part` on its stream.
void enqueue_batch_step(zfvm_batch *b, int part = -1) {
  if (b->n_clock == 0) return;
  const Part *pt = part < 0 ? nullptr : &b->parts[part];
  const int k0 = pt ? pt->clk_lo : 0, k1 = pt ? pt->clk_hi : b->n_clock;
  const int s0 = pt ? pt->slot_lo : 0, s1 = pt ? pt->slot_hi : (int)b->slots.size();
  cudaStream_t stream = pt ? pt->stream : b->stream;
  if (k1 <= k0) return;
  k_clock_multi<<<(k1 - k0 + 127) / 128, 128, 0, stream>>>(b->clock_ptrs.p + k0, b->cfls.p + k0, k1 - k0, 0);
  CK(cudaGetLastError());
  // slots with step rejection put back the start of a rejected step
  for (int k = s0; k < s1; ++k)
    if (b->slots[k] && b->slots[k]->uprev.p) solver_restore_on(b->slots[k], stream);
  int stages = 0;
  for (auto &kv : b->groups) stages = std::max(stages, kv.second->key.stages);
  for (int st = 0; st < stages; ++st) {
    for (auto &kv : b->groups)
      if (kv.second->n_ct > 0 && st < kv.second->key.stages) launch_group_stage(b, *kv.second, st, nullptr, part, stream);
    // advected variables: the slot's own three kernels after the stage, which
    // read the stage's face states before the next stage overwrites them
    for (int k = s0; k < s1; ++k) {
      zfvm_solver *s = b->slots[k];
      if (s && s->na && st < s->P.n_stages) solver_tracers_on(s, st, stream);
    }
  }
}

void drop_graphs(zfvm_batch *b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->graph_tail) cudaGraphExecDestroy(b->graph_tail);
  b->graph = b->graph_tail = nullptr;
  b->graph_steps = b->graph_tail_steps = 0;
  for (Part &pt : b->parts) {
    if (pt.graph) cudaGraphExecDestroy(pt.graph);
    if (pt.graph_tail) cudaGraphExecDestroy(pt.graph_tail);
    pt.graph = pt.graph_tail = nullptr;
    pt.graph_steps = pt.graph_tail_steps = 0;
  }
}

// Rebuild the device tables of every group from the current slots.
void rebuild(zfvm_batch *b) {
  drop_graphs(b);
  for (auto &kv : b->groups) kv.second->slots.clear();
  // parts: consecutive slot ranges of about equal cell counts
  {
    int64_t total = 0;
    int active = 0;
    for (zfvm_solver *s : b->slots)
      if (s) total += s->n_cells, ++active;
    const int np = std::min(kIoParts, active);
    b->parts.assign(np, Part{});
    int64_t acc = 0;
    int q = 0;
    for (int k = 0; k < (int)b->slots.size() && np > 0; ++k) {
      if (!b->slots[k]) continue;
      // part q ends once it holds its share of the cells (every part keeps a slot)
      if (q < np - 1 && acc >= total * (q + 1) / np) {
        b->parts[q].slot_hi = k;
        b->parts[++q].slot_lo = k;
      }
      acc += b->slots[k]->n_cells;
    }
    if (np > 0) {
      b->parts[0].slot_lo = 0;
      b->parts[np - 1].slot_hi = (int)b->slots.size();
      b->parts.resize(q + 1);
      b->parts[q].slot_hi = (int)b->slots.size();
    }
  }
  std::vector<Clock *> clocks;
  std::vector<double> cfls;
  std::vector<int> clock_slot;
  for (int k = 0; k < (int)b->slots.size(); ++k) {
    zfvm_solver *s = b->slots[k];
    if (!s) continue;
    GroupKey key{s->shape_id, s->has_eq, s->has_src, s->mixed, s->scheme.flux == ZFVM_FLUX_HLLC ? 0 : 1,
                 s->P.n_stages};
    auto &g = b->groups[key];
    if (!g) {
      g = std::make_unique<Group>();
      g->key = key;
    }
    g->slots.push_back(k);
    clocks.push_back(s->clock.p);
    cfls.push_back(s->P.cfl);
    clock_slot.push_back(k);
  }
  for (auto &kv : b->groups) {
    Group &g = *kv.second;
    std::vector<BatchInst> inst;
    std::vector<SlotIO> io;
    std::vector<Tile> ct, ft;
    std::vector<int> ct_at(g.slots.size() + 1), ft_at(g.slots.size() + 1);  // first tile of each instance
    for (size_t j = 0; j < g.slots.size(); ++j) {
      zfvm_solver *s = b->slots[g.slots[j]];
      ct_at[j] = (int)ct.size();
      ft_at[j] = (int)ft.size();
      io.push_back(SlotIO{s->aos.p, s->qsplit.p, s->src_map.p, g.slots[j], s->nv});
      BatchInst I{};
      I.d = s->D;
      I.P = s->P;
      for (int st = 0; st < 3; ++st) I.a[st] = stage_args(s, std::min(st, s->P.n_stages - 1), nullptr);
      inst.push_back(I);
      for (int c = 0; c < s->n_cells; c += g.block) ct.push_back(Tile{(int)j, c});
      for (int e = 0; e < s->n_edges; e += g.block) ft.push_back(Tile{(int)j, e});
    }
    ct_at[g.slots.size()] = (int)ct.size();
    ft_at[g.slots.size()] = (int)ft.size();
    // tile boundaries of the parts: the group's instances are in slot order
    g.part_ct.assign(b->parts.size() + 1, (int)ct.size());
    g.part_ft.assign(b->parts.size() + 1, (int)ft.size());
    for (size_t q = 0; q < b->parts.size(); ++q) {
      size_t j = 0;
      while (j < g.slots.size() && g.slots[j] < b->parts[q].slot_lo) ++j;
      g.part_ct[q] = ct_at[j];
      g.part_ft[q] = ft_at[j];
    }
    g.inst.upload(inst);
    g.io.upload(io);
    g.cell_tiles.upload(ct);
    g.face_tiles.upload(ft);
    g.n_ct = (int)ct.size();
    g.n_ft = (int)ft.size();
  }
  b->clock_ptrs.upload(clocks);
  b->cfls.upload(cfls);
  b->clock_slot.upload(clock_slot);
  b->n_clock = (int)clocks.size();
  for (Part &pt : b->parts) {
    pt.clk_lo = (int)(std::lower_bound(clock_slot.begin(), clock_slot.end(), pt.slot_lo) - clock_slot.begin());
    pt.clk_hi = (int)(std::lower_bound(clock_slot.begin(), clock_slot.end(), pt.slot_hi) - clock_slot.begin());
  }
  b->dirty = false;
}

void capture_steps(zfvm_batch *b, int steps, cudaGraphExec_t *out, int part = -1) {
  cudaGraph_t g;
  cudaStream_t stream = part < 0 ? b->stream : b->parts[part].stream;
  CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
  try {
    for (int k = 0; k < steps; ++k) enqueue_batch_step(b, part);
  } catch (...) {
    // end the capture, so the thread and the stream are usable again
    cudaGraph_t broken = nullptr;
    cudaStreamEndCapture(stream, &broken);
    if (broken) cudaGraphDestroy(broken);
    throw;
  }
  CK(cudaStreamEndCapture(stream, &g));
  CK(cudaGraphInstantiate(out, g, 0));
  cudaGraphDestroy(g);
}

// Streams and graphs of the parts for `n_steps` steps (at most 8 per graph).
int prepare_part_graphs(zfvm_batch *b, int n_steps) {
  if (b->dirty) rebuild(b);
  if (b->part_streams.size() < b->parts.size()) {
    // earlier parts first: their copies back overlap the later parts' steps
    int lo = 0, hi = 0;
    CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    while (b->part_streams.size() < b->parts.size()) {
      const int q = (int)b->part_streams.size();
      cudaStream_t st = nullptr;
      cudaEvent_t ev = nullptr;
      CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, std::min(lo, hi + q)));
      CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      b->part_streams.push_back(st);
      b->part_events.push_back(ev);
    }
  }
  if (!b->ev_fork) CK(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
  const int chunk = std::min(n_steps, 8), tail = n_steps % chunk;
  for (size_t q = 0; q < b->parts.size(); ++q) {
    Part &pt = b->parts[q];
    pt.stream = b->part_streams[q];
    pt.done = b->part_events[q];
    if (!pt.graph || pt.graph_steps != chunk) {
      if (pt.graph) cudaGraphExecDestroy(pt.graph);
      pt.graph = nullptr;
      capture_steps(b, chunk, &pt.graph, (int)q);
      pt.graph_steps = chunk;
    }
    if (tail && (!pt.graph_tail || pt.graph_tail_steps != tail)) {
      if (pt.graph_tail) cudaGraphExecDestroy(pt.graph_tail);
      pt.graph_tail = nullptr;
      capture_steps(b, tail, &pt.graph_tail, (int)q);
      pt.graph_tail_steps = tail;
    }
  }
  return chunk;
}

// The graphs that replay exactly n_steps steps: n_steps / chunk replays of a
// `chunk`-step graph (chunk = min(n_steps, chunk_max)) and one graph of the rest.
int prepare_graphs(zfvm_batch *b, int n_steps, int chunk_max) {
  if (b->dirty) rebuild(b);
  const int chunk = std::min(n_steps, chunk_max), tail = n_steps % chunk;
  if (!b->graph || b->graph_steps != chunk) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    capture_steps(b, chunk, &b->graph);
    b->graph_steps = chunk;
  }
  if (tail && (!b->graph_tail || b->graph_tail_steps != tail)) {
    if (b->graph_tail) cudaGraphExecDestroy(b->graph_tail);
    b->graph_tail = nullptr;
    capture_steps(b, tail, &b->graph_tail);
    b->graph_tail_steps = tail;
  }
  return chunk;
}

void launch_graphs(zfvm_batch *b, int n_steps, int chunk) {
  for (int k = 0; k + chunk <= n_steps; k += chunk) CK(cudaGraphLaunch(b->graph, b->stream));
  if (n_steps % chunk) CK(cudaGraphLaunch(b->graph_tail, b->stream));
}

// Work a caller queued on a slot's own stream (the layout and CFL kernels of
// zfvm_set_state, which returns once its host buffer is read) comes before the
// batch's next launch on the batch stream.
void wait_for_slots(zfvm_batch *b) {
  for (zfvm_solver *s : b->slots)
    if (s) {
      CK(cudaEventRecord(s->ev_sync, s->stream));
      CK(cudaStreamWaitEvent(b->stream, s->ev_sync, 0));
    }
}

int running_count(zfvm_batch *b) {
  if (b->n_clock == 0) return 0;
  CK(cudaMemsetAsync(b->running.p, 0, sizeof(int), b->stream));
  k_count_running<<<(b->n_clock + 127) / 128, 128, 0, b->stream>>>(b->clock_ptrs.p, b->n_clock, b->running.p);
  int r = 0;
  CK(cudaMemcpyAsync(&r, b->running.p, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return r;
}

int fail_cuda(const CudaError &e) { return fail(ZFVM_ECUDA, e.where + ": " + cudaGetErrorString(e.err)); }

}  // namespace

#define BATCH_GUARD_BEGIN try {
#define BATCH_GUARD_END                                  \
  }                                                      \
  catch (const CudaError &e) {                           \
    return fail_cuda(e);                                 \
  }                                                      \
  catch (const std::bad_alloc &) {                       \
    return fail(ZFVM_ENOMEM, "host allocation failed");  \
  }

extern "C" int zfvm_batch_create(int32_t max_slots, zfvm_batch **out) {
  if (!out || max_slots <= 0) return fail(ZFVM_EINVAL, "bad argument");
  auto b = std::make_unique<zfvm_batch>();
  BATCH_GUARD_BEGIN
  b->max_slots = max_slots;
  b->slots.assign(max_slots, nullptr);
  CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  b->running.alloc(1);
  int dev = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev));
  *out = b.release();
  return ZFVM_OK;
  BATCH_GUARD_END
}

extern "C" int zfvm_batch_destroy(zfvm_batch *b) {
  if (!b) return ZFVM_OK;
  drop_graphs(b);
  if (b->stream) {
    cudaStreamSynchronize(b->stream);
    cudaStreamDestroy(b->stream);
  }
  for (cudaStream_t st : b->part_streams) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  for (cudaEvent_t ev : b->part_events) cudaEventDestroy(ev);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  delete b;
  return ZFVM_OK;
}

extern "C" int zfvm_batch_add(zfvm_batch *b, zfvm_solver *s, int64_t n_steps, double t_end, int32_t *slot) {
  if (!b || !s) return fail(ZFVM_EINVAL, "null argument");
  if (n_steps <= 0 && !(t_end > 0.0)) return fail(ZFVM_EINVAL, "need n_steps > 0 or t_end > 0");
  BATCH_GUARD_BEGIN
  int k = -1;
  for (int j = 0; j < b->max_slots; ++j) {
    if (b->slots[j] == s) return fail(ZFVM_EINVAL, "solver already in the batch");
    if (k < 0 && !b->slots[j]) k = j;
  }
  if (k < 0) return fail(ZFVM_ENOMEM, "no free batch slot");
  CK(cudaStreamSynchronize(s->stream));
  reset_clock_for_run(s, n_steps, t_end, 0.0);
  CK(cudaStreamSynchronize(s->stream));
  b->slots[k] = s;
  b->dirty = true;
  if (slot) *slot = k;
  return ZFVM_OK;
  BATCH_GUARD_END
}

extern "C" int zfvm_batch_remove(zfvm_batch *b, int32_t slot) {
  if (!b || slot < 0 || slot >= b->max_slots || !b->slots[slot]) return fail(ZFVM_EINVAL, "bad slot");
  BATCH_GUARD_BEGIN
  CK(cudaStreamSynchronize(b->stream));
  zfvm_solver *s = b->slots[slot];
  // close the slot's last step so its clock reads the final time (and a
  // rejected last step is put back), as zfvm_advance does
  solver_close_step(s);
  CK(cudaStreamSynchronize(s->stream));
  b->slots[slot] = nullptr;
  b->dirty = true;
  return ZFVM_OK;
  BATCH_GUARD_END
}

extern "C" int zfvm_batch_advance(zfvm_batch *b, int32_t max_steps, int32_t *n_running) {
  if (!b || max_steps <= 0) return fail(ZFVM_EINVAL, "bad argument");
  BATCH_GUARD_BEGIN
  const int chunk = prepare_graphs(b, max_steps, 8);
  wait_for_slots(b);
  launch_graphs(b, max_steps, chunk);
  int r = running_count(b);
  if (n_running) *n_running = r;
  return ZFVM_OK;
  BATCH_GUARD_END
}

// The batch form of zfvm_step_host: one host round trip for every slot.
// Slots with a state in states_in[slot] take it at the time their clock holds
// (the open step of every slot is closed first, a rejected one put back, as
// zfvm_batch_remove does), the batch advances up to max_steps steps, and slots
// with a buffer in states_out[slot] are read back after their last step is
// closed (a rejected step put back).  The slots run in parts
// (consecutive slot ranges of about equal cell counts), each on its own stream
// with its own step graphs, so one part's copies overlap the other parts'
// steps; the layout and CFL work is one launch per part, kernel group and
// direction.  The host synchronises once, at the end.
extern "C" int zfvm_batch_step_host(zfvm_batch *b, const double *const *states_in, double *const *states_out,
                                    int32_t max_steps, int32_t *n_running) {
  if (!b || max_steps <= 0) return fail(ZFVM_EINVAL, "bad argument");
  BATCH_GUARD_BEGIN
  if (b->dirty) rebuild(b);
  const int n_slots = (int)b->slots.size();
  std::vector<int> &mask = b->io_mask_host;
  mask.assign(n_slots, 0);
  bool any_in = false, any_out = false;
  for (int k = 0; k < n_slots; ++k) {
    if (!b->slots[k]) continue;
    if (states_in && states_in[k]) mask[k] |= 1, any_in = true;
    if (states_out && states_out[k]) mask[k] |= 2, any_out = true;
  }
  if (b->n_clock == 0) {
    if (n_running) *n_running = 0;
    return ZFVM_OK;
  }
  const int chunk = prepare_part_graphs(b, max_steps);
  wait_for_slots(b);
  if (any_in || any_out) {
    if (b->io_mask.n < (size_t)n_slots) b->io_mask.alloc(n_slots);
    CK(cudaMemcpyAsync(b->io_mask.p, mask.data(), n_slots * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  }
  CK(cudaEventRecord(b->ev_fork, b->stream));
  for (size_t q = 0; q < b->parts.size(); ++q) {
    Part &pt = b->parts[q];
    cudaStream_t st = pt.stream;
    CK(cudaStreamWaitEvent(st, b->ev_fork, 0));
    if (any_in && pt.clk_hi > pt.clk_lo) {
      const int nk = pt.clk_hi - pt.clk_lo;
      k_clock_close_multi<<<(nk + 127) / 128, 128, 0, st>>>(b->clock_ptrs.p + pt.clk_lo, b->cfls.p + pt.clk_lo,
                                                            b->clock_slot.p + pt.clk_lo, b->io_mask.p, nk);
      CK(cudaGetLastError());
      for (int k = pt.slot_lo; k < pt.slot_hi; ++k)
        if (b->slots[k] && b->slots[k]->uprev.p) solver_restore_on(b->slots[k], st);
      for (int k = pt.slot_lo; k < pt.slot_hi; ++k)
        if (mask[k] & 1) {
          zfvm_solver *s = b->slots[k];
          CK(cudaMemcpyAsync(s->aos.p, states_in[k], (size_t)s->n_cells * 5 * sizeof(double),
                             cudaMemcpyHostToDevice, st));
        }
      for (auto &kv : b->groups) {
        Group &g = *kv.second;
        const int c0 = g.part_ct[q], nc = g.part_ct[q + 1] - c0;
        if (nc <= 0) continue;
        if (g.key.shape >= 2)
          km_io_state_in<5><<<nc, g.block, 0, st>>>(g.inst.p, g.io.p, g.cell_tiles.p + c0, b->io_mask.p, g.key.mixed);
        else
          km_io_state_in<4><<<nc, g.block, 0, st>>>(g.inst.p, g.io.p, g.cell_tiles.p + c0, b->io_mask.p, g.key.mixed);
        CK(cudaGetLastError());
      }
    }
    for (int k = 0; k + chunk <= max_steps; k += chunk) CK(cudaGraphLaunch(pt.graph, st));
    if (max_steps % chunk) CK(cudaGraphLaunch(pt.graph_tail, st));
    if (any_out) {
      // close the last step first, so a rejected one is put back before its
      // state goes out (the next step then opens with the shorter retry step)
      if (pt.clk_hi > pt.clk_lo) {
        const int nk = pt.clk_hi - pt.clk_lo;
        k_clock_multi<<<(nk + 127) / 128, 128, 0, st>>>(b->clock_ptrs.p + pt.clk_lo, b->cfls.p + pt.clk_lo, nk, 1);
        CK(cudaGetLastError());
        for (int k = pt.slot_lo; k < pt.slot_hi; ++k)
          if (b->slots[k] && b->slots[k]->uprev.p) solver_restore_on(b->slots[k], st);
      }
      for (auto &kv : b->groups) {
        Group &g = *kv.second;
        const int c0 = g.part_ct[q], nc = g.part_ct[q + 1] - c0;
        if (nc <= 0) continue;
        if (g.key.shape >= 2)
          km_io_state_out<5><<<nc, g.block, 0, st>>>(g.inst.p, g.io.p, g.cell_tiles.p + c0, b->io_mask.p);
        else
          km_io_state_out<4><<<nc, g.block, 0, st>>>(g.inst.p, g.io.p, g.cell_tiles.p + c0, b->io_mask.p);
        CK(cudaGetLastError());
      }
      for (int k = pt.slot_lo; k < pt.slot_hi; ++k)
        if (mask[k] & 2) {
          zfvm_solver *s = b->slots[k];
          CK(cudaMemcpyAsync(states_out[k], s->aos.p, (size_t)s->n_cells * 5 * sizeof(double),
                             cudaMemcpyDeviceToHost, st));
        }
    }
    CK(cudaEventRecord(pt.done, st));
    CK(cudaStreamWaitEvent(b->stream, pt.done, 0));
  }
  const int r = running_count(b);
  if (n_running) *n_running = r;
  return ZFVM_OK;
  BATCH_GUARD_END
}

extern "C" int zfvm_batch_advance_timed(zfvm_batch *b, int32_t n_steps, float *ms) {
  if (!b || !ms || n_steps <= 0) return fail(ZFVM_EINVAL, "bad argument");
  BATCH_GUARD_BEGIN
  const int chunk = prepare_graphs(b, n_steps, 8);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  wait_for_slots(b);
  CK(cudaStreamSynchronize(b->stream));
  CK(cudaEventRecord(e0, b->stream));
  launch_graphs(b, n_steps, chunk);
  CK(cudaEventRecord(e1, b->stream));
  CK(cudaEventSynchronize(e1));
  CK(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ZFVM_OK;
  BATCH_GUARD_END
}

// Autotuner: for each group, every tile size / block size (64, 128, 256 cells
// or faces per tile and threads per block) with every grid (one block per
// tile, or a persistent grid of 1x or 2x the occupancy limit times the SM
// count), timed over `trial_steps` steps; the fastest is kept.  The slots'
// states advance.
extern "C" int zfvm_batch_autotune(zfvm_batch *b, int32_t trial_steps, float *best_ms) {
  if (!b || trial_steps <= 0) return fail(ZFVM_EINVAL, "bad argument");
  BATCH_GUARD_BEGIN
  if (b->dirty) rebuild(b);
  wait_for_slots(b);
  float overall = 0.0f;
  for (auto &kv : b->groups) {
    Group &g = *kv.second;
    if (g.n_ct == 0) continue;
    float best = 1e30f;
    int best_block = g.block;
    std::array<int, 3> pick{0, 0, 0};
    for (int block : {64, 128, 256}) {
      g.block = block;
      rebuild(b);  // the group's tile lists for this tile size
      BatchCfg c{};
      c.mixed = g.key.mixed;
      c.block = block;
      int occ[3] = {1, 1, 1};
      switch (g.key.shape) {
        case 0: batch_occupancy_s2o3(c, occ); break;
        case 1: batch_occupancy_s2o2(c, occ); break;
        case 2: batch_occupancy_s3o3(c, occ); break;
        case 3: batch_occupancy_s3o2(c, occ); break;
      }
      std::vector<std::array<int, 3>> cands;
      cands.push_back({0, 0, 0});  // one block per tile
      for (int m : {1, 2})
        cands.push_back({std::max(1, occ[0] * m) * b->sms, std::max(1, occ[1] * m) * b->sms,
                         std::max(1, occ[2] * m) * b->sms});
      for (auto &cand : cands) {
        for (int j = 0; j < 3; ++j) g.grid[j] = cand[j];
        drop_graphs(b);
        float ms = 0;
        int st = zfvm_batch_advance_timed(b, trial_steps, &ms);
        if (st) return st;
        if (ms < best) best = ms, best_block = block, pick = cand;
      }
    }
    g.block = best_block;
    for (int j = 0; j < 3; ++j) g.grid[j] = pick[j];
    g.tuned = true;
    rebuild(b);
    overall += best;
  }
  drop_graphs(b);
  if (best_ms) *best_ms = overall;
  return ZFVM_OK;
  BATCH_GUARD_END
}

// The launch shape of every group: shape id, threads per block (= tile size),
// the grids of the reconstruction, face and update kernels (0: one block per
// tile), and whether the autotuner chose them.
extern "C" int zfvm_batch_launch_shapes(const zfvm_batch *b, int32_t max_groups, int32_t *shapes,
                                        int32_t *n_groups) {
  if (!b || !n_groups || (max_groups > 0 && !shapes)) return fail(ZFVM_EINVAL, "null argument");
  int k = 0;
  for (const auto &kv : b->groups) {
    const Group &g = *kv.second;
    if (g.slots.empty()) continue;
    if (k < max_groups) {
      int32_t *o = shapes + 6 * k;
      o[0] = g.key.shape, o[1] = g.block, o[2] = g.grid[0], o[3] = g.grid[1], o[4] = g.grid[2], o[5] = g.tuned;
    }
    ++k;
  }
  *n_groups = k;
  return ZFVM_OK;
}

// Average device time (ms) of one launch of each of the three stage kernels
// {reconstruct, face flux, update} over `n_steps` steps (no graph; events
// around every launch on the batch stream).  The slots' states advance.
extern "C" int zfvm_batch_kernel_times(zfvm_batch *b, int32_t n_steps, float *ms) {
  if (!b || !ms || n_steps <= 0) return fail(ZFVM_EINVAL, "bad argument");
  BATCH_GUARD_BEGIN
  if (b->dirty) rebuild(b);
  wait_for_slots(b);
  drop_graphs(b);
  cudaEvent_t ev[4];
  for (auto &e : ev) CK(cudaEventCreate(&e));
  double acc[3] = {0.0, 0.0, 0.0};
  int n = 0;
  int stages = 0;
  for (auto &kv : b->groups) stages = std::max(stages, kv.second->key.stages);
  for (int k = 0; k < n_steps && b->n_clock > 0; ++k) {
    k_clock_multi<<<(b->n_clock + 127) / 128, 128, 0, b->stream>>>(b->clock_ptrs.p, b->cfls.p, b->n_clock, 0);
    CK(cudaGetLastError());
    for (int st = 0; st < stages; ++st)
      for (auto &kv : b->groups) {
        if (kv.second->n_ct == 0 || st >= kv.second->key.stages) continue;
        launch_group_stage(b, *kv.second, st, ev);
        CK(cudaEventSynchronize(ev[3]));
        for (int j = 0; j < 3; ++j) {
          float t = 0.f;
          CK(cudaEventElapsedTime(&t, ev[j], ev[j + 1]));
          acc[j] += t;
        }
        ++n;
      }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  for (int j = 0; j < 3; ++j) ms[j] = n ? float(acc[j] / n) : 0.f;
  return ZFVM_OK;
  BATCH_GUARD_END
}

extern "C" int zfvm_batch_slot_status(zfvm_batch *b, int32_t slot, double *t, int64_t *steps, int32_t *done,
                                      int32_t *status) {
  if (!b || slot < 0 || slot >= b->max_slots || !b->slots[slot]) return fail(ZFVM_EINVAL, "bad slot");
  BATCH_GUARD_BEGIN
  CK(cudaStreamSynchronize(b->stream));
  Clock c = read_clock(b->slots[slot]);
  if (t) *t = c.t + (c.started ? c.dt : 0.0);
  if (steps) *steps = c.step + (c.started ? 1 : 0);
  if (done) *done = c.done;
  if (status) *status = c.status;
  return ZFVM_OK;
  BATCH_GUARD_END
}

extern "C" int zfvm_batch_slots(const zfvm_batch *b, int32_t *n_active) {
  if (!b || !n_active) return fail(ZFVM_EINVAL, "null argument");
  int n = 0;
  for (auto *s : b->slots) n += s != nullptr;
  *n_active = n;
  return ZFVM_OK;
}
