// Serving engine: a request loop with continuous batching over the batch engine.
//
// Callers submit solves (mesh, scheme, initial state, end condition) from any
// thread; one worker thread owns the device work.  Every round it
//   1. admits queued requests in arrival order while their device footprint
//      (the exact bytes zfvm_solver_create will allocate) fits the memory
//      budget and a batch slot is free -- a request that does not fit may be
//      overtaken by smaller ones behind it, but only kMaxOvertaken times,
//      after which admission waits for it;
//   2. hands them to a set-up thread, which creates their solvers and uploads
//      their states while the batch keeps stepping, and adds the solvers that
//      are ready to the batch, so new requests join the solves on the device;
//   3. replays `steps_per_round` batched steps (one persistent launch per phase
//      per RK stage for all running requests of one kernel configuration);
//   4. retires finished requests: their final state is copied to the host,
//      the budget is returned and waiters are woken; the set-up thread frees
//      the solver.
// The state of every running request stays on the device between rounds.
// There is no counterpart in the reference, which runs one solve per process.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "solver_obj.hpp"

using namespace zfvm;

namespace {

using SteadyClock = std::chrono::steady_clock;

enum ReqState { kQueued = 0, kRunning = 1, kDone = 2, kFailed = 3 };
constexpr int kMaxOvertaken = 8;

struct Request {
  int64_t id = 0;
  zfvm_mesh *mesh = nullptr;
  zfvm_scheme_desc scheme{};
  std::vector<double> gravity_table;  // a tabulated potential, owned here (scheme points into it)
  std::vector<double> state;  // initial state; the final state once done
  double t0 = 0.0, t_end = 0.0;
  int64_t n_steps = 0;
  int64_t bytes = 0;  // device footprint reserved while admitted
  int64_t n_cells = 0;
  int phase = kQueued;
  int overtaken = 0;
  int error_code = 0;
  std::string error;
  zfvm_solver *solver = nullptr;
  int32_t slot = -1;
  double t_out = 0.0;
  int64_t steps_out = 0;
  SteadyClock::time_point t_submit, t_admit, t_finish;
};

double ms_between(SteadyClock::time_point a, SteadyClock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

struct zfvm_server {
  zfvm_server_desc desc{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_setup;
  std::map<int64_t, std::unique_ptr<Request>> reqs;
  std::deque<int64_t> queue;
  std::vector<Request *> running;  // worker thread only
  // set-up thread hand-over (under mu): admitted requests to create, created
  // ones ready for the batch, retired solvers to free
  std::deque<Request *> to_create, ready;
  std::deque<zfvm_solver *> to_destroy;
  int creating = 0;      // admitted requests not yet ready
  uint64_t changes = 0;  // bumped by anything that can make admission possible
  int64_t next_id = 1;
  bool stop = false, setup_stop = false;
  zfvm_batch *batch = nullptr;
  std::thread worker, setup;
  // statistics (under mu)
  int64_t submitted = 0, completed = 0, failed = 0, bytes_in_use = 0, bytes_peak = 0, cell_stages = 0;
  int64_t rounds = 0;
  double busy_s = 0.0, setup_s = 0.0;
  std::string fatal;
};

namespace {

void finish(zfvm_server *S, Request *r, int code, const std::string &msg) {
  // caller holds S->mu
  r->t_finish = SteadyClock::now();
  if (r->phase == kRunning) S->bytes_in_use -= r->bytes;  // queued requests hold no budget
  r->phase = code == ZFVM_OK ? kDone : kFailed;
  r->error_code = code;
  r->error = msg;
  if (code == ZFVM_OK) {
    ++S->completed;
    S->cell_stages += r->n_cells * r->scheme.rk_stages * r->steps_out;
  } else {
    ++S->failed;
  }
  ++S->changes;
  S->cv_done.notify_all();
  S->cv_work.notify_all();
}

// Pick queued requests that fit: arrival order, bounded overtaking.
std::vector<Request *> pick_admissions(zfvm_server *S) {
  std::vector<Request *> out;
  int64_t free_bytes = S->desc.hbm_budget_bytes - S->bytes_in_use;
  int free_slots = S->desc.max_slots - (int)S->running.size() - S->creating;
  std::vector<Request *> skipped;
  for (auto it = S->queue.begin(); it != S->queue.end() && free_slots > 0;) {
    Request *r = S->reqs[*it].get();
    if (r->bytes <= free_bytes) {
      bool blocked = false;
      for (Request *q : skipped) blocked = blocked || q->overtaken >= kMaxOvertaken;
      if (blocked) break;
      for (Request *q : skipped) ++q->overtaken;
      out.push_back(r);
      free_bytes -= r->bytes;
      --free_slots;
      r->phase = kRunning;
      r->t_admit = SteadyClock::now();
      S->bytes_in_use += r->bytes;
      S->bytes_peak = std::max(S->bytes_peak, S->bytes_in_use);
      it = S->queue.erase(it);
    } else {
      skipped.push_back(r);
      ++it;
    }
  }
  return out;
}

std::string last_error_str() { return std::string(zfvm_last_error()); }

std::string stopped_message(const zfvm_server *S) {
  return S->fatal.empty() ? "server stopped" : "server failed: " + S->fatal;
}

// Set-up thread: create the solvers of admitted requests, free retired ones.
void setup_main(zfvm_server *S) {
  cudaSetDevice(S->device);
  for (;;) {
    Request *r = nullptr;
    zfvm_solver *dead = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_setup.wait(lk, [&] { return S->setup_stop || !S->to_create.empty() || !S->to_destroy.empty(); });
      if (!S->to_destroy.empty()) {
        dead = S->to_destroy.front();
        S->to_destroy.pop_front();
      } else if (!S->to_create.empty()) {
        r = S->to_create.front();
        S->to_create.pop_front();
      } else {
        break;  // stopping and nothing left
      }
    }
    if (dead) {
      zfvm_solver_destroy(dead);
      continue;
    }
    const auto t0 = SteadyClock::now();
    zfvm_solver *s = nullptr;
    int st = zfvm_solver_create(r->mesh, &r->scheme, &s);
    if (st == ZFVM_OK) st = zfvm_set_state(s, r->state.data(), r->t0);
    const std::string msg = st == ZFVM_OK ? std::string() : last_error_str();
    if (st != ZFVM_OK && s) {
      zfvm_solver_destroy(s);
      s = nullptr;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    S->setup_s += std::chrono::duration<double>(SteadyClock::now() - t0).count();
    --S->creating;
    if (st != ZFVM_OK) {
      finish(S, r, st, msg);
    } else if (S->stop) {
      // the worker has stopped and drained the ready list already
      S->to_destroy.push_back(s);
      finish(S, r, ZFVM_EINVAL, stopped_message(S));
    } else {
      r->solver = s;
      S->ready.push_back(r);
      ++S->changes;
      S->cv_work.notify_all();
    }
  }
}

// Worker: put a created solver into the batch.
void add_ready(zfvm_server *S, Request *r) {
  int32_t slot = -1;
  const int st = zfvm_batch_add(S->batch, r->solver, r->n_steps, r->t_end, &slot);
  if (st != ZFVM_OK) {
    const std::string msg = last_error_str();
    std::lock_guard<std::mutex> lk(S->mu);
    S->to_destroy.push_back(r->solver);
    r->solver = nullptr;
    S->cv_setup.notify_all();
    finish(S, r, st, msg);
    return;
  }
  r->slot = slot;
  S->running.push_back(r);
}

// Move finished requests out of the batch.
int retire(zfvm_server *S, bool all) {
  int n = 0;
  for (size_t k = 0; k < S->running.size();) {
    Request *r = S->running[k];
    double t = 0.0;
    int64_t steps = 0;
    int32_t done = 0, status = 0;
    int st = zfvm_batch_slot_status(S->batch, r->slot, &t, &steps, &done, &status);
    if (st == ZFVM_OK && !done && !all) {
      ++k;
      continue;
    }
    std::string msg;
    int code = st;
    if (st == ZFVM_OK) code = zfvm_batch_remove(S->batch, r->slot);
    if (code == ZFVM_OK) code = zfvm_get_state(r->solver, r->state.data(), &r->t_out);
    if (code != ZFVM_OK) msg = last_error_str();
    if (code == ZFVM_OK && status != 0) code = status_to_code(status, msg);
    if (code == ZFVM_OK && all && !done) code = ZFVM_EINVAL, msg = "server stopped before the solve finished";
    r->steps_out = steps;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->to_destroy.push_back(r->solver);
      r->solver = nullptr;
      S->cv_setup.notify_all();
      finish(S, r, code, msg);
    }
    S->running.erase(S->running.begin() + k);
    ++n;
  }
  return n;
}

void worker_main(zfvm_server *S) {
  cudaSetDevice(S->device);
  uint64_t seen = ~uint64_t(0);
  for (;;) {
    std::vector<Request *> ready;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      // with nothing on the device, sleep until something can change:
      // a submission, a released budget or a solver becoming ready
      if (S->running.empty())
        S->cv_work.wait(lk, [&] { return S->stop || !S->ready.empty() || S->changes != seen; });
      if (S->stop) break;
      seen = S->changes;
      for (Request *r : pick_admissions(S)) {
        S->to_create.push_back(r);
        ++S->creating;
      }
      if (!S->to_create.empty()) S->cv_setup.notify_all();
      ready.assign(S->ready.begin(), S->ready.end());
      S->ready.clear();
    }
    for (Request *r : ready) add_ready(S, r);
    if (S->running.empty()) continue;
    const auto t0 = SteadyClock::now();
    int32_t n_run = 0;
    const int st = zfvm_batch_advance(S->batch, S->desc.steps_per_round, &n_run);
    if (st != ZFVM_OK) {
      const std::string msg = last_error_str();
      {
        std::lock_guard<std::mutex> lk(S->mu);
        S->fatal = msg;
      }
      retire(S, true);
      std::lock_guard<std::mutex> lk(S->mu);
      S->stop = true;
      break;
    }
    if (n_run < (int32_t)S->running.size()) retire(S, false);
    std::lock_guard<std::mutex> lk(S->mu);
    S->busy_s += std::chrono::duration<double>(SteadyClock::now() - t0).count();
    ++S->rounds;
  }
  retire(S, true);
  // S->stop is set: fail what is queued or waiting for the set-up thread; a
  // solver the set-up thread is still creating is failed when it is done
  std::lock_guard<std::mutex> lk(S->mu);
  const std::string msg = stopped_message(S);
  for (int64_t id : S->queue) {
    Request *r = S->reqs[id].get();
    r->t_admit = r->t_submit;
    finish(S, r, ZFVM_EINVAL, msg);
  }
  S->queue.clear();
  for (Request *r : S->to_create) {
    --S->creating;
    finish(S, r, ZFVM_EINVAL, msg);
  }
  S->to_create.clear();
  for (Request *r : S->ready) {
    S->to_destroy.push_back(r->solver);
    r->solver = nullptr;
    finish(S, r, ZFVM_EINVAL, msg);
  }
  S->ready.clear();
  S->cv_setup.notify_all();
}

}  // namespace

extern "C" int zfvm_server_create(const zfvm_server_desc *desc, zfvm_server **out) {
  if (!desc || !out) return fail(ZFVM_EINVAL, "null argument");
  if (desc->max_slots <= 0 || desc->steps_per_round <= 0) return fail(ZFVM_EINVAL, "bad max_slots or steps_per_round");
  try {
    auto S = std::make_unique<zfvm_server>();
    S->desc = *desc;
    CK(cudaGetDevice(&S->device));
    if (S->desc.hbm_budget_bytes <= 0) {
      size_t free_b = 0, total_b = 0;
      CK(cudaMemGetInfo(&free_b, &total_b));
      S->desc.hbm_budget_bytes = (int64_t)(0.8 * (double)free_b);
    }
    const int st = zfvm_batch_create(desc->max_slots, &S->batch);
    if (st != ZFVM_OK) return st;
    try {
      S->setup = std::thread(setup_main, S.get());
    } catch (const std::system_error &e) {
      zfvm_batch_destroy(S->batch);
      return fail(ZFVM_ENOMEM, std::string("cannot start the set-up thread: ") + e.what());
    }
    try {
      S->worker = std::thread(worker_main, S.get());
    } catch (const std::system_error &e) {
      {
        std::lock_guard<std::mutex> lk(S->mu);
        S->setup_stop = true;
      }
      S->cv_setup.notify_all();
      S->setup.join();
      zfvm_batch_destroy(S->batch);
      return fail(ZFVM_ENOMEM, std::string("cannot start the worker thread: ") + e.what());
    }
    *out = S.release();
    return ZFVM_OK;
  } catch (const CudaError &e) {
    return fail(ZFVM_ECUDA, e.where + ": " + cudaGetErrorString(e.err));
  }
}

extern "C" int zfvm_server_destroy(zfvm_server *S) {
  if (!S) return ZFVM_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  if (S->worker.joinable()) S->worker.join();
  // the set-up thread frees the solvers handed to it, then exits
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->setup_stop = true;
  }
  S->cv_setup.notify_all();
  if (S->setup.joinable()) S->setup.join();
  zfvm_batch_destroy(S->batch);
  delete S;
  return ZFVM_OK;
}

extern "C" int zfvm_server_submit(zfvm_server *S, zfvm_mesh *mesh, const zfvm_scheme_desc *scheme,
                                  const double *cvars, double t0, int64_t n_steps, double t_end, int64_t *id) {
  if (!S || !mesh || !scheme || !cvars || !id) return fail(ZFVM_EINVAL, "null argument");
  if (n_steps <= 0 && !(t_end > t0)) return fail(ZFVM_EINVAL, "need n_steps > 0 or t_end > t0");
  if (scheme->n_avars != 0)
    return fail(ZFVM_EINVAL, "server requests carry no advected variables (zfvm_server_submit takes cvars only)");
  const int64_t bytes = solver_footprint(mesh, *scheme);
  if (bytes < 0) return fail(ZFVM_EINVAL, "the mesh has fewer than two stencils");
  if (bytes > S->desc.hbm_budget_bytes)
    return fail(ZFVM_ENOMEM, "the solve needs " + std::to_string(bytes) + " device bytes, more than the server's budget of " +
                                 std::to_string(S->desc.hbm_budget_bytes));
  try {
    auto r = std::make_unique<Request>();
    r->mesh = mesh;
    r->scheme = *scheme;
    if (scheme->gravity == ZFVM_GRAVITY_RADIAL_TABLE && scheme->gravity_table_n > 0 && scheme->gravity_table_r &&
        scheme->gravity_table_phi) {
      // the solver is created later, on the set-up thread: keep the caller's table
      const size_t n = (size_t)scheme->gravity_table_n;
      r->gravity_table.assign(scheme->gravity_table_r, scheme->gravity_table_r + n);
      r->gravity_table.insert(r->gravity_table.end(), scheme->gravity_table_phi, scheme->gravity_table_phi + n);
      r->scheme.gravity_table_r = r->gravity_table.data();
      r->scheme.gravity_table_phi = r->gravity_table.data() + n;
    }
    r->n_cells = mesh->grid.n_cells;
    r->state.assign(cvars, cvars + (size_t)r->n_cells * 5);
    r->t0 = t0;
    r->t_end = t_end;
    r->n_steps = n_steps;
    r->bytes = bytes;
    r->t_submit = SteadyClock::now();
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return fail(ZFVM_EINVAL, stopped_message(S));
    r->id = S->next_id++;
    *id = r->id;
    S->queue.push_back(r->id);
    S->reqs[r->id] = std::move(r);
    ++S->submitted;
    ++S->changes;
  } catch (const std::bad_alloc &) {
    return fail(ZFVM_ENOMEM, "host allocation failed");
  }
  S->cv_work.notify_all();
  return ZFVM_OK;
}

extern "C" int zfvm_server_poll(zfvm_server *S, int64_t id, int32_t *phase) {
  if (!S || !phase) return fail(ZFVM_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) return fail(ZFVM_EINVAL, "unknown request id");
  *phase = it->second->phase;
  return ZFVM_OK;
}

extern "C" int zfvm_server_wait(zfvm_server *S, int64_t id, double timeout_s, double *cvars, double *t,
                                int64_t *steps, double *times_ms) {
  if (!S) return fail(ZFVM_EINVAL, "null argument");
  std::unique_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return fail(ZFVM_EINVAL, "unknown request id");
    Request *p = it->second.get();
    auto finished = [&] { return p->phase == kDone || p->phase == kFailed; };
    if (timeout_s < 0.0) {
      S->cv_done.wait(lk, finished);
    } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished)) {
      return fail(ZFVM_ETIMEDOUT, "request " + std::to_string(id) + " not finished within the timeout");
    }
    r = std::move(it->second);
    S->reqs.erase(it);
  }
  if (times_ms) {
    times_ms[0] = ms_between(r->t_submit, r->t_admit);
    times_ms[1] = ms_between(r->t_admit, r->t_finish);
    times_ms[2] = ms_between(r->t_submit, r->t_finish);
  }
  if (r->phase == kFailed) return fail(r->error_code ? r->error_code : ZFVM_EINVAL, r->error);
  if (cvars) std::copy(r->state.begin(), r->state.end(), cvars);
  if (t) *t = r->t_out;
  if (steps) *steps = r->steps_out;
  return ZFVM_OK;
}

extern "C" int zfvm_server_get_stats(zfvm_server *S, zfvm_server_stats *st) {
  if (!S || !st) return fail(ZFVM_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  st->submitted = S->submitted;
  st->completed = S->completed;
  st->failed = S->failed;
  st->queued = (int64_t)S->queue.size();
  int64_t running = 0;
  for (auto &kv : S->reqs) running += kv.second->phase == kRunning;
  st->running = running;
  st->bytes_in_use = S->bytes_in_use;
  st->bytes_peak = S->bytes_peak;
  st->budget_bytes = S->desc.hbm_budget_bytes;
  st->cell_stage_updates = S->cell_stages;
  st->rounds = S->rounds;
  st->busy_s = S->busy_s;
  st->setup_s = S->setup_s;
  return ZFVM_OK;
}
