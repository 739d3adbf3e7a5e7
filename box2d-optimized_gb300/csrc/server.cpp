// server.cpp - continuous-batching rollout server.
//
// A request is a seeded scene (the batch-world recipe with a body count) plus K steps. Requests
// wait in a FIFO queue. Each tick runs ONE batched Step of every active world, so requests that
// arrive while others are running join a later Step instead of waiting for the batch to drain.
//
// Admission is taken off the step's critical path. The tick admits FIFO within the world slots and
// the device memory budget, but building an admitted request's world (the scene recipe on the
// host, about a microsecond per body) runs on builder threads, each on its own host-only batch.
// A built world moves into the served batch while a step runs on the device (no record is
// copied), the tick packs the new worlds into device layout in the same window, and the next
// tick's step uploads them: that step leaves them out of the solve (its closing broadphase gives
// them their first contacts) and they step from the tick after. When nothing is running, the tick
// waits for the builds it started and uploads them at once. A request finishes after its K steps:
// its final state is summarised, its world retired, and retired worlds are compacted away in
// bulk. World state stays resident on the device between ticks.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/b2g_capi.h"
#include "engine.h"

namespace {

// Device bytes budgeted per body of an admitted world: body and fixture records, contact
// buffers (about three contacts per body, both lists, pair list, solver scratch) and broadphase
// scratch, rounded up.
const uint64_t kBytesPerBody = 2304;
const int kDefaultBuilders = 2;

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  int64_t id;
  uint32_t seed;
  int32_t bodies;
  int32_t steps;
  int32_t done = 0;
  int32_t world = -1;
  double submit = 0, admit = 0;
  uint64_t bytes = 0;
  bool uploaded = false;  // its world is on the device (a step has uploaded it)
  bool stepped = false;   // stepped by the current tick
};

// An admitted request whose world has been built on the host.
struct Built {
  Request r;
  int status = B2G_OK;
  b2g::HostWorld world;
  float checksum[4] = {0, 0, 0, 0};  // K = 0 requests: the initial state's summary
};

// Sum of x, y, angle and |v| over the world's bodies, accumulated in creation order.
int world_checksum(b2g_batch* batch, int world, float* out4) {
  int32_t nb = 0;
  int st = b2g_world_sizes(batch, world, &nb, nullptr, nullptr, nullptr);
  if (st != B2G_OK) return st;
  std::vector<b2g_body> bodies(nb);
  if (nb) {
    st = b2g_bodies_read(batch, world, 0, nb, bodies.data());
    if (st != B2G_OK) return st;
  }
  double acc[4] = {0, 0, 0, 0};
  for (const b2g_body& b : bodies) {
    acc[0] += b.c[0];
    acc[1] += b.c[1];
    acc[2] += b.a;
    acc[3] += sqrt((double)b.v[0] * b.v[0] + (double)b.v[1] * b.v[1]);
  }
  for (int k = 0; k < 4; ++k) out4[k] = (float)acc[k];
  return B2G_OK;
}

// Builds a request's world on a host-only batch and moves it out into o->world.
void build_world(b2g_batch* scratch, Built* o) {
  const Request& r = o->r;
  int32_t n = 0, w = -1;
  float gx = 0, gy = -10;
  b2g_batch_world_params(r.seed, &n, &gx, &gy);
  int st = b2g_world_add(scratch, gx, gy, &w);
  if (st == B2G_OK) st = b2g_world_set_flags(scratch, w, 0, 1, 0, 1);
  if (st == B2G_OK) st = b2g_scene_build(scratch, w, B2G_SCENE_BATCH_WORLD, r.seed, r.bodies, 0, 0, nullptr);
  if (st == B2G_OK && r.steps == 0) st = world_checksum(scratch, w, o->checksum);
  if (w >= 0) {
    int t = b2g::take_world(scratch, w, &o->world);
    if (st == B2G_OK) st = t;
  }
  o->status = st;
}

}  // namespace

struct b2g_server {
  b2g_batch* batch = nullptr;
  int32_t max_worlds = 0;
  float dt = 1.0f / 60.0f;
  int32_t vi = 8, pi = 3;
  uint64_t budget = 0;
  uint64_t in_use = 0;
  std::deque<Request> queue;
  std::vector<Request> active;
  std::vector<uint8_t> mask;  // per world: stepped in this tick
  std::vector<b2g_request_result> finished;
  int64_t next_id = 1, completed = 0, rejected = 0;
  int32_t retired = 0;
  // world building: requests admitted and not yet in `active` (to build, building or built)
  b2g_batch* scratch = nullptr;  // the tick thread's own host-only batch (no builder threads)
  std::vector<std::thread> builders;
  std::mutex m;
  std::condition_variable cv_todo, cv_built;
  std::deque<Built*> todo;    // guarded by m
  std::vector<Built*> built;  // guarded by m
  int32_t unbuilt = 0;        // guarded by m: in todo or being built
  bool stop = false;          // guarded by m
  int32_t admitted = 0;       // admitted, not yet joined (tick thread only)
  std::unordered_map<int64_t, Request> admitted_reqs;  // admitted, not yet joined, by id
  std::unordered_set<int64_t> cancelled;
};

namespace {

void builder_main(b2g_server* s) {
  b2g_batch* scratch = nullptr;
  b2g_batch_create(B2G_HOST_ONLY, 0, &scratch);
  for (;;) {
    Built* o = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->m);
      s->cv_todo.wait(lk, [&] { return s->stop || !s->todo.empty(); });
      if (s->stop) break;
      o = s->todo.front();
      s->todo.pop_front();
    }
    if (scratch) build_world(scratch, o);
    else o->status = B2G_E_OUT_OF_MEMORY;
    {
      std::lock_guard<std::mutex> lk(s->m);
      s->built.push_back(o);
      --s->unbuilt;
    }
    s->cv_built.notify_all();
  }
  b2g_batch_destroy(scratch);
}

void stop_builders(b2g_server* s) {
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->stop = true;
  }
  s->cv_todo.notify_all();
  for (std::thread& t : s->builders) t.join();
  s->builders.clear();
  s->stop = false;
}

void start_builders(b2g_server* s, int n) {
  for (int i = 0; i < n; ++i) s->builders.emplace_back(builder_main, s);
}

}  // namespace

extern "C" {

B2G_API int b2g_server_create(int device, uint64_t budget_bytes, int32_t max_worlds, float dt,
                              int32_t velocity_iterations, int32_t position_iterations, b2g_server** out) {
  if (!out || max_worlds <= 0 || !(dt > 0.0f) || velocity_iterations < 0 || position_iterations < 0)
    return B2G_E_INVALID_ARG;
  b2g_server* s = new b2g_server();
  // the budget governs admission (per-body estimate); the batch itself gets no hard cap, since
  // its fixed scratch (sort temporaries, counters) does not scale with the admitted bodies
  int st = b2g_batch_create(device, 0, &s->batch);
  if (st == B2G_OK) st = b2g_batch_create(B2G_HOST_ONLY, 0, &s->scratch);
  if (st != B2G_OK) {
    if (s->batch) b2g_batch_destroy(s->batch);
    delete s;
    return st;
  }
  b2g_batch_set_graphs(s->batch, 0);  // the layout changes on most ticks; launch eagerly
  s->max_worlds = max_worlds;
  s->dt = dt;
  s->vi = velocity_iterations;
  s->pi = position_iterations;
  s->budget = budget_bytes;
  start_builders(s, kDefaultBuilders);
  *out = s;
  return B2G_OK;
}

B2G_API int b2g_server_destroy(b2g_server* s) {
  if (!s) return B2G_E_INVALID_ARG;
  stop_builders(s);
  for (Built* o : s->todo) delete o;
  for (Built* o : s->built) delete o;
  b2g_batch_destroy(s->scratch);
  b2g_batch_destroy(s->batch);
  delete s;
  return B2G_OK;
}

B2G_API int b2g_server_set_builders(b2g_server* s, int32_t n) {
  if (!s || n < 0 || n > 64) return B2G_E_INVALID_ARG;
  if (s->admitted) return B2G_E_LOCKED;  // only with no admitted world still to join
  stop_builders(s);
  start_builders(s, n);
  return B2G_OK;
}

B2G_API int b2g_server_submit(b2g_server* s, uint32_t seed, int32_t bodies, int32_t steps, int64_t* out_id) {
  if (!s || bodies < 1 || steps < 0) return B2G_E_INVALID_ARG;
  Request r;
  r.id = s->next_id++;
  r.seed = seed;
  r.bodies = bodies;
  r.steps = steps;
  r.submit = now_s();
  r.bytes = (uint64_t)bodies * kBytesPerBody;
  s->queue.push_back(r);
  if (out_id) *out_id = r.id;
  return B2G_OK;
}

static void finish(b2g_server* s, const Request& r, int status, const float* checksum) {
  b2g_request_result o;
  memset(&o, 0, sizeof(o));
  o.request_id = r.id;
  o.status = status;
  o.bodies = r.bodies;
  o.steps = r.done;
  o.submit_time_s = r.submit;
  o.admit_time_s = r.admit;
  o.finish_time_s = now_s();
  if (checksum)
    for (int k = 0; k < 4; ++k) o.checksum[k] = checksum[k];
  s->finished.push_back(o);
}

// Admits queued requests FIFO while world slots and the budget allow (a request larger than the
// whole budget is rejected) and hands them to the builders. Without builder threads the tick
// builds them itself: with `overlap`, only while the device is still busy with the step in flight
// (after at least one, so the queue always moves).
static void admit(b2g_server* s, bool overlap) {
  int built_here = 0;
  while (!s->queue.empty() && (int32_t)s->active.size() + s->admitted < s->max_worlds) {
    Request r = s->queue.front();
    if (s->budget && r.bytes > s->budget) {
      s->queue.pop_front();
      ++s->rejected;
      finish(s, r, B2G_E_OUT_OF_MEMORY, nullptr);
      continue;
    }
    if (s->budget && s->in_use + r.bytes > s->budget) break;
    if (s->builders.empty() && overlap && built_here > 0) {
      int32_t done = 1;
      b2g_step_poll(s->batch, &done);
      if (done) break;
    }
    s->queue.pop_front();
    s->in_use += r.bytes;
    ++s->admitted;
    s->admitted_reqs[r.id] = r;
    Built* o = new Built();
    o->r = r;
    if (s->builders.empty()) {
      build_world(s->scratch, o);
      ++built_here;
      std::lock_guard<std::mutex> lk(s->m);
      s->built.push_back(o);
    } else {
      {
        std::lock_guard<std::mutex> lk(s->m);
        s->todo.push_back(o);
        ++s->unbuilt;
      }
      s->cv_todo.notify_one();
    }
  }
}

// Moves the built worlds into the served batch (they are uploaded by the next step); with
// `wait`, first waits until every admitted world is built. Returns how many joined `active`.
static int join_built(b2g_server* s, bool wait) {
  std::vector<Built*> got;
  {
    std::unique_lock<std::mutex> lk(s->m);
    if (wait) s->cv_built.wait(lk, [&] { return s->unbuilt == 0; });
    got.swap(s->built);
  }
  int joined = 0;
  for (Built* o : got) {
    Request r = o->r;
    --s->admitted;
    s->admitted_reqs.erase(r.id);
    r.admit = now_s();
    if (s->cancelled.erase(r.id)) {  // cancelled while it was built: already reported
      s->in_use -= r.bytes;
    } else if (o->status != B2G_OK) {
      s->in_use -= r.bytes;
      ++s->rejected;
      finish(s, r, o->status, nullptr);
    } else if (r.steps == 0) {  // nothing to step: the initial state's summary is the result
      s->in_use -= r.bytes;
      ++s->completed;
      finish(s, r, B2G_OK, o->checksum);
    } else {
      int st = b2g::append_world(s->batch, std::move(o->world), &r.world);
      if (st != B2G_OK) {
        s->in_use -= r.bytes;
        ++s->rejected;
        finish(s, r, st, nullptr);
      } else {
        s->active.push_back(r);
        ++joined;
      }
    }
    delete o;
  }
  return joined;
}

B2G_API int b2g_server_tick(b2g_server* s, int32_t* active, double* step_ms) {
  if (!s) return B2G_E_INVALID_ARG;
  if (step_ms) *step_ms = 0.0;
  // nothing running to overlap with: admit, wait for the builds, and let this step upload them
  if (s->active.empty()) {
    admit(s, false);
    join_built(s, true);
  }
  if (!s->active.empty()) {
    // every active request has at least one step left (K = 0 requests finish at admission).
    // Worlds not on the device yet are uploaded by this step but left out of its solve.
    int32_t nw = 0;
    b2g_world_count(s->batch, &nw);
    s->mask.assign((size_t)nw, 0);
    for (Request& r : s->active) {
      r.stepped = r.uploaded;
      if (r.stepped) s->mask[r.world] = 1;
    }
    double t0 = now_s();
    int st = b2g_step_begin(s->batch, s->dt, s->vi, s->pi, s->mask.data());
    if (st != B2G_OK) return st;
    for (Request& r : s->active) r.uploaded = true;
    // while the device steps: admit, take in the built worlds and pack them for the next upload
    admit(s, true);
    if (join_built(s, false) > 0) b2g_batch_stage(s->batch);
    st = b2g_step_end(s->batch);
    if (step_ms) *step_ms = (now_s() - t0) * 1e3;
    if (st != B2G_OK) return st;
  }
  if (active) *active = (int32_t)s->active.size();
  // retire finished requests; a request whose world faulted (non-finite state) ends with that
  // status, the others run on unaffected
  std::vector<Request> still;
  bool waiting = false;  // some admitted world is not on the device yet
  for (Request& r : s->active) {
    if (!r.stepped) {
      waiting |= !r.uploaded;
      still.push_back(r);
      continue;
    }
    r.stepped = false;
    ++r.done;
    int32_t wst = B2G_OK;
    b2g_world_status(s->batch, r.world, &wst);
    if (wst != B2G_OK) {
      b2g_world_retire(s->batch, r.world);
      ++s->retired;
      s->in_use -= r.bytes;
      ++s->rejected;
      finish(s, r, wst, nullptr);
      continue;
    }
    if (r.done >= r.steps) {
      float cs[4];
      int st = world_checksum(s->batch, r.world, cs);
      b2g_world_retire(s->batch, r.world);
      ++s->retired;
      s->in_use -= r.bytes;
      ++s->completed;
      finish(s, r, st, st == B2G_OK ? cs : nullptr);
    } else {
      still.push_back(r);
    }
  }
  s->active.swap(still);
  // reclaim retired worlds in bulk once they outnumber the running ones, in a tick that leaves no
  // admitted world waiting for its upload (compaction renumbers worlds, which would discard the
  // staged pack)
  if (!waiting && s->retired >= 4 && s->retired >= (int32_t)s->active.size()) {
    int32_t nw = 0;
    b2g_world_count(s->batch, &nw);
    std::vector<int32_t> map(nw);
    int st = b2g_compact(s->batch, map.data(), nw);
    if (st != B2G_OK) return st;
    for (Request& r : s->active) r.world = map[r.world];
    s->retired = 0;
  }
  return B2G_OK;
}

B2G_API int b2g_server_batch(b2g_server* s, b2g_batch** out) {
  if (!s || !out) return B2G_E_INVALID_ARG;
  *out = s->batch;
  return B2G_OK;
}

B2G_API int b2g_server_cancel(b2g_server* s, int64_t request_id) {
  if (!s) return B2G_E_INVALID_ARG;
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
    if (it->id != request_id) continue;
    Request r = *it;
    s->queue.erase(it);
    finish(s, r, B2G_E_CANCELLED, nullptr);
    return B2G_OK;
  }
  auto adm = s->admitted_reqs.find(request_id);
  if (adm != s->admitted_reqs.end() && !s->cancelled.count(request_id)) {
    // admitted, its world still being built: reported now, the world dropped once built
    s->cancelled.insert(request_id);
    finish(s, adm->second, B2G_E_CANCELLED, nullptr);
    return B2G_OK;
  }
  for (auto it = s->active.begin(); it != s->active.end(); ++it) {
    if (it->id != request_id) continue;
    Request r = *it;
    s->active.erase(it);
    b2g_world_retire(s->batch, r.world);
    ++s->retired;
    s->in_use -= r.bytes;
    finish(s, r, B2G_E_CANCELLED, nullptr);
    return B2G_OK;
  }
  return B2G_E_INVALID_ARG;
}

B2G_API int b2g_server_poll(b2g_server* s, b2g_request_result* out, int32_t cap, int32_t* n) {
  if (!s || !n) return B2G_E_INVALID_ARG;
  int32_t k = (int32_t)std::min<size_t>(s->finished.size(), (size_t)std::max(cap, 0));
  if (out)
    for (int32_t i = 0; i < k; ++i) out[i] = s->finished[i];
  s->finished.erase(s->finished.begin(), s->finished.begin() + k);
  *n = k;
  return B2G_OK;
}

B2G_API int b2g_server_stats(b2g_server* s, int64_t* queued, int64_t* active, int64_t* completed, int64_t* rejected,
                             int64_t* hbm_bytes) {
  if (!s) return B2G_E_INVALID_ARG;
  if (queued) *queued = (int64_t)s->queue.size();
  if (active) *active = (int64_t)s->active.size() + s->admitted;
  if (completed) *completed = s->completed;
  if (rejected) *rejected = s->rejected;
  if (hbm_bytes) *hbm_bytes = (int64_t)b2g::batch_allocated_bytes(s->batch);
  return B2G_OK;
}

}  // extern "C"
