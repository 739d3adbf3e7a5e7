// server.cpp - continuous-batching rollout server.
//
// A request is a seeded scene (the batch-world recipe with a body count) plus K steps. Requests
// wait in a FIFO queue; each tick admits as many as fit (world slots and the device memory
// budget), then runs ONE batched Step of every active world, so requests that arrive while
// others are running join the next Step instead of waiting for the batch to drain. A request
// finishes after its K steps: its final state is summarised, its world retired, and retired
// worlds are compacted away in bulk. World state stays resident on the device between ticks.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <vector>

#include "../../include/b2g_capi.h"
#include "engine.h"

namespace {

// Device bytes budgeted per body of an admitted world: body and fixture records, contact
// buffers (about three contacts per body, both lists, pair list, solver scratch) and broadphase
// scratch, rounded up.
const uint64_t kBytesPerBody = 2048;

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
};

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
  std::vector<b2g_request_result> finished;
  int64_t next_id = 1, completed = 0, rejected = 0;
  int32_t retired = 0;
};

extern "C" {

B2G_API int b2g_server_create(int device, uint64_t budget_bytes, int32_t max_worlds, float dt,
                              int32_t velocity_iterations, int32_t position_iterations, b2g_server** out) {
  if (!out || max_worlds <= 0 || !(dt > 0.0f) || velocity_iterations < 0 || position_iterations < 0)
    return B2G_E_INVALID_ARG;
  b2g_server* s = new b2g_server();
  // the budget governs admission (per-body estimate); the batch itself gets no hard cap, since
  // its fixed scratch (sort temporaries, counters) does not scale with the admitted bodies
  int st = b2g_batch_create(device, 0, &s->batch);
  if (st != B2G_OK) {
    delete s;
    return st;
  }
  b2g_batch_set_graphs(s->batch, 0);  // the layout changes on most ticks; launch eagerly
  s->max_worlds = max_worlds;
  s->dt = dt;
  s->vi = velocity_iterations;
  s->pi = position_iterations;
  s->budget = budget_bytes;
  *out = s;
  return B2G_OK;
}

B2G_API int b2g_server_destroy(b2g_server* s) {
  if (!s) return B2G_E_INVALID_ARG;
  b2g_batch_destroy(s->batch);
  delete s;
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

// Sum of x, y, angle and |v| over the world's bodies, accumulated in creation order.
static int world_checksum(b2g_server* s, int world, float* out4) {
  int32_t nb = 0;
  int st = b2g_world_sizes(s->batch, world, &nb, nullptr, nullptr, nullptr);
  if (st != B2G_OK) return st;
  std::vector<b2g_body> bodies(nb);
  if (nb) {
    st = b2g_bodies_read(s->batch, world, 0, nb, bodies.data());
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

B2G_API int b2g_server_tick(b2g_server* s, int32_t* active, double* step_ms) {
  if (!s) return B2G_E_INVALID_ARG;
  // admit while slots and budget allow (FIFO; a request larger than the whole budget is rejected)
  while (!s->queue.empty() && (int32_t)s->active.size() < s->max_worlds) {
    Request r = s->queue.front();
    if (s->budget && r.bytes > s->budget) {
      s->queue.pop_front();
      ++s->rejected;
      finish(s, r, B2G_E_OUT_OF_MEMORY, nullptr);
      continue;
    }
    if (s->budget && s->in_use + r.bytes > s->budget) break;
    s->queue.pop_front();
    int32_t n = 0;
    float gx = 0, gy = -10;
    b2g_batch_world_params(r.seed, &n, &gx, &gy);
    int st = b2g_world_add(s->batch, gx, gy, &r.world);
    if (st == B2G_OK) st = b2g_world_set_flags(s->batch, r.world, 0, 1, 0, 1);
    if (st == B2G_OK) st = b2g_scene_build(s->batch, r.world, B2G_SCENE_BATCH_WORLD, r.seed, r.bodies, 0, 0, nullptr);
    if (st != B2G_OK) {
      ++s->rejected;
      if (r.world >= 0) b2g_world_retire(s->batch, r.world);
      finish(s, r, st, nullptr);
      continue;
    }
    r.admit = now_s();
    if (r.steps == 0) {  // nothing to step: summarise the initial state and retire at once
      float cs[4];
      st = world_checksum(s, r.world, cs);
      b2g_world_retire(s->batch, r.world);
      ++s->retired;
      ++s->completed;
      finish(s, r, st, st == B2G_OK ? cs : nullptr);
      continue;
    }
    s->in_use += r.bytes;
    s->active.push_back(r);
  }
  if (active) *active = (int32_t)s->active.size();
  if (step_ms) *step_ms = 0.0;
  if (!s->active.empty()) {
    // every active request has at least one step left (K = 0 requests finish at admission)
    double t0 = now_s();
    int st = b2g_step(s->batch, s->dt, s->vi, s->pi, nullptr);
    if (step_ms) *step_ms = (now_s() - t0) * 1e3;
    if (st != B2G_OK) return st;
  }
  // retire finished requests; a request whose world faulted (non-finite state) ends with that
  // status, the others run on unaffected
  std::vector<Request> still;
  for (Request& r : s->active) {
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
      int st = world_checksum(s, r.world, cs);
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
  // reclaim retired worlds in bulk once they outnumber the running ones
  if (s->retired >= 4 && s->retired >= (int32_t)s->active.size()) {
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

B2G_API int b2g_server_cancel(b2g_server* s, int64_t request_id) {
  if (!s) return B2G_E_INVALID_ARG;
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
    if (it->id != request_id) continue;
    Request r = *it;
    s->queue.erase(it);
    finish(s, r, B2G_E_CANCELLED, nullptr);
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
  if (active) *active = (int64_t)s->active.size();
  if (completed) *completed = s->completed;
  if (rejected) *rejected = s->rejected;
  if (hbm_bytes) *hbm_bytes = (int64_t)b2g::batch_allocated_bytes(s->batch);
  return B2G_OK;
}

}  // extern "C"
