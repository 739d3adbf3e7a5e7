// dev_common.cuh - device helpers shared by the Step kernels.
#pragma once

#include "engine.h"
#include "kernels.h"

namespace b2g {

// Manifold records are 64 bytes at 64-byte aligned positions in the device contact arrays:
// move them as four 16-byte words instead of sixteen 4-byte fields.
static_assert(sizeof(b2g_manifold) == 64, "manifold record size");
__device__ __forceinline__ b2g_manifold ld_manifold(const b2g_manifold* p) {
  const int4* q = reinterpret_cast<const int4*>(p);
  int4 t[4] = {q[0], q[1], q[2], q[3]};
  b2g_manifold m;
  memcpy(&m, t, sizeof(m));
  return m;
}
__device__ __forceinline__ void st_manifold(b2g_manifold* p, const b2g_manifold& m) {
  int4 t[4];
  memcpy(t, &m, sizeof(m));
  int4* q = reinterpret_cast<int4*>(p);
  q[0] = t[0]; q[1] = t[1]; q[2] = t[2]; q[3] = t[3];
}
__device__ __forceinline__ void copy_manifold(b2g_manifold* dst, const b2g_manifold* src) {
  const int4* s = reinterpret_cast<const int4*>(src);
  int4* d = reinterpret_cast<int4*>(dst);
  int4 t0 = s[0], t1 = s[1], t2 = s[2], t3 = s[3];
  d[0] = t0; d[1] = t1; d[2] = t2; d[3] = t3;
}

__device__ __forceinline__ void raise_status(unsigned int* status, unsigned int bit) { atomicOr(status, bit); }

// Appends one listener event; events past the buffer capacity are counted but dropped.
__device__ __forceinline__ void record_event(const KernelArgs& a, int kind, int world, int fa, int fb, int pc,
                                             const float* ni, const float* ti, const b2g_manifold* old) {
  unsigned long long slot = atomicAdd(&a.counters[1], 1ull);
  if ((int64_t)slot >= a.event_cap) return;
  EventDev& e = a.events[slot];
  e.kind = kind;
  e.world = world;
  e.fixtureA = fa;
  e.fixtureB = fb;
  e.pointCount = pc;
  e.normalImpulses[0] = ni ? ni[0] : 0.0f;
  e.normalImpulses[1] = ni ? ni[1] : 0.0f;
  e.tangentImpulses[0] = ti ? ti[0] : 0.0f;
  e.tangentImpulses[1] = ti ? ti[1] : 0.0f;
  if (old) e.old = *old;
  else memset(&e.old, 0, sizeof(e.old));
}

}  // namespace b2g
