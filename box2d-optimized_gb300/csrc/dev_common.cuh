// dev_common.cuh - device helpers shared by the Step kernels.
#pragma once

#include "engine.h"
#include "kernels.h"

namespace b2g {

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
