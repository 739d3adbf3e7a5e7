// query.cu - batched world queries against the per-world LBVH of the last broadphase:
// b2World::QueryAABB (src/dynamics/b2_world.cpp:1193-1207, b2BroadPhase::Query
// include/box2d/b2_broad_phase.h:622-644) and b2World::RayCast with a closest-hit callback
// (b2_world.cpp:1209-1238, b2BroadPhase::RayCast b2_broad_phase.h:646-710). One thread per query;
// each traverses its world's subtree with the child boxes stored in the parent record.
#include "b2g_math.cuh"
#include "dev_common.cuh"
#include "kernels.h"

namespace b2g {

#define Q_LEAF 0x80000000u
#define Q_STACK 96

static inline unsigned qgrid(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

__device__ __forceinline__ AABB box_of(float4 b) {
  AABB r;
  r.lo = mk(b.x, b.y);
  r.hi = mk(b.z, b.w);
  return r;
}

// Calls leaf(f, box) for every fixture of world w whose tree box passes `keep_node` (applied to
// internal and leaf boxes alike, as the reference's traversal does); a guard that trips raises
// the status word and ends the walk.
// A world of one fixture has that fixture's leaf as its root: the ray cast tests it like any node,
// while b2BroadPhase::QueryAABB reports a leaf root without testing it (test_leaf_root = false).
template <class KeepNode, class Leaf>
__device__ __forceinline__ void traverse_world(const KernelArgs& a, int w, bool test_leaf_root, KeepNode keep_node,
                                               Leaf leaf) {
  const int root = a.wroot[w];
  if (root == -1) return;  // no fixtures (a leaf root has the top bit set, so it is negative too)
  if (root & Q_LEAF) {
    int li = root & ~Q_LEAF;
    float4 b = a.laabb[li];
    if (!test_leaf_root || keep_node(b)) leaf(a.mval_sorted[li], b);
    return;
  }
  if (!keep_node(a.naabb[root])) return;
  int stack[Q_STACK];
  int sp = 0;
  stack[sp++] = root;
  int visits = 0;
  const int maxVisits = 2 * a.wb[w].w + 8;
  while (sp > 0) {
    if (++visits > maxVisits) {
      raise_status(a.status, B2G_DEV_STACK_OVERFLOW);
      return;
    }
    int node = stack[--sp];
    int2 ch = a.nchild[node];
    int kids[2] = {ch.x, ch.y};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      float4 b = a.nrec[3 * (int64_t)node + q];
      if (!keep_node(b)) continue;
      int c = kids[q];
      if (c & Q_LEAF) {
        leaf(a.mval_sorted[c & ~Q_LEAF], b);
      } else if (sp < Q_STACK) {
        stack[sp++] = c;
      } else {
        raise_status(a.status, B2G_DEV_STACK_OVERFLOW);
      }
    }
  }
}

__device__ __forceinline__ bool query_world_ok(const KernelArgs& a, int w) {
  return w >= 0 && w < a.nw && !(a.wflags[w] & B2G_WF_RETIRED);
}

// Count (EMIT = false) or write (EMIT = true, ascending world-local fixture indices) the fixtures
// whose box overlaps the query box (b2TestOverlap, bounds inclusive).
template <bool EMIT>
__global__ void k_query_aabb(KernelArgs a, int n, const int* qw, const float4* qbox, int* counts, const int64_t* offs,
                             int* out) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int w = qw[q];
  int cnt = 0;
  int* seg = EMIT ? out + offs[q] : nullptr;
  if (query_world_ok(a, w)) {
    const int fo = a.wb[w].z;
    const AABB qb = box_of(qbox[q]);
    const int limit = EMIT ? counts[q] : 0;
    traverse_world(
        a, w, false, [&](float4 b) { return overlap(box_of(b), qb); },
        [&](int f, float4) {
          if (EMIT && cnt < limit) seg[cnt] = f - fo;
          ++cnt;
        });
  }
  if (!EMIT) {
    counts[q] = cnt;
    return;
  }
  for (int x = 1; x < cnt; ++x) {
    int v = seg[x];
    int y = x - 1;
    while (y >= 0 && seg[y] > v) {
      seg[y + 1] = seg[y];
      --y;
    }
    seg[y + 1] = v;
  }
}

// Closest hit of each ray p1 -> p2: the callback returns the hit fraction, so later leaves are
// tested against the shortened segment; the result is the smallest fraction (ties: the lowest
// fixture index).
__global__ void k_raycast(KernelArgs a, int n, const int* qw, const float4* rays, b2g_ray_hit* out) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  b2g_ray_hit res;
  res.fixture = -1;
  res.point[0] = res.point[1] = res.normal[0] = res.normal[1] = 0.0f;
  res.fraction = 1.0f;
  int w = qw[q];
  float4 ry = rays[q];
  V2 p1 = mk(ry.x, ry.y), p2 = mk(ry.z, ry.w);
  V2 r = p2 - p1;
  if (query_world_ok(a, w) && normalize(r) > 0.0f) {
    const int fo = a.wb[w].z;
    V2 v = cross(1.0f, r);
    V2 absV = mk(fabs2(v.x), fabs2(v.y));
    float maxFraction = 1.0f;
    AABB segment = raySegmentBox(p1, p2, maxFraction);
    int best = -1;
    RayHit bestHit;
    bestHit.fraction = 0.0f;
    bestHit.normal = mk(0.0f, 0.0f);
    traverse_world(
        a, w, true, [&](float4 b) { return !rayPrunes(box_of(b), segment, p1, v, absV); },
        [&](int f, float4) {
          const b2g_shape& sh = a.shape[f];
          float4 t = a.xf[a.fbody[f]];
          Xf xf;
          xf.p = mk(t.x, t.y);
          xf.q.s = t.z;
          xf.q.c = t.w;
          RayHit h;
          if (!rayShape(sh, xf, p1, p2, maxFraction, &h)) return;
          if (best >= 0 && h.fraction == bestHit.fraction && f > best) return;
          best = f;
          bestHit = h;
          maxFraction = h.fraction;
          segment = raySegmentBox(p1, p2, maxFraction);
        });
    if (best >= 0) {
      float fr = bestHit.fraction;
      V2 point = (1.0f - fr) * p1 + fr * p2;
      res.fixture = best - fo;
      res.point[0] = point.x;
      res.point[1] = point.y;
      res.normal[0] = bestHit.normal.x;
      res.normal[1] = bestHit.normal.y;
      res.fraction = fr;
    }
  }
  out[q] = res;
}

void launch_query_count(const KernelArgs& a, int n, const int* qw, const float4* qbox, int* counts, cudaStream_t s) {
  if (n > 0) k_query_aabb<false><<<qgrid(n, 128), 128, 0, s>>>(a, n, qw, qbox, counts, nullptr, nullptr);
}
void launch_query_emit(const KernelArgs& a, int n, const int* qw, const float4* qbox, int* counts, const int64_t* offs,
                       int* out, cudaStream_t s) {
  if (n > 0) k_query_aabb<true><<<qgrid(n, 128), 128, 0, s>>>(a, n, qw, qbox, counts, offs, out);
}
void launch_raycast(const KernelArgs& a, int n, const int* qw, const float4* rays, b2g_ray_hit* out, cudaStream_t s) {
  if (n > 0) k_raycast<<<qgrid(n, 128), 128, 0, s>>>(a, n, qw, rays, out);
}

}  // namespace b2g
