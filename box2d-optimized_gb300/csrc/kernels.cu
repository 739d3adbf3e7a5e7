// kernels.cu - the Step's device kernels over a packed batch of worlds.
//
//   k_collide      narrowphase + contact update for every contact of every active world
//                  (b2ContactManager::Collide / b2Contact::Update, src/dynamics/b2_contact_manager.cpp:66-116,
//                  src/dynamics/b2_contact.cpp:126-210)
//   (the island solver, one CTA per world, is in solve.cu)
//   broadphase     fixture AABBs, 30-bit Morton codes, radix sort, Karras LBVH (one subtree per world),
//                  bottom-up bounds, stack traversal emitting the sorted, filtered pair list, and the
//                  sorted diff of that list against the live contacts (b2BroadPhase::UpdateAndQuery +
//                  b2ContactManager::QueryCallback / RemoveDeadContacts).
//   k_solve_toi    continuous collision: b2World::SolveTOI for the worlds that run it, one warp per
//                  world (src/dynamics/b2_world.cpp:859-1106)
#include <cub/cub.cuh>
#include <cuda/atomic>

#include "b2g_math.cuh"
#include "engine.h"
#include "dev_common.cuh"
#include "kernels.h"
#include "solver_dev.cuh"
#include "toi.cuh"

namespace b2g {

#define LEAF_BIT 0x80000000u
#define FULL_MASK 0xffffffffu

__device__ __forceinline__ Xf ldXf(const float4* xf, int i) {
  float4 t = xf[i];
  Xf x;
  x.p = mk(t.x, t.y);
  x.q.s = t.z;
  x.q.c = t.w;
  return x;
}

// ================================================================================ narrowphase
#define B2G_CONTACT_CLOSURE 0x40000000u  // scratch: updated by the wake closure of this step

// A sensor contact is touching when the shapes overlap (b2TestOverlap); kept out of line so that
// its GJK state does not weigh on the registers of the manifold path.
__device__ __noinline__ bool sensor_overlap(const b2g_shape& A, Xf xfA, const b2g_shape& B, Xf xfB) {
  return testOverlap(A, xfA, B, xfB);
}

// b2Contact::Update for contact i: evaluate the manifold, carry impulses by feature id, set
// touching, record Begin/End/PreSolve when events are on. Returns whether touching changed on a
// non-sensor contact (which wakes both bodies, src/dynamics/b2_contact.cpp:183-188).
__device__ __forceinline__ bool update_contact(const KernelArgs& a, int64_t i, int w, int2 f, int ba, int bb,
                                               uint32_t extra_flags, bool sensor) {
  uint32_t flags = a.cflags[i];
  bool wasTouching = (flags & B2G_CONTACT_TOUCHING) != 0;
  flags |= B2G_CONTACT_ENABLED | extra_flags;
  b2g_manifold old = ld_manifold(&a.cman[i]);
  bool touching = false;
  b2g_manifold nm;
  if (sensor) {  // no manifold: touching is the shapes' overlap (b2_contact.cpp:145-152)
    nm = old;
    nm.point_count = 0;
    touching = sensor_overlap(a.shape[f.x], ldXf(a.xf, ba), a.shape[f.y], ldXf(a.xf, bb));
  } else {
    const b2g_shape& sA = a.shape[f.x];
    const b2g_shape& sB = a.shape[f.y];
    Xf xfA = ldXf(a.xf, ba);
    Xf xfB = ldXf(a.xf, bb);
    Man m;
    evaluate(&m, sA, xfA, sB, xfB);
    touching = m.pointCount > 0;
    nm.type = m.type;
    nm.point_count = m.pointCount;
    nm.local_normal[0] = m.localNormal.x; nm.local_normal[1] = m.localNormal.y;
    nm.local_point[0] = m.localPoint.x; nm.local_point[1] = m.localPoint.y;
    for (int j = 0; j < 2; ++j) {
      nm.points[j].local_point[0] = m.lp[j].x;
      nm.points[j].local_point[1] = m.lp[j].y;
      nm.points[j].id = m.id[j];
      nm.points[j].normal_impulse = 0.0f;
      nm.points[j].tangent_impulse = 0.0f;
    }
    for (int j = 0; j < m.pointCount; ++j) {
      for (int k = 0; k < old.point_count; ++k) {
        if (old.points[k].id == nm.points[j].id) {
          nm.points[j].normal_impulse = old.points[k].normal_impulse;
          nm.points[j].tangent_impulse = old.points[k].tangent_impulse;
          break;
        }
      }
    }
  }
  if (touching) flags |= B2G_CONTACT_TOUCHING;
  else flags &= ~B2G_CONTACT_TOUCHING;
  st_manifold(&a.cman[i], nm);
  a.cflags[i] = flags;
  if (a.events_on) {
    int fo = a.wb[w].z;
    if (!wasTouching && touching) record_event(a, B2G_EVENT_BEGIN, w, f.x - fo, f.y - fo, 0, 0, 0, 0);
    if (wasTouching && !touching) record_event(a, B2G_EVENT_END, w, f.x - fo, f.y - fo, 0, 0, 0, 0);
    if (!sensor && touching) record_event(a, B2G_EVENT_PRESOLVE, w, f.x - fo, f.y - fo, 0, 0, 0, &old);
  }
  return !sensor && touching != wasTouching;
}

// Marks a non-static body woken in this step's narrowphase; returns whether the mark is new.
__device__ __forceinline__ bool mark_wake(const KernelArgs& a, int b) {
  if (a.btype[b] == B2G_STATIC || a.bwake[b]) return false;
  a.bwake[b] = 1;
  return true;
}

// b2ContactManager::Collide (src/dynamics/b2_contact_manager.cpp:66-116) over every contact of
// every active world. In sleep-mode worlds a contact is updated only when one of its bodies is
// awake (static bodies never are); wakes are marked, not applied, so every contact of this pass
// sees the awake flags the step started with. Sensor contacts go through a pass of their own
// (SENSORS = true, launched only when the layout has sensors), which keeps the overlap test's
// state out of the manifold pass's registers. Four 256-thread blocks per SM (64 registers): the
// pass waits on its shape and manifold loads, and the extra warps hide more of that than the few
// spilled registers cost (against 128-thread blocks at 75 registers: -1.5% on the bench's short
// window, the settled step unchanged; measured on the same worlds).
template <bool SENSORS>
__global__ void __launch_bounds__(256, 4) k_collide(KernelArgs a) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)a.counters[B2G_CNT_CONTACTS]) return;
  int2 f = a.cfix[i];
  // without sensor fixtures in the layout every contact is the manifold pass's
  if ((SENSORS || a.any_sensor) && (a.fsensor[f.x] || a.fsensor[f.y]) != SENSORS) return;
  int w = a.fworld[f.x];
  const int wf = a.wflags[w];
  if ((wf & B2G_WF_ACTIVE) == 0) return;
  const int ba = a.fbody[f.x], bb = a.fbody[f.y];
  const bool sleepMode = (wf & B2G_WF_SLEEPMODE) != 0;
  if (sleepMode && !((a.bstate[ba].x | a.bstate[bb].x) & B2G_BS_AWAKE)) return;
  if (update_contact(a, i, w, f, ba, bb, 0u, SENSORS)) {
    a.isl_dirty[w] = 1;  // a solid contact began or stopped touching (kept for any later sleep mode)
    if (sleepMode) {
      mark_wake(a, ba);
      mark_wake(a, bb);
    }
  }
}

// The wake closure of a sleep-mode world (one CTA per world): a contact whose bodies were both
// asleep at the start of the step is updated once one of them has been woken by another
// contact's touching change in this step, and may wake further bodies, until nothing changes.
// The reference updates its contacts in one sequential pass in which a wake takes effect for the
// contacts after it; the closure gives that result for every order in which a waking contact
// precedes the contacts it wakes (the reference keeps its newest contacts first), and it does not
// depend on the order of the contact list.
__global__ void k_collide_closure(KernelArgs a) {
  const int w = blockIdx.x;
  const int wf = a.wflags[w];
  if (!(wf & B2G_WF_ACTIVE) || !(wf & B2G_WF_SLEEPMODE)) return;
  // a contact joins only through a body that slept at the start of the step and has been woken
  // since: nothing to do unless the world has one
  const int4 wb = a.wb[w];
  int trigger = 0;
  for (int i = threadIdx.x; i < wb.y && !trigger; i += blockDim.x)
    trigger = a.bwake[wb.x + i] && !(a.bstate[wb.x + i].x & B2G_BS_AWAKE);
  if (!__syncthreads_or(trigger)) return;
  const int2 wc = a.wc[w];
  const int c0 = wc.x, n = wc.y;
  for (int round = 0; round <= n; ++round) {
    int changed = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      const int64_t i = c0 + k;
      if (a.cflags[i] & B2G_CONTACT_CLOSURE) continue;
      const int2 f = a.cfix[i];
      const int ba = a.fbody[f.x], bb = a.fbody[f.y];
      if ((a.bstate[ba].x | a.bstate[bb].x) & B2G_BS_AWAKE) continue;  // updated by k_collide
      if (!a.bwake[ba] && !a.bwake[bb]) continue;
      if (update_contact(a, i, w, f, ba, bb, B2G_CONTACT_CLOSURE, a.fsensor[f.x] || a.fsensor[f.y])) {
        if (mark_wake(a, ba)) changed = 1;
        if (mark_wake(a, bb)) changed = 1;
        a.isl_dirty[w] = 1;
      }
    }
    if (!__syncthreads_or(changed)) break;
  }
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int64_t i = c0 + k;
    const uint32_t fl = a.cflags[i];
    if (fl & B2G_CONTACT_CLOSURE) a.cflags[i] = fl & ~B2G_CONTACT_CLOSURE;
  }
}

__global__ void k_clear_forces(KernelArgs a, int nbodies) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbodies) return;
  int w = a.bworld[i];
  int wf = a.wflags[w];
  if ((wf & B2G_WF_ACTIVE) && (wf & B2G_WF_CLEAR_FORCES)) a.force[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if ((wf & B2G_WF_SLEEPMODE) && a.bwake[i]) {  // wakes of a step without a solve (dt = 0)
    a.bwake[i] = 0;
    if (a.btype[i] != B2G_STATIC) a.bstate[i] = make_int2(a.bstate[i].x | B2G_BS_AWAKE, 0);
  }
}

// ================================================================================ broadphase
// Fixture AABBs, and the packed attributes the pair filter reads for every candidate partner:
// (body, group index, category | mask << 16, shape type | body type << 8).
// The attributes change only with the layout, which rebuilds every tree: ATTR is set for the
// broadphases that build trees and clear for refits.
template <bool ATTR>
__global__ void k_aabb(KernelArgs a, int n) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  int i = a.bp_f0 + idx;
  int body = a.fbody[i];
  const b2g_shape& sh = a.shape[i];
  AABB bb = shapeAABB(sh, ldXf(a.xf, body));
  a.aabb[i] = make_float4(bb.lo.x, bb.lo.y, bb.hi.x, bb.hi.y);
  if (ATTR) a.fattr[i] = make_int4(body, a.fgroup[i], (int)a.ffilter[i], sh.type | (a.btype[body] << 8));
}

// Per-world bounds of AABB centres (lower + upper, the reference's GetCenter2) for Morton codes.
__global__ void k_world_bounds(KernelArgs a) {
  int w = a.bp_w0 + blockIdx.x;
  int4 wb = a.wb[w];
  float mnx = B2G_MAX_FLOAT, mny = B2G_MAX_FLOAT, mxx = -B2G_MAX_FLOAT, mxy = -B2G_MAX_FLOAT;
  for (int i = threadIdx.x; i < wb.w; i += blockDim.x) {
    float4 bb = a.aabb[wb.z + i];
    float cx = bb.x + bb.z, cy = bb.y + bb.w;
    mnx = fminf(mnx, cx); mny = fminf(mny, cy); mxx = fmaxf(mxx, cx); mxy = fmaxf(mxy, cy);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mnx = fminf(mnx, __shfl_xor_sync(FULL_MASK, mnx, o));
    mny = fminf(mny, __shfl_xor_sync(FULL_MASK, mny, o));
    mxx = fmaxf(mxx, __shfl_xor_sync(FULL_MASK, mxx, o));
    mxy = fmaxf(mxy, __shfl_xor_sync(FULL_MASK, mxy, o));
  }
  __shared__ float s[4][32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { s[0][wid] = mnx; s[1][wid] = mny; s[2][wid] = mxx; s[3][wid] = mxy; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int nw = (blockDim.x + 31) / 32;
    for (int k = 1; k < nw; ++k) {
      mnx = fminf(mnx, s[0][k]); mny = fminf(mny, s[1][k]); mxx = fmaxf(mxx, s[2][k]); mxy = fmaxf(mxy, s[3][k]);
    }
    a.wbounds[w] = make_float4(mnx, mny, mxx, mxy);
  }
}

__device__ __forceinline__ uint32_t expand_bits15(uint32_t v) {
  v &= 0x7fffu;
  v = (v | (v << 8)) & 0x00ff00ffu;
  v = (v | (v << 4)) & 0x0f0f0f0fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}

// 30-bit Morton code of the AABB centre normalised to its world's bounds; sort key
// world << 32 | code so that each world's fixtures form one contiguous sorted range.
__global__ void k_morton(KernelArgs a, int n) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  int i = a.bp_f0 + idx;
  int w = a.fworld[i];
  float4 wbnd = a.wbounds[w];
  float4 bb = a.aabb[i];
  float cx = bb.x + bb.z, cy = bb.y + bb.w;
  float ex = fmaxf(wbnd.z - wbnd.x, 1e-30f), ey = fmaxf(wbnd.w - wbnd.y, 1e-30f);
  float ux = fminf(fmaxf((cx - wbnd.x) / ex, 0.0f), 1.0f);
  float uy = fminf(fmaxf((cy - wbnd.y) / ey, 0.0f), 1.0f);
  uint32_t qx = (uint32_t)fminf(ux * 32768.0f, 32767.0f);
  uint32_t qy = (uint32_t)fminf(uy * 32768.0f, 32767.0f);
  uint32_t code = (expand_bits15(qx) << 1) | expand_bits15(qy);
  a.mkey[i] = ((uint64_t)(uint32_t)w << 32) | code;
  a.mval[i] = i;
}

__device__ __forceinline__ int lbvh_delta(const uint64_t* k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  uint64_t x = k[i], y = k[j];
  if (x == y) return 64 + __clz((unsigned)(i ^ j));
  return __clzll((long long)(x ^ y));
}

// Karras (2012) binary radix tree: internal node i covers a range of sorted leaves; its split is
// the highest differing bit. The node whose range is exactly a world's fixtures is that world's root.
__global__ void k_lbvh_internal(KernelArgs a, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int f0 = a.bp_f0;  // the tree is built over sorted leaves [f0, f0 + n); ids are global
  const uint64_t* k = a.mkey_sorted + f0;
  int d = (lbvh_delta(k, n, i, i + 1) - lbvh_delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = lbvh_delta(k, n, i, i - d);
  int lmax = 2;
  while (lbvh_delta(k, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (lbvh_delta(k, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = lbvh_delta(k, n, i, j);
  int s = 0;
  int t = l;
  do {
    t = (t + 1) >> 1;
    if (lbvh_delta(k, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  int gamma = i + s * d + min(d, 0);
  int lo = min(i, j), hi = max(i, j);
  const int gi = f0 + i, gg = f0 + gamma;
  int left = (lo == gamma) ? (int)(gg | LEAF_BIT) : gg;
  int right = (hi == gamma + 1) ? (int)((gg + 1) | LEAF_BIT) : gg + 1;
  a.nchild[gi] = make_int2(left, right);
  a.nrange[gi] = make_int2(f0 + lo, f0 + hi);
  if (lo == gamma) a.lparent[gg] = gi; else a.nparent[gg] = gi;
  if (hi == gamma + 1) a.lparent[gg + 1] = gi; else a.nparent[gg + 1] = gi;
  int w = (int)(k[lo] >> 32);
  if ((int)(k[hi] >> 32) == w) {
    int4 wb = a.wb[w];
    if (f0 + lo == wb.z && f0 + hi == wb.z + wb.w - 1) a.wroot[w] = gi;
  }
}

// Sorted-leaf attributes: x fixture, y body, z group << 16 | shape type | body type << 8, w filter
// (category | mask << 16), from the fixture's packed attributes (k_aabb). The pair search reads
// a leaf's fixture and filter data from its sorted position, with no indirection.
__device__ __forceinline__ int4 leaf_attr(int f, int4 fa) {
  return make_int4(f, fa.x, (int)(((uint32_t)fa.y << 16) | ((uint32_t)fa.w & 0xffffu)), fa.z);
}
__device__ __forceinline__ bool leaf_static(int4 la) { return ((la.z >> 8) & 0xff) == B2G_STATIC; }

// A node's or leaf's meta: the last sorted leaf of its range, with the top bit set when the
// range holds a static fixture.
__device__ __forceinline__ int leaf_meta(int j, int4 la) { return j | (leaf_static(la) ? (int)0x80000000 : 0); }

__global__ void k_lbvh_init(KernelArgs a, int n, int nw) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) {
    int i = a.bp_f0 + idx;
    const int f = a.mval_sorted[i];
    a.laabb[i] = a.aabb[f];
    a.lattr[i] = leaf_attr(f, a.fattr[f]);
    a.lparent[i] = -1;
    if (idx < n - 1) {
      a.nparent[i] = -1;
      a.nflag[i] = 0;
    }
  }
  if (idx < nw) {
    int w = a.bp_w0 + idx;
    int4 wb = a.wb[w];
    a.wroot[w] = wb.w == 1 ? (int)(wb.z | LEAF_BIT) : -1;
  }
}

// Refit of existing trees: leaf boxes from the fixtures' new AABBs in the trees' leaf order, node
// arrival counters cleared (internal nodes of every tree built over [0, n) lie in [0, n)). The
// sorted leaf attributes stay those of the build: they change only with the layout.
__global__ void k_lbvh_refit_init(KernelArgs a, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  a.laabb[i] = a.aabb[a.mval_sorted[i]];
  a.nflag[i] = 0;
}

// Node p's box, meta and record from its children (the second arrival at p does this).
__device__ __forceinline__ void lbvh_combine(const KernelArgs& a, int p, int2 ch) {
  float4 l, r;
  int ml, mr;
  if (ch.x & LEAF_BIT) {
    const int j = ch.x & ~LEAF_BIT;
    l = a.laabb[j];
    ml = leaf_meta(j, a.lattr[j]);
  } else {
    l = __ldcg(&a.naabb[ch.x]);
    ml = __ldcg(&a.nhi[ch.x]);
  }
  if (ch.y & LEAF_BIT) {
    const int j = ch.y & ~LEAF_BIT;
    r = a.laabb[j];
    mr = leaf_meta(j, a.lattr[j]);
  } else {
    r = __ldcg(&a.naabb[ch.y]);
    mr = __ldcg(&a.nhi[ch.y]);
  }
  float4 u = make_float4(fminf(l.x, r.x), fminf(l.y, r.y), fmaxf(l.z, r.z), fmaxf(l.w, r.w));
  __stcg(&a.naabb[p], u);
  // the range's last leaf is its right child's; the static bit is either child's
  __stcg(&a.nhi[p], (mr & 0x7fffffff) | ((ml | mr) & (int)0x80000000));
  float4* rec = a.nrec + 3 * (int64_t)p;
  rec[0] = l;
  rec[1] = r;
  rec[2] = make_float4(__int_as_float(ch.x), __int_as_float(ch.y), __int_as_float(ml), __int_as_float(mr));
}

// Bottom-up node bounds over the forest: a thread per leaf climbs towards its world's root and
// the second thread to reach a node combines its children (lbvh_combine). Walks stop at their
// world's root (the traversal never reads nodes above it). A block's leaves are a contiguous
// range of the sorted leaves, so the nodes whose leaf range lies inside it are reached only by
// its own threads: their arrival counters are block-scope acquire-release atomics in shared
// memory (fast, and the block's threads see each other's node boxes); the nodes above them have
// device-scope counters (nflag), through which the first arrival's child bounds and meta become
// visible to the second. A node's links and range are read before its arrival (they do not
// change during the pass).
constexpr int kBoundsThreads = 256;
__global__ void __launch_bounds__(kBoundsThreads) k_lbvh_bounds(KernelArgs a, int n) {
  __shared__ int arrivals[kBoundsThreads];
  const int B0 = a.bp_f0 + (int)blockIdx.x * kBoundsThreads;
  const int B1 = min(B0 + kBoundsThreads, a.bp_f0 + n);
  arrivals[threadIdx.x] = 0;
  __syncthreads();
  const int i = B0 + (int)threadIdx.x;
  if (i >= B1) return;
  const int w = a.fworld[a.mval_sorted[i]];
  const int root = a.wroot[w];
  if (root < 0 || (root & LEAF_BIT)) return;  // single-fixture world: the leaf is the root
  int p = a.lparent[i];
  int guard = 0;
  while (p >= 0) {
    if (++guard > 256) {  // deeper than any valid tree over 2^31 leaves: the tree is malformed
      raise_status(a.status, B2G_DEV_STACK_OVERFLOW);
      return;
    }
    const int2 ch = a.nchild[p];
    const int pp = a.nparent[p];
    const int2 rg = a.nrange[p];
    bool second;
    if (rg.x >= B0 && rg.y < B1) {  // p's index is one end of its range, so p - B0 is in the block
      cuda::atomic_ref<int, cuda::thread_scope_block> arrived(arrivals[p - B0]);
      second = arrived.fetch_add(1, cuda::memory_order_acq_rel) != 0;
    } else {
      cuda::atomic_ref<int, cuda::thread_scope_device> arrived(a.nflag[p]);
      second = arrived.fetch_add(1, cuda::memory_order_acq_rel) != 0;
    }
    if (!second) return;
    lbvh_combine(a, p, ch);
    if (p == root) return;
    p = pp;
  }
}

__device__ __forceinline__ bool aabb_overlap4(float4 a, float4 b) {
  return (a.z >= b.x) & (a.x <= b.z) & (a.w >= b.y) & (a.y <= b.w);
}

__device__ __forceinline__ bool nocollide_has(const uint64_t* keys, int n, uint64_t key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (keys[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo < n && keys[lo] == key;
}

// Would the pair of sorted leaves x, y (leaf_attr records) be reported? The filters of
// b2ContactManager::QueryCallback (src/dynamics/b2_contact_manager.cpp:136-188): same body,
// b2Body::ShouldCollide (a dynamic body, no collideConnected=false joint: `nocol` is the world's
// slice of the no-collide list, first and count), the default b2ContactFilter (group / category /
// mask, src/dynamics/b2_world_callbacks.cpp:28-39) and the collider table. Symmetric in x and y;
// which fixture emits the pair is decided by the caller.
__device__ __forceinline__ bool accept_leaves(const KernelArgs& a, int4 x, int4 y, int2 nocol) {
  if (x.y == y.y) return false;  // the same body (or the same fixture)
  const int tx = (x.z >> 8) & 0xff, ty = (y.z >> 8) & 0xff;
  if (tx != B2G_DYNAMIC && ty != B2G_DYNAMIC) return false;
  if (nocol.y > 0) {
    uint32_t lo = (uint32_t)min(x.y, y.y), hi = (uint32_t)max(x.y, y.y);
    if (nocollide_has(a.nocollide + nocol.x, nocol.y, ((uint64_t)lo << 32) | hi)) return false;
  }
  const int gx = x.z >> 16, gy = y.z >> 16;
  if (gx == gy && gx != 0) {
    if (!(gx > 0)) return false;
  } else {
    const uint32_t fx = (uint32_t)x.w, fy = (uint32_t)y.w;
    const uint32_t catX = fx & 0xffffu, maskX = fx >> 16, catY = fy & 0xffffu, maskY = fy >> 16;
    if (!((maskX & catY) != 0 && (catX & maskY) != 0)) return false;
  }
  const int sx = x.z & 0xff, sy = y.z & 0xff;
  return hasCollider(sx, sy) || hasCollider(sy, sx);
}

#define BP_STACK 96
#define BP_SLOTS 8  // partners recorded per fixture by the counting pass

// Every partner of emitter fixture f (non-static) over its world's subtree, for the emit pass of
// fixtures with more partners than slots: f emits (f, g) when g is static or g > f. Calls
// on_pair(g, j) for the j-th accepted partner (traversal order) and returns the number.
template <class OnPair>
__device__ __forceinline__ int traverse_pairs(const KernelArgs& a, int f, OnPair&& on_pair) {
  const int4 fa = a.fattr[f];
  int wf = a.fworld[f];
  int cnt = 0;
  if ((fa.w >> 8) == B2G_STATIC || (a.wflags[wf] & B2G_WF_RETIRED)) return 0;
  int root = a.wroot[wf];
  if (root < 0 || (root & LEAF_BIT)) return 0;
  const int4 la = leaf_attr(f, fa);
  float4 box = a.aabb[f];
  const int4 wjw = a.wj[wf];
  const int2 nocol = make_int2(wjw.z, wjw.w);
  int stack[BP_STACK];
  int sp = 0;
  stack[sp++] = root;
  int visits = 0;
  const int maxVisits = 2 * a.wb[wf].w + 8;  // each internal node of the world at most once
  while (sp > 0) {
    if (++visits > maxVisits) {
      raise_status(a.status, B2G_DEV_STACK_OVERFLOW);
      break;
    }
    int node = stack[--sp];
    const float4* rec = a.nrec + 3 * (int64_t)node;
    const float4 cbox[2] = {rec[0], rec[1]};
    const float4 m4 = rec[2];
    const int kids[2] = {__float_as_int(m4.x), __float_as_int(m4.y)};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      int c = kids[q];
      if (!aabb_overlap4(box, cbox[q])) continue;
      if (c & LEAF_BIT) {
        const int4 lg = a.lattr[c & ~LEAF_BIT];
        const int g = lg.x;
        if ((leaf_static(lg) || g > f) && accept_leaves(a, la, lg, nocol)) {
          on_pair(g, cnt);
          ++cnt;
        }
      } else {
        if (sp < BP_STACK) stack[sp++] = c;
        else raise_status(a.status, B2G_DEV_STACK_OVERFLOW);
      }
    }
  }
  return cnt;
}

// Counting pass over the sorted leaves (threads in Morton order, so that a warp's walks follow
// neighbouring tree paths). Each overlapping pair is found once: a pair of non-static fixtures by
// the leaf that sorts first (the walk skips every range that ends at or before its own leaf and
// holds no static fixture), a static pair by its non-static leaf (static leaves do not walk). The
// pair is counted for its emitter (the non-static fixture of a static pair, else the lower
// index), whose first BP_SLOTS partners are kept in arrival order (the emit pass sorts them).
// pcount holds zeros for the range beforehand.
__global__ void k_pairs_count(KernelArgs a, int n) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int i = a.bp_f0 + idx;
  const int4 la = a.lattr[i];
  if (leaf_static(la)) return;
  const int f = la.x;
  const int wf = a.fworld[f];
  if (a.wflags[wf] & B2G_WF_RETIRED) return;
  const int root = a.wroot[wf];
  if (root < 0 || (root & LEAF_BIT)) return;
  const float4 box = a.laabb[i];
  const int4 wjw = a.wj[wf];
  const int2 nocol = make_int2(wjw.z, wjw.w);
  int stack[BP_STACK];
  int sp = 0;
  stack[sp++] = root;
  int visits = 0;
  const int maxVisits = 2 * a.wb[wf].w + 8;  // each internal node of the world at most once
  while (sp > 0) {
    if (++visits > maxVisits) {
      raise_status(a.status, B2G_DEV_STACK_OVERFLOW);
      break;
    }
    const int node = stack[--sp];
    const float4* rec = a.nrec + 3 * (int64_t)node;
    const float4 cbox[2] = {rec[0], rec[1]};
    const float4 m4 = rec[2];
    const int kids[2] = {__float_as_int(m4.x), __float_as_int(m4.y)};
    const int meta[2] = {__float_as_int(m4.z), __float_as_int(m4.w)};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (meta[q] >= 0 && meta[q] <= i) continue;  // ends at or before this leaf, no static fixture
      if (!aabb_overlap4(box, cbox[q])) continue;
      const int c = kids[q];
      if (c & LEAF_BIT) {
        const int4 lg = a.lattr[c & ~LEAF_BIT];
        if (!accept_leaves(a, la, lg, nocol)) continue;
        const int g = lg.x;
        const bool fe = meta[q] < 0 || f < g;  // a leaf's meta is negative when it is static
        const int e = fe ? f : g, p = fe ? g : f;
        const int k = atomicAdd(&a.pcount[e], 1);
        if (k < BP_SLOTS) a.pslots[(int64_t)e * BP_SLOTS + k] = (uint32_t)p;
      } else {
        if (sp < BP_STACK) stack[sp++] = c;
        else raise_status(a.status, B2G_DEV_STACK_OVERFLOW);
      }
    }
  }
}

// Emit pass: each fixture's partners, ascending, as keys f << 32 | g at its scanned offset (the
// pair list comes out sorted). Fixtures with more partners than slots search again.
__global__ void k_pairs_emit(KernelArgs a, int n) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  int f = a.bp_f0 + idx;
  if ((int64_t)a.poff[a.nf] > a.ccap) return;  // overflow: the host grows the buffers and redoes this pass
  if (a.counters[B2G_CNT_OVERFLOW]) return;    // an earlier pair update of the step overflowed
  int64_t off = a.poff[f];
  int cnt = (int)(a.poff[f + 1] - off);
  if (cnt == 0) return;
  uint64_t* seg = a.pairs + off;
  const uint64_t hi = (uint64_t)(uint32_t)f << 32;
  if (cnt <= BP_SLOTS) {
    uint32_t v[BP_SLOTS];
    const uint32_t* slots = a.pslots + (int64_t)f * BP_SLOTS;
#pragma unroll
    for (int j = 0; j < BP_SLOTS; ++j) v[j] = j < cnt ? slots[j] : 0xffffffffu;
    // odd-even transposition sort, fully unrolled so that v stays in registers
#pragma unroll
    for (int r = 0; r < BP_SLOTS; ++r) {
#pragma unroll
      for (int j = r & 1; j + 1 < BP_SLOTS; j += 2) {
        uint32_t x = v[j], y = v[j + 1];
        v[j] = x < y ? x : y;
        v[j + 1] = x < y ? y : x;
      }
    }
#pragma unroll
    for (int j = 0; j < BP_SLOTS; ++j)
      if (j < cnt) seg[j] = hi | v[j];
    return;
  }
  int got = traverse_pairs(a, f, [&](int g, int j) {
    if (j < cnt) seg[j] = hi | (uint32_t)g;
  });
  if (got != cnt) raise_status(a.status, B2G_DEV_STACK_OVERFLOW);  // cannot happen: same tree, same test
  for (int x = 1; x < cnt; ++x) {
    uint64_t v = seg[x];
    int y = x - 1;
    while (y >= 0 && seg[y] > v) {
      seg[y + 1] = seg[y];
      --y;
    }
    seg[y + 1] = v;
  }
}

__global__ void k_world_contacts(KernelArgs a, int nw) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nw || a.counters[B2G_CNT_OVERFLOW]) return;
  int w = a.bp_w0 + idx;
  int4 wb = a.wb[w];
  int s = a.poff[wb.z], e = a.poff[wb.z + wb.w];
  a.wc[w] = make_int2(s, e - s);
}

__device__ __forceinline__ int64_t find_key(const uint64_t* keys, int64_t n, uint64_t key) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (keys[mid] < key) lo = mid + 1; else hi = mid;
  }
  return (lo < n && keys[lo] == key) ? lo : -1;
}

// A new contact for pair `key` at index k of contact buffer `dst`, like b2Contact's constructor
// (src/dynamics/b2_contact.cpp:96-122) in b2Contact::Create's orientation: fixture order by the
// collider table, mixed friction / restitution / threshold, enabled, empty manifold.
__device__ __forceinline__ void init_new_contact(const KernelArgs& a, int dst, int64_t k, uint64_t key) {
  a.ckeyB[dst][k] = key;
  int e = (int)(key >> 32), p = (int)(uint32_t)key;
  int fa, fb;
  if (hasCollider(a.shape[e].type, a.shape[p].type)) { fa = e; fb = p; }
  else { fa = p; fb = e; }
  float4 ma = a.fmat[fa], mb = a.fmat[fb];
  a.cfixB[dst][k] = make_int2(fa, fb);
  a.cflagsB[dst][k] = B2G_CONTACT_ENABLED;
  a.cmatB[dst][k] = make_float4(sqrtf(ma.x * mb.x), ma.y > mb.y ? ma.y : mb.y, ma.z < mb.z ? ma.z : mb.z, 0.0f);
  int4* m = reinterpret_cast<int4*>(&a.cmanB[dst][k]);
  m[0] = m[1] = m[2] = m[3] = make_int4(0, 0, 0, 0);
}

// New contact list = the new pair list; persisting contacts keep their orientation, flags,
// mixed material and manifold (impulses included); new ones are created as new contacts.
__global__ void k_contact_diff(KernelArgs a, int src, int dst) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t nnew = a.poff[a.nf];
  int64_t nold = (int64_t)a.counters[B2G_CNT_CONTACTS];
  if (nnew > a.ccap || k >= nnew || a.counters[B2G_CNT_OVERFLOW]) return;
  uint64_t key = a.pairs[k];
  int64_t o;
  if (a.poff_old) {  // the live list's entries of this emitter
    int e = (int)(key >> 32);
    int64_t lo = a.poff_old[e], hi = a.poff_old[e + 1];
    int64_t r = find_key(a.ckeyB[src] + lo, hi - lo, key);
    o = r >= 0 ? lo + r : -1;
  } else {
    o = find_key(a.ckeyB[src], nold, key);
  }
  if (o >= 0) {
    a.ckeyB[dst][k] = key;
    a.cfixB[dst][k] = a.cfixB[src][o];
    a.cflagsB[dst][k] = a.cflagsB[src][o];
    a.cmatB[dst][k] = a.cmatB[src][o];
    copy_manifold(&a.cmanB[dst][k], &a.cmanB[src][o]);
  } else {
    init_new_contact(a, dst, k, key);
    a.isl_dirty[a.fworld[(int)(key >> 32)]] = 1;  // a body may have gained its first contact
  }
}

// ---- broadphase of appended worlds only (fixtures [bp_f0, nf), worlds [bp_w0, nw)): their keys
// sort after every live contact, so their pairs are appended to the live list of buffer `dst`.
// poff holds the appended pairs' offsets relative to the first appended fixture.
__global__ void k_tail_append(KernelArgs a, int dst) {
  const int64_t total = (int64_t)a.poff[a.nf];
  const int64_t nc0 = (int64_t)a.counters[B2G_CNT_CONTACTS];
  if (nc0 + total > a.ccap) return;  // overflow: the host grows the buffers and redoes this pass
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x)
    init_new_contact(a, dst, nc0 + k, a.pairs[k]);
}

// Contact ranges of the appended worlds and, when the live list's per-fixture offsets are kept,
// their entries for the appended fixtures.
__global__ void k_tail_ranges(KernelArgs a, int nw, int nfix, int* poff_live) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t total = (int64_t)a.poff[a.nf];
  const int nc0 = (int)a.counters[B2G_CNT_CONTACTS];
  if (nc0 + total > a.ccap) return;
  if (idx < nw) {
    int4 wb = a.wb[a.bp_w0 + idx];
    int s = a.poff[wb.z], e = a.poff[wb.z + wb.w];
    a.wc[a.bp_w0 + idx] = make_int2(nc0 + s, e - s);
  }
  if (poff_live && idx <= nfix) poff_live[a.bp_f0 + idx] = nc0 + a.poff[a.bp_f0 + idx];
}

__global__ void k_tail_commit(KernelArgs a) {
  unsigned long long total = (unsigned long long)a.poff[a.nf];
  unsigned long long nc = a.counters[B2G_CNT_CONTACTS] + total;
  if ((int64_t)nc > a.ccap) a.counters[B2G_CNT_OVERFLOW] = nc;
  else a.counters[B2G_CNT_CONTACTS] = nc;
}

// Contacts that disappeared: EndContact if they were touching (b2ContactManager::Destroy,
// src/dynamics/b2_contact_manager.cpp:48-61), and in sleep-mode worlds a destroyed contact with
// manifold points wakes both bodies (b2Contact::Destroy, src/dynamics/b2_contact.cpp:80-91).
__global__ void k_contact_dead(KernelArgs a, int src) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t nnew = a.poff[a.nf];
  int64_t nold = (int64_t)a.counters[B2G_CNT_CONTACTS];
  if (nnew > a.ccap || k >= nold || a.counters[B2G_CNT_OVERFLOW]) return;
  uint64_t key = a.ckeyB[src][k];
  int e = (int)(key >> 32);
  int64_t lo = a.poff[e];
  if (find_key(a.pairs + lo, (int64_t)a.poff[e + 1] - lo, key) >= 0) return;
  a.isl_dirty[a.fworld[e]] = 1;  // a body may have lost its last contact, or a solid edge
  if ((a.cflagsB[src][k] & B2G_CONTACT_TOUCHING) == 0) return;
  int2 f = a.cfixB[src][k];
  int w = a.fworld[f.x];
  if (a.wflags[w] & B2G_WF_RETIRED) return;
  if (a.events_on) {
    int fo = a.wb[w].z;
    record_event(a, B2G_EVENT_END, w, f.x - fo, f.y - fo, 0, 0, 0, 0);
  }
  if ((a.wflags[w] & B2G_WF_SLEEPMODE) && !a.fsensor[f.x] && !a.fsensor[f.y]) {
    const int bodies[2] = {a.fbody[f.x], a.fbody[f.y]};
    for (int q = 0; q < 2; ++q)
      if (a.btype[bodies[q]] != B2G_STATIC) a.bstate[bodies[q]] = make_int2(a.bstate[bodies[q]].x | B2G_BS_AWAKE, 0);
  }
}

// The new list becomes the live one, or the needed capacity is recorded for the host.
__global__ void k_commit_contacts(KernelArgs a) {
  if (a.counters[B2G_CNT_OVERFLOW]) return;  // kept from an earlier pair update of the step
  unsigned long long total = (unsigned long long)a.poff[a.nf];
  if ((int64_t)total > a.ccap) a.counters[B2G_CNT_OVERFLOW] = total;
  else a.counters[B2G_CNT_CONTACTS] = total;
}

// ================================================================================ continuous collision
// b2World::SolveTOI (src/dynamics/b2_world.cpp:859-1106) for one world per warp, after the
// step's pair update: the times of impact of the world's contacts (b2Contact::CalculateTOI,
// src/dynamics/b2_contact.cpp:212-280) in a min-heap (b2TOIMinHeap, b2_world.cpp:671-850); the
// earliest impact advances its two bodies (b2Body::Advance), gathers the static, kinematic and
// bullet bodies touching them into a small island that b2Island::SolveTOI
// (src/dynamics/b2_island.cpp:486-619) solves over the rest of the step, moves the island's
// fixture boxes, refreshes the TOIs of their contacts and queries the boxes for new contacts,
// until no impact is left before the step's end. The lanes compute the first TOIs of all the
// world's contacts; lane 0 runs the event loop. The heap is built in contact order, a body's
// contacts are visited in contact order, and a moved fixture meets its partners in fixture order.
// Contacts made inside the loop live in shared memory (at most TOI_MADE per world and step) and
// are made again by the pair update that follows the kernel.
#define TOI_MADE 32
#define TOI_BODIES 64    // 2 * b2_maxTOIContacts
#define TOI_CONTACTS 32  // b2_maxTOIContacts
#define TOI_ISLAND 1u
#define TOI_PERSIST 2u

struct ToiMade {
  b2g_manifold man;
  float4 mat;
  int2 fix;
  uint32_t flags;
  int hpos;
  uint32_t fl;
};
struct ToiSmem {
  ToiMade made[TOI_MADE];
  float4 P[TOI_BODIES], V[TOI_BODIES];
  int ib[TOI_BODIES];
  int ic[TOI_CONTACTS];
};

// b2Contact::CalculateTOI (src/dynamics/b2_contact.cpp:212-280) of the contact between fixtures
// f.x and f.y with flags `cflags`: 1 unless both bodies are non-static (and awake in sleep-mode
// worlds) and one is a bullet or kinematic; the sweeps are first put on the same alpha0 (which
// advances the earlier one). Out of line, so that the TOI loop's state stays in registers.
__device__ __noinline__ float contactTOI(const KernelArgs& a, int2 f, uint32_t cflags, bool sleepMode) {
  if (a.fsensor[f.x] || a.fsensor[f.y] || !(cflags & B2G_CONTACT_ENABLED)) return 1.0f;
  const int A = a.fbody[f.x], B = a.fbody[f.y];
  const int tA = a.btype[A], tB = a.btype[B];
  const int sA = a.bstate[A].x, sB = a.bstate[B].x;
  const bool active = sleepMode ? ((sA & B2G_BS_AWAKE) && tA != B2G_STATIC && (sB & B2G_BS_AWAKE) && tB != B2G_STATIC)
                                : (tA != B2G_STATIC && tB != B2G_STATIC);
  if (!active) return 1.0f;
  const bool collideA = (sA & B2G_BS_BULLET) || tA != B2G_DYNAMIC;
  const bool collideB = (sB & B2G_BS_BULLET) || tB != B2G_DYNAMIC;
  if (!collideA && !collideB) return 1.0f;
  auto sweepOfBody = [&](int b) {
    float4 s = a.sweep0[b], p = a.pos[b];
    float2 l = a.lc[b];
    Sweep o;
    o.lc = mk(l.x, l.y);
    o.c0 = mk(s.x, s.y);
    o.c = mk(p.x, p.y);
    o.a0 = s.z;
    o.a = p.z;
    o.alpha0 = s.w;
    return o;
  };
  Sweep swA = sweepOfBody(A), swB = sweepOfBody(B);
  float alpha0 = swA.alpha0;
  if (swA.alpha0 < swB.alpha0) {
    alpha0 = swB.alpha0;
    sweepAdvance(swA, alpha0);
    a.sweep0[A] = make_float4(swA.c0.x, swA.c0.y, swA.a0, swA.alpha0);
  } else if (swB.alpha0 < swA.alpha0) {
    alpha0 = swA.alpha0;
    sweepAdvance(swB, alpha0);
    a.sweep0[B] = make_float4(swB.c0.x, swB.c0.y, swB.a0, swB.alpha0);
  }
  float t;
  const int state = timeOfImpact(a.shape[f.x], a.shape[f.y], swA, swB, 1.0f, &t);
  return state == B2G_TOI_TOUCHING ? fmin2(alpha0 + (1.0f - alpha0) * t, 1.0f) : 1.0f;
}

struct ToiWorld {
  const KernelArgs& a;
  ToiSmem& S;
  int w, c0, nc, nmade, b0, nb, f0, nf, fo;
  int4* heap;
  int hn;
  bool sleepMode;
  int2 nocol;
  int *boff, *blist, *foff, *flist;  // per-body contact / fixture lists (valid once `adj`)
  bool adj;
  VCDev* vcs;  // the island's contact constraints (global scratch: TOI_CONTACTS per world)

  __device__ ToiWorld(const KernelArgs& a_, ToiSmem& S_) : a(a_), S(S_) {}

  // Per-body lists of the live contacts and of the fixtures, each in ascending order: counts at
  // off[A + 1], prefix sums (off[A + 1] = end of A's list, off[nb + 1] = the total), then a
  // descending fill that moves off[A + 1] to the start of A's list: list A = [off[A + 1], off[A + 2]).
  __device__ void buildLists(int* off, int* list, int n, bool contacts) {
    for (int i = 0; i < nb + 2; ++i) off[i] = 0;
    for (int k = 0; k < n; ++k) {
      if (contacts) {
        const int2 f = fix(k);
        ++off[a.fbody[f.x] - b0 + 1];
        ++off[a.fbody[f.y] - b0 + 1];
      } else {
        ++off[a.fbody[f0 + k] - b0 + 1];
      }
    }
    for (int i = 1; i <= nb; ++i) off[i] += off[i - 1];
    off[nb + 1] = off[nb];
    for (int k = n - 1; k >= 0; --k) {
      if (contacts) {
        const int2 f = fix(k);
        list[--off[a.fbody[f.x] - b0 + 1]] = k;
        list[--off[a.fbody[f.y] - b0 + 1]] = k;
      } else {
        list[--off[a.fbody[f0 + k] - b0 + 1]] = k;
      }
    }
  }
  __device__ void ensureLists() {
    if (adj) return;
    buildLists(boff, blist, nc, true);
    buildLists(foff, flist, nf, false);
    adj = true;
  }
  // Calls fn(k) for body b's contacts in contact order (the live list's, then those made in the
  // loop) until fn returns false; returns whether it ran to the end.
  template <class F>
  __device__ bool forContacts(int b, F&& fn) {
    const int A = b - b0;
    for (int j = boff[A + 1]; j < boff[A + 2]; ++j)
      if (!fn(blist[j])) return false;
    for (int m = 0; m < nmade; ++m) {
      const int2 f = S.made[m].fix;
      if ((a.fbody[f.x] == b || a.fbody[f.y] == b) && !fn(nc + m)) return false;
    }
    return true;
  }

  // contact k of the world: its live slot below nc, else a contact made inside the loop
  __device__ int2 fix(int k) const { return k < nc ? a.cfix[c0 + k] : S.made[k - nc].fix; }
  __device__ uint32_t& flags(int k) { return k < nc ? a.cflags[c0 + k] : S.made[k - nc].flags; }
  __device__ b2g_manifold* man(int k) { return k < nc ? &a.cman[c0 + k] : &S.made[k - nc].man; }
  __device__ float4 mat(int k) const { return k < nc ? a.cmat[c0 + k] : S.made[k - nc].mat; }
  __device__ int& hpos(int k) { return k < nc ? a.toi_hpos[c0 + k] : S.made[k - nc].hpos; }
  __device__ uint32_t getFl(int k) const { return k < nc ? (uint32_t)a.toi_cfl[c0 + k] : S.made[k - nc].fl; }
  __device__ void setFl(int k, uint32_t v) {
    if (k < nc) a.toi_cfl[c0 + k] = (uint8_t)v;
    else S.made[k - nc].fl = v;
  }
  __device__ int count() const { return nc + nmade; }

  __device__ bool awake(int b) const { return (a.bstate[b].x & B2G_BS_AWAKE) != 0; }
  __device__ bool bullet(int b) const { return (a.bstate[b].x & B2G_BS_BULLET) != 0; }
  // SET_AWAKE_OR_NONE / b2Body::SetAwake(true): sleep-mode worlds only
  __device__ void wake(int b) {
    if (sleepMode && a.btype[b] != B2G_STATIC) a.bstate[b] = make_int2(a.bstate[b].x | B2G_BS_AWAKE, 0);
  }

  __device__ Sweep sweep(int b) const {
    float4 s = a.sweep0[b], p = a.pos[b];
    float2 l = a.lc[b];
    Sweep o;
    o.lc = mk(l.x, l.y);
    o.c0 = mk(s.x, s.y);
    o.c = mk(p.x, p.y);
    o.a0 = s.z;
    o.a = p.z;
    o.alpha0 = s.w;
    return o;
  }
  __device__ void advanceSweep(int b, float alpha) {
    Sweep s = sweep(b);
    sweepAdvance(s, alpha);
    a.sweep0[b] = make_float4(s.c0.x, s.c0.y, s.a0, s.alpha0);
  }
  // b2Body::SynchronizeTransform
  __device__ void syncXf(int b) {
    float4 p = a.pos[b];
    float2 l = a.lc[b];
    Rot q = rotOf(p.z);
    V2 o = mk(p.x, p.y) - mul(q, mk(l.x, l.y));
    a.xf[b] = make_float4(o.x, o.y, q.s, q.c);
  }
  // b2Body::Advance (include/box2d/b2_body.h:963-971)
  __device__ void advanceBody(int b, float alpha) {
    advanceSweep(b, alpha);
    float4 s = a.sweep0[b];
    a.pos[b] = make_float4(s.x, s.y, s.z, 0.0f);
    syncXf(b);
  }

  // b2Contact::CalculateTOI
  __device__ float calcTOI(int k) { return contactTOI(a, fix(k), flags(k), sleepMode); }

  // b2TOIMinHeap
  __device__ float key(int i) const { return __int_as_float(heap[i].x); }
  __device__ void swapNodes(int i, int j) {
    int4 x = heap[i], y = heap[j];
    hpos(x.z) = j;
    hpos(y.z) = i;
    heap[i] = y;
    heap[j] = x;
  }
  __device__ void down(int i) {
    for (;;) {
      int m = i, l = 2 * i + 1, r = 2 * i + 2;
      if (l < hn && key(l) < key(m)) m = l;
      if (r < hn && key(r) < key(m)) m = r;
      if (m == i) return;
      swapNodes(i, m);
      i = m;
    }
  }
  __device__ void up(int i) {
    while (i > 0 && key(i) < key((i - 1) / 2)) {
      swapNodes(i, (i - 1) / 2);
      i = (i - 1) / 2;
    }
  }
  __device__ void setKey(int i, float toi) {
    const bool u = toi < key(i), d = toi > key(i);
    heap[i].x = __float_as_int(toi);
    if (u) up(i);
    else if (d) down(i);
  }
  __device__ void update(int k) {
    const int i = hpos(k);
    setKey(i, heap[i].y > 8 ? 1.0f : calcTOI(k));  // b2_maxSubSteps
  }
  __device__ void insert(int k) {
    const float toi = calcTOI(k);
    if (toi < 1.0f) {
      heap[hn] = make_int4(__float_as_int(toi), 0, k, 0);
      hpos(k) = hn;
      ++hn;
      up(hn - 1);
    }
  }

  // b2Contact::Update of a non-sensor contact at the bodies' current transforms; returns whether
  // touching changed (which wakes both bodies in sleep-mode worlds)
  __device__ bool updateContact(int k) {
    const int2 f = fix(k);
    uint32_t fl = flags(k);
    const bool wasTouching = (fl & B2G_CONTACT_TOUCHING) != 0;
    fl |= B2G_CONTACT_ENABLED;
    b2g_manifold* mp = man(k);
    const b2g_manifold old = *mp;
    const int A = a.fbody[f.x], B = a.fbody[f.y];
    Man m;
    evaluate(&m, a.shape[f.x], ldXf(a.xf, A), a.shape[f.y], ldXf(a.xf, B));
    const bool touching = m.pointCount > 0;
    b2g_manifold nm;
    nm.type = m.type;
    nm.point_count = m.pointCount;
    nm.local_normal[0] = m.localNormal.x; nm.local_normal[1] = m.localNormal.y;
    nm.local_point[0] = m.localPoint.x; nm.local_point[1] = m.localPoint.y;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      nm.points[j].local_point[0] = m.lp[j].x;
      nm.points[j].local_point[1] = m.lp[j].y;
      nm.points[j].id = m.id[j];
      nm.points[j].normal_impulse = 0.0f;
      nm.points[j].tangent_impulse = 0.0f;
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      if (j >= m.pointCount) break;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        if (q >= old.point_count) break;
        if (old.points[q].id == nm.points[j].id) {
          nm.points[j].normal_impulse = old.points[q].normal_impulse;
          nm.points[j].tangent_impulse = old.points[q].tangent_impulse;
          break;
        }
      }
    }
    *mp = nm;
    if (touching) fl |= B2G_CONTACT_TOUCHING;
    else fl &= ~B2G_CONTACT_TOUCHING;
    flags(k) = fl;
    if (a.events_on) {
      if (!wasTouching && touching) record_event(a, B2G_EVENT_BEGIN, w, f.x - fo, f.y - fo, 0, 0, 0, 0);
      if (wasTouching && !touching) record_event(a, B2G_EVENT_END, w, f.x - fo, f.y - fo, 0, 0, 0, 0);
      if (touching) record_event(a, B2G_EVENT_PRESOLVE, w, f.x - fo, f.y - fo, 0, 0, 0, &old);
    }
    if (touching != wasTouching) {
      a.isl_dirty[w] = 1;
      wake(A);
      wake(B);
      return true;
    }
    return false;
  }

  __device__ int islandIndex(int b, int nbI) const {
    for (int i = 0; i < nbI; ++i)
      if (S.ib[i] == b) return i;
    return 0;
  }

  // b2ContactSolver::SolveTOIPositionConstraints (src/dynamics/b2_contact_solver.cpp:790-878) for
  // one constraint over island positions P: only island bodies 0 and 1 (the impact's) move.
  __device__ float solveTOIPosition(const VCDev& vc) {
    float minSeparation = 0.0f;
    float mA = 0.0f, iA = 0.0f, mB = 0.0f, iB = 0.0f;
    if (vc.indexA == 0 || vc.indexA == 1) { mA = vc.invMassA; iA = vc.invIA; }
    if (vc.indexB == 0 || vc.indexB == 1) { mB = vc.invMassB; iB = vc.invIB; }
    V2 lcA = ld2(vc.localCenterA), lcB = ld2(vc.localCenterB);
    float4 pa = S.P[vc.indexA], pb = S.P[vc.indexB];
    V2 cA = mk(pa.x, pa.y), cB = mk(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    for (int j = 0; j < vc.pcPointCount; ++j) {
      Xf xfA, xfB;
      xfA.q = rotOf(aA);
      xfB.q = rotOf(aB);
      xfA.p = cA - mul(xfA.q, lcA);
      xfB.p = cB - mul(xfB.q, lcB);
      V2 normal, point;
      float separation;
      if (vc.type == B2G_MANIFOLD_CIRCLES) {
        V2 pointA = mul(xfA, ld2(vc.localPoint));
        V2 pointB = mul(xfB, ld2(vc.localPoints[0]));
        normal = pointB - pointA;
        normalize(normal);
        point = 0.5f * (pointA + pointB);
        separation = (dot(pointB - pointA, normal) - vc.radiusA) - vc.radiusB;
      } else if (vc.type == B2G_MANIFOLD_FACE_A) {
        normal = mul(xfA.q, ld2(vc.localNormal));
        V2 clipPoint = mul(xfB, ld2(vc.localPoints[j]));
        separation = (dot(clipPoint - mul(xfA, ld2(vc.localPoint)), normal) - vc.radiusA) - vc.radiusB;
        point = clipPoint;
      } else {
        normal = mul(xfB.q, ld2(vc.localNormal));
        V2 clipPoint = mul(xfA, ld2(vc.localPoints[j]));
        separation = (dot(clipPoint - mul(xfB, ld2(vc.localPoint)), normal) - vc.radiusA) - vc.radiusB;
        point = clipPoint;
        normal = -normal;
      }
      V2 rA = point - cA, rB = point - cB;
      minSeparation = fmin2(minSeparation, separation);
      float C = fclamp(0.75f * (separation + B2G_LINEAR_SLOP), -B2G_MAX_LINEAR_CORRECTION, 0.0f);  // b2_toiBaumgarte
      float rnA = cross(rA, normal), rnB = cross(rB, normal);
      float K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
      float impulse = K > 0.0f ? -C / K : 0.0f;
      V2 P = impulse * normal;
      subFrom(cA, mA * P);
      aA -= iA * cross(rA, P);
      addTo(cB, mB * P);
      aB += iB * cross(rB, P);
    }
    S.P[vc.indexA] = make_float4(cA.x, cA.y, aA, 0.0f);
    S.P[vc.indexB] = make_float4(cB.x, cB.y, aB, 0.0f);
    return minSeparation;
  }

  __device__ void prepare(int nbI, int ncI) {
    for (int j = 0; j < ncI; ++j) {
      const int k = S.ic[j];
      const int2 f = fix(k);
      const int A = a.fbody[f.x], B = a.fbody[f.y];
      const int ia = islandIndex(A, nbI), ib = islandIndex(B, nbI);
      prepareContact(vcs[j], *man(k), mat(k), a.frad[f.x], a.frad[f.y], ia, ib, a.massd[A], a.massd[B], a.lc[A],
                     a.lc[B], S.P[ia], S.V[ia], S.P[ib], S.V[ib], 1.0f, false, k);
    }
  }

  // b2Island::SolveTOI over the island's bodies S.ib[0, nbI) and contacts S.ic[0, ncI)
  __device__ void solveIsland(int nbI, int ncI, float minAlpha) {
    const float h = (1.0f - minAlpha) * a.dt;
    for (int i = 0; i < nbI; ++i) {
      S.P[i] = a.pos[S.ib[i]];
      S.V[i] = a.vel[S.ib[i]];
    }
    prepare(nbI, ncI);
    for (int it = 0; it < 20; ++it) {  // b2TimeStep::positionIterations of the sub-step
      float minSep = 0.0f;
      for (int j = 0; j < ncI; ++j) minSep = fmin2(minSep, solveTOIPosition(vcs[j]));
      if (minSep >= -1.5f * B2G_LINEAR_SLOP) break;
    }
    for (int k = 0; k < 2; ++k) {
      float4 s = a.sweep0[S.ib[k]];
      a.sweep0[S.ib[k]] = make_float4(S.P[k].x, S.P[k].y, S.P[k].z, s.w);
    }
    prepare(nbI, ncI);  // InitializeVelocityConstraints at the corrected positions
    for (int it = 0; it < a.vi; ++it)
      for (int j = 0; j < ncI; ++j) solveContactVelocity(vcs[j], S.V);
    for (int i = 0; i < nbI; ++i) {
      V2 c = mk(S.P[i].x, S.P[i].y), v = mk(S.V[i].x, S.V[i].y);
      float an = S.P[i].z, wv = S.V[i].z;
      V2 translation = h * v;
      if (dot(translation, translation) > B2G_MAX_TRANSLATION_SQ) {
        float ratio = B2G_MAX_TRANSLATION / lengthOf(translation);
        v.x *= ratio;
        v.y *= ratio;
      }
      float rotation = h * wv;
      if (rotation * rotation > B2G_MAX_ROTATION_SQ) {
        float ratio = B2G_MAX_ROTATION / fabs2(rotation);
        wv *= ratio;
      }
      addTo(c, h * v);
      an += h * wv;
      const int b = S.ib[i];
      a.pos[b] = make_float4(c.x, c.y, an, 0.0f);
      a.vel[b] = make_float4(v.x, v.y, wv, 0.0f);
      syncXf(b);
    }
    if (a.events_on)  // b2Island::Report (src/dynamics/b2_island.cpp:621-647)
      for (int j = 0; j < ncI; ++j) {
        const VCDev& vc = vcs[j];
        const int2 f = fix(S.ic[j]);
        float ni[2] = {vc.normalImpulse[0], vc.pointCount > 1 ? vc.normalImpulse[1] : 0.0f};
        float ti[2] = {vc.tangentImpulse[0], vc.pointCount > 1 ? vc.tangentImpulse[1] : 0.0f};
        record_event(a, B2G_EVENT_POSTSOLVE, w, f.x - fo, f.y - fo, vc.pointCount, ni, ti, 0);
      }
  }

  __device__ void run() {
    while (hn > 0) {
      heap[0].y += 1;
      const int mc = heap[0].z;
      const float minAlpha = key(0);
      if (1.0f - 10.0f * B2G_EPSILON < minAlpha) break;
      const int2 mf = fix(mc);
      const int ia = a.fbody[mf.x], ib = a.fbody[mf.y];
      const float4 sA = a.sweep0[ia], pA = a.pos[ia], sB = a.sweep0[ib], pB = a.pos[ib];
      advanceBody(ia, minAlpha);
      advanceBody(ib, minAlpha);
      updateContact(mc);
      update(mc);
      if (!(flags(mc) & B2G_CONTACT_ENABLED) || !(flags(mc) & B2G_CONTACT_TOUCHING)) {
        flags(mc) &= ~B2G_CONTACT_ENABLED;
        a.sweep0[ia] = sA; a.pos[ia] = pA;
        a.sweep0[ib] = sB; a.pos[ib] = pB;
        syncXf(ia);
        syncXf(ib);
        update(mc);
        continue;
      }
      wake(ia);
      wake(ib);
      int nbI = 2, ncI = 1;
      S.ib[0] = ia;
      S.ib[1] = ib;
      S.ic[0] = mc;
      a.toi_bfl[ia] = 1;
      a.toi_bfl[ib] = 1;
      setFl(mc, getFl(mc) | TOI_ISLAND);
      ensureLists();
      for (int side = 0; side < 2; ++side) {
        const int body = side ? ib : ia;
        if (a.btype[body] != B2G_DYNAMIC) continue;
        forContacts(body, [&](int ci) {
          if (nbI == TOI_BODIES || ncI == TOI_CONTACTS) return false;
          const int2 f = fix(ci);
          const int ca = a.fbody[f.x], cb = a.fbody[f.y];
          const uint32_t cf = getFl(ci);
          if ((cf & TOI_ISLAND) || !(cf & TOI_PERSIST)) return true;
          const int other = ca == body ? cb : ca;
          if (a.btype[other] == B2G_DYNAMIC && !bullet(body) && !bullet(other)) return true;
          if (a.fsensor[f.x] || a.fsensor[f.y]) return true;
          const float4 so = a.sweep0[other], po = a.pos[other];
          if (!a.toi_bfl[other]) advanceBody(other, minAlpha);
          updateContact(ci);
          const uint32_t fl = flags(ci);
          if (!(fl & B2G_CONTACT_ENABLED) || !(fl & B2G_CONTACT_TOUCHING)) {
            a.sweep0[other] = so;
            a.pos[other] = po;
            syncXf(other);
            return true;
          }
          setFl(ci, cf | TOI_ISLAND);
          S.ic[ncI++] = ci;
          if (a.toi_bfl[other]) return true;
          a.toi_bfl[other] = 1;
          wake(other);
          S.ib[nbI++] = other;
          return true;
        });
      }
      solveIsland(nbI, ncI, minAlpha);
      a.toi_flags[0] = 1;
      // reset the island flags, move the dynamic bodies' fixture boxes, refresh their contacts' TOIs
      for (int i = 0; i < nbI; ++i) {
        const int b = S.ib[i];
        a.toi_bfl[b] = 0;
        if (a.btype[b] != B2G_DYNAMIC) continue;
        const int A = b - b0;
        for (int j = foff[A + 1]; j < foff[A + 2]; ++j) {
          const int f = f0 + flist[j];
          AABB bb = shapeAABB(a.shape[f], ldXf(a.xf, b));
          a.aabb[f] = make_float4(bb.lo.x, bb.lo.y, bb.hi.x, bb.hi.y);
        }
        forContacts(b, [&](int ci) {
          if (getFl(ci) & TOI_PERSIST) {
            if (hpos(ci) == -1) insert(ci);
            else update(ci);
          }
          setFl(ci, 0);
          return true;
        });
      }
      // b2BroadPhase::Query with each moved fixture's box (b2ContactManager::QueryCallback)
      for (int i = 0; i < nbI; ++i) {
        const int b = S.ib[i];
        if (a.btype[b] != B2G_DYNAMIC) continue;
        const int A = b - b0;
        for (int j = foff[A + 1]; j < foff[A + 2]; ++j) {
          const int f = f0 + flist[j];
          const float4 fb = a.aabb[f];
          for (int g = f0; g < f0 + nf; ++g) {
            if (a.fbody[g] == b || !aabb_overlap4(fb, a.aabb[g])) continue;
            int found = -1;
            forContacts(b, [&](int ci) {
              const int2 cf = fix(ci);
              if ((cf.x == f && cf.y == g) || (cf.x == g && cf.y == f)) found = ci;
              return found < 0;
            });
            if (found >= 0) {
              setFl(found, getFl(found) | TOI_PERSIST);
              if (hpos(found) == -1) insert(found);
              continue;
            }
            const bool sg = a.btype[a.fbody[g]] == B2G_STATIC;
            const int e = sg ? f : min(f, g), p = sg ? g : max(f, g);
            if (!accept_leaves(a, leaf_attr(e, a.fattr[e]), leaf_attr(p, a.fattr[p]), nocol)) continue;
            if (nmade == TOI_MADE) continue;
            ToiMade& m = S.made[nmade];
            int fa = e, fb2 = p;
            if (!hasCollider(a.shape[e].type, a.shape[p].type)) { fa = p; fb2 = e; }
            const float4 ma = a.fmat[fa], mb = a.fmat[fb2];
            m.fix = make_int2(fa, fb2);
            m.flags = B2G_CONTACT_ENABLED;
            m.mat = make_float4(sqrtf(ma.x * mb.x), ma.y > mb.y ? ma.y : mb.y, ma.z < mb.z ? ma.z : mb.z, 0.0f);
            memset(&m.man, 0, sizeof(m.man));
            m.hpos = -1;
            m.fl = TOI_PERSIST;
            ++nmade;
            insert(nc + nmade - 1);
          }
        }
      }
    }
  }
};

__global__ void __launch_bounds__(32, 27) k_solve_toi(KernelArgs a) {
  __shared__ ToiSmem S;
  const int w = blockIdx.x;
  const int wf = a.wflags[w];
  // the pair update before this kernel skipped its list when it overflowed: nothing to work on,
  // and the host redoes both after growing the buffers
  const bool overflowed = a.counters[B2G_CNT_OVERFLOW] != 0;
  if (w == 0 && threadIdx.x == 0 && !overflowed) a.toi_flags[1] = 1;
  if (!(wf & B2G_WF_ACTIVE) || !(wf & B2G_WF_CONTINUOUS) || (wf & B2G_WF_RETIRED) || overflowed) return;
  const int lane = threadIdx.x;
  ToiWorld T(a, S);
  const int4 wb = a.wb[w];
  const int2 wc = a.wc[w];
  const int4 wj = a.wj[w];
  T.w = w;
  T.c0 = wc.x;
  T.nc = wc.y;
  T.nmade = 0;
  T.b0 = wb.x;
  T.nb = wb.y;
  T.f0 = wb.z;
  T.nf = wb.w;
  T.fo = wb.z;
  T.heap = a.toi_heap + wc.x + (int64_t)TOI_MADE * w;
  T.hn = 0;
  T.sleepMode = (wf & B2G_WF_SLEEPMODE) != 0;
  T.nocol = make_int2(wj.z, wj.w);
  T.boff = a.toi_boff + wb.x + 2 * w;
  T.foff = a.toi_foff + wb.x + 2 * w;
  T.blist = a.toi_blist + 2 * (int64_t)wc.x;
  T.flist = a.toi_flist + wb.z;
  T.adj = false;
  T.vcs = a.toi_vc + (int64_t)TOI_CONTACTS * w;
  if (T.nc == 0) return;
  for (int i = lane; i < T.nb; i += 32) {
    a.sweep0[T.b0 + i].w = 0.0f;
    a.toi_bfl[T.b0 + i] = 0;
  }
  __syncwarp();
  // the contacts' first TOIs (no sweep is advanced here: every alpha0 is 0)
  for (int k = lane; k < T.nc; k += 32) {
    a.toi_cfl[T.c0 + k] = (uint8_t)TOI_PERSIST;
    const float toi = (a.cflags[T.c0 + k] & B2G_CONTACT_ENABLED) ? T.calcTOI(k) : 1.0f;
    a.toi_hpos[T.c0 + k] = __float_as_int(toi);
  }
  __syncwarp();
  if (lane != 0) return;
  for (int k = 0; k < T.nc; ++k) {
    const float toi = __int_as_float(a.toi_hpos[T.c0 + k]);
    a.toi_hpos[T.c0 + k] = -1;
    if (toi < 1.0f) T.heap[T.hn++] = make_int4(__float_as_int(toi), 0, k, 0);
  }
  for (int i = T.hn / 2 - 1; i >= 0; --i) T.down(i);
  for (int i = 0; i < T.hn; ++i) a.toi_hpos[T.c0 + T.heap[i].z] = i;
  T.run();
}

void launch_solve_toi(const KernelArgs& a, int nw, cudaStream_t s) {
  if (nw > 0) k_solve_toi<<<nw, 32, 0, s>>>(a);
}

// ================================================================================ standalone
__global__ void k_collide_pairs(const b2g_shape* sa, const float* xa, const b2g_shape* sb, const float* xb, int n,
                                b2g_manifold* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Xf A, B;
  A.p = mk(xa[4 * i], xa[4 * i + 1]); A.q.s = xa[4 * i + 2]; A.q.c = xa[4 * i + 3];
  B.p = mk(xb[4 * i], xb[4 * i + 1]); B.q.s = xb[4 * i + 2]; B.q.c = xb[4 * i + 3];
  Man m;
  evaluate(&m, sa[i], A, sb[i], B);
  b2g_manifold r;
  r.type = m.type;
  r.point_count = m.pointCount;
  r.local_normal[0] = m.localNormal.x; r.local_normal[1] = m.localNormal.y;
  r.local_point[0] = m.localPoint.x; r.local_point[1] = m.localPoint.y;
  for (int j = 0; j < 2; ++j) {
    r.points[j].local_point[0] = m.lp[j].x;
    r.points[j].local_point[1] = m.lp[j].y;
    r.points[j].id = m.id[j];
    r.points[j].normal_impulse = 0.0f;
    r.points[j].tangent_impulse = 0.0f;
  }
  out[i] = r;
}

// ================================================================================ launchers
static inline unsigned grid_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

void launch_collide(const KernelArgs& a, int nw, cudaStream_t s) {
  if (a.ccap > 0) k_collide<false><<<grid_for(a.ccap, 256), 256, 0, s>>>(a);
  if (a.ccap > 0 && a.any_sensor) k_collide<true><<<grid_for(a.ccap, 128), 128, 0, s>>>(a);
  if (a.ccap > 0 && a.any_sleep && nw > 0) k_collide_closure<<<nw, 256, 0, s>>>(a);
}
void launch_clear_forces(const KernelArgs& a, int nb, cudaStream_t s) {
  if (nb > 0) k_clear_forces<<<grid_for(nb, 256), 256, 0, s>>>(a, nb);
}
void launch_bp_build(const KernelArgs& a, int nf, int nw, size_t cub_bytes, int sort_bits, cudaStream_t s,
                     bool pairs) {
  if (nf <= 0) {
    if (!pairs) {
      k_lbvh_init<<<grid_for(nw, 256), 256, 0, s>>>(a, 0, nw);
      return;
    }
    cudaMemsetAsync(a.poff, 0, sizeof(int), s);
    k_world_contacts<<<grid_for(nw, 128), 128, 0, s>>>(a, nw);
    return;
  }
  k_aabb<true><<<grid_for(nf, 128), 128, 0, s>>>(a, nf);
  k_world_bounds<<<nw, 256, 0, s>>>(a);
  k_morton<<<grid_for(nf, 256), 256, 0, s>>>(a, nf);
  size_t bytes = cub_bytes;
  cub::DeviceRadixSort::SortPairs(a.cub_tmp, bytes, a.mkey, a.mkey_sorted, a.mval, a.mval_sorted, nf, 0, sort_bits, s);
  int m = nf > nw ? nf : nw;
  k_lbvh_init<<<grid_for(m, 256), 256, 0, s>>>(a, nf, nw);
  if (nf > 1) {
    k_lbvh_internal<<<grid_for(nf - 1, 256), 256, 0, s>>>(a, nf);
    k_lbvh_bounds<<<grid_for(nf, kBoundsThreads), kBoundsThreads, 0, s>>>(a, nf);
  }
  if (!pairs) return;
  cudaMemsetAsync(a.pcount, 0, sizeof(int) * (size_t)nf, s);
  k_pairs_count<<<grid_for(nf, 128), 128, 0, s>>>(a, nf);
  bytes = cub_bytes;
  cub::DeviceScan::ExclusiveSum(a.cub_tmp, bytes, a.pcount, a.poff, nf + 1, s);
  k_world_contacts<<<grid_for(nw, 128), 128, 0, s>>>(a, nw);
}
void launch_bp_tail(const KernelArgs& a0, int f0, int nf, int w0, int nw, size_t cub_bytes, int sort_bits, int dst,
                    int* poff_live, cudaStream_t s) {
  KernelArgs a = a0;
  a.bp_f0 = f0;
  a.bp_w0 = w0;
  const int n = nf - f0, nwt = nw - w0;
  if (n <= 0) {  // appended worlds without fixtures: empty ranges at the end of the live list
    cudaMemsetAsync(a.poff + f0, 0, sizeof(int), s);
    k_tail_ranges<<<grid_for(nwt + 1, 128), 128, 0, s>>>(a, nwt, 0, nullptr);
    return;
  }
  k_aabb<true><<<grid_for(n, 128), 128, 0, s>>>(a, n);
  k_world_bounds<<<nwt, 256, 0, s>>>(a);
  k_morton<<<grid_for(n, 256), 256, 0, s>>>(a, n);
  size_t bytes = cub_bytes;
  cub::DeviceRadixSort::SortPairs(a.cub_tmp, bytes, a.mkey + f0, a.mkey_sorted + f0, a.mval + f0, a.mval_sorted + f0, n,
                                  0, sort_bits, s);
  int m = n > nwt ? n : nwt;
  k_lbvh_init<<<grid_for(m, 256), 256, 0, s>>>(a, n, nwt);
  if (n > 1) {
    k_lbvh_internal<<<grid_for(n - 1, 256), 256, 0, s>>>(a, n);
    k_lbvh_bounds<<<grid_for(n, kBoundsThreads), kBoundsThreads, 0, s>>>(a, n);
  }
  cudaMemsetAsync(a.pcount + f0, 0, sizeof(int) * (size_t)n, s);
  k_pairs_count<<<grid_for(n, 128), 128, 0, s>>>(a, n);
  bytes = cub_bytes;
  cub::DeviceScan::ExclusiveSum(a.cub_tmp, bytes, a.pcount + f0, a.poff + f0, n + 1, s);
  k_pairs_emit<<<grid_for(n, 128), 128, 0, s>>>(a, n);
  k_tail_append<<<1024, 256, 0, s>>>(a, dst);
  int r = (n + 1 > nwt ? n + 1 : nwt);
  k_tail_ranges<<<grid_for(r, 128), 128, 0, s>>>(a, nwt, n, poff_live);
  k_tail_commit<<<1, 1, 0, s>>>(a);
}
void launch_bp_refit(const KernelArgs& a, int tree_nf, int tree_nw, int nf, int nw, size_t cub_bytes, int sort_bits,
                     cudaStream_t s) {
  if (nf <= 0) {
    launch_bp_build(a, nf, nw, cub_bytes, sort_bits, s, true);
    return;
  }
  const int n = nf - tree_nf, nwt = nw - tree_nw;
  k_aabb<false><<<grid_for(tree_nf, 128), 128, 0, s>>>(a, tree_nf);
  if (tree_nf > 0) {
    k_lbvh_refit_init<<<grid_for(tree_nf, 256), 256, 0, s>>>(a, tree_nf);
    if (tree_nf > 1) k_lbvh_bounds<<<grid_for(tree_nf, kBoundsThreads), kBoundsThreads, 0, s>>>(a, tree_nf);
  }
  if (nwt > 0) {  // worlds appended after the kept trees: trees of their own over [tree_nf, nf)
    KernelArgs t = a;
    t.bp_f0 = tree_nf;
    t.bp_w0 = tree_nw;
    if (n > 0) {
      k_aabb<true><<<grid_for(n, 128), 128, 0, s>>>(t, n);
      k_world_bounds<<<nwt, 256, 0, s>>>(t);
      k_morton<<<grid_for(n, 256), 256, 0, s>>>(t, n);
      size_t bytes = cub_bytes;
      cub::DeviceRadixSort::SortPairs(a.cub_tmp, bytes, a.mkey + tree_nf, a.mkey_sorted + tree_nf, a.mval + tree_nf,
                                      a.mval_sorted + tree_nf, n, 0, sort_bits, s);
    }
    int m = n > nwt ? n : nwt;
    k_lbvh_init<<<grid_for(m, 256), 256, 0, s>>>(t, n, nwt);
    if (n > 1) {
      k_lbvh_internal<<<grid_for(n - 1, 256), 256, 0, s>>>(t, n);
      k_lbvh_bounds<<<grid_for(n, kBoundsThreads), kBoundsThreads, 0, s>>>(t, n);
    }
  }
  cudaMemsetAsync(a.pcount, 0, sizeof(int) * (size_t)nf, s);
  k_pairs_count<<<grid_for(nf, 128), 128, 0, s>>>(a, nf);
  size_t bytes = cub_bytes;
  cub::DeviceScan::ExclusiveSum(a.cub_tmp, bytes, a.pcount, a.poff, nf + 1, s);
  k_world_contacts<<<grid_for(nw, 128), 128, 0, s>>>(a, nw);
}
void launch_bp_emit(const KernelArgs& a, int nf, cudaStream_t s) {
  if (nf > 0) k_pairs_emit<<<grid_for(nf, 128), 128, 0, s>>>(a, nf);
}
void launch_contact_diff(const KernelArgs& a, int src, int dst, cudaStream_t s) {
  k_contact_diff<<<grid_for(a.ccap, 256), 256, 0, s>>>(a, src, dst);
  if (a.events_on || a.any_sleep) k_contact_dead<<<grid_for(a.ccap, 256), 256, 0, s>>>(a, src);
  k_commit_contacts<<<1, 1, 0, s>>>(a);
}
size_t cub_temp_bytes(int nf) {
  size_t b1 = 0, b2 = 0;
  cub::DeviceRadixSort::SortPairs((void*)nullptr, b1, (uint64_t*)nullptr, (uint64_t*)nullptr, (int*)nullptr,
                                  (int*)nullptr, nf, 0, 64);
  cub::DeviceScan::ExclusiveSum((void*)nullptr, b2, (int*)nullptr, (int*)nullptr, nf + 1);
  return (b1 > b2 ? b1 : b2) + 256;
}
void launch_collide_pairs(const b2g_shape* sa, const float* xa, const b2g_shape* sb, const float* xb, int n,
                          b2g_manifold* out, cudaStream_t s) {
  if (n > 0) k_collide_pairs<<<grid_for(n, 128), 128, 0, s>>>(sa, xa, sb, xb, n, out);
}

}  // namespace b2g
