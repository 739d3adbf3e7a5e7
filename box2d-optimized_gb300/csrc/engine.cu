// engine.cu - host orchestration of the batched Step and the C ABI (include/b2g_capi.h).
//
// The host keeps the structure of every world (bodies, fixtures, joints, mass data) in
// HostWorld records; the device holds the live dynamic state in packed world-major arrays
// (engine.h). A structural change (new world, body, fixture, joint) downloads the live state,
// edits the host records, and re-uploads the whole layout before the next step; steps
// themselves never touch the host copy.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cstdarg>
#include <chrono>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "b2g_math.cuh"
#include "engine.h"
#include "kernels.h"

namespace b2g {

// Host-side NVTX range around an engine phase (upload, tail broadphase, step, readback,
// compaction, queries). NVTX is header-only and costs a branch when no profiler is attached;
// under a profiler the ranges group each phase's launches on the timeline.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

static thread_local std::string g_last_error;

void set_error(Batch* b, const std::string& msg) {
  g_last_error = msg;
  if (b) b->error = msg;
}

static int locked(Batch* b) {
  set_error(b, "the batch is in a step (between b2g_step_begin and b2g_step_end)");
  return B2G_E_LOCKED;
}

#define CUDA_TRY(b, call)                                                                       \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) {                                                                    \
      set_error(b, std::string(#call) + ": " + cudaGetErrorString(e_));                         \
      return B2G_E_CUDA;                                                                        \
    }                                                                                           \
  } while (0)

template <typename T>
static int ensure(Batch* b, DBuf<T>& buf, size_t n, bool keep = false) {
  if (n == 0) n = 1;
  if (buf.cap >= n) return B2G_OK;
  size_t cap = n + n / 4 + 16;
  size_t bytes = cap * sizeof(T);
  if (b->budget && b->allocated - buf.cap * sizeof(T) + bytes > b->budget) {
    set_error(b, "device memory budget exceeded");
    return B2G_E_OUT_OF_MEMORY;
  }
  T* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();  // a failed allocation leaves the context usable: clear the error
    set_error(b, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? B2G_E_OUT_OF_MEMORY : B2G_E_CUDA;
  }
  if (keep && buf.p && buf.cap) cudaMemcpyAsync(p, buf.p, buf.cap * sizeof(T), cudaMemcpyDeviceToDevice, b->stream);
  if (buf.p) {
    cudaStreamSynchronize(b->stream);
    cudaFree(buf.p);
    b->allocated -= buf.cap * sizeof(T);
  }
  buf.p = p;
  buf.cap = cap;
  b->allocated += bytes;
  return B2G_OK;
}

// Reallocates `buf` at exactly n elements (keeping the first min(n, old) when `keep`).
template <typename T>
static int resize_exact(Batch* b, DBuf<T>& buf, size_t n, bool keep) {
  if (b->budget && b->allocated - buf.cap * sizeof(T) + n * sizeof(T) > b->budget) {
    set_error(b, "device memory budget exceeded");
    return B2G_E_OUT_OF_MEMORY;
  }
  T* p = nullptr;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(b, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? B2G_E_OUT_OF_MEMORY : B2G_E_CUDA;
  }
  if (keep && buf.p) cudaMemcpyAsync(p, buf.p, std::min(n, buf.cap) * sizeof(T), cudaMemcpyDeviceToDevice, b->stream);
  cudaStreamSynchronize(b->stream);
  if (buf.p) {
    cudaFree(buf.p);
    b->allocated -= buf.cap * sizeof(T);
  }
  buf.p = p;
  buf.cap = n;
  b->allocated += n * sizeof(T);
  return B2G_OK;
}

template <typename T>
static void release(Batch* b, DBuf<T>& buf) {
  if (buf.p) {
    cudaFree(buf.p);
    b->allocated -= buf.cap * sizeof(T);
  }
  buf.p = nullptr;
  buf.cap = 0;
}

#define TRY(x)            \
  do {                    \
    int s_ = (x);         \
    if (s_ != B2G_OK) return s_; \
  } while (0)

template <typename T>
static int upload(Batch* b, DBuf<T>& buf, const std::vector<T>& v) {
  TRY(ensure(b, buf, v.size()));
  if (!v.empty()) CUDA_TRY(b, cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, b->stream));
  return B2G_OK;
}

static KernelArgs make_args(Batch* b) {
  KernelArgs a;
  memset(&a, 0, sizeof(a));
  a.wb = b->wb.p; a.wj = b->wj.p; a.wg = b->wg.p; a.wflags = b->wflags.p; a.wc = b->wc.p; a.wfault = b->wfault.p; a.isl_dirty = b->isl_dirty.p;
  a.world_order = b->world_order.p;
  a.xf = b->xf.p; a.pos = b->pos.p; a.vel = b->vel.p; a.massd = b->massd.p; a.damp = b->damp.p;
  a.force = b->force.p; a.lc = b->lc.p; a.btype = b->btype.p; a.bworld = b->bworld.p;
  a.bstate = b->bstate.p; a.bwake = b->bwake.p; a.sl = b->sl.p; a.any_sleep = b->any_sleep ? 1 : 0;
  if (b->step_ccd) {
    a.sweep0 = b->sweep0.p; a.toi_hpos = b->toi_hpos.p; a.toi_cfl = b->toi_cfl.p; a.toi_heap = b->toi_heap.p;
    a.toi_bfl = b->toi_bfl.p; a.toi_flags = b->toi_flags.p;
    const int64_t nbw = (int64_t)b->NB + 2 * (int64_t)b->NW;
    a.toi_boff = b->toi_adj.p; a.toi_foff = b->toi_adj.p + nbw; a.toi_blist = b->toi_adj.p + 2 * nbw;
    a.toi_flist = a.toi_blist + 2 * b->ccap;
    a.toi_vc = b->toi_vc.p;
  }
  a.any_sensor = b->any_sensor ? 1 : 0;
  a.shape = b->shape.p; a.fbody = b->fbody.p; a.fgroup = b->fgroup.p; a.fsensor = b->fsensor.p;
  a.fworld = b->fworld.p; a.frad = b->frad.p; a.ffilter = b->ffilter.p; a.fmat = b->fmat.p; a.aabb = b->aabb.p;
  a.joints = b->joints.p; a.nocollide = b->nocollide.p; a.n_nocollide = b->n_nocollide;
  int c = b->cur;
  a.ckey = b->ckey[c].p; a.cfix = b->cfix[c].p; a.cflags = b->cflags[c].p; a.cmat = b->cmat[c].p;
  a.cman = b->cman[c].p;
  for (int k = 0; k < 2; ++k) {
    a.ckeyB[k] = b->ckey[k].p; a.cfixB[k] = b->cfix[k].p; a.cflagsB[k] = b->cflags[k].p;
    a.cmatB[k] = b->cmat[k].p; a.cmanB[k] = b->cman[k].p;
  }
  a.wbounds = b->wbounds.p; a.mkey = b->mkey.p; a.mkey_sorted = b->mkey_sorted.p; a.mval = b->mval.p;
  a.mval_sorted = b->mval_sorted.p; a.nchild = b->nchild.p; a.nrange = b->nrange.p; a.nparent = b->nparent.p; a.lparent = b->lparent.p;
  a.naabb = b->naabb.p; a.nrec = b->nrec.p; a.nhi = b->nhi.p; a.laabb = b->laabb.p; a.lattr = b->lattr.p; a.fattr = b->fattr.p; a.nflag = b->nflag.p; a.wroot = b->wroot.p; a.pcount = b->pcount.p; a.pslots = b->pslots.p; a.poff = b->poffB[b->cur ^ 1].p; a.poff_old = nullptr;
  a.pairs = b->pairs.p; a.cub_tmp = b->cub_tmp.p;
  a.sc_list = b->sc_list.p; a.scb = b->scb.p; a.srad = b->srad.p; a.cslot = b->cslot.p; a.ccol = b->ccol.p; a.corder = b->corder.p; a.cprio = b->cprio.p;
  a.sp.nf = b->sp_nf.p; a.sp.cid = b->sp_cid.p; a.sp.r0 = b->sp_r0.p; a.sp.r1 = b->sp_r1.p;
  a.sp.nmtm = b->sp_nmtm.p; a.sp.bk = b->sp_bk.p; a.sp.kn = b->sp_kn.p; a.sp.imp = b->sp_imp.p;
  a.sp.idx = b->sp_idx.p; a.sp.lcs = b->sp_lcs.p; a.sp.lnp = b->sp_lnp.p; a.sp.lps = b->sp_lps.p;
  a.sp.rad = b->sp_rad.p;
  a.cready = b->cready.p; a.inc_cnt = b->inc_cnt.p; a.inc_head = b->inc_head.p;
  a.inc_mask = b->inc_mask.p; a.inc_list = b->inc_list.p; a.jinc_list = b->jinc_list.p; a.cwork = b->cwork.p; a.jwork = b->jwork.p; a.jcb = b->jcb.p;
  a.jcol = b->jcol.p; a.jorder = b->jorder.p; a.jranges = b->jranges.p; a.cranges = b->cranges.p; a.jprio = b->jprio.p;
  a.jready = b->jready.p; a.ncolors = b->ncolors.p;
  a.jplanes = b->jplanes.p; a.jstride = b->NJ;
  a.events = b->events.p; a.event_cap = b->event_cap; a.events_on = b->events_on ? 1 : 0;
  a.counters = b->counters.p; a.status = b->status.p;
  return a;
}

// ------------------------------------------------------------------------------ layout upload
// Per-joint constants set by the reference's joint constructors: the prismatic and wheel axes
// (b2_prismatic_joint.cpp:84-90, b2_wheel_joint.cpp:44-45) and the pulley's rope constant
// (b2_pulley_joint.cpp:67).
// A gear's device record from its world's two coupled joints (bo: the world's first body).
static void init_gear_dev(const HostWorld& hw, const b2g_joint_def& def, int bo, JointDev* d) {
  const b2g_joint_def& j1 = hw.joints[def.joint_1].def;
  const b2g_joint_def& j2 = hw.joints[def.joint_2].def;
  JointDev::Gear& g = d->g;
  g.iC = bo + j1.body_a;
  g.iD = bo + j2.body_a;
  g.typeA = j1.type;
  g.typeB = j2.type;
  g.lC[0] = j1.local_anchor_a[0]; g.lC[1] = j1.local_anchor_a[1];
  g.lA[0] = j1.local_anchor_b[0]; g.lA[1] = j1.local_anchor_b[1];
  g.lD[0] = j2.local_anchor_a[0]; g.lD[1] = j2.local_anchor_a[1];
  g.lB[0] = j2.local_anchor_b[0]; g.lB[1] = j2.local_anchor_b[1];
  g.refA = j1.reference_angle;
  g.refB = j2.reference_angle;
  g.axC[0] = g.axC[1] = g.axD[0] = g.axD[1] = 0.0f;
  if (j1.type == B2G_JOINT_PRISMATIC) { g.axC[0] = j1.local_axis_a[0]; g.axC[1] = j1.local_axis_a[1]; }
  if (j2.type == B2G_JOINT_PRISMATIC) { g.axD[0] = j2.local_axis_a[0]; g.axD[1] = j2.local_axis_a[1]; }
}

static void init_joint_dev(const b2g_joint_def& def, JointDev* d) {
  if (def.type == B2G_JOINT_PRISMATIC || def.type == B2G_JOINT_WHEEL) {
    V2 ax = mk(def.local_axis_a[0], def.local_axis_a[1]);
    V2 ay = cross(1.0f, ax);
    d->localXAxisA[0] = ax.x; d->localXAxisA[1] = ax.y;
    d->localYAxisA[0] = ay.x; d->localYAxisA[1] = ay.y;
  } else if (def.type == B2G_JOINT_PULLEY) {
    d->constant = def.length_a + def.ratio * def.length_b;
  }
}

// Device world flags: the host flags without the per-step ones, plus the sleep bits.
static int device_world_flags(const HostWorld& hw) {
  int f = hw.flags & ~(B2G_WF_ACTIVE | B2G_WF_NEW_CONTACTS | B2G_WF_SLEEPMODE | B2G_WF_ALLOW_SLEEP | B2G_WF_CONTINUOUS);
  if (hw.allow_sleep || hw.sleepers) f |= B2G_WF_SLEEPMODE;
  if (hw.allow_sleep) f |= B2G_WF_ALLOW_SLEEP;
  // SolveTOI finds times of impact only between two non-static bodies of which one is a bullet or
  // kinematic (b2Contact::CalculateTOI, src/dynamics/b2_contact.cpp:222-246): without such a body
  // it does nothing
  // (found once per upload: every change to a body reaches the device through one)
  if (hw.continuous) {
    if (hw.toi_bodies < 0) {
      hw.toi_bodies = 0;
      for (const b2g_body& bd : hw.bodies)
        if (bd.type == B2G_KINEMATIC || (bd.type == B2G_DYNAMIC && (bd.flags & B2G_BODY_BULLET))) {
          hw.toi_bodies = 1;
          break;
        }
    }
    if (hw.toi_bodies) f |= B2G_WF_CONTINUOUS;
  }
  return f;
}

// Device sleep state of body i: awake / auto-sleep flags and the sleep timer.
static int2 body_state(const HostWorld& hw, size_t i) {
  const b2g_body& s = hw.bodies[i];
  int fl = 0;
  if ((s.flags & B2G_BODY_AWAKE) && s.type != B2G_STATIC) fl |= B2G_BS_AWAKE;
  if (s.flags & B2G_BODY_AUTO_SLEEP) fl |= B2G_BS_AUTO_SLEEP;
  if (s.flags & B2G_BODY_BULLET) fl |= B2G_BS_BULLET;
  float t = i < hw.body_sleep.size() ? hw.body_sleep[i] : 0.0f;
  int bits;
  memcpy(&bits, &t, sizeof(bits));
  return make_int2(fl, bits);
}

static uint64_t emitter_key(const HostWorld& w, int fo, int fa, int fb) {
  bool sa = w.bodies[w.fixtures[fa].body].type == B2G_STATIC;
  bool sb = w.bodies[w.fixtures[fb].body].type == B2G_STATIC;
  int e, p;
  if (sa) { e = fb; p = fa; }
  else if (sb) { e = fa; p = fb; }
  else { e = std::min(fa, fb); p = std::max(fa, fb); }
  return ((uint64_t)(uint32_t)(e + fo) << 32) | (uint32_t)(p + fo);
}

// Solver launch classes from the world order and the per-class thread counts.
static void replan_solver(Batch* b) {
  std::vector<int> nbw(b->worlds.size());
  for (size_t w = 0; w < b->worlds.size(); ++w) nbw[w] = (int)b->worlds[w].bodies.size();
  int cl = b->cluster_ctas < 0 ? solver_max_cluster_ctas() : std::min(b->cluster_ctas, solver_max_cluster_ctas());
  b->solve_classes = plan_solve_classes(b->h_world_order, nbw, b->class_threads, b->wide_waves, cl);
}

// Solver constraints address bodies by a 24-bit world-local index.
static const size_t kMaxWorldBodies = size_t(1) << 24;

// Reads the status word after the upload's joint colouring (the upload synchronises anyway).
// Each world's slice of the sorted no-collide list (its bodies are contiguous, so its pairs are) in
// the world table's joint record: z = first entry, w = count. The pair filter searches only there.
static void nocollide_ranges(const std::vector<uint64_t>& nocol, const std::vector<int>& body_off,
                             std::vector<int4>& wj) {
  for (size_t w = 0; w < wj.size(); ++w) {
    auto lo = std::lower_bound(nocol.begin(), nocol.end(), (uint64_t)(uint32_t)body_off[w] << 32);
    auto hi = std::lower_bound(lo, nocol.end(), (uint64_t)(uint32_t)body_off[w + 1] << 32);
    wj[w].z = (int)(lo - nocol.begin());
    wj[w].w = (int)(hi - lo);
  }
}

// The broadphase forest no longer matches the fixture layout: the next broadphase builds every tree.
static void forest_reset(Batch* b) { b->tree_nf = b->tree_nw = b->tree_age = 0; }

static int check_upload_status(Batch* b) {
  unsigned int st = 0;
  CUDA_TRY(b, cudaMemcpyAsync(&st, b->status.p, sizeof(st), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(b, cudaStreamSynchronize(b->stream));
  if (st & B2G_DEV_COLOR_ROUNDS) {
    set_error(b, "joint colouring did not complete");
    return B2G_E_CAPACITY;
  }
  return B2G_OK;
}

int upload_all(Batch* b) {
  CUDA_TRY(b, cudaSetDevice(b->device));
  int NW = (int)b->worlds.size();
  std::vector<int4> wb(NW), wj(NW);
  std::vector<float4> wg(NW);
  std::vector<int> wflags(NW);
  b->h_body_off.assign(NW + 1, 0);
  b->h_fix_off.assign(NW + 1, 0);
  b->h_joint_off.assign(NW + 1, 0);
  int NB = 0, NF = 0, NJ = 0;
  int64_t NC = 0;
  for (int w = 0; w < NW; ++w) {
    const HostWorld& hw = b->worlds[w];
    if (hw.bodies.size() >= kMaxWorldBodies) {
      set_error(b, "a world has more bodies than the solver's 24-bit body index allows");
      return B2G_E_CAPACITY;
    }
    b->h_body_off[w] = NB; b->h_fix_off[w] = NF; b->h_joint_off[w] = NJ;
    wb[w] = make_int4(NB, (int)hw.bodies.size(), NF, (int)hw.fixtures.size());
    wj[w] = make_int4(NJ, (int)hw.joints.size(), 0, 0);
    wg[w] = make_float4(hw.gx, hw.gy, hw.inv_dt0, 0.0f);
    hw.toi_bodies = -1;
    wflags[w] = device_world_flags(hw);
    NB += (int)hw.bodies.size();
    NF += (int)hw.fixtures.size();
    NJ += (int)hw.joints.size();
    NC += (int64_t)hw.contacts.size();
  }
  b->h_body_off[NW] = NB; b->h_fix_off[NW] = NF; b->h_joint_off[NW] = NJ;
  std::vector<float4> xf(NB), pos(NB), vel(NB), massd(NB), damp(NB), force(NB);
  std::vector<float2> lc(NB);
  std::vector<int> btype(NB), bworld(NB);
  std::vector<int2> bstate(NB);
  std::vector<b2g_shape> shape(NF);
  std::vector<int> fbody(NF), fgroup(NF), fsensor(NF), fworld(NF);
  std::vector<float> frad(NF);
  std::vector<uint32_t> ffilter(NF);
  std::vector<float4> fmat(NF);
  std::vector<JointDev> joints(NJ);
  std::vector<uint64_t> nocol;
  std::vector<std::pair<uint64_t, size_t>> ckeys;
  std::vector<b2g_contact> call;
  ckeys.reserve(NC);
  call.reserve(NC);
  for (int w = 0; w < NW; ++w) {
    const HostWorld& hw = b->worlds[w];
    int bo = b->h_body_off[w], fo = b->h_fix_off[w], jo = b->h_joint_off[w];
    for (size_t i = 0; i < hw.bodies.size(); ++i) {
      const b2g_body& s = hw.bodies[i];
      size_t k = bo + i;
      xf[k] = make_float4(s.xf[0], s.xf[1], s.xf[2], s.xf[3]);
      pos[k] = make_float4(s.c[0], s.c[1], s.a, 0.0f);
      vel[k] = make_float4(s.v[0], s.v[1], s.w, 0.0f);
      massd[k] = make_float4(s.mass, s.inv_mass, s.inertia, s.inv_inertia);
      damp[k] = make_float4(s.linear_damping, s.angular_damping, s.gravity_scale, 0.0f);
      force[k] = make_float4(s.force[0], s.force[1], s.torque, 0.0f);
      lc[k] = make_float2(s.local_center[0], s.local_center[1]);
      btype[k] = s.type;
      bworld[k] = w;
      bstate[k] = body_state(hw, i);
    }
    for (size_t i = 0; i < hw.fixtures.size(); ++i) {
      const b2g_fixture& f = hw.fixtures[i];
      size_t k = fo + i;
      shape[k] = f.shape;
      frad[k] = f.shape.radius;
      fbody[k] = bo + f.body;
      fgroup[k] = f.group_index;
      fsensor[k] = f.is_sensor ? 1 : 0;
      fworld[k] = w;
      ffilter[k] = (uint32_t)f.category_bits | ((uint32_t)f.mask_bits << 16);
      fmat[k] = make_float4(f.friction, f.restitution, f.restitution_threshold, f.density);
    }
    for (size_t i = 0; i < hw.joints.size(); ++i) {
      const b2g_joint& j = hw.joints[i];
      JointDev& d = joints[jo + i];
      memset(&d, 0, sizeof(d));
      d.d = j.def;
      d.d.body_a += bo;
      d.d.body_b += bo;
      d.impulse[0] = j.impulse[0]; d.impulse[1] = j.impulse[1]; d.impulse[2] = j.impulse[2];
      d.motorImpulse = j.motor_impulse; d.lowerImpulse = j.lower_impulse; d.upperImpulse = j.upper_impulse;
      init_joint_dev(j.def, &d);
      if (j.def.type == B2G_JOINT_GEAR) init_gear_dev(hw, j.def, bo, &d);
      if (!j.def.collide_connected) {
        uint32_t x = (uint32_t)(bo + j.def.body_a), y = (uint32_t)(bo + j.def.body_b);
        if (x > y) std::swap(x, y);
        nocol.push_back(((uint64_t)x << 32) | y);
      }
    }
    for (const b2g_contact& c : hw.contacts) {
      ckeys.push_back({emitter_key(hw, fo, c.fixture_a, c.fixture_b), call.size()});
      b2g_contact g = c;
      g.fixture_a += fo;
      g.fixture_b += fo;
      call.push_back(g);
    }
  }
  std::sort(nocol.begin(), nocol.end());
  nocol.erase(std::unique(nocol.begin(), nocol.end()), nocol.end());
  std::sort(ckeys.begin(), ckeys.end());
  std::vector<uint64_t> ckey(NC);
  std::vector<int2> cfix(NC);
  std::vector<uint32_t> cflags(NC);
  std::vector<float4> cmat(NC);
  std::vector<b2g_manifold> cman(NC);
  for (int64_t i = 0; i < NC; ++i) {
    const b2g_contact& c = call[ckeys[i].second];
    ckey[i] = ckeys[i].first;
    cfix[i] = make_int2(c.fixture_a, c.fixture_b);
    cflags[i] = c.flags;
    cmat[i] = make_float4(c.friction, c.restitution, c.restitution_threshold, c.tangent_speed);
    cman[i] = c.manifold;
  }
  // worlds by body count, largest first: solver launch classes are contiguous ranges of it
  std::vector<int> order(NW);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return b->worlds[x].bodies.size() > b->worlds[y].bodies.size(); });
  b->h_world_order = order;
  replan_solver(b);
  nocollide_ranges(nocol, b->h_body_off, wj);
  TRY(upload(b, b->wb, wb)); TRY(upload(b, b->wj, wj)); TRY(upload(b, b->wg, wg)); TRY(upload(b, b->wflags, wflags));
  TRY(upload(b, b->world_order, order));
  // per-world live contact ranges: the sorted contact list groups by world (keys hold global
  // fixture indices, and each world's fixtures are contiguous)
  {
    std::vector<int2> wc(NW);
    int64_t off = 0;
    for (int w = 0; w < NW; ++w) {
      int cnt = (int)b->worlds[w].contacts.size();
      wc[w] = make_int2((int)off, cnt);
      off += cnt;
    }
    TRY(upload(b, b->wc, wc));
  }
  TRY(ensure(b, b->wbounds, NW)); TRY(ensure(b, b->wroot, NW));
  TRY(ensure(b, b->ncolors, 4 * (size_t)NW)); TRY(ensure(b, b->jranges, 65 * (size_t)NW)); TRY(ensure(b, b->cranges, 65 * (size_t)NW));
  TRY(ensure(b, b->wfault, NW));
  CUDA_TRY(b, cudaMemsetAsync(b->wfault.p, 0, b->wfault.cap, b->stream));
  TRY(ensure(b, b->isl_dirty, NW));  // a new layout labels every world's islands afresh
  CUDA_TRY(b, cudaMemsetAsync(b->isl_dirty.p, 1, b->isl_dirty.cap, b->stream));
  TRY(upload(b, b->xf, xf)); TRY(upload(b, b->pos, pos)); TRY(upload(b, b->vel, vel)); TRY(upload(b, b->massd, massd));
  TRY(upload(b, b->damp, damp)); TRY(upload(b, b->force, force)); TRY(upload(b, b->lc, lc));
  TRY(upload(b, b->btype, btype)); TRY(upload(b, b->bworld, bworld)); TRY(upload(b, b->bstate, bstate));
  TRY(ensure(b, b->bwake, NB)); TRY(ensure(b, b->sl, NB));
  CUDA_TRY(b, cudaMemsetAsync(b->bwake.p, 0, b->bwake.cap, b->stream));
  TRY(upload(b, b->shape, shape)); TRY(upload(b, b->fbody, fbody)); TRY(upload(b, b->fgroup, fgroup));
  TRY(upload(b, b->fsensor, fsensor)); TRY(upload(b, b->fworld, fworld)); TRY(upload(b, b->ffilter, ffilter));
  b->any_sensor = std::find(fsensor.begin(), fsensor.end(), 1) != fsensor.end();
  TRY(upload(b, b->frad, frad));
  TRY(upload(b, b->fmat, fmat)); TRY(ensure(b, b->aabb, NF));
  TRY(upload(b, b->joints, joints)); TRY(upload(b, b->nocollide, nocol));
  b->n_nocollide = (int)nocol.size();
  b->h_nocol.swap(nocol);
  b->cur = 0;
  TRY(upload(b, b->ckey[0], ckey)); TRY(upload(b, b->cfix[0], cfix)); TRY(upload(b, b->cflags[0], cflags));
  TRY(upload(b, b->cmat[0], cmat)); TRY(upload(b, b->cman[0], cman));
  // per-body and per-fixture scratch
  TRY(ensure(b, b->mkey, NF)); TRY(ensure(b, b->mkey_sorted, NF)); TRY(ensure(b, b->mval, NF));
  TRY(ensure(b, b->mval_sorted, NF)); TRY(ensure(b, b->nchild, NF)); TRY(ensure(b, b->nrange, NF)); TRY(ensure(b, b->nparent, NF));
  TRY(ensure(b, b->lparent, NF)); TRY(ensure(b, b->naabb, NF)); TRY(ensure(b, b->nflag, NF));
  TRY(ensure(b, b->nrec, 3 * (size_t)NF)); TRY(ensure(b, b->nhi, NF)); TRY(ensure(b, b->laabb, NF)); TRY(ensure(b, b->lattr, NF)); TRY(ensure(b, b->fattr, NF));
  TRY(ensure(b, b->pcount, (size_t)NF + 1)); TRY(ensure(b, b->pslots, 8 * (size_t)NF));
  TRY(ensure(b, b->poffB[0], (size_t)NF + 1)); TRY(ensure(b, b->poffB[1], (size_t)NF + 1));
  b->poff_valid[0] = b->poff_valid[1] = false;
  TRY(ensure(b, b->cub_tmp, cub_temp_bytes(NF)));
  TRY(ensure(b, b->inc_cnt, NB)); TRY(ensure(b, b->inc_head, NB)); TRY(ensure(b, b->inc_mask, NB));
  TRY(ensure(b, b->jinc_list, 2 * (size_t)NJ)); TRY(ensure(b, b->jwork, 4 * (size_t)NJ)); TRY(ensure(b, b->jcol, NJ)); TRY(ensure(b, b->jorder, NJ));
  TRY(ensure(b, b->jcb, NJ)); TRY(ensure(b, b->jprio, NJ)); TRY(ensure(b, b->jready, NJ));
  TRY(ensure(b, b->jplanes, (size_t)B2G_JV_ROWS * NJ));
  TRY(ensure(b, b->status, 1)); TRY(ensure(b, b->counters, 5));
  b->NW = NW; b->NB = NB; b->NF = NF; b->NJ = NJ; b->NC = NC;
  {
    unsigned long long cnt[4] = {(unsigned long long)NC, 0, 0, 0};
    CUDA_TRY(b, cudaMemcpyAsync(b->counters.p, cnt, sizeof(cnt), cudaMemcpyHostToDevice, b->stream));
  }
  b->h_wflags = wflags;
  b->ccap = 0;
  // joint colours are fixed for the layout
  CUDA_TRY(b, cudaMemsetAsync(b->status.p, 0, sizeof(unsigned int), b->stream));
  launch_joint_colour(make_args(b), 0, NW, b->stream);
  TRY(check_upload_status(b));
  b->tree_valid = false;
  forest_reset(b);
  b->layout_version++;
  b->structure_dirty = false;
  b->device_state_valid = true;
  b->host_state_stale = false;
  CUDA_TRY(b, cudaStreamSynchronize(b->stream));
  return B2G_OK;
}

// Copies v into buf at element offset `off`, growing buf (keeping its contents) as needed.
template <typename T>
static int upload_at(Batch* b, DBuf<T>& buf, size_t off, const std::vector<T>& v) {
  TRY(ensure(b, buf, off + v.size(), true));
  if (!v.empty()) CUDA_TRY(b, cudaMemcpyAsync(buf.p + off, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, b->stream));
  return B2G_OK;
}

// Host -> device copies of host vectors through one pinned staging buffer: the copies are
// asynchronous (no pageable-memory staging on the copy path) and the buffer is reused only once
// the previous batch of copies has completed.
struct Stager {
  struct Item {
    void* dst;
    const void* src;
    size_t bytes;
  };
  std::vector<Item> items;
  size_t total = 0;
  template <typename T>
  int add(Batch* b, DBuf<T>& buf, size_t off, const std::vector<T>& v) {
    TRY(ensure(b, buf, off + v.size(), true));
    if (!v.empty()) {
      items.push_back({buf.p + off, v.data(), v.size() * sizeof(T)});
      total += (v.size() * sizeof(T) + 15) & ~(size_t)15;
    }
    return B2G_OK;
  }
  int flush(Batch* b) {
    if (b->stage_ev) CUDA_TRY(b, cudaEventSynchronize(b->stage_ev));
    if (total > b->h_stage_cap) {
      if (b->h_stage) cudaFreeHost(b->h_stage);
      b->h_stage = nullptr;
      b->h_stage_cap = 0;
      size_t cap = total + total / 2 + 4096;
      CUDA_TRY(b, cudaMallocHost(&b->h_stage, cap));
      b->h_stage_cap = cap;
    }
    char* p = (char*)b->h_stage;
    for (const Item& it : items) {
      memcpy(p, it.src, it.bytes);
      CUDA_TRY(b, cudaMemcpyAsync(it.dst, p, it.bytes, cudaMemcpyHostToDevice, b->stream));
      p += (it.bytes + 15) & ~(size_t)15;
    }
    if (!b->stage_ev) CUDA_TRY(b, cudaEventCreateWithFlags(&b->stage_ev, cudaEventDisableTiming));
    CUDA_TRY(b, cudaEventRecord(b->stage_ev, b->stream));
    return B2G_OK;
  }
};

// Packs the worlds [NW, worlds.size()) that are not on the device yet into device layout, after
// the current layout: host work only, so that it can run while a step executes on the device.
static int pack_tail(Batch* b, TailPack& P) {
  P = TailPack();
  P.w0 = b->NW;
  P.w1 = (int)b->worlds.size();
  P.NB0 = b->NB; P.NF0 = b->NF; P.NJ0 = b->NJ;
  int NB = P.NB0, NF = P.NF0, NJ = P.NJ0;
  size_t nb = 0, nf = 0, nj = 0;
  for (int w = P.w0; w < P.w1; ++w) {
    nb += b->worlds[w].bodies.size(); nf += b->worlds[w].fixtures.size(); nj += b->worlds[w].joints.size();
  }
  P.xf.reserve(nb); P.pos.reserve(nb); P.vel.reserve(nb); P.massd.reserve(nb); P.damp.reserve(nb);
  P.force.reserve(nb); P.lc.reserve(nb); P.btype.reserve(nb); P.bworld.reserve(nb); P.bstate.reserve(nb);
  P.shape.reserve(nf); P.frad.reserve(nf); P.fbody.reserve(nf); P.fgroup.reserve(nf); P.fsensor.reserve(nf);
  P.fworld.reserve(nf); P.ffilter.reserve(nf); P.fmat.reserve(nf); P.joints.reserve(nj);
  for (int w = P.w0; w < P.w1; ++w) {
    const HostWorld& hw = b->worlds[w];
    if (hw.bodies.size() >= kMaxWorldBodies) {
      set_error(b, "a world has more bodies than the solver's 24-bit body index allows");
      return B2G_E_CAPACITY;
    }
    int bo = NB;
    P.body_off.push_back(NB); P.fix_off.push_back(NF); P.joint_off.push_back(NJ);
    for (size_t i = 0; i < hw.bodies.size(); ++i) {
      const b2g_body& s = hw.bodies[i];
      P.bstate.push_back(body_state(hw, i));
      P.xf.push_back(make_float4(s.xf[0], s.xf[1], s.xf[2], s.xf[3]));
      P.pos.push_back(make_float4(s.c[0], s.c[1], s.a, 0.0f));
      P.vel.push_back(make_float4(s.v[0], s.v[1], s.w, 0.0f));
      P.massd.push_back(make_float4(s.mass, s.inv_mass, s.inertia, s.inv_inertia));
      P.damp.push_back(make_float4(s.linear_damping, s.angular_damping, s.gravity_scale, 0.0f));
      P.force.push_back(make_float4(s.force[0], s.force[1], s.torque, 0.0f));
      P.lc.push_back(make_float2(s.local_center[0], s.local_center[1]));
      P.btype.push_back(s.type);
      P.bworld.push_back(w);
    }
    for (const b2g_fixture& f : hw.fixtures) {
      P.shape.push_back(f.shape);
      P.frad.push_back(f.shape.radius);
      P.fbody.push_back(bo + f.body);
      P.fgroup.push_back(f.group_index);
      P.fsensor.push_back(f.is_sensor ? 1 : 0);
      P.fworld.push_back(w);
      P.ffilter.push_back((uint32_t)f.category_bits | ((uint32_t)f.mask_bits << 16));
      P.fmat.push_back(make_float4(f.friction, f.restitution, f.restitution_threshold, f.density));
    }
    for (const b2g_joint& j : hw.joints) {
      JointDev d;
      memset(&d, 0, sizeof(d));
      d.d = j.def;
      d.d.body_a += bo;
      d.d.body_b += bo;
      d.impulse[0] = j.impulse[0]; d.impulse[1] = j.impulse[1]; d.impulse[2] = j.impulse[2];
      d.motorImpulse = j.motor_impulse; d.lowerImpulse = j.lower_impulse; d.upperImpulse = j.upper_impulse;
      init_joint_dev(j.def, &d);
      if (j.def.type == B2G_JOINT_GEAR) init_gear_dev(hw, j.def, bo, &d);
      P.joints.push_back(d);
      if (!j.def.collide_connected) {
        uint32_t x = (uint32_t)(bo + j.def.body_a), y = (uint32_t)(bo + j.def.body_b);
        if (x > y) std::swap(x, y);
        P.nocol.push_back(((uint64_t)x << 32) | y);
      }
    }
    NB += (int)hw.bodies.size();
    NF += (int)hw.fixtures.size();
    NJ += (int)hw.joints.size();
  }
  std::sort(P.nocol.begin(), P.nocol.end());
  P.nocol.erase(std::unique(P.nocol.begin(), P.nocol.end()), P.nocol.end());
  P.NB = NB; P.NF = NF; P.NJ = NJ;
  P.valid = true;
  return B2G_OK;
}

// Uploads the packed worlds after the existing layout without touching the live state of the
// others: body / fixture / joint arrays grow in place and only the new segments are copied; the
// world table is rewritten (small); the new worlds' contacts are found by a broadphase of their
// own or by the step's closing broadphase.
static int flush_tail(Batch* b, TailPack& P) {
  CUDA_TRY(b, cudaSetDevice(b->device));
  const int w0 = P.w0, NW = P.w1;
  const int NB0 = P.NB0, NF0 = P.NF0, NJ0 = P.NJ0, NB = P.NB, NF = P.NF, NJ = P.NJ;
  b->h_body_off.resize(NW + 1);
  b->h_fix_off.resize(NW + 1);
  b->h_joint_off.resize(NW + 1);
  std::vector<float4> wg_tail;
  for (int w = w0; w < NW; ++w) {
    b->h_body_off[w] = P.body_off[w - w0]; b->h_fix_off[w] = P.fix_off[w - w0];
    b->h_joint_off[w] = P.joint_off[w - w0];
    const HostWorld& hw = b->worlds[w];
    wg_tail.push_back(make_float4(hw.gx, hw.gy, hw.inv_dt0, 0.0f));
  }
  b->h_body_off[NW] = NB; b->h_fix_off[NW] = NF; b->h_joint_off[NW] = NJ;
  // world table: offsets are static, gravity/inv_dt0 of existing worlds stay as the device has them
  std::vector<int4> wb(NW), wj(NW);
  std::vector<int> wflags(NW);
  for (int w = 0; w < NW; ++w) {
    const HostWorld& hw = b->worlds[w];
    wb[w] = make_int4(b->h_body_off[w], (int)hw.bodies.size(), b->h_fix_off[w], (int)hw.fixtures.size());
    wj[w] = make_int4(b->h_joint_off[w], (int)hw.joints.size(), 0, 0);
    hw.toi_bodies = -1;
    wflags[w] = device_world_flags(hw);
  }
  std::vector<int> order(NW);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return b->worlds[x].bodies.size() > b->worlds[y].bodies.size(); });
  b->h_world_order = order;
  replan_solver(b);
  std::vector<int2> wc_tail(NW - w0, make_int2(0, 0));
  Stager st;
  b->h_nocol.insert(b->h_nocol.end(), P.nocol.begin(), P.nocol.end());  // appended bodies sort last
  nocollide_ranges(b->h_nocol, b->h_body_off, wj);
  TRY(st.add(b, b->wb, 0, wb)); TRY(st.add(b, b->wj, 0, wj)); TRY(st.add(b, b->wg, w0, wg_tail));
  TRY(st.add(b, b->wflags, 0, wflags)); TRY(st.add(b, b->world_order, 0, order)); TRY(st.add(b, b->wc, w0, wc_tail));
  b->h_wflags = wflags;
  // the broadphase forest's structure (world roots, leaf order, links) survives growth: the next
  // broadphase refits it and builds trees for the appended worlds only
  TRY(ensure(b, b->wbounds, NW)); TRY(ensure(b, b->wroot, NW, true)); TRY(ensure(b, b->ncolors, 4 * (size_t)NW, true));
  TRY(ensure(b, b->isl_dirty, NW, true));  // the appended worlds label their islands afresh
  CUDA_TRY(b, cudaMemsetAsync(b->isl_dirty.p + w0, 1, (size_t)(NW - w0), b->stream));
  if (b->wfault.cap < (size_t)NW) {  // flags are zero between steps: a grown array starts zeroed
    TRY(ensure(b, b->wfault, NW));
    CUDA_TRY(b, cudaMemsetAsync(b->wfault.p, 0, b->wfault.cap, b->stream));
  }
  TRY(ensure(b, b->jranges, 65 * (size_t)NW, true)); TRY(ensure(b, b->cranges, 65 * (size_t)NW));
  TRY(st.add(b, b->xf, NB0, P.xf)); TRY(st.add(b, b->pos, NB0, P.pos)); TRY(st.add(b, b->vel, NB0, P.vel));
  TRY(st.add(b, b->massd, NB0, P.massd)); TRY(st.add(b, b->damp, NB0, P.damp)); TRY(st.add(b, b->force, NB0, P.force));
  TRY(st.add(b, b->lc, NB0, P.lc)); TRY(st.add(b, b->btype, NB0, P.btype)); TRY(st.add(b, b->bworld, NB0, P.bworld));
  TRY(st.add(b, b->bstate, NB0, P.bstate));
  TRY(st.add(b, b->shape, NF0, P.shape)); TRY(st.add(b, b->fbody, NF0, P.fbody)); TRY(st.add(b, b->fgroup, NF0, P.fgroup));
  TRY(st.add(b, b->fsensor, NF0, P.fsensor)); TRY(st.add(b, b->fworld, NF0, P.fworld));
  if (std::find(P.fsensor.begin(), P.fsensor.end(), 1) != P.fsensor.end()) b->any_sensor = true;
  TRY(st.add(b, b->frad, NF0, P.frad));
  TRY(st.add(b, b->ffilter, NF0, P.ffilter)); TRY(st.add(b, b->fmat, NF0, P.fmat));
  TRY(st.add(b, b->joints, NJ0, P.joints)); TRY(st.add(b, b->nocollide, b->n_nocollide, P.nocol));
  TRY(st.flush(b));
  b->n_nocollide += (int)P.nocol.size();
  TRY(ensure(b, b->bwake, NB, true)); TRY(ensure(b, b->sl, NB));  // wake marks are zero between steps
  if (b->bwake.cap > (size_t)NB0) CUDA_TRY(b, cudaMemsetAsync(b->bwake.p + NB0, 0, b->bwake.cap - NB0, b->stream));
  TRY(ensure(b, b->aabb, NF)); TRY(ensure(b, b->mkey, NF)); TRY(ensure(b, b->mkey_sorted, NF));
  TRY(ensure(b, b->mval, NF)); TRY(ensure(b, b->mval_sorted, NF, true)); TRY(ensure(b, b->nchild, NF, true)); TRY(ensure(b, b->nrange, NF, true));
  TRY(ensure(b, b->nparent, NF, true)); TRY(ensure(b, b->lparent, NF, true)); TRY(ensure(b, b->naabb, NF));
  TRY(ensure(b, b->nrec, 3 * (size_t)NF)); TRY(ensure(b, b->nhi, NF)); TRY(ensure(b, b->laabb, NF)); TRY(ensure(b, b->lattr, NF, true));
  TRY(ensure(b, b->fattr, NF, true));  // kept trees keep their leaf attributes (a refit does not rewrite them)
  TRY(ensure(b, b->nflag, NF)); TRY(ensure(b, b->pcount, (size_t)NF + 1));
  // the live list's per-fixture offsets stay valid for the existing fixtures; the appended
  // fixtures' entries come from their broadphase in the next step
  TRY(ensure(b, b->poffB[0], (size_t)NF + 1, true)); TRY(ensure(b, b->poffB[1], (size_t)NF + 1, true));
  TRY(ensure(b, b->pslots, 8 * (size_t)NF));
  TRY(ensure(b, b->cub_tmp, cub_temp_bytes(NF)));
  TRY(ensure(b, b->inc_cnt, NB)); TRY(ensure(b, b->inc_head, NB)); TRY(ensure(b, b->inc_mask, NB));
  TRY(ensure(b, b->jinc_list, 2 * (size_t)NJ)); TRY(ensure(b, b->jwork, 4 * (size_t)NJ)); TRY(ensure(b, b->jcol, NJ, true)); TRY(ensure(b, b->jorder, NJ, true));
  TRY(ensure(b, b->jcb, NJ, true)); TRY(ensure(b, b->jprio, NJ, true)); TRY(ensure(b, b->jready, NJ));
  TRY(ensure(b, b->jplanes, (size_t)B2G_JV_ROWS * NJ));
  b->NW = NW; b->NB = NB; b->NF = NF; b->NJ = NJ;
  // joint colours of the appended worlds; a colouring failure reaches the step's status check
  launch_joint_colour(make_args(b), w0, NW - w0, b->stream);
  b->layout_version++;
  P.valid = false;
  return B2G_OK;
}

// Uploads every world not on the device yet, from a pack prepared by b2g_batch_stage when it
// still matches the layout (it then covers the worlds that existed when it was made), else from a
// pack made now.
int upload_tail(Batch* b) {
  TailPack& P = b->tail_pack;
  if (P.valid && P.w0 == b->NW && P.NB0 == b->NB && P.NF0 == b->NF && P.NJ0 == b->NJ &&
      P.w1 <= (int)b->worlds.size())
    TRY(flush_tail(b, P));
  if ((int)b->worlds.size() > b->NW) {
    TRY(pack_tail(b, P));
    TRY(flush_tail(b, P));
  }
  return B2G_OK;
}

// Copies the live device state (bodies, joints, contacts, inv_dt0) into the host records.
int download_state(Batch* b) {
  if (b->in_step) return locked(b);
  if (b->device < 0 || !b->device_state_valid || !b->host_state_stale) return B2G_OK;
  CUDA_TRY(b, cudaSetDevice(b->device));
  int NB = b->NB, NJ = b->NJ, NW = b->NW;
  int64_t NC = b->NC;
  std::vector<float4> xf(NB), pos(NB), vel(NB), force(NB), wg(NW);
  std::vector<int2> bstate(NB);
  std::vector<JointDev> joints(NJ);
  std::vector<uint64_t> ckey(NC);
  std::vector<int2> cfix(NC);
  std::vector<uint32_t> cflags(NC);
  std::vector<float4> cmat(NC);
  std::vector<b2g_manifold> cman(NC);
  cudaStream_t s = b->stream;
  int c = b->cur;
  if (NB) {
    CUDA_TRY(b, cudaMemcpyAsync(xf.data(), b->xf.p, NB * sizeof(float4), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(pos.data(), b->pos.p, NB * sizeof(float4), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(vel.data(), b->vel.p, NB * sizeof(float4), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(force.data(), b->force.p, NB * sizeof(float4), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(bstate.data(), b->bstate.p, NB * sizeof(int2), cudaMemcpyDeviceToHost, s));
  }
  if (NW) CUDA_TRY(b, cudaMemcpyAsync(wg.data(), b->wg.p, NW * sizeof(float4), cudaMemcpyDeviceToHost, s));
  if (NJ) CUDA_TRY(b, cudaMemcpyAsync(joints.data(), b->joints.p, NJ * sizeof(JointDev), cudaMemcpyDeviceToHost, s));
  if (NC) {
    CUDA_TRY(b, cudaMemcpyAsync(ckey.data(), b->ckey[c].p, NC * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(cfix.data(), b->cfix[c].p, NC * sizeof(int2), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(cflags.data(), b->cflags[c].p, NC * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(cmat.data(), b->cmat[c].p, NC * sizeof(float4), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(cman.data(), b->cman[c].p, NC * sizeof(b2g_manifold), cudaMemcpyDeviceToHost, s));
  }
  CUDA_TRY(b, cudaStreamSynchronize(s));
  for (int w = 0; w < NW; ++w) {
    HostWorld& hw = b->worlds[w];
    int bo = b->h_body_off[w], fo = b->h_fix_off[w], jo = b->h_joint_off[w];
    int nbw = std::min((int)hw.bodies.size(), b->h_body_off[w + 1] - bo);
    for (int i = 0; i < nbw; ++i) {
      b2g_body& r = hw.bodies[i];
      int k = bo + i;
      r.xf[0] = xf[k].x; r.xf[1] = xf[k].y; r.xf[2] = xf[k].z; r.xf[3] = xf[k].w;
      r.c[0] = pos[k].x; r.c[1] = pos[k].y; r.a = pos[k].z;
      r.v[0] = vel[k].x; r.v[1] = vel[k].y; r.w = vel[k].z;
      r.force[0] = force[k].x; r.force[1] = force[k].y; r.torque = force[k].z;
      if (r.type != B2G_STATIC)
        r.flags = (r.flags & ~B2G_BODY_AWAKE) | ((bstate[k].x & B2G_BS_AWAKE) ? B2G_BODY_AWAKE : 0u);
      if (hw.body_sleep.size() < hw.bodies.size()) hw.body_sleep.resize(hw.bodies.size(), 0.0f);
      memcpy(&hw.body_sleep[i], &bstate[k].y, sizeof(float));
    }
    hw.inv_dt0 = wg[w].z;
    int njw = std::min((int)hw.joints.size(), b->h_joint_off[w + 1] - jo);
    for (int i = 0; i < njw; ++i) {
      const JointDev& d = joints[jo + i];
      b2g_joint& r = hw.joints[i];
      r.impulse[0] = d.impulse[0]; r.impulse[1] = d.impulse[1]; r.impulse[2] = d.impulse[2];
      r.motor_impulse = d.motorImpulse; r.lower_impulse = d.lowerImpulse; r.upper_impulse = d.upperImpulse;
      // reaction impulses (GetReactionForce / GetReactionTorque without the inv_dt factor)
      if (r.def.type == B2G_JOINT_REVOLUTE) {
        r.reaction_impulse[0] = d.impulse[0];
        r.reaction_impulse[1] = d.impulse[1];
        r.reaction_angular_impulse = (d.motorImpulse + d.lowerImpulse) - d.upperImpulse;
      } else if (r.def.type == B2G_JOINT_PRISMATIC) {
        V2 perp = mk(d.perp[0], d.perp[1]), axis = mk(d.axis[0], d.axis[1]);
        V2 f = d.impulse[0] * perp + ((d.motorImpulse + d.lowerImpulse) - d.upperImpulse) * axis;
        r.reaction_impulse[0] = f.x; r.reaction_impulse[1] = f.y;
        r.reaction_angular_impulse = d.impulse[1];
      } else if (r.def.type == B2G_JOINT_DISTANCE) {
        V2 u = mk(d.u[0], d.u[1]);
        V2 f = ((d.impulse[0] + d.lowerImpulse) - d.upperImpulse) * u;
        r.reaction_impulse[0] = f.x; r.reaction_impulse[1] = f.y;
        r.reaction_angular_impulse = 0.0f;
      } else if (r.def.type == B2G_JOINT_WHEEL) {  // b2_wheel_joint.cpp:448-456
        V2 f = d.impulse[0] * mk(d.perp[0], d.perp[1]) +
               ((d.impulse[1] + d.lowerImpulse) - d.upperImpulse) * mk(d.axis[0], d.axis[1]);
        r.reaction_impulse[0] = f.x; r.reaction_impulse[1] = f.y;
        r.reaction_angular_impulse = d.motorImpulse;
      } else if (r.def.type == B2G_JOINT_PULLEY) {  // b2_pulley_joint.cpp:276-286
        V2 f = d.impulse[0] * mk(d.uB[0], d.uB[1]);
        r.reaction_impulse[0] = f.x; r.reaction_impulse[1] = f.y;
        r.reaction_angular_impulse = 0.0f;
      } else if (r.def.type == B2G_JOINT_GEAR) {  // b2_gear_joint.cpp:387-397
        r.reaction_impulse[0] = d.impulse[0] * d.g.JvAC[0];
        r.reaction_impulse[1] = d.impulse[0] * d.g.JvAC[1];
        r.reaction_angular_impulse = d.impulse[0] * d.g.JwA;
      } else {  // weld, motor, friction (x, y, angular), mouse (x, y)
        r.reaction_impulse[0] = d.impulse[0];
        r.reaction_impulse[1] = d.impulse[1];
        r.reaction_angular_impulse = r.def.type == B2G_JOINT_MOUSE ? 0.0f : d.impulse[2];
      }
    }
    hw.contacts.clear();
  }
  for (int64_t i = 0; i < NC; ++i) {
    int ga = cfix[i].x, gb = cfix[i].y;
    int w = (int)(std::upper_bound(b->h_fix_off.begin(), b->h_fix_off.end() - 1, ga) - b->h_fix_off.begin()) - 1;
    int fo = b->h_fix_off[w];
    b2g_contact r;
    memset(&r, 0, sizeof(r));
    r.fixture_a = ga - fo;
    r.fixture_b = gb - fo;
    r.flags = cflags[i];
    r.friction = cmat[i].x; r.restitution = cmat[i].y; r.restitution_threshold = cmat[i].z; r.tangent_speed = cmat[i].w;
    r.manifold = cman[i];
    b->worlds[w].contacts.push_back(r);
  }
  b->host_state_stale = false;
  return B2G_OK;
}

// Contact-sized buffers (both contact lists, the pair list, solver scratch) at capacity `cap`.
static int ensure_contact_capacity(Batch* b, int64_t want) {
  if (want < b->ccap && b->ccap > 0) return B2G_OK;
  int64_t cap = std::max<int64_t>(want + want / 2 + 1024, 4 * (int64_t)b->NF + 1024);
  for (int k = 0; k < 2; ++k) {
    bool keep = (k == b->cur);
    TRY(ensure(b, b->ckey[k], (size_t)cap, keep)); TRY(ensure(b, b->cfix[k], (size_t)cap, keep));
    TRY(ensure(b, b->cflags[k], (size_t)cap, keep)); TRY(ensure(b, b->cmat[k], (size_t)cap, keep));
    TRY(ensure(b, b->cman[k], (size_t)cap, keep));
  }
  TRY(ensure(b, b->pairs, (size_t)cap));
  TRY(ensure(b, b->sc_list, (size_t)cap)); TRY(ensure(b, b->scb, (size_t)cap)); TRY(ensure(b, b->srad, (size_t)cap)); TRY(ensure(b, b->cslot, (size_t)cap)); TRY(ensure(b, b->ccol, (size_t)cap));
  TRY(ensure(b, b->corder, (size_t)cap)); TRY(ensure(b, b->cprio, (size_t)cap)); TRY(ensure(b, b->cready, (size_t)cap));
  TRY(ensure(b, b->inc_list, 2 * (size_t)cap)); TRY(ensure(b, b->cwork, 4 * (size_t)cap));
  TRY(ensure(b, b->sp_nf, (size_t)cap)); TRY(ensure(b, b->sp_cid, (size_t)cap)); TRY(ensure(b, b->sp_r0, (size_t)cap));
  TRY(ensure(b, b->sp_r1, (size_t)cap)); TRY(ensure(b, b->sp_nmtm, (size_t)cap)); TRY(ensure(b, b->sp_bk, (size_t)cap));
  TRY(ensure(b, b->sp_kn, (size_t)cap)); TRY(ensure(b, b->sp_imp, (size_t)cap)); TRY(ensure(b, b->sp_idx, (size_t)cap));
  TRY(ensure(b, b->sp_lcs, (size_t)cap)); TRY(ensure(b, b->sp_lnp, (size_t)cap)); TRY(ensure(b, b->sp_lps, (size_t)cap));
  TRY(ensure(b, b->sp_rad, (size_t)cap));
  if (b->events_on) {
    TRY(ensure(b, b->events, (size_t)(4 * cap + 1024)));
    b->event_cap = (int64_t)b->events.cap;
  }
  b->ccap = cap;
  b->layout_version++;
  return B2G_OK;
}

static KernelArgs step_args(Batch* b, float dt, int vi, int pi) {
  KernelArgs a = make_args(b);
  a.dt = dt;
  a.inv_dt = dt > 0.0f ? 1.0f / dt : 0.0f;
  a.vi = vi;
  a.pi = pi;
  a.nf = b->NF;
  a.nw = b->NW;
  a.ccap = b->ccap;
  return a;
}

static int sort_bits(Batch* b) {
  int bits = 32;
  while ((1ll << (bits - 32)) < (long long)b->NW) ++bits;
  return bits;
}

// Broadphase modes: a full build sorts every fixture's Morton code and builds every world's tree;
// a refit keeps the trees of the forest (b->tree_nf fixtures), refits their boxes and builds trees
// only for the fixtures appended after them. Both give the same pairs; the full build restores
// the trees' spatial order, so it runs every b->tree_period broadphases.
enum { BP_FULL = 0, BP_REFIT = 1 };

static int bp_mode(const Batch* b) {
  return (b->tree_nf > 0 && b->tree_nf <= b->NF && b->tree_nw <= b->NW && b->tree_age < b->tree_period)
             ? BP_REFIT : BP_FULL;
}

// The forest after a broadphase of `mode`: every fixture has a tree.
static void bp_done(Batch* b, int mode) {
  b->tree_age = mode == BP_FULL ? 1 : b->tree_age + 1;
  b->tree_nf = b->NF;
  b->tree_nw = b->NW;
}

// Broadphase + contact diff enqueued on the stream with no host synchronisation: pair counts,
// scan, emission and the diff read their sizes from device memory; when the pairs exceed the
// buffers, emission and diff are skipped and the needed size is left in the overflow counter.
// The live contact list moves to buffer cur ^ 1. `tree_nf` / `tree_nw` give the forest a refit
// keeps (ignored by a full build).
static void enqueue_broadphase(Batch* b, const KernelArgs& a0, int src, int mode, int tree_nf, int tree_nw) {
  KernelArgs a = a0;
  // the new list goes to buffer src ^ 1; the diff finds persisting contacts through the live
  // list's per-fixture offsets when the last broadphase left them
  a.poff = b->poffB[src ^ 1].p;
  a.poff_old = b->poff_valid[src] ? b->poffB[src].p : nullptr;
  b->poff_valid[src ^ 1] = true;
  if (mode == BP_REFIT)
    launch_bp_refit(a, tree_nf, tree_nw, b->NF, b->NW, b->cub_tmp.cap, sort_bits(b), b->stream);
  else
    launch_bp_build(a, b->NF, b->NW, b->cub_tmp.cap, sort_bits(b), b->stream);
  launch_bp_emit(a, b->NF, b->stream);
  launch_contact_diff(a, src, src ^ 1, b->stream);
}

// An eagerly launched broadphase in the mode the forest allows; the forest then covers every fixture.
static void enqueue_broadphase(Batch* b, const KernelArgs& a0, int src) {
  const int mode = bp_mode(b);
  enqueue_broadphase(b, a0, src, mode, b->tree_nf, b->tree_nw);
  bp_done(b, mode);
}

// One Step enqueued: [broadphase if fixtures were added] -> collide -> solve -> broadphase ->
// clear forces. `src` is the live contact buffer at entry; it flips once per broadphase. The
// closing broadphase runs in the mode the forest allows, or (graph capture, `capture_mode` >= 0)
// in that mode over a forest that covers every fixture.
static void enqueue_step(Batch* b, float dt, int vi, int pi, bool initial_bp, int src, bool record_profile,
                         int capture_mode = -1) {
  KernelArgs a = step_args(b, dt, vi, pi);
  if (record_profile) cudaEventRecord(b->ev[0], b->stream);
  if (initial_bp) {
    b->cur = src;
    enqueue_broadphase(b, step_args(b, dt, vi, pi), src);
    src ^= 1;
  }
  b->cur = src;
  a = step_args(b, dt, vi, pi);
  launch_collide(a, b->NW, b->stream);
  if (record_profile) cudaEventRecord(b->ev[1], b->stream);
  if (dt > 0.0f) {
    // the forces' copy of b2g_step_io (an event recorded outside the graph when captured)
    const bool captured = capture_mode >= 0;
    cudaStreamWaitEvent(b->stream, b->io_in, captured ? cudaEventWaitExternal : 0);
    launch_solve(a, b->solve_classes, b->stream, b->side, b->fork_ev);
    if (b->debug_checks) launch_colour_check(a, b->NW, b->stream);
    cudaEventRecordWithFlags(b->io_solved, b->stream, captured ? cudaEventRecordExternal : cudaEventRecordDefault);
    b->last_solve_buf = src;
    if (record_profile) cudaEventRecord(b->ev[2], b->stream);
    if (capture_mode >= 0) enqueue_broadphase(b, a, src, capture_mode, b->NF, b->NW);
    else enqueue_broadphase(b, a, src);
    src ^= 1;
    if (b->step_ccd) {
      // b2World::SolveTOI (src/dynamics/b2_world.cpp:1152-1156) on the list the pair update made,
      // then a pair update over the moved bodies' boxes (a refit: the forest covers every fixture)
      b->cur = src;
      KernelArgs t = step_args(b, dt, vi, pi);
      cudaMemsetAsync(b->toi_flags.p, 0, 2 * sizeof(int), b->stream);
      if (!captured) cudaEventRecord(b->ev[6], b->stream);
      launch_solve_toi(t, b->NW, b->stream);
      if (!captured) cudaEventRecord(b->ev[7], b->stream);
      enqueue_broadphase(b, t, src, BP_REFIT, b->NF, b->NW);
      if (!captured) bp_done(b, BP_REFIT);
      src ^= 1;
    }
  } else if (record_profile) {
    cudaEventRecord(b->ev[2], b->stream);
  }
  if (record_profile) cudaEventRecord(b->ev[3], b->stream);
  b->cur = src;
  launch_clear_forces(step_args(b, dt, vi, pi), b->NB, b->stream);
  if (record_profile) cudaEventRecord(b->ev[4], b->stream);
}

// Worlds whose state became non-finite in the last step are frozen (retired: no kernel touches
// them again) and marked faulted; the other worlds of the batch are unaffected.
static int freeze_faulted_worlds(Batch* b) {
  std::vector<uint8_t> f(b->NW);
  if (b->NW > 0) {
    CUDA_TRY(b, cudaMemcpyAsync(f.data(), b->wfault.p, b->NW, cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(b, cudaMemsetAsync(b->wfault.p, 0, b->NW, b->stream));
    CUDA_TRY(b, cudaStreamSynchronize(b->stream));
  }
  for (int w = 0; w < b->NW; ++w)
    if (f[w]) b->worlds[w].flags |= B2G_WF_RETIRED | B2G_WF_FAULTED;
  return B2G_OK;
}

static int check_status(Batch* b, unsigned int st) {
  if (st & B2G_DEV_NONFINITE) {
    set_error(b, "a world produced a non-finite body state");
    return B2G_E_WORLD_FAULT;
  }
  if (st & B2G_DEV_ISLAND_CHECK) {
    set_error(b, "island check failed: inconsistent island labels");
    return B2G_E_CAPACITY;
  }
  if (st & B2G_DEV_COLOUR_CONFLICT) {
    set_error(b, "colouring check failed: a regular colour holds two constraints of one body");
    return B2G_E_CAPACITY;
  }
  if (st & (B2G_DEV_STACK_OVERFLOW | B2G_DEV_COLOR_ROUNDS)) {
    set_error(b, "device capacity check failed (status " + std::to_string(st) + ")");
    return B2G_E_CAPACITY;
  }
  return B2G_OK;
}

static int drain_device_events(Batch* b, unsigned long long n) {
  if (!b->events_on) return B2G_OK;
  int64_t cnt = std::min<int64_t>((int64_t)n, b->event_cap);
  std::vector<EventDev> ev(cnt);
  if (cnt) CUDA_TRY(b, cudaMemcpy(ev.data(), b->events.p, cnt * sizeof(EventDev), cudaMemcpyDeviceToHost));
  for (const EventDev& e : ev) {
    b2g_event o;
    memset(&o, 0, sizeof(o));
    o.kind = e.kind; o.world = e.world; o.fixture_a = e.fixtureA; o.fixture_b = e.fixtureB;
    o.point_count = e.pointCount;
    o.normal_impulses[0] = e.normalImpulses[0]; o.normal_impulses[1] = e.normalImpulses[1];
    o.tangent_impulses[0] = e.tangentImpulses[0]; o.tangent_impulses[1] = e.tangentImpulses[1];
    o.old_manifold = e.old;
    b->host_events.push_back(o);
  }
  return B2G_OK;
}

// Reads the step's counters and status word (one small copy), and recovers from a pair-buffer
// overflow: the overflowing broadphase skipped its emission, so the live list is still the
// pre-broadphase one (with this step's manifolds); grow the buffers and redo the broadphase.
static int finish_step(Batch* b, int live_before_last_bp) {
  NvtxRange range("b2g.readback");
  b->h_readback[5] = 0;
  CUDA_TRY(b, cudaMemcpyAsync(b->h_readback, b->counters.p, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                              b->stream));
  CUDA_TRY(b, cudaMemcpyAsync(b->h_readback + 5, b->status.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(b, cudaStreamSynchronize(b->stream));
  unsigned long long* r = b->h_readback;
  unsigned long long overflow = r[B2G_CNT_OVERFLOW];
  unsigned int status_word = (unsigned int)(r[5] & 0xffffffffull);
  b->profile.colors_max = (int64_t)r[B2G_CNT_MAXCOLORS];
  int guard = 0;
  while (overflow) {
    if (++guard > 8) {
      set_error(b, "pair buffer kept overflowing");
      return B2G_E_CAPACITY;
    }
    b->cur = live_before_last_bp;
    TRY(ensure_contact_capacity(b, (int64_t)overflow));
    CUDA_TRY(b, cudaMemsetAsync(b->counters.p + B2G_CNT_OVERFLOW, 0, sizeof(unsigned long long), b->stream));
    KernelArgs a = step_args(b, b->last_dt, b->last_vi, b->last_pi);
    enqueue_broadphase(b, a, b->cur, BP_FULL, 0, 0);
    bp_done(b, BP_FULL);
    b->cur ^= 1;
    CUDA_TRY(b, cudaMemcpyAsync(b->h_readback, b->counters.p, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                b->stream));
    CUDA_TRY(b, cudaStreamSynchronize(b->stream));
    overflow = r[B2G_CNT_OVERFLOW];
  }
  b->NC = (int64_t)r[B2G_CNT_CONTACTS];
  if (status_word & B2G_DEV_NONFINITE) {
    TRY(freeze_faulted_worlds(b));
    status_word &= ~B2G_DEV_NONFINITE;
  }
  TRY(drain_device_events(b, r[B2G_CNT_EVENTS]));
  b->profile.touching = (int64_t)r[B2G_CNT_TOUCHING];
  b->profile.touching_total += (int64_t)r[B2G_CNT_TOUCHING];
  return check_status(b, status_word);
}

// Contacts of worlds appended since the last step (b2World::Step's FindNewContacts for their new
// fixtures, src/dynamics/b2_world.cpp:1113-1122): a broadphase over the appended fixtures only,
// appended to the live list (the other worlds' bodies have not moved since their broadphase).
static int tail_broadphase(Batch* b, float dt, int vi, int pi, int f0, int w0) {
  NvtxRange range("b2g.tail_broadphase");
  for (int guard = 0;; ++guard) {
    if (guard > 8) {
      set_error(b, "pair buffer kept overflowing");
      return B2G_E_CAPACITY;
    }
    KernelArgs a = step_args(b, dt, vi, pi);
    a.poff = b->poffB[b->cur ^ 1].p;  // scratch: the next full broadphase rewrites it
    launch_bp_tail(a, f0, b->NF, w0, b->NW, b->cub_tmp.cap, sort_bits(b), b->cur,
                   b->poff_valid[b->cur] ? b->poffB[b->cur].p : nullptr, b->stream);
    CUDA_TRY(b, cudaGetLastError());
    CUDA_TRY(b, cudaMemcpyAsync(b->h_readback, b->counters.p, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                b->stream));
    CUDA_TRY(b, cudaStreamSynchronize(b->stream));
    unsigned long long overflow = b->h_readback[B2G_CNT_OVERFLOW];
    if (!overflow) break;
    TRY(ensure_contact_capacity(b, (int64_t)overflow));
    CUDA_TRY(b, cudaMemsetAsync(b->counters.p + B2G_CNT_OVERFLOW, 0, sizeof(unsigned long long), b->stream));
  }
  b->NC = (int64_t)b->h_readback[B2G_CNT_CONTACTS];
  // the appended fixtures' trees join the forest when it covered every fixture before them
  if (b->tree_nf == f0 && b->tree_nw == w0) {
    b->tree_nf = b->NF;
    b->tree_nw = b->NW;
  } else {
    forest_reset(b);
  }
  return B2G_OK;
}

static void invalidate_graphs(Batch* b) {
  for (int m = 0; m < 2; ++m)
    for (int k = 0; k < 2; ++k) {
      if (b->graph_exec[m][k]) cudaGraphExecDestroy(b->graph_exec[m][k]);
      b->graph_exec[m][k] = nullptr;
    }
}

// Captures one Step per live-buffer parity and closing-broadphase mode; a replay does the whole
// Step with no host work.
static int capture_graphs(Batch* b, float dt, int vi, int pi) {
  invalidate_graphs(b);
  int saved = b->cur;
  for (int mode = 0; mode < 2; ++mode)
    for (int parity = 0; parity < 2; ++parity) {
      cudaGraph_t g = nullptr;
      CUDA_TRY(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      enqueue_step(b, dt, vi, pi, false, parity, false, mode);
      const cudaError_t launched = cudaGetLastError();  // a launch refused during capture
      CUDA_TRY(b, cudaStreamEndCapture(b->stream, &g));
      if (launched != cudaSuccess) {
        cudaGraphDestroy(g);
        CUDA_TRY(b, launched);
      }
      CUDA_TRY(b, cudaGraphInstantiate(&b->graph_exec[mode][parity], g, 0));
      cudaGraphDestroy(g);
    }
  b->cur = saved;
  b->graph_dt = dt;
  b->graph_vi = vi;
  b->graph_pi = pi;
  b->graph_ccd = b->step_ccd;
  b->graph_version = b->layout_version;
  return B2G_OK;
}

// One b2World::Step (src/dynamics/b2_world.cpp:1108-1171) for the worlds selected by mask.
static double host_ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// The first half of one b2World::Step (src/dynamics/b2_world.cpp:1108-1171) for the worlds
// selected by mask: uploads, flags, and the step's launches (or graph replay), without waiting
// for the device; step_end waits and reads the step's counters.
// Scratch of the SolveTOI kernel for the current layout and contact capacity.
static int ensure_toi_scratch(Batch* b) {
  const void* before[8] = {b->sweep0.p, b->toi_bfl.p, b->toi_hpos.p, b->toi_cfl.p, b->toi_heap.p, b->toi_flags.p,
                           b->toi_adj.p, b->toi_vc.p};
  TRY(ensure(b, b->sweep0, (size_t)std::max(b->NB, 1)));
  TRY(ensure(b, b->toi_bfl, (size_t)std::max(b->NB, 1)));
  TRY(ensure(b, b->toi_hpos, (size_t)std::max<int64_t>(b->ccap, 1)));
  TRY(ensure(b, b->toi_cfl, (size_t)std::max<int64_t>(b->ccap, 1)));
  TRY(ensure(b, b->toi_heap, (size_t)std::max<int64_t>(b->ccap, 1) + 32 * (size_t)b->NW));
  TRY(ensure(b, b->toi_flags, 2));
  TRY(ensure(b, b->toi_adj, 2 * ((size_t)b->NB + 2 * (size_t)b->NW) + 2 * (size_t)std::max<int64_t>(b->ccap, 1) +
                                (size_t)b->NF + 1));
  TRY(ensure(b, b->toi_vc, 32 * (size_t)std::max(b->NW, 1)));
  const void* after[8] = {b->sweep0.p, b->toi_bfl.p, b->toi_hpos.p, b->toi_cfl.p, b->toi_heap.p, b->toi_flags.p,
                          b->toi_adj.p, b->toi_vc.p};
  for (int i = 0; i < 8; ++i)
    if (before[i] != after[i]) b->layout_version++;  // captured graphs hold the old addresses
  return B2G_OK;
}

// The SolveTOI stage of a step run on its own, after a pair update that had overflowed was redone
// (a step normally runs it inside enqueue_step): the TOI kernel on the live list, then, when an
// island moved bodies, a second pair update that moves their proxies and makes and drops their
// contacts (the UpdateNoRebuild / Query / RemoveDeadContacts inside SolveTOI).
static int toi_stage(Batch* b) {
  NvtxRange range("b2g.solve_toi");
  TRY(ensure_toi_scratch(b));  // the pair update may have grown the contact capacity
  CUDA_TRY(b, cudaMemsetAsync(b->counters.p + 1, 0, 4 * sizeof(unsigned long long), b->stream));
  CUDA_TRY(b, cudaMemsetAsync(b->toi_flags.p, 0, 2 * sizeof(int), b->stream));
  KernelArgs a = step_args(b, b->last_dt, b->last_vi, b->last_pi);
  cudaEventRecord(b->ev[6], b->stream);
  launch_solve_toi(a, b->NW, b->stream);
  CUDA_TRY(b, cudaGetLastError());
  cudaEventRecord(b->ev[7], b->stream);
  // no impact solved in any world: the contacts' boxes are those of the step's pair update
  int* moved = reinterpret_cast<int*>(b->h_readback + 6);
  CUDA_TRY(b, cudaMemcpyAsync(moved, b->toi_flags.p, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(b, cudaStreamSynchronize(b->stream));
  if (*moved) {
    enqueue_broadphase(b, a, b->cur);
    b->cur ^= 1;
  }
  // the step's solver counters were read by the first readback
  const int64_t touching = b->profile.touching, colors = b->profile.colors_max;
  const int st = finish_step(b, b->cur ^ 1);
  b->profile.touching = touching;
  b->profile.colors_max = colors;
  return st;
}

static int step_begin(Batch* b, float dt, int vi, int pi, const uint8_t* mask) {
  NvtxRange range("b2g.step");
  if (b->in_step) return locked(b);
  b->step_t0 = std::chrono::steady_clock::now();
  b->profile.host_admit_upload = 0.0f;
  b->profile.host_admit_broadphase = 0.0f;
  b->profile.host_grow = 0.0f;
  if (!(dt >= 0.0f) || vi < 0 || pi < 0) {
    set_error(b, "invalid step arguments");
    return B2G_E_INVALID_ARG;
  }
  if (b->device < 0) {
    set_error(b, "host-only batch cannot step");
    return B2G_E_CUDA;
  }
  CUDA_TRY(b, cudaSetDevice(b->device));
  int tail_w0 = -1, tail_f0 = 0;
  if (b->status.p) CUDA_TRY(b, cudaMemsetAsync(b->status.p, 0, sizeof(unsigned int), b->stream));
  if (b->structure_dirty) {
    NvtxRange upload_range("b2g.upload");
    TRY(upload_all(b));
    invalidate_graphs(b);
  } else if ((int)b->worlds.size() > b->NW) {
    NvtxRange upload_range("b2g.upload_tail");
    const auto t0 = std::chrono::steady_clock::now();
    tail_w0 = b->NW;
    tail_f0 = b->NF;
    TRY(upload_tail(b));
    invalidate_graphs(b);
    b->profile.host_admit_upload = (float)host_ms_since(t0);
  }
  if (b->NW == 0) return B2G_OK;
  if (!b->h_readback) CUDA_TRY(b, cudaMallocHost(&b->h_readback, 8 * sizeof(unsigned long long)));
  bool need_bp = false;
  bool all_active = true;
  bool any_sleep = false;
  std::vector<int> wflags(b->NW);
  for (int w = 0; w < b->NW; ++w) {
    HostWorld& hw = b->worlds[w];
    int f = device_world_flags(hw);
    if ((!mask || mask[w]) && !(hw.flags & B2G_WF_RETIRED)) f |= B2G_WF_ACTIVE;
    if (f & B2G_WF_SLEEPMODE) any_sleep = true;
    if (mask && !mask[w]) all_active = false;
    wflags[w] = f;
    // appended worlds get their first contacts from the broadphase of the appended range below
    if ((hw.flags & B2G_WF_NEW_CONTACTS) && (tail_w0 < 0 || w < tail_w0)) need_bp = true;
    hw.flags &= ~B2G_WF_NEW_CONTACTS;
  }
  if (wflags != b->h_wflags) {
    TRY(upload(b, b->wflags, wflags));
    b->h_wflags = wflags;
  }
  if (any_sleep != b->any_sleep) {
    b->any_sleep = any_sleep;
    b->layout_version++;  // captured graphs hold the kernel arguments
  }
  // appended worlds that this step leaves out (masked) need no broadphase of their own: the
  // end-of-step broadphase creates their contacts, as FindNewContacts would before their first
  // step (a step without one keeps them flagged for the next step's initial broadphase)
  bool tail_masked = false;
  if (tail_w0 >= 0 && mask) {
    tail_masked = true;
    for (int w = tail_w0; w < b->NW; ++w) tail_masked = tail_masked && !mask[w];
  }
  if (tail_masked) {
    b->poff_valid[b->cur] = false;  // the live list's per-fixture offsets do not cover them
    if (!(dt > 0.0f))
      for (int w = tail_w0; w < b->NW; ++w) b->worlds[w].flags |= B2G_WF_NEW_CONTACTS;
  }
  {
    const auto t0 = std::chrono::steady_clock::now();
    TRY(ensure_contact_capacity(b, b->NC));
    b->profile.host_grow = (float)host_ms_since(t0);
  }
  CUDA_TRY(b, cudaMemsetAsync(b->counters.p + 1, 0, 4 * sizeof(unsigned long long), b->stream));
  if (b->events_on) b->host_events.clear();
  b->last_dt = dt;
  b->last_vi = vi;
  b->last_pi = pi;
  if (tail_w0 >= 0 && !tail_masked) {
    const auto t0 = std::chrono::steady_clock::now();
    TRY(tail_broadphase(b, dt, vi, pi, tail_f0, tail_w0));
    b->profile.host_admit_broadphase = (float)host_ms_since(t0);
    CUDA_TRY(b, cudaMemsetAsync(b->counters.p + 1, 0, 4 * sizeof(unsigned long long), b->stream));
  }
  // continuous collision (b2World::SolveTOI) runs eagerly after the step's pair update
  b->step_ccd = false;
  if (dt > 0.0f)
    for (int w = 0; w < b->NW && !b->step_ccd; ++w)
      b->step_ccd = (wflags[w] & B2G_WF_CONTINUOUS) && (wflags[w] & B2G_WF_ACTIVE) && !(wflags[w] & B2G_WF_RETIRED);
  if (b->step_ccd) TRY(ensure_toi_scratch(b));
  int entry = b->cur;
  bool graph = b->use_graphs && !need_bp && !b->events_on && all_active && dt > 0.0f;
  if (graph && (!b->graph_exec[0][0] || b->graph_version != b->layout_version || b->graph_dt != dt ||
                b->graph_vi != vi || b->graph_pi != pi || b->graph_ccd != b->step_ccd))
    TRY(capture_graphs(b, dt, vi, pi));
  if (need_bp) {
    // fixtures were added or bodies moved: find contacts first (b2_world.cpp:1113-1122), and
    // make sure the list is complete before any kernel reads it
    KernelArgs a = step_args(b, dt, vi, pi);
    enqueue_broadphase(b, a, b->cur);
    b->cur ^= 1;
    TRY(finish_step(b, b->cur ^ 1));
    CUDA_TRY(b, cudaMemsetAsync(b->counters.p + 1, 0, 4 * sizeof(unsigned long long), b->stream));
    entry = b->cur;
  }
  if (graph) {
    // the refit graph assumes a forest over every fixture (captured with it)
    const int mode = (bp_mode(b) == BP_REFIT && b->tree_nf == b->NF && b->tree_nw == b->NW) ? BP_REFIT : BP_FULL;
    cudaEventRecord(b->ev[0], b->stream);
    CUDA_TRY(b, cudaGraphLaunch(b->graph_exec[mode][entry], b->stream));
    bp_done(b, mode);
    if (b->step_ccd) bp_done(b, BP_REFIT);
    cudaEventRecord(b->ev[4], b->stream);
    b->cur = b->step_ccd ? entry : entry ^ 1;  // a step with SolveTOI has two pair updates
    b->last_solve_buf = entry;
  } else {
    enqueue_step(b, dt, vi, pi, false, entry, true);
  }
  CUDA_TRY(b, cudaGetLastError());
  b->host_state_stale = true;
  if (dt > 0.0f || need_bp) b->tree_valid = true;  // a full broadphase rebuilt every world's tree
  b->step_graph = graph;
  b->in_step = true;
  cudaEventRecord(b->ev[5], b->stream);  // b2g_step_poll's marker
  return B2G_OK;
}

// The second half: waits for the step, reads its counters and status (recovering from a pair
// buffer overflow), and fills the profile.
static int step_end(Batch* b) {
  if (!b->in_step) {
    set_error(b, "no step in flight");
    return B2G_E_INVALID_ARG;
  }
  b->in_step = false;
  int live_before_last_bp = b->cur ^ 1;
  bool toi_ran = true;
  if (b->step_ccd) {
    // the TOI kernel found the first pair update overflowed: both pair updates skipped their
    // lists, the live list is the step's first, and the TOI stage runs once it is redone
    int* flags = reinterpret_cast<int*>(b->h_readback + 6);
    CUDA_TRY(b, cudaMemcpyAsync(flags, b->toi_flags.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(b, cudaStreamSynchronize(b->stream));
    toi_ran = flags[1] != 0;
    if (!toi_ran) live_before_last_bp = b->cur;
  }
  int st = finish_step(b, live_before_last_bp);
  float t_toi = 0.0f;
  if (st == B2G_OK && b->step_ccd && !toi_ran) st = toi_stage(b);
  if (b->step_ccd && (!b->step_graph || !toi_ran)) cudaEventElapsedTime(&t_toi, b->ev[6], b->ev[7]);
  if (!b->step_graph) {
    float t_col = 0, t_sol = 0, t_bp = 0;
    cudaEventElapsedTime(&t_col, b->ev[0], b->ev[1]);
    cudaEventElapsedTime(&t_sol, b->ev[1], b->ev[2]);
    cudaEventElapsedTime(&t_bp, b->ev[2], b->ev[3]);
    b->profile.collide = t_col;
    b->profile.solve = t_sol;
    b->profile.broadphase = t_bp;
  }
  float t_all = 0;
  cudaEventElapsedTime(&t_all, b->ev[0], b->ev[4]);
  b->profile.step = t_all;
  b->profile.solve_toi = t_toi;
  b->profile.bodies = b->NB;
  b->profile.fixtures = b->NF;
  b->profile.contacts = b->NC;
  b->profile.joints = b->NJ;
  b->profile.host_step = (float)host_ms_since(b->step_t0);
  return st;
}

int step_batch(Batch* b, float dt, int vi, int pi, const uint8_t* mask, bool sync) {
  (void)sync;
  TRY(step_begin(b, dt, vi, pi, mask));
  return step_end(b);
}

static int world_index_ok(Batch* b, int32_t w) { return b && w >= 0 && w < (int32_t)b->worlds.size(); }

// Before a structural edit: bring the host copy up to date, mark the layout for re-upload.
static int begin_edit(Batch* b) {
  if (b->in_step) return locked(b);
  TRY(download_state(b));
  b->structure_dirty = true;
  return B2G_OK;
}

}  // namespace b2g

// =============================================================================== C ABI
using namespace b2g;

struct b2g_batch : public Batch {};

uint64_t b2g::batch_allocated_bytes(const b2g_batch* b) { return b ? b->allocated : 0; }

int b2g::take_world(b2g_batch* src, int32_t world, HostWorld* out) {
  if (!world_index_ok(src, world) || !out || world < src->NW) return B2G_E_INVALID_ARG;
  if (src->in_step) return locked(src);
  *out = std::move(src->worlds[world]);
  if (world + 1 == (int32_t)src->worlds.size()) {
    src->worlds.pop_back();
  } else {
    src->worlds[world] = HostWorld();
    src->worlds[world].flags |= B2G_WF_RETIRED;
  }
  src->tail_pack.valid = false;
  return B2G_OK;
}

int b2g::append_world(b2g_batch* dst, HostWorld&& w, int32_t* out_world) {
  if (!dst) return B2G_E_INVALID_ARG;
  // after the device layout: the next step uploads it with the other new worlds
  w.flags &= ~(B2G_WF_ACTIVE | B2G_WF_FAULTED);
  dst->worlds.push_back(std::move(w));
  if (out_world) *out_world = (int32_t)dst->worlds.size() - 1;
  return B2G_OK;
}

static const char* kStatusNames[] = {"OK",   "INVALID_ARG", "OUT_OF_MEMORY", "TIMEOUT",  "WORLD_FAULT",
                                     "CUDA", "LOCKED",      "CAPACITY",      "CANCELLED"};

extern "C" {

B2G_API const char* b2g_status_string(int status) {
  if (status < 0 || status >= (int)(sizeof(kStatusNames) / sizeof(kStatusNames[0]))) return "UNKNOWN";
  return kStatusNames[status];
}

B2G_API const char* b2g_last_error(void) { return g_last_error.c_str(); }

B2G_API int b2g_device_count(int32_t* n) {
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (n) *n = (e == cudaSuccess) ? c : 0;
  return e == cudaSuccess ? B2G_OK : B2G_E_CUDA;
}

B2G_API int b2g_batch_create(int device, uint64_t budget_bytes, b2g_batch** out) {
  if (!out) return B2G_E_INVALID_ARG;
  *out = nullptr;
  if (device == B2G_HOST_ONLY) {
    // host-only batch: worlds can be built, edited and read back, but not stepped
    b2g_batch* b = new b2g_batch();
    b->device = -1;
    b->budget = budget_bytes;
    *out = b;
    return B2G_OK;
  }
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || device < 0 || device >= n) {
    set_error(nullptr, std::string("no CUDA device ") + std::to_string(device) + ": " + cudaGetErrorString(e));
    return B2G_E_CUDA;
  }
  b2g_batch* b = new b2g_batch();
  b->device = device;
  b->budget = budget_bytes;
  cudaSetDevice(device);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return B2G_E_CUDA;
  }
  for (int i = 0; i < 8; ++i) cudaEventCreate(&b->ev[i]);
  cudaStreamCreateWithFlags(&b->io_stream, cudaStreamNonBlocking);
  cudaEventCreateWithFlags(&b->io_in, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&b->io_solved, cudaEventDisableTiming);
  cudaEventRecord(b->io_in, b->io_stream);  // complete: a step without b2g_step_io waits for nothing
  for (int i = 0; i < B2G_SOLVE_CLASSES; ++i) cudaStreamCreateWithFlags(&b->side[i], cudaStreamNonBlocking);
  for (int i = 0; i <= B2G_SOLVE_CLASSES; ++i) cudaEventCreateWithFlags(&b->fork_ev[i], cudaEventDisableTiming);
  solver_setup();
  *out = b;
  return B2G_OK;
}

B2G_API int b2g_batch_destroy(b2g_batch* b) {
  if (!b) return B2G_E_INVALID_ARG;
  if (b->device < 0) {
    delete b;
    return B2G_OK;
  }
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  invalidate_graphs(b);
  if (b->h_readback) cudaFreeHost(b->h_readback);
  if (b->h_stage) cudaFreeHost(b->h_stage);
  if (b->stage_ev) cudaEventDestroy(b->stage_ev);
  release(b, b->wb); release(b, b->wj); release(b, b->wg); release(b, b->wflags); release(b, b->wc); release(b, b->wfault); release(b, b->isl_dirty);
  release(b, b->world_order); release(b, b->xf); release(b, b->pos); release(b, b->vel); release(b, b->massd);
  release(b, b->damp); release(b, b->force); release(b, b->lc); release(b, b->btype); release(b, b->bworld);
  release(b, b->bstate); release(b, b->bwake); release(b, b->sl);
  release(b, b->sweep0); release(b, b->toi_hpos); release(b, b->toi_cfl); release(b, b->toi_heap); release(b, b->toi_bfl); release(b, b->toi_flags); release(b, b->toi_adj); release(b, b->toi_vc);
  release(b, b->shape); release(b, b->fbody); release(b, b->fgroup); release(b, b->fsensor); release(b, b->fworld);
  release(b, b->ffilter); release(b, b->fmat); release(b, b->aabb); release(b, b->joints); release(b, b->nocollide);
  for (int k = 0; k < 2; ++k) {
    release(b, b->ckey[k]); release(b, b->cfix[k]); release(b, b->cflags[k]); release(b, b->cmat[k]);
    release(b, b->cman[k]);
  }
  release(b, b->wbounds); release(b, b->mkey); release(b, b->mkey_sorted); release(b, b->mval);
  release(b, b->mval_sorted); release(b, b->nchild); release(b, b->nrange); release(b, b->nparent); release(b, b->lparent);
  release(b, b->naabb); release(b, b->nrec); release(b, b->nhi); release(b, b->laabb); release(b, b->lattr); release(b, b->fattr); release(b, b->nflag); release(b, b->wroot); release(b, b->pcount); release(b, b->pslots); release(b, b->poffB[0]); release(b, b->poffB[1]); release(b, b->pairs);
  release(b, b->cub_tmp); release(b, b->status); release(b, b->counters); release(b, b->sc_list); release(b, b->scb); release(b, b->srad); release(b, b->cslot); release(b, b->frad);
  release(b, b->ccol); release(b, b->corder); release(b, b->cprio); release(b, b->cready); release(b, b->inc_cnt);
  release(b, b->inc_head); release(b, b->inc_mask); release(b, b->inc_list); release(b, b->cwork); release(b, b->jwork);
  release(b, b->sp_nf); release(b, b->sp_cid); release(b, b->sp_r0); release(b, b->sp_r1); release(b, b->sp_nmtm);
  release(b, b->sp_bk); release(b, b->sp_kn); release(b, b->sp_imp); release(b, b->sp_idx); release(b, b->sp_lcs);
  release(b, b->sp_lnp); release(b, b->sp_lps); release(b, b->sp_rad);
  release(b, b->jinc_list); release(b, b->jcol); release(b, b->jorder); release(b, b->jcb); release(b, b->jranges); release(b, b->cranges);
  release(b, b->jprio); release(b, b->jready); release(b, b->jplanes);
  release(b, b->ncolors); release(b, b->events);
  release(b, b->q_world); release(b, b->q_counts); release(b, b->q_out); release(b, b->q_box); release(b, b->q_offs);
  release(b, b->q_hits);
  {
    Batch::Spare& sp = b->spare;
    release(b, sp.xf); release(b, sp.pos); release(b, sp.vel); release(b, sp.massd); release(b, sp.damp);
    release(b, sp.force); release(b, sp.fmat); release(b, sp.lc); release(b, sp.btype); release(b, sp.bworld); release(b, sp.bstate);
    release(b, sp.fbody); release(b, sp.fgroup); release(b, sp.fsensor); release(b, sp.fworld); release(b, sp.tables);
    release(b, sp.shape); release(b, sp.ffilter); release(b, sp.frad); release(b, sp.joints);
  }
  for (int i = 0; i < B2G_SOLVE_CLASSES; ++i) {
    if (b->side[i]) cudaStreamDestroy(b->side[i]);
    if (b->fork_ev[i]) cudaEventDestroy(b->fork_ev[i]);
  }
  if (b->fork_ev[B2G_SOLVE_CLASSES]) cudaEventDestroy(b->fork_ev[B2G_SOLVE_CLASSES]);
  for (int i = 0; i < 8; ++i)
    if (b->ev[i]) cudaEventDestroy(b->ev[i]);
  if (b->io_in) cudaEventDestroy(b->io_in);
  if (b->io_solved) cudaEventDestroy(b->io_solved);
  if (b->io_stream) cudaStreamDestroy(b->io_stream);
  cudaStreamDestroy(b->stream);
  delete b;
  return B2G_OK;
}

B2G_API int b2g_world_add(b2g_batch* b, float gx, float gy, int32_t* out_world) {
  if (!b || !isfinite(gx) || !isfinite(gy)) return B2G_E_INVALID_ARG;
  // a new world goes after the device layout: the next step uploads only the new worlds
  HostWorld w;
  w.gx = gx;
  w.gy = gy;
  b->worlds.push_back(std::move(w));
  if (out_world) *out_world = (int32_t)b->worlds.size() - 1;
  return B2G_OK;
}

// ---- checkpoint / resume: one world's complete state as a self-describing byte blob
extern "C++" {
namespace {
const uint32_t kSnapMagic = 0x53473242u;  // "B2GS"
const uint32_t kSnapVersion = 3;  // 2: body sleep timers; 3: gear joint fields
struct SnapshotHeader {
  uint32_t magic, version;
  uint32_t nb, nf, nj, nc;
  float gx, gy, inv_dt0;
  int32_t flags;
  uint8_t allow_sleep, continuous, sleepers, pad;
  uint32_t record_size[4];  // b2g_body, b2g_fixture, b2g_joint, b2g_contact
};
uint64_t snapshot_bytes(const HostWorld& w) {
  return sizeof(SnapshotHeader) + w.bodies.size() * (sizeof(b2g_body) + 8 + sizeof(float)) +
         w.fixtures.size() * (sizeof(b2g_fixture) + 8) + w.joints.size() * sizeof(b2g_joint) +
         w.contacts.size() * sizeof(b2g_contact);
}
template <typename T>
void put(uint8_t*& p, const std::vector<T>& v) {
  if (!v.empty()) memcpy(p, v.data(), v.size() * sizeof(T));
  p += v.size() * sizeof(T);
}
template <typename T>
void get(const uint8_t*& p, std::vector<T>& v, size_t n) {
  v.resize(n);
  if (n) memcpy(v.data(), p, n * sizeof(T));
  p += n * sizeof(T);
}
}  // namespace
}  // extern "C++"

B2G_API int b2g_world_snapshot(b2g_batch* b, int32_t world, void* buf, uint64_t cap, uint64_t* size) {
  if (!world_index_ok(b, world) || !size || (cap > 0 && !buf)) return B2G_E_INVALID_ARG;
  TRY(download_state(b));  // the host records hold the live state, contacts and impulses included
  const HostWorld& w = b->worlds[world];
  *size = snapshot_bytes(w);
  if (cap < *size) {
    set_error(b, "snapshot buffer too small");
    return B2G_E_CAPACITY;
  }
  SnapshotHeader h;
  memset(&h, 0, sizeof(h));
  h.magic = kSnapMagic;
  h.version = kSnapVersion;
  h.nb = (uint32_t)w.bodies.size(); h.nf = (uint32_t)w.fixtures.size();
  h.nj = (uint32_t)w.joints.size(); h.nc = (uint32_t)w.contacts.size();
  h.gx = w.gx; h.gy = w.gy; h.inv_dt0 = w.inv_dt0;
  h.flags = w.flags & ~(B2G_WF_ACTIVE | B2G_WF_RETIRED | B2G_WF_FAULTED);
  h.allow_sleep = w.allow_sleep; h.continuous = w.continuous; h.sleepers = w.sleepers;
  h.record_size[0] = sizeof(b2g_body); h.record_size[1] = sizeof(b2g_fixture);
  h.record_size[2] = sizeof(b2g_joint); h.record_size[3] = sizeof(b2g_contact);
  uint8_t* p = (uint8_t*)buf;
  memcpy(p, &h, sizeof(h));
  p += sizeof(h);
  std::vector<float> sleep(w.bodies.size(), 0.0f);
  for (size_t i = 0; i < sleep.size() && i < w.body_sleep.size(); ++i) sleep[i] = w.body_sleep[i];
  put(p, w.bodies); put(p, w.body_user); put(p, sleep); put(p, w.fixtures); put(p, w.fixture_user);
  put(p, w.joints); put(p, w.contacts);
  return B2G_OK;
}

B2G_API int b2g_world_restore(b2g_batch* b, const void* buf, uint64_t size, int32_t* out_world) {
  if (!b || !buf || size < sizeof(SnapshotHeader)) return B2G_E_INVALID_ARG;
  SnapshotHeader h;
  memcpy(&h, buf, sizeof(h));
  if (h.magic != kSnapMagic || h.version != kSnapVersion || h.record_size[0] != sizeof(b2g_body) ||
      h.record_size[1] != sizeof(b2g_fixture) || h.record_size[2] != sizeof(b2g_joint) ||
      h.record_size[3] != sizeof(b2g_contact)) {
    set_error(b, "not a world snapshot of this format");
    return B2G_E_INVALID_ARG;
  }
  HostWorld w;
  w.gx = h.gx; w.gy = h.gy; w.inv_dt0 = h.inv_dt0; w.flags = h.flags;
  w.allow_sleep = h.allow_sleep != 0; w.continuous = h.continuous != 0; w.sleepers = h.sleepers != 0;
  if (sizeof(SnapshotHeader) + (uint64_t)h.nb * (sizeof(b2g_body) + 8 + sizeof(float)) + (uint64_t)h.nf * (sizeof(b2g_fixture) + 8) +
          (uint64_t)h.nj * sizeof(b2g_joint) + (uint64_t)h.nc * sizeof(b2g_contact) != size) {
    set_error(b, "snapshot size does not match its counts");
    return B2G_E_INVALID_ARG;
  }
  const uint8_t* p = (const uint8_t*)buf + sizeof(SnapshotHeader);
  get(p, w.bodies, h.nb); get(p, w.body_user, h.nb); get(p, w.body_sleep, h.nb);
  get(p, w.fixtures, h.nf); get(p, w.fixture_user, h.nf);
  get(p, w.joints, h.nj); get(p, w.contacts, h.nc);
  // indices must stay inside the world
  for (const b2g_fixture& f : w.fixtures)
    if (f.body < 0 || f.body >= (int32_t)h.nb) return B2G_E_INVALID_ARG;
  for (const b2g_joint& j : w.joints)
    if (j.def.body_a < 0 || j.def.body_a >= (int32_t)h.nb || j.def.body_b < 0 || j.def.body_b >= (int32_t)h.nb)
      return B2G_E_INVALID_ARG;
  for (const b2g_contact& c : w.contacts)
    if (c.fixture_a < 0 || c.fixture_a >= (int32_t)h.nf || c.fixture_b < 0 || c.fixture_b >= (int32_t)h.nf)
      return B2G_E_INVALID_ARG;
  w.body_fixtures.assign(h.nb, {});
  for (uint32_t f = 0; f < h.nf; ++f) w.body_fixtures[w.fixtures[f].body].push_back((int)f);
  // the restored contacts (with their impulses) enter through a full layout upload
  TRY(begin_edit(b));
  b->worlds.push_back(std::move(w));
  if (out_world) *out_world = (int32_t)b->worlds.size() - 1;
  return B2G_OK;
}

B2G_API int b2g_world_count(b2g_batch* b, int32_t* out_n) {
  if (!b || !out_n) return B2G_E_INVALID_ARG;
  *out_n = (int32_t)b->worlds.size();
  return B2G_OK;
}

B2G_API int b2g_world_set_gravity(b2g_batch* b, int32_t world, float gx, float gy) {
  if (!world_index_ok(b, world) || !isfinite(gx) || !isfinite(gy)) return B2G_E_INVALID_ARG;
  if (b->in_step && world < b->NW) return locked(b);
  b->worlds[world].gx = gx;
  b->worlds[world].gy = gy;
  if (world < b->NW && b->device_state_valid && !b->structure_dirty) {
    float g2[2] = {gx, gy};
    CUDA_TRY(b, cudaMemcpyAsync((char*)(b->wg.p + world), g2, sizeof(g2), cudaMemcpyHostToDevice, b->stream));
    CUDA_TRY(b, cudaStreamSynchronize(b->stream));
  }
  return B2G_OK;
}

// Retires a world: it is no longer stepped, its contacts are dropped at the next broadphase, and
// its memory is reclaimed by the next b2g_compact.
B2G_API int b2g_world_retire(b2g_batch* b, int32_t world) {
  if (!world_index_ok(b, world)) return B2G_E_INVALID_ARG;
  b->worlds[world].flags |= B2G_WF_RETIRED;
  return B2G_OK;
}

// Device compaction of a batch whose device layout is current: kept worlds move down in every
// array (compact.cu), the small world table and the joint-no-collide list are rebuilt on the
// host, and the joint colouring is recomputed; no body, fixture or contact state crosses the bus.
static int compact_device(Batch* b, int32_t* old_to_new, int32_t n) {
  NvtxRange range("b2g.compact");
  CUDA_TRY(b, cudaSetDevice(b->device));
  cudaStream_t s = b->stream;
  const int NW = b->NW;
  std::vector<int2> wc(NW);
  std::vector<float4> wg(NW);
  if (NW > 0) {
    CUDA_TRY(b, cudaMemcpyAsync(wc.data(), b->wc.p, NW * sizeof(int2), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(wg.data(), b->wg.p, NW * sizeof(float4), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaStreamSynchronize(s));
  }
  // per old world: new index and offsets; tables packed as off_old | off_new | wnew | con_old | con_new
  std::vector<int> tab(11 * (size_t)std::max(NW, 1), 0);
  int4* off_old = reinterpret_cast<int4*>(tab.data());
  int4* off_new = off_old + NW;
  int* wnew = tab.data() + 8 * (size_t)NW;
  int* con_old = wnew + NW;
  int* con_new = con_old + NW;
  int NB2 = 0, NF2 = 0, NJ2 = 0, kept = 0;
  int64_t NC2 = 0;
  for (int w = 0; w < NW; ++w) {
    const HostWorld& hw = b->worlds[w];
    off_old[w] = make_int4(b->h_body_off[w], b->h_fix_off[w], b->h_joint_off[w], 0);
    wnew[w] = -1;
    if (hw.flags & B2G_WF_RETIRED) continue;
    wnew[w] = kept++;
    off_new[w] = make_int4(NB2, NF2, NJ2, 0);
    con_old[w] = wc[w].x;
    con_new[w] = (int)NC2;
    NB2 += (int)hw.bodies.size();
    NF2 += (int)hw.fixtures.size();
    NJ2 += (int)hw.joints.size();
    NC2 += wc[w].y;
  }
  TRY(upload(b, b->spare.tables, tab));
  const int* tp = b->spare.tables.p;
  CompactTables t{tp + 8 * (size_t)NW, reinterpret_cast<const int4*>(tp), reinterpret_cast<const int4*>(tp) + NW,
                  tp + 9 * (size_t)NW, tp + 10 * (size_t)NW};
  Batch::Spare& sp = b->spare;
  // the spare arrays take at least the live arrays' capacity: after the swap the live layout keeps
  // the room it had, so worlds appended after a compaction do not regrow every array
  auto room = [](auto& spare, const auto& live, int n) { return std::max((size_t)n, live.cap); };
  auto fit = [&](auto& spare, const auto& live, int n) -> int {
    size_t want = room(spare, live, n);
    return spare.cap >= want ? B2G_OK : resize_exact(b, spare, want, false);
  };
  TRY(fit(sp.xf, b->xf, NB2)); TRY(fit(sp.pos, b->pos, NB2)); TRY(fit(sp.vel, b->vel, NB2));
  TRY(fit(sp.massd, b->massd, NB2)); TRY(fit(sp.damp, b->damp, NB2)); TRY(fit(sp.force, b->force, NB2));
  TRY(fit(sp.lc, b->lc, NB2)); TRY(fit(sp.btype, b->btype, NB2)); TRY(fit(sp.bworld, b->bworld, NB2));
  TRY(fit(sp.bstate, b->bstate, NB2));
  TRY(fit(sp.shape, b->shape, NF2)); TRY(fit(sp.fbody, b->fbody, NF2)); TRY(fit(sp.fgroup, b->fgroup, NF2));
  TRY(fit(sp.fsensor, b->fsensor, NF2)); TRY(fit(sp.fworld, b->fworld, NF2)); TRY(fit(sp.ffilter, b->ffilter, NF2));
  TRY(fit(sp.fmat, b->fmat, NF2)); TRY(fit(sp.frad, b->frad, NF2)); TRY(fit(sp.joints, b->joints, NJ2));
  BodyRecs sb{b->xf.p, b->pos.p, b->vel.p, b->massd.p, b->damp.p, b->force.p, b->lc.p, b->btype.p, b->bworld.p,
              b->bstate.p};
  BodyRecs db{sp.xf.p, sp.pos.p, sp.vel.p, sp.massd.p, sp.damp.p, sp.force.p, sp.lc.p, sp.btype.p, sp.bworld.p,
              sp.bstate.p};
  FixRecs sf{b->shape.p, b->fbody.p, b->fgroup.p, b->fsensor.p, b->fworld.p, b->ffilter.p, b->fmat.p, b->frad.p};
  FixRecs df{sp.shape.p, sp.fbody.p, sp.fgroup.p, sp.fsensor.p, sp.fworld.p, sp.ffilter.p, sp.fmat.p, sp.frad.p};
  const int c = b->cur, d = c ^ 1;  // the live list moves into the other (scratch) contact buffer
  ConRecs sc{b->ckey[c].p, b->cfix[c].p, b->cflags[c].p, b->cmat[c].p, b->cman[c].p};
  ConRecs dc{b->ckey[d].p, b->cfix[d].p, b->cflags[d].p, b->cmat[d].p, b->cman[d].p};
  launch_compact(t, b->NB, sb, db, b->NF, sf, df, b->NJ, b->joints.p, sp.joints.p, b->NC, sc, dc, s);
  CUDA_TRY(b, cudaGetLastError());
  std::swap(b->xf, sp.xf); std::swap(b->pos, sp.pos); std::swap(b->vel, sp.vel); std::swap(b->massd, sp.massd);
  std::swap(b->damp, sp.damp); std::swap(b->force, sp.force); std::swap(b->lc, sp.lc);
  std::swap(b->btype, sp.btype); std::swap(b->bworld, sp.bworld); std::swap(b->bstate, sp.bstate);
  std::swap(b->shape, sp.shape); std::swap(b->fbody, sp.fbody); std::swap(b->fgroup, sp.fgroup);
  std::swap(b->fsensor, sp.fsensor); std::swap(b->fworld, sp.fworld); std::swap(b->ffilter, sp.ffilter);
  std::swap(b->fmat, sp.fmat); std::swap(b->frad, sp.frad); std::swap(b->joints, sp.joints);
  b->cur = d;
  // host records and the world table
  std::vector<HostWorld> keep;
  keep.reserve(kept);
  std::vector<int4> wb(kept), wj(kept);
  std::vector<float4> wg2(kept);
  std::vector<int2> wc2(kept);
  std::vector<int> wflags(kept);
  const int trailing = (int)b->worlds.size() - NW;  // worlds not uploaded yet keep their order
  for (int w = 0; w < NW; ++w) {
    int to = wnew[w];
    if (w < n) old_to_new[w] = to;
    if (to < 0) continue;
    HostWorld& hw = b->worlds[w];
    wb[to] = make_int4(off_new[w].x, (int)hw.bodies.size(), off_new[w].y, (int)hw.fixtures.size());
    wj[to] = make_int4(off_new[w].z, (int)hw.joints.size(), 0, 0);
    wg2[to] = wg[w];
    wc2[to] = make_int2(con_new[w], wc[w].y);
    wflags[to] = device_world_flags(hw);
    keep.push_back(std::move(hw));
  }
  for (int k = 0; k < trailing; ++k) {
    if (NW + k < n) old_to_new[NW + k] = kept + k;
    keep.push_back(std::move(b->worlds[NW + k]));
  }
  b->worlds.swap(keep);
  b->h_body_off.assign(kept + 1, 0);
  b->h_fix_off.assign(kept + 1, 0);
  b->h_joint_off.assign(kept + 1, 0);
  std::vector<uint64_t> nocol;
  for (int w = 0; w < kept; ++w) {
    b->h_body_off[w] = wb[w].x; b->h_fix_off[w] = wb[w].z; b->h_joint_off[w] = wj[w].x;
    for (const b2g_joint& j : b->worlds[w].joints) {
      if (j.def.collide_connected) continue;
      uint32_t x = (uint32_t)(wb[w].x + j.def.body_a), y = (uint32_t)(wb[w].x + j.def.body_b);
      if (x > y) std::swap(x, y);
      nocol.push_back(((uint64_t)x << 32) | y);
    }
  }
  b->h_body_off[kept] = NB2; b->h_fix_off[kept] = NF2; b->h_joint_off[kept] = NJ2;
  std::sort(nocol.begin(), nocol.end());
  nocol.erase(std::unique(nocol.begin(), nocol.end()), nocol.end());
  nocollide_ranges(nocol, b->h_body_off, wj);
  TRY(upload(b, b->wb, wb)); TRY(upload(b, b->wj, wj)); TRY(upload(b, b->wg, wg2)); TRY(upload(b, b->wc, wc2));
  TRY(upload(b, b->wflags, wflags)); TRY(upload(b, b->nocollide, nocol));
  b->n_nocollide = (int)nocol.size();
  b->h_nocol.swap(nocol);
  std::vector<int> order(kept);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return b->worlds[x].bodies.size() > b->worlds[y].bodies.size(); });
  TRY(upload(b, b->world_order, order));
  b->h_world_order = order;
  b->NW = kept; b->NB = NB2; b->NF = NF2; b->NJ = NJ2; b->NC = NC2;
  replan_solver(b);
  {
    unsigned long long cnt = (unsigned long long)NC2;
    CUDA_TRY(b, cudaMemcpyAsync(b->counters.p, &cnt, sizeof(cnt), cudaMemcpyHostToDevice, s));
  }
  b->h_wflags = wflags;
  b->poff_valid[0] = b->poff_valid[1] = false;
  b->last_solve_buf = -1;
  b->tree_valid = false;
  forest_reset(b);
  CUDA_TRY(b, cudaMemsetAsync(b->status.p, 0, sizeof(unsigned int), s));
  launch_joint_colour(make_args(b), 0, kept, s);
  TRY(check_upload_status(b));
  if (b->isl_dirty.p) CUDA_TRY(b, cudaMemsetAsync(b->isl_dirty.p, 1, b->isl_dirty.cap, s));  // bodies moved
  b->layout_version++;
  return B2G_OK;
}

B2G_API int b2g_world_status(b2g_batch* b, int32_t world, int32_t* status) {
  if (!world_index_ok(b, world) || !status) return B2G_E_INVALID_ARG;
  *status = (b->worlds[world].flags & B2G_WF_FAULTED) ? B2G_E_WORLD_FAULT : B2G_OK;
  return B2G_OK;
}

// Removes retired worlds; old_to_new[w] receives each world's new index (-1 if removed).
B2G_API int b2g_compact(b2g_batch* b, int32_t* old_to_new, int32_t n) {
  if (!b || (n > 0 && !old_to_new)) return B2G_E_INVALID_ARG;
  if (b->in_step) return locked(b);
  if (b->device >= 0 && b->device_state_valid && !b->structure_dirty && (int)b->worlds.size() >= b->NW &&
      b->NW > 0)
    return compact_device(b, old_to_new, n);
  TRY(download_state(b));
  std::vector<HostWorld> keep;
  int nw = (int)b->worlds.size();
  for (int w = 0; w < nw; ++w) {
    int to = -1;
    if (!(b->worlds[w].flags & B2G_WF_RETIRED)) {
      to = (int)keep.size();
      keep.push_back(std::move(b->worlds[w]));
    }
    if (w < n) old_to_new[w] = to;
  }
  b->worlds.swap(keep);
  b->structure_dirty = true;
  return B2G_OK;
}

B2G_API int b2g_world_set_flags(b2g_batch* b, int32_t world, int32_t allow_sleep, int32_t warm_starting,
                                int32_t continuous, int32_t auto_clear_forces) {
  if (!world_index_ok(b, world)) return B2G_E_INVALID_ARG;
  // flags travel with the per-step world flags upload; no re-layout
  if (!allow_sleep && (b->worlds[world].allow_sleep || b->worlds[world].sleepers)) {
    // b2World::SetAllowSleeping(false) wakes every body (src/dynamics/b2_world.cpp:474-488)
    if (world < b->NW) TRY(begin_edit(b));
    else b->tail_pack.valid = false;  // a staged upload of this world is stale
    HostWorld& hw = b->worlds[world];
    for (size_t i = 0; i < hw.bodies.size(); ++i)
      if (hw.bodies[i].type != B2G_STATIC) hw.bodies[i].flags |= B2G_BODY_AWAKE;
    hw.body_sleep.assign(hw.bodies.size(), 0.0f);
    hw.sleepers = false;
  }
  HostWorld& w = b->worlds[world];
  w.allow_sleep = allow_sleep != 0;
  w.continuous = continuous != 0;
  w.flags = (w.flags & ~(B2G_WF_WARM | B2G_WF_CLEAR_FORCES)) | (warm_starting ? B2G_WF_WARM : 0) |
            (auto_clear_forces ? B2G_WF_CLEAR_FORCES : 0);
  return B2G_OK;
}

B2G_API int b2g_world_get_flags(b2g_batch* b, int32_t world, int32_t* allow_sleep, int32_t* warm_starting,
                                int32_t* continuous, int32_t* auto_clear_forces) {
  if (!world_index_ok(b, world)) return B2G_E_INVALID_ARG;
  const HostWorld& w = b->worlds[world];
  if (allow_sleep) *allow_sleep = w.allow_sleep ? 1 : 0;
  if (warm_starting) *warm_starting = (w.flags & B2G_WF_WARM) ? 1 : 0;
  if (continuous) *continuous = w.continuous ? 1 : 0;
  if (auto_clear_forces) *auto_clear_forces = (w.flags & B2G_WF_CLEAR_FORCES) ? 1 : 0;
  return B2G_OK;
}

// b2Body::b2Body (src/dynamics/b2_body.cpp:29-122)
B2G_API int b2g_bodies_add(b2g_batch* b, int32_t world, const b2g_body_def* defs, int32_t n, int32_t* out_ids) {
  if (!world_index_ok(b, world) || n < 0 || (n > 0 && !defs)) return B2G_E_INVALID_ARG;
  if (world >= b->NW) b->tail_pack.valid = false;  // a staged upload of this world is stale
  for (int i = 0; i < n; ++i) {
    const b2g_body_def& d = defs[i];
    if (d.type < 0 || d.type > 2 || !isfinite(d.position[0]) || !isfinite(d.position[1]) || !isfinite(d.angle) ||
        !isfinite(d.linear_velocity[0]) || !isfinite(d.linear_velocity[1]) || !isfinite(d.angular_velocity) ||
        !(d.linear_damping >= 0.0f) || !(d.angular_damping >= 0.0f)) {
      set_error(b, "malformed body definition");
      return B2G_E_INVALID_ARG;
    }
  }
  if (world < b->NW) TRY(begin_edit(b));
  HostWorld& w = b->worlds[world];
  for (int i = 0; i < n; ++i) {
    const b2g_body_def& d = defs[i];
    b2g_body r;
    memset(&r, 0, sizeof(r));
    r.xf[0] = d.position[0];
    r.xf[1] = d.position[1];
    r.xf[2] = sinf(d.angle);
    r.xf[3] = cosf(d.angle);
    r.c[0] = d.position[0];
    r.c[1] = d.position[1];
    r.a = d.angle;
    r.v[0] = d.linear_velocity[0];
    r.v[1] = d.linear_velocity[1];
    r.w = d.angular_velocity;
    r.linear_damping = d.linear_damping;
    r.angular_damping = d.angular_damping;
    r.gravity_scale = d.gravity_scale;
    r.type = d.type;
    uint32_t fl = 0;
    if (d.bullet) fl |= B2G_BODY_BULLET;
    if (d.fixed_rotation) fl |= B2G_BODY_FIXED_ROTATION;
    if (d.allow_sleep) fl |= B2G_BODY_AUTO_SLEEP;
    if (d.awake && d.type != B2G_STATIC) fl |= B2G_BODY_AWAKE;
    if (d.enabled) fl |= B2G_BODY_ENABLED;
    r.flags = fl;
    if (out_ids) out_ids[i] = (int32_t)w.bodies.size();
    if (d.type != B2G_STATIC && !(fl & B2G_BODY_AWAKE)) w.sleepers = true;
    w.body_sleep.resize(w.bodies.size(), 0.0f);
    w.bodies.push_back(r);
    w.body_sleep.push_back(0.0f);
    w.body_user.push_back(d.user_data);
    w.body_fixtures.emplace_back();
  }
  return B2G_OK;
}

// b2Body::CreateFixture (src/dynamics/b2_body.cpp:230-269)
B2G_API int b2g_fixtures_add(b2g_batch* b, int32_t world, const b2g_fixture_def* defs, int32_t n, int32_t* out_ids) {
  if (!world_index_ok(b, world) || n < 0 || (n > 0 && !defs)) return B2G_E_INVALID_ARG;
  if (world >= b->NW) b->tail_pack.valid = false;  // a staged upload of this world is stale
  HostWorld& w0 = b->worlds[world];
  std::vector<b2g_fixture> made(n);
  for (int i = 0; i < n; ++i) {
    if (defs[i].body < 0 || defs[i].body >= (int)w0.bodies.size()) {
      set_error(b, "fixture body index out of range");
      return B2G_E_INVALID_ARG;
    }
    int st = process_fixture_def(defs[i], &made[i]);
    if (st != B2G_OK) {
      set_error(b, "malformed fixture definition");
      return st;
    }
  }
  if (world < b->NW) TRY(begin_edit(b));
  HostWorld& w = b->worlds[world];
  for (int i = 0; i < n; ++i) {
    int fi = (int)w.fixtures.size();
    w.fixtures.push_back(made[i]);
    w.fixture_user.push_back(defs[i].user_data);
    w.body_fixtures[made[i].body].push_back(fi);
    if (made[i].density > 0.0f) reset_mass_data(w, made[i].body);
    if (out_ids) out_ids[i] = fi;
  }
  w.flags |= B2G_WF_NEW_CONTACTS;
  return B2G_OK;
}

// b2World::CreateJoint (src/dynamics/b2_world.cpp:268-324) + joint constructors.
B2G_API int b2g_joints_add(b2g_batch* b, int32_t world, const b2g_joint_def* defs, int32_t n, int32_t* out_ids) {
  if (!world_index_ok(b, world) || n < 0 || (n > 0 && !defs)) return B2G_E_INVALID_ARG;
  if (world >= b->NW) b->tail_pack.valid = false;  // a staged upload of this world is stale
  HostWorld& w0 = b->worlds[world];
  for (int i = 0; i < n; ++i) {
    const b2g_joint_def& d = defs[i];
    const int t = d.type;
    if (t != B2G_JOINT_REVOLUTE && t != B2G_JOINT_PRISMATIC && t != B2G_JOINT_DISTANCE && t != B2G_JOINT_PULLEY &&
        t != B2G_JOINT_MOUSE && t != B2G_JOINT_WHEEL && t != B2G_JOINT_WELD && t != B2G_JOINT_FRICTION &&
        t != B2G_JOINT_MOTOR && t != B2G_JOINT_GEAR) {
      set_error(b, "unsupported joint type");
      return B2G_E_INVALID_ARG;
    }
    if (t == B2G_JOINT_GEAR) {  // two earlier revolute / prismatic joints, their bodies B dynamic
      const int have = (int)w0.joints.size() + i;
      auto typeOf = [&](int k) { return k < (int)w0.joints.size() ? w0.joints[k].def.type : defs[k - w0.joints.size()].type; };
      auto bodyB = [&](int k) { return k < (int)w0.joints.size() ? w0.joints[k].def.body_b : defs[k - w0.joints.size()].body_b; };
      bool ok = d.joint_1 >= 0 && d.joint_1 < have && d.joint_2 >= 0 && d.joint_2 < have && d.joint_1 != d.joint_2 &&
                std::isfinite(d.ratio);
      for (int k : {d.joint_1, d.joint_2}) {
        if (!ok) break;
        const int tk = typeOf(k);
        ok = (tk == B2G_JOINT_REVOLUTE || tk == B2G_JOINT_PRISMATIC) && bodyB(k) >= 0 &&
             bodyB(k) < (int)w0.bodies.size() && w0.bodies[bodyB(k)].type == B2G_DYNAMIC;
      }
      if (!ok) {
        set_error(b, "a gear joint needs two earlier revolute or prismatic joints with dynamic bodies B");
        return B2G_E_INVALID_ARG;
      }
      continue;
    }
    if (t == B2G_JOINT_PULLEY && !(d.ratio != 0.0f)) {  // b2PulleyJoint ctor asserts ratio != 0
      set_error(b, "pulley ratio must be non-zero");
      return B2G_E_INVALID_ARG;
    }
    if (d.body_a < 0 || d.body_a >= (int)w0.bodies.size() || d.body_b < 0 || d.body_b >= (int)w0.bodies.size() ||
        d.body_a == d.body_b) {
      set_error(b, "joint body index out of range");
      return B2G_E_INVALID_ARG;
    }
  }
  if (world < b->NW) TRY(begin_edit(b));
  HostWorld& w = b->worlds[world];
  for (int i = 0; i < n; ++i) {
    b2g_joint j;
    memset(&j, 0, sizeof(j));
    j.def = defs[i];
    if (j.def.type == B2G_JOINT_PRISMATIC) {
      // b2PrismaticJoint ctor normalises the axis (b2_prismatic_joint.cpp:84-90)
      V2 ax = mk(j.def.local_axis_a[0], j.def.local_axis_a[1]);
      normalize(ax);
      j.def.local_axis_a[0] = ax.x;
      j.def.local_axis_a[1] = ax.y;
    } else if (j.def.type == B2G_JOINT_DISTANCE) {
      // b2DistanceJoint ctor (b2_distance_joint.cpp:56-64)
      j.def.length = fmax2(j.def.length, B2G_LINEAR_SLOP);
      j.def.min_length = fmax2(j.def.min_length, B2G_LINEAR_SLOP);
      j.def.max_length = fmax2(j.def.max_length, j.def.min_length);
    } else if (j.def.type == B2G_JOINT_GEAR) {
      // b2GearJoint ctor (src/dynamics/b2_gear_joint.cpp:48-139): bodies A, B from the joints'
      // bodies B, C, D from their bodies A; the constant from the joints' coordinates now
      const b2g_joint_def& j1 = w.joints[j.def.joint_1].def;
      const b2g_joint_def& j2 = w.joints[j.def.joint_2].def;
      auto coordinate = [&](const b2g_joint_def& jd) {
        const b2g_body& bx = w.bodies[jd.body_b];  // the gear's A (or B)
        const b2g_body& by = w.bodies[jd.body_a];  // the gear's C (or D)
        if (jd.type == B2G_JOINT_REVOLUTE) return (bx.a - by.a) - jd.reference_angle;
        Rot qx, qy;
        qx.s = bx.xf[2]; qx.c = bx.xf[3];
        qy.s = by.xf[2]; qy.c = by.xf[3];
        const V2 pC = mk(jd.local_anchor_a[0], jd.local_anchor_a[1]);
        const V2 pA = mulT(qy, mul(qx, mk(jd.local_anchor_b[0], jd.local_anchor_b[1])) +
                                   (mk(bx.xf[0], bx.xf[1]) - mk(by.xf[0], by.xf[1])));
        return dot(pA - pC, mk(jd.local_axis_a[0], jd.local_axis_a[1]));
      };
      j.def.body_a = j1.body_b;
      j.def.body_b = j2.body_b;
      const float coordinateA = coordinate(j1), coordinateB = coordinate(j2);
      j.def.gear_constant = coordinateA + j.def.ratio * coordinateB;
    } else if (j.def.type == B2G_JOINT_MOUSE) {
      // b2MouseJoint ctor: the target in body B's frame (b2_mouse_joint.cpp:38-40, b2MulT)
      const b2g_body& bB = w.bodies[j.def.body_b];
      float px = j.def.target[0] - bB.xf[0], py = j.def.target[1] - bB.xf[1];
      j.def.local_anchor_b[0] = bB.xf[3] * px + bB.xf[2] * py;
      j.def.local_anchor_b[1] = -bB.xf[2] * px + bB.xf[3] * py;
    }
    if (out_ids) out_ids[i] = (int32_t)w.joints.size();
    w.joints.push_back(j);
  }
  w.flags |= B2G_WF_NEW_CONTACTS;
  return B2G_OK;
}

// ---- structural removal (b2World::DestroyBody / DestroyJoint, b2Body::DestroyFixture)
//
// Removes the marked bodies, fixtures and joints of one world from its host records and
// renumbers the rest (creation order is kept), as the reference's destroy calls do:
//  * destroying a body destroys its joints, contacts and fixtures (src/dynamics/b2_world.cpp:178-266);
//  * destroying a contact that was touching ends it (EndContact, b2_contact_manager.cpp:48-61), and
//    one with manifold points and no sensor wakes both bodies (b2_contact.cpp:80-91);
//  * destroying a joint wakes both bodies (b2_world.cpp:326-410);
//  * destroying a fixture resets its body's mass data (b2_body.cpp:280-350).
// The End callbacks of the destroyed contacts are returned at once (the reference calls them
// inside the destroy call), with the fixture indices from before the removal. The world is
// re-uploaded by its next step; the surviving contacts keep their manifolds and impulses.
static void wake_body(HostWorld& w, int bi) {
  b2g_body& r = w.bodies[bi];
  if (r.type == B2G_STATIC) return;
  r.flags |= B2G_BODY_AWAKE;
  if ((size_t)bi < w.body_sleep.size()) w.body_sleep[bi] = 0.0f;
}

static int remove_structure(Batch* b, int32_t world, std::vector<char> deadBody, std::vector<char> deadFix,
                            std::vector<char> deadJoint, b2g_event* ended, int32_t cap, int32_t* n_ended) {
  if (world < b->NW) TRY(begin_edit(b));
  else b->tail_pack.valid = false;  // not on the device yet: its host records are the state
  HostWorld& w = b->worlds[world];
  const int nb = (int)w.bodies.size(), nf = (int)w.fixtures.size(), nj = (int)w.joints.size();
  for (int f = 0; f < nf; ++f)
    if (deadBody[w.fixtures[f].body]) deadFix[f] = 1;
  for (int j = 0; j < nj; ++j)
    if (deadBody[w.joints[j].def.body_a] || deadBody[w.joints[j].def.body_b]) deadJoint[j] = 1;
  // a gear goes with either joint it couples (gears follow their joints in creation order)
  for (int j = 0; j < nj; ++j)
    if (w.joints[j].def.type == B2G_JOINT_GEAR && (deadJoint[w.joints[j].def.joint_1] || deadJoint[w.joints[j].def.joint_2]))
      deadJoint[j] = 1;
  w.body_sleep.resize(nb, 0.0f);
  for (int j = 0; j < nj; ++j)
    if (deadJoint[j]) {
      wake_body(w, w.joints[j].def.body_a);
      wake_body(w, w.joints[j].def.body_b);
    }
  // contacts: End for the touching ones, wakes for those with points
  int32_t ne = 0;
  std::vector<b2g_contact> kept;
  kept.reserve(w.contacts.size());
  for (const b2g_contact& c : w.contacts) {
    if (!deadFix[c.fixture_a] && !deadFix[c.fixture_b]) {
      kept.push_back(c);
      continue;
    }
    if ((c.flags & B2G_CONTACT_TOUCHING) && ended && ne < cap) {
      b2g_event e;
      memset(&e, 0, sizeof(e));
      e.kind = B2G_EVENT_END;
      e.world = world;
      e.fixture_a = c.fixture_a;
      e.fixture_b = c.fixture_b;
      ended[ne] = e;
    }
    if (c.flags & B2G_CONTACT_TOUCHING) ++ne;
    const b2g_fixture& fa = w.fixtures[c.fixture_a];
    const b2g_fixture& fb = w.fixtures[c.fixture_b];
    if (c.manifold.point_count > 0 && !fa.is_sensor && !fb.is_sensor) {
      wake_body(w, fa.body);
      wake_body(w, fb.body);
    }
  }
  if (n_ended) *n_ended = ne;
  // renumbering maps (-1: removed)
  std::vector<int> bmap(nb), fmap(nf), jmap(nj);
  int k = 0;
  for (int i = 0; i < nb; ++i) bmap[i] = deadBody[i] ? -1 : k++;
  k = 0;
  for (int i = 0; i < nf; ++i) fmap[i] = deadFix[i] ? -1 : k++;
  k = 0;
  for (int i = 0; i < nj; ++i) jmap[i] = deadJoint[i] ? -1 : k++;
  std::vector<int> massReset;
  for (int f = 0; f < nf; ++f)
    if (deadFix[f] && !deadBody[w.fixtures[f].body] && w.fixtures[f].density > 0.0f) massReset.push_back(w.fixtures[f].body);
  // compact every per-body, per-fixture and per-joint array
  auto compact = [](auto& v, const std::vector<int>& map) {
    size_t o = 0;
    for (size_t i = 0; i < map.size() && i < v.size(); ++i) {
      if (map[i] < 0) continue;
      if (o != i) v[o] = std::move(v[i]);  // never self-move: it would empty a vector element
      ++o;
    }
    v.resize(o);
  };
  compact(w.bodies, bmap);
  compact(w.body_sleep, bmap);
  compact(w.body_user, bmap);
  compact(w.body_fixtures, bmap);
  compact(w.fixtures, fmap);
  compact(w.fixture_user, fmap);
  compact(w.joints, jmap);
  for (b2g_fixture& f : w.fixtures) f.body = bmap[f.body];
  for (b2g_joint& j : w.joints) {
    j.def.body_a = bmap[j.def.body_a];
    j.def.body_b = bmap[j.def.body_b];
    if (j.def.type == B2G_JOINT_GEAR) {
      j.def.joint_1 = jmap[j.def.joint_1];
      j.def.joint_2 = jmap[j.def.joint_2];
    }
  }
  for (std::vector<int>& lst : w.body_fixtures) {
    size_t o = 0;
    for (int f : lst)
      if (fmap[f] >= 0) lst[o++] = fmap[f];
    lst.resize(o);
  }
  for (b2g_contact& c : kept) {
    c.fixture_a = fmap[c.fixture_a];
    c.fixture_b = fmap[c.fixture_b];
  }
  w.contacts.swap(kept);
  for (int bi : massReset) reset_mass_data(w, bmap[bi]);
  // undelivered events of this world name fixtures by their old indices
  std::vector<b2g_event>& ev = b->host_events;
  size_t o = 0;
  for (size_t i = 0; i < ev.size(); ++i) {
    b2g_event e = ev[i];
    if (e.world == world) {
      if (fmap[e.fixture_a] < 0 || fmap[e.fixture_b] < 0) continue;
      e.fixture_a = fmap[e.fixture_a];
      e.fixture_b = fmap[e.fixture_b];
    }
    ev[o++] = e;
  }
  ev.resize(o);
  return B2G_OK;
}

static int remove_args_ok(Batch* b, int32_t world, const int32_t* ids, int32_t n, size_t count) {
  if (!world_index_ok(b, world) || n < 0 || (n > 0 && !ids)) return B2G_E_INVALID_ARG;
  for (int32_t i = 0; i < n; ++i)
    if (ids[i] < 0 || (size_t)ids[i] >= count) {
      set_error(b, "index out of range in a removal");
      return B2G_E_INVALID_ARG;
    }
  return B2G_OK;
}

B2G_API int b2g_bodies_remove(b2g_batch* b, int32_t world, const int32_t* bodies, int32_t n, b2g_event* ended,
                              int32_t cap, int32_t* n_ended) {
  if (n_ended) *n_ended = 0;
  if (!b || cap < 0 || (cap > 0 && !ended)) return B2G_E_INVALID_ARG;
  TRY(remove_args_ok(b, world, bodies, n, world_index_ok(b, world) ? b->worlds[world].bodies.size() : 0));
  if (b->in_step) return locked(b);
  const HostWorld& w = b->worlds[world];
  std::vector<char> db(w.bodies.size(), 0), df(w.fixtures.size(), 0), dj(w.joints.size(), 0);
  for (int32_t i = 0; i < n; ++i) db[bodies[i]] = 1;
  return remove_structure(b, world, std::move(db), std::move(df), std::move(dj), ended, cap, n_ended);
}

B2G_API int b2g_fixtures_remove(b2g_batch* b, int32_t world, const int32_t* fixtures, int32_t n, b2g_event* ended,
                                int32_t cap, int32_t* n_ended) {
  if (n_ended) *n_ended = 0;
  if (!b || cap < 0 || (cap > 0 && !ended)) return B2G_E_INVALID_ARG;
  TRY(remove_args_ok(b, world, fixtures, n, world_index_ok(b, world) ? b->worlds[world].fixtures.size() : 0));
  if (b->in_step) return locked(b);
  const HostWorld& w = b->worlds[world];
  std::vector<char> db(w.bodies.size(), 0), df(w.fixtures.size(), 0), dj(w.joints.size(), 0);
  for (int32_t i = 0; i < n; ++i) df[fixtures[i]] = 1;
  return remove_structure(b, world, std::move(db), std::move(df), std::move(dj), ended, cap, n_ended);
}

B2G_API int b2g_joints_remove(b2g_batch* b, int32_t world, const int32_t* joints, int32_t n) {
  if (!b) return B2G_E_INVALID_ARG;
  TRY(remove_args_ok(b, world, joints, n, world_index_ok(b, world) ? b->worlds[world].joints.size() : 0));
  if (b->in_step) return locked(b);
  const HostWorld& w = b->worlds[world];
  std::vector<char> db(w.bodies.size(), 0), df(w.fixtures.size(), 0), dj(w.joints.size(), 0);
  for (int32_t i = 0; i < n; ++i) dj[joints[i]] = 1;
  return remove_structure(b, world, std::move(db), std::move(df), std::move(dj), nullptr, 0, nullptr);
}

// ---- b2World::Dump (src/dynamics/b2_world.cpp:1469-1531): the world as C++ source that rebuilds it
// through the b2World API, in the reference's text format (an interchange format: the same lines,
// numbers printed with %.9g, bodies in the reference's list order - non-static bodies newest first,
// then static bodies oldest first - fixtures newest first, joints newest first with gears last).
namespace {
struct DumpText {
  std::string s;
  void operator()(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    const int n = vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (n > 0) s.append(buf, (size_t)std::min(n, (int)sizeof(buf) - 1));
  }
};
}  // namespace

static void dump_world(const HostWorld& w, DumpText& D) {
  const int nb = (int)w.bodies.size(), nj = (int)w.joints.size();
  D("b2Vec2 g(%.9g, %.9g);\n", w.gx, w.gy);
  D("m_world->SetGravity(g);\n");
  D("b2Body** bodies = (b2Body**)b2Alloc(%d * sizeof(b2Body*));\n", nb);
  D("b2Joint** joints = (b2Joint**)b2Alloc(%d * sizeof(b2Joint*));\n", nj);
  std::vector<int> order, index(nb);
  for (int i = nb - 1; i >= 0; --i)
    if (w.bodies[i].type != B2G_STATIC) order.push_back(i);
  for (int i = 0; i < nb; ++i)
    if (w.bodies[i].type == B2G_STATIC) order.push_back(i);
  for (int k = 0; k < nb; ++k) index[order[k]] = k;
  // reference b2Body flags (include/box2d/b2_body.h:478-484)
  auto flag = [](uint32_t f, uint32_t ours, int theirs) { return (f & ours) ? theirs : 0; };
  for (int k = 0; k < nb; ++k) {
    const b2g_body& b = w.bodies[order[k]];
    D("{\n");
    D("  b2BodyDef bd;\n");
    D("  bd.type = b2BodyType(%d);\n", b.type);
    D("  bd.position.Set(%.9g, %.9g);\n", b.xf[0], b.xf[1]);
    D("  bd.angle = %.9g;\n", b.a);
    D("  bd.linearVelocity.Set(%.9g, %.9g);\n", b.v[0], b.v[1]);
    D("  bd.angularVelocity = %.9g;\n", b.w);
    D("  bd.linearDamping = %.9g;\n", b.linear_damping);
    D("  bd.angularDamping = %.9g;\n", b.angular_damping);
    D("  bd.allowSleep = bool(%d);\n", flag(b.flags, B2G_BODY_AUTO_SLEEP, 0x0004));
    D("  bd.awake = bool(%d);\n", flag(b.flags, B2G_BODY_AWAKE, 0x0002));
    D("  bd.fixedRotation = bool(%d);\n", flag(b.flags, B2G_BODY_FIXED_ROTATION, 0x0010));
    D("  bd.bullet = bool(%d);\n", flag(b.flags, B2G_BODY_BULLET, 0x0008));
    D("  bd.enabled = bool(%d);\n", flag(b.flags, B2G_BODY_ENABLED, 0x0020));
    D("  bd.gravityScale = %.9g;\n", b.gravity_scale);
    D("  bodies[%d] = m_world->CreateBody(&bd);\n", k);
    D("\n");
    const std::vector<int>& fl = w.body_fixtures[order[k]];
    for (int q = (int)fl.size() - 1; q >= 0; --q) {
      const b2g_fixture& f = w.fixtures[fl[q]];
      const b2g_shape& sh = f.shape;
      D("  {\n");
      D("    b2FixtureDef fd;\n");
      D("    fd.friction = %.9g;\n", f.friction);
      D("    fd.restitution = %.9g;\n", f.restitution);
      D("    fd.restitutionThreshold = %.9g;\n", f.restitution_threshold);
      D("    fd.density = %.9g;\n", f.density);
      D("    fd.isSensor = bool(%d);\n", f.is_sensor ? 1 : 0);
      D("    fd.filter.categoryBits = uint16(%d);\n", (int)f.category_bits);
      D("    fd.filter.maskBits = uint16(%d);\n", (int)f.mask_bits);
      D("    fd.filter.groupIndex = int16(%d);\n", (int)f.group_index);
      if (sh.type == B2G_SHAPE_CIRCLE) {
        D("    b2CircleShape shape;\n");
        D("    shape.m_radius = %.9g;\n", sh.radius);
        D("    shape.m_p.Set(%.9g, %.9g);\n", sh.vertices[0][0], sh.vertices[0][1]);
      } else if (sh.type == B2G_SHAPE_EDGE) {  // record vertices: v1, v2, v0, v3
        D("    b2EdgeShape shape;\n");
        D("    shape.m_radius = %.9g;\n", sh.radius);
        D("    shape.m_vertex0.Set(%.9g, %.9g);\n", sh.vertices[2][0], sh.vertices[2][1]);
        D("    shape.m_vertex1.Set(%.9g, %.9g);\n", sh.vertices[0][0], sh.vertices[0][1]);
        D("    shape.m_vertex2.Set(%.9g, %.9g);\n", sh.vertices[1][0], sh.vertices[1][1]);
        D("    shape.m_vertex3.Set(%.9g, %.9g);\n", sh.vertices[3][0], sh.vertices[3][1]);
        D("    shape.m_oneSided = bool(%d);\n", sh.one_sided ? 1 : 0);
      } else {
        D("    b2PolygonShape shape;\n");
        D("    b2Vec2 vs[%d];\n", B2G_MAX_POLYGON_VERTICES);
        for (int i = 0; i < sh.count; ++i) D("    vs[%d].Set(%.9g, %.9g);\n", i, sh.vertices[i][0], sh.vertices[i][1]);
        D("    shape.Set(vs, %d);\n", sh.count);
      }
      D("\n");
      D("    fd.shape = &shape;\n");
      D("\n");
      D("    bodies[%d]->CreateFixture(&fd);\n", k);
      D("  }\n");
    }
    D("}\n");
  }
  auto joint = [&](int ji) {  // b2*Joint::Dump, the joint's index in the reference's list order
    const b2g_joint_def& d = w.joints[ji].def;
    const int jindex = nj - 1 - ji;
    D("{\n");
    const char* names[] = {"", "b2RevoluteJointDef", "b2PrismaticJointDef", "b2DistanceJointDef", "b2PulleyJointDef",
                           "", "b2GearJointDef", "b2WheelJointDef", "b2WeldJointDef", "b2FrictionJointDef", "", "b2MotorJointDef"};
    if (d.type != B2G_JOINT_MOUSE) {  // b2MouseJoint::Dump writes to the log only
      D("  %s jd;\n", names[d.type]);
      D("  jd.bodyA = bodies[%d];\n", index[d.body_a]);
      D("  jd.bodyB = bodies[%d];\n", index[d.body_b]);
      D("  jd.collideConnected = bool(%d);\n", d.collide_connected ? 1 : 0);
    }
    switch (d.type) {
      case B2G_JOINT_REVOLUTE:
        D("  jd.localAnchorA.Set(%.9g, %.9g);\n", d.local_anchor_a[0], d.local_anchor_a[1]);
        D("  jd.localAnchorB.Set(%.9g, %.9g);\n", d.local_anchor_b[0], d.local_anchor_b[1]);
        D("  jd.referenceAngle = %.9g;\n", d.reference_angle);
        D("  jd.enableLimit = bool(%d);\n", d.enable_limit ? 1 : 0);
        D("  jd.lowerAngle = %.9g;\n", d.lower);
        D("  jd.upperAngle = %.9g;\n", d.upper);
        D("  jd.enableMotor = bool(%d);\n", d.enable_motor ? 1 : 0);
        D("  jd.motorSpeed = %.9g;\n", d.motor_speed);
        D("  jd.maxMotorTorque = %.9g;\n", d.max_motor);
        break;
      case B2G_JOINT_PRISMATIC:
        D("  jd.localAnchorA.Set(%.9g, %.9g);\n", d.local_anchor_a[0], d.local_anchor_a[1]);
        D("  jd.localAnchorB.Set(%.9g, %.9g);\n", d.local_anchor_b[0], d.local_anchor_b[1]);
        D("  jd.localAxisA.Set(%.9g, %.9g);\n", d.local_axis_a[0], d.local_axis_a[1]);
        D("  jd.referenceAngle = %.9g;\n", d.reference_angle);
        D("  jd.enableLimit = bool(%d);\n", d.enable_limit ? 1 : 0);
        D("  jd.lowerTranslation = %.9g;\n", d.lower);
        D("  jd.upperTranslation = %.9g;\n", d.upper);
        D("  jd.enableMotor = bool(%d);\n", d.enable_motor ? 1 : 0);
        D("  jd.motorSpeed = %.9g;\n", d.motor_speed);
        D("  jd.maxMotorForce = %.9g;\n", d.max_motor);
        break;
      case B2G_JOINT_DISTANCE:
        D("  jd.localAnchorA.Set(%.9g, %.9g);\n", d.local_anchor_a[0], d.local_anchor_a[1]);
        D("  jd.localAnchorB.Set(%.9g, %.9g);\n", d.local_anchor_b[0], d.local_anchor_b[1]);
        D("  jd.length = %.9g;\n", d.length);
        D("  jd.minLength = %.9g;\n", d.min_length);
        D("  jd.maxLength = %.9g;\n", d.max_length);
        D("  jd.stiffness = %.9g;\n", d.stiffness);
        D("  jd.damping = %.9g;\n", d.damping);
        break;
      case B2G_JOINT_WELD:
        D("  jd.localAnchorA.Set(%.9g, %.9g);\n", d.local_anchor_a[0], d.local_anchor_a[1]);
        D("  jd.localAnchorB.Set(%.9g, %.9g);\n", d.local_anchor_b[0], d.local_anchor_b[1]);
        D("  jd.referenceAngle = %.9g;\n", d.reference_angle);
        D("  jd.stiffness = %.9g;\n", d.stiffness);
        D("  jd.damping = %.9g;\n", d.damping);
        break;
      case B2G_JOINT_WHEEL:
        D("  jd.localAnchorA.Set(%.9g, %.9g);\n", d.local_anchor_a[0], d.local_anchor_a[1]);
        D("  jd.localAnchorB.Set(%.9g, %.9g);\n", d.local_anchor_b[0], d.local_anchor_b[1]);
        D("  jd.localAxisA.Set(%.9g, %.9g);\n", d.local_axis_a[0], d.local_axis_a[1]);
        D("  jd.enableMotor = bool(%d);\n", d.enable_motor ? 1 : 0);
        D("  jd.motorSpeed = %.9g;\n", d.motor_speed);
        D("  jd.maxMotorTorque = %.9g;\n", d.max_motor);
        D("  jd.stiffness = %.9g;\n", d.stiffness);
        D("  jd.damping = %.9g;\n", d.damping);
        break;
      case B2G_JOINT_MOTOR:
        D("  jd.linearOffset.Set(%.9g, %.9g);\n", d.linear_offset[0], d.linear_offset[1]);
        D("  jd.angularOffset = %.9g;\n", d.reference_angle);
        D("  jd.maxForce = %.9g;\n", d.max_force);
        D("  jd.maxTorque = %.9g;\n", d.max_torque);
        D("  jd.correctionFactor = %.9g;\n", d.correction_factor);
        break;
      case B2G_JOINT_FRICTION:
        D("  jd.localAnchorA.Set(%.9g, %.9g);\n", d.local_anchor_a[0], d.local_anchor_a[1]);
        D("  jd.localAnchorB.Set(%.9g, %.9g);\n", d.local_anchor_b[0], d.local_anchor_b[1]);
        D("  jd.maxForce = %.9g;\n", d.max_force);
        D("  jd.maxTorque = %.9g;\n", d.max_torque);
        break;
      case B2G_JOINT_PULLEY:
        D("  jd.groundAnchorA.Set(%.9g, %.9g);\n", d.ground_anchor_a[0], d.ground_anchor_a[1]);
        D("  jd.groundAnchorB.Set(%.9g, %.9g);\n", d.ground_anchor_b[0], d.ground_anchor_b[1]);
        D("  jd.localAnchorA.Set(%.9g, %.9g);\n", d.local_anchor_a[0], d.local_anchor_a[1]);
        D("  jd.localAnchorB.Set(%.9g, %.9g);\n", d.local_anchor_b[0], d.local_anchor_b[1]);
        D("  jd.lengthA = %.9g;\n", d.length_a);
        D("  jd.lengthB = %.9g;\n", d.length_b);
        D("  jd.ratio = %.9g;\n", d.ratio);
        break;
      case B2G_JOINT_GEAR:
        D("  jd.joint1 = joints[%d];\n", nj - 1 - d.joint_1);
        D("  jd.joint2 = joints[%d];\n", nj - 1 - d.joint_2);
        D("  jd.ratio = %.9g;\n", d.ratio);
        break;
      default:
        break;
    }
    if (d.type != B2G_JOINT_MOUSE) D("  joints[%d] = m_world->CreateJoint(&jd);\n", jindex);
    D("}\n");
  };
  for (int ji = nj - 1; ji >= 0; --ji)
    if (w.joints[ji].def.type != B2G_JOINT_GEAR) joint(ji);
  for (int ji = nj - 1; ji >= 0; --ji)
    if (w.joints[ji].def.type == B2G_JOINT_GEAR) joint(ji);
  D("b2Free(joints);\n");
  D("b2Free(bodies);\n");
  D("joints = nullptr;\n");
  D("bodies = nullptr;\n");
}

B2G_API int b2g_world_dump(b2g_batch* b, int32_t world, char* out, uint64_t cap, uint64_t* n) {
  if (!world_index_ok(b, world) || !n || (cap > 0 && !out)) return B2G_E_INVALID_ARG;
  if (world < b->NW) TRY(download_state(b));
  DumpText D;
  dump_world(b->worlds[world], D);
  *n = D.s.size();
  if (cap > 0) {
    const size_t k = std::min<size_t>(D.s.size(), (size_t)cap - 1);
    memcpy(out, D.s.data(), k);
    out[k] = 0;
  }
  return D.s.size() < cap ? B2G_OK : B2G_E_CAPACITY;
}

B2G_API int b2g_world_sizes(b2g_batch* b, int32_t world, int32_t* bodies, int32_t* fixtures, int32_t* joints,
                            int32_t* contacts) {
  if (!world_index_ok(b, world)) return B2G_E_INVALID_ARG;
  const HostWorld& w = b->worlds[world];
  if (bodies) *bodies = (int32_t)w.bodies.size();
  if (fixtures) *fixtures = (int32_t)w.fixtures.size();
  if (joints) *joints = (int32_t)w.joints.size();
  if (contacts) {
    if (b->host_state_stale && !b->structure_dirty && world < b->NW) {
      std::vector<int2> wc(b->NW);
      if (cudaMemcpy(wc.data(), b->wc.p, b->NW * sizeof(int2), cudaMemcpyDeviceToHost) != cudaSuccess) return B2G_E_CUDA;
      *contacts = wc[world].y;
    } else {
      *contacts = (int32_t)w.contacts.size();
    }
  }
  return B2G_OK;
}

B2G_API int b2g_step(b2g_batch* b, float dt, int32_t vi, int32_t pi, const uint8_t* world_mask) {
  if (!b) return B2G_E_INVALID_ARG;
  return step_batch(b, dt, vi, pi, world_mask, true);
}

B2G_API int b2g_step_begin(b2g_batch* b, float dt, int32_t vi, int32_t pi, const uint8_t* world_mask) {
  if (!b) return B2G_E_INVALID_ARG;
  return step_begin(b, dt, vi, pi, world_mask);
}

B2G_API int b2g_step_poll(b2g_batch* b, int32_t* done) {
  if (!b || !done) return B2G_E_INVALID_ARG;
  if (!b->in_step) {
    *done = 1;
    return B2G_OK;
  }
  cudaError_t e = cudaEventQuery(b->ev[5]);
  if (e == cudaErrorNotReady) {
    *done = 0;
    return B2G_OK;
  }
  CUDA_TRY(b, e);
  *done = 1;
  return B2G_OK;
}

B2G_API int b2g_step_end(b2g_batch* b) {
  if (!b) return B2G_E_INVALID_ARG;
  return step_end(b);
}

B2G_API int b2g_batch_stage(b2g_batch* b) {
  if (!b) return B2G_E_INVALID_ARG;
  if (b->device < 0 || b->structure_dirty || (int)b->worlds.size() <= b->NW) return B2G_OK;
  return pack_tail(b, b->tail_pack);
}

B2G_API int b2g_step_n(b2g_batch* b, float dt, int32_t vi, int32_t pi, int32_t n, int32_t use_graph) {
  if (!b || n < 0) return B2G_E_INVALID_ARG;
  bool saved = b->use_graphs;
  b->use_graphs = use_graph != 0;
  int st = B2G_OK;
  for (int i = 0; i < n && st == B2G_OK; ++i) st = step_batch(b, dt, vi, pi, nullptr, i == n - 1);
  b->use_graphs = saved;
  return st;
}

B2G_API int b2g_debug_set_contact_capacity(b2g_batch* b, int64_t cap) {
  if (!b || cap < 1 || b->device < 0) return B2G_E_INVALID_ARG;
  if (b->structure_dirty) TRY(upload_all(b));
  if (cap < b->NC) return B2G_E_INVALID_ARG;
  // shrink: reallocate every contact-sized buffer at exactly `cap` (the live list is kept)
  for (int k = 0; k < 2; ++k) {
    bool keep = (k == b->cur);
    TRY(resize_exact(b, b->ckey[k], (size_t)cap, keep)); TRY(resize_exact(b, b->cfix[k], (size_t)cap, keep));
    TRY(resize_exact(b, b->cflags[k], (size_t)cap, keep)); TRY(resize_exact(b, b->cmat[k], (size_t)cap, keep));
    TRY(resize_exact(b, b->cman[k], (size_t)cap, keep));
  }
  TRY(resize_exact(b, b->pairs, (size_t)cap, false));
  b->ccap = cap;
  b->layout_version++;
  return B2G_OK;
}

B2G_API int b2g_batch_set_graphs(b2g_batch* b, int32_t enable) {
  if (!b) return B2G_E_INVALID_ARG;
  b->use_graphs = enable != 0;
  return B2G_OK;
}

B2G_API int b2g_batch_set_debug_checks(b2g_batch* b, int32_t enable) {
  if (!b) return B2G_E_INVALID_ARG;
  if (b->debug_checks != (enable != 0)) b->layout_version++;  // captured graphs lack or hold the check
  b->debug_checks = enable != 0;
  return B2G_OK;
}

B2G_API int b2g_batch_set_solver_threads(b2g_batch* b, const int32_t* threads) {
  if (!b || !threads) return B2G_E_INVALID_ARG;
  for (int c = 0; c < B2G_SOLVE_CLASSES; ++c)
    if (!solver_threads_valid(threads[c])) return B2G_E_INVALID_ARG;
  for (int c = 0; c < B2G_SOLVE_CLASSES; ++c) b->class_threads[c] = threads[c];
  if (!b->h_world_order.empty()) {
    replan_solver(b);
    b->layout_version++;  // captured graphs hold the old launch shapes
  }
  return B2G_OK;
}

B2G_API int b2g_batch_set_tree_rebuild_period(b2g_batch* b, int32_t period) {
  if (!b || period < 1) return B2G_E_INVALID_ARG;
  b->tree_period = period;
  return B2G_OK;
}

B2G_API int b2g_batch_set_solver_waves(b2g_batch* b, float waves) {
  if (!b || !(waves >= 0.0f)) return B2G_E_INVALID_ARG;
  b->wide_waves = waves;
  if (!b->h_world_order.empty()) {
    replan_solver(b);
    b->layout_version++;  // captured graphs hold the old launch shapes
  }
  return B2G_OK;
}

B2G_API int b2g_batch_set_cluster_solve(b2g_batch* b, int32_t ctas) {
  if (!b || !(ctas == -1 || ctas == 0 || ctas == 1 || ctas == 2 || ctas == 4 || ctas == 8 || ctas == 16))
    return B2G_E_INVALID_ARG;
  b->cluster_ctas = ctas;
  if (!b->h_world_order.empty()) {
    replan_solver(b);
    b->layout_version++;  // captured graphs hold the old launch shapes
  }
  return B2G_OK;
}

B2G_API int b2g_batch_get_cluster_solve(b2g_batch* b, int32_t* ctas) {
  if (!b || !ctas) return B2G_E_INVALID_ARG;
  const int dmax = solver_max_cluster_ctas();
  const int c = b->cluster_ctas < 0 ? dmax : std::min(b->cluster_ctas, dmax);
  *ctas = c > 1 ? c : 1;
  return B2G_OK;
}

B2G_API int b2g_batch_get_solver_threads(b2g_batch* b, int32_t* threads) {
  if (!b || !threads) return B2G_E_INVALID_ARG;
  for (int c = 0; c < B2G_SOLVE_CLASSES; ++c) threads[c] = b->class_threads[c];
  return B2G_OK;
}

// Median device time of the solver over `steps` eager steps (real steps: the worlds advance).
static int time_solver(Batch* b, int steps, float dt, int vi, int pi, float* ms, int* taken) {
  std::vector<float> t;
  for (int i = 0; i < steps; ++i) {
    TRY(step_batch(b, dt, vi, pi, nullptr, true));
    ++*taken;
    t.push_back(b->profile.solve);
  }
  std::sort(t.begin(), t.end());
  *ms = t.empty() ? 0.0f : t[t.size() / 2];
  return B2G_OK;
}

B2G_API int b2g_batch_autotune(b2g_batch* b, int32_t steps, float dt, int32_t vi, int32_t pi, int32_t* threads_out,
                               int32_t* steps_taken) {
  if (!b || steps < 1 || !(dt > 0.0f) || vi < 0 || pi < 0 || b->device < 0) return B2G_E_INVALID_ARG;
  bool graphs = b->use_graphs;
  b->use_graphs = false;  // eager steps carry the per-phase events
  int st = B2G_OK;
  int taken = 0;
  if (b->structure_dirty || (int)b->worlds.size() > b->NW) {
    st = step_batch(b, dt, vi, pi, nullptr, true);
    ++taken;
  }
  // coordinate descent, largest worlds first: each class tries half and double its threads
  for (int c = B2G_SOLVE_CLASSES - 1; c >= 0 && st == B2G_OK; --c) {
    bool present = false;
    for (const SolveClass& k : b->solve_classes) present = present || k.cls == c;
    if (!present) continue;
    int best = b->class_threads[c];
    float best_ms = 0.0f;
    st = time_solver(b, steps, dt, vi, pi, &best_ms, &taken);
    for (int cand : {best / 2, best * 2}) {
      if (st != B2G_OK || !solver_threads_valid(cand)) continue;
      int keep = b->class_threads[c];
      b->class_threads[c] = cand;
      replan_solver(b);
      float ms = 0.0f;
      st = time_solver(b, steps, dt, vi, pi, &ms, &taken);
      if (st == B2G_OK && ms < 0.97f * best_ms) {
        best = cand;
        best_ms = ms;
      } else {
        b->class_threads[c] = keep;
        replan_solver(b);
      }
    }
    b->class_threads[c] = best;
    replan_solver(b);
  }
  b->layout_version++;
  b->use_graphs = graphs;
  if (threads_out)
    for (int c = 0; c < B2G_SOLVE_CLASSES; ++c) threads_out[c] = b->class_threads[c];
  if (steps_taken) *steps_taken = taken;
  return st;
}

B2G_API int b2g_step_timed(b2g_batch* b, float dt, int32_t vi, int32_t pi, int32_t n, float* device_ms) {
  if (!b || n < 0 || b->device < 0) return B2G_E_INVALID_ARG;
  if (b->structure_dirty) TRY(upload_all(b));
  cudaEvent_t e0, e1;
  cudaSetDevice(b->device);
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, b->stream);
  int st = B2G_OK;
  for (int i = 0; i < n && st == B2G_OK; ++i) st = step_batch(b, dt, vi, pi, nullptr, i == n - 1);
  cudaEventRecord(e1, b->stream);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (device_ms) *device_ms = ms;
  return st;
}

B2G_API int b2g_batch_set_forces(b2g_batch* b, const float* f4, int64_t n_bodies) {
  if (!b || !f4 || n_bodies < 0 || b->device < 0) return B2G_E_INVALID_ARG;
  if (b->in_step) return locked(b);
  if (b->structure_dirty) TRY(upload_all(b));
  if (n_bodies != b->NB) return B2G_E_INVALID_ARG;
  if (n_bodies) CUDA_TRY(b, cudaMemcpyAsync(b->force.p, f4, n_bodies * sizeof(float4), cudaMemcpyHostToDevice, b->stream));
  b->host_state_stale = true;
  return B2G_OK;
}

B2G_API int b2g_reserve(b2g_batch* b, int64_t contacts) {
  if (!b || contacts < 0 || b->device < 0) return B2G_E_INVALID_ARG;
  if (b->structure_dirty) TRY(upload_all(b));
  return ensure_contact_capacity(b, contacts);
}

B2G_API int b2g_bodies_read(b2g_batch* b, int32_t world, int32_t first, int32_t n, b2g_body* out) {
  if (!world_index_ok(b, world) || first < 0 || n < 0 || (n > 0 && !out)) return B2G_E_INVALID_ARG;
  const HostWorld& w = b->worlds[world];
  if (first + n > (int)w.bodies.size()) return B2G_E_INVALID_ARG;
  if (b->in_step && world < b->NW) return locked(b);
  for (int i = 0; i < n; ++i) out[i] = w.bodies[first + i];
  if (n > 0 && b->host_state_stale && b->device_state_valid && world < b->NW) {
    // the host copy is older than the device: fetch this world's slice only
    int bo = b->h_body_off[world] + first;
    std::vector<float4> xf(n), pos(n), vel(n), force(n);
    std::vector<int2> bst(n);
    CUDA_TRY(b, cudaMemcpyAsync(bst.data(), b->bstate.p + bo, n * sizeof(int2), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(b, cudaMemcpyAsync(xf.data(), b->xf.p + bo, n * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(b, cudaMemcpyAsync(pos.data(), b->pos.p + bo, n * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(b, cudaMemcpyAsync(vel.data(), b->vel.p + bo, n * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(b, cudaMemcpyAsync(force.data(), b->force.p + bo, n * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(b, cudaStreamSynchronize(b->stream));
    for (int i = 0; i < n; ++i) {
      b2g_body& r = out[i];
      r.xf[0] = xf[i].x; r.xf[1] = xf[i].y; r.xf[2] = xf[i].z; r.xf[3] = xf[i].w;
      r.c[0] = pos[i].x; r.c[1] = pos[i].y; r.a = pos[i].z;
      r.v[0] = vel[i].x; r.v[1] = vel[i].y; r.w = vel[i].z;
      r.force[0] = force[i].x; r.force[1] = force[i].y; r.torque = force[i].z;
      if (r.type != B2G_STATIC)
        r.flags = (r.flags & ~B2G_BODY_AWAKE) | ((bst[i].x & B2G_BS_AWAKE) ? B2G_BODY_AWAKE : 0u);
    }
  }
  return B2G_OK;
}

// b2Body::SetTransform / SetLinearVelocity / SetAngularVelocity / ApplyForce: kinematic state of
// each record is taken as given (xf, c, a, v, w, force, torque); a moved body's fixtures get
// their contacts re-found at the start of the next step (b2_body.cpp:482-504).
B2G_API int b2g_bodies_write(b2g_batch* b, int32_t world, int32_t first, int32_t n, const b2g_body* in) {
  if (!world_index_ok(b, world) || first < 0 || n < 0 || (n > 0 && !in)) return B2G_E_INVALID_ARG;
  HostWorld& w0 = b->worlds[world];
  if (first + n > (int)w0.bodies.size()) return B2G_E_INVALID_ARG;
  if (world < b->NW) TRY(begin_edit(b));
  else b->tail_pack.valid = false;  // not on the device yet: its host records are the state
  HostWorld& w = b->worlds[world];
  for (int i = 0; i < n; ++i) {
    b2g_body& r = w.bodies[first + i];
    const b2g_body& s = in[i];
    memcpy(r.xf, s.xf, sizeof(r.xf));
    memcpy(r.c, s.c, sizeof(r.c));
    r.a = s.a;
    memcpy(r.v, s.v, sizeof(r.v));
    r.w = s.w;
    memcpy(r.force, s.force, sizeof(r.force));
    r.torque = s.torque;
    // b2Body::SetLinearVelocity / SetAngularVelocity: a non-zero velocity wakes the body and
    // restarts its sleep timer (include/box2d/b2_body.h:580-612)
    if (r.type != B2G_STATIC && (r.v[0] * r.v[0] + r.v[1] * r.v[1] > 0.0f || r.w * r.w > 0.0f)) {
      r.flags |= B2G_BODY_AWAKE;
      if ((size_t)(first + i) < w.body_sleep.size()) w.body_sleep[first + i] = 0.0f;
    }
  }
  w.flags |= B2G_WF_NEW_CONTACTS;
  return B2G_OK;
}

// b2Body::SetAwake (include/box2d/b2_body.h:719-740); a static body ignores it.
B2G_API int b2g_body_set_awake(b2g_batch* b, int32_t world, int32_t body, int32_t awake) {
  if (!world_index_ok(b, world) || body < 0 || body >= (int32_t)b->worlds[world].bodies.size())
    return B2G_E_INVALID_ARG;
  if (world < b->NW) TRY(begin_edit(b));
  else b->tail_pack.valid = false;  // not on the device yet: its host records are the state
  HostWorld& w = b->worlds[world];
  b2g_body& r = w.bodies[body];
  if (r.type == B2G_STATIC) return B2G_OK;
  w.body_sleep.resize(w.bodies.size(), 0.0f);
  w.body_sleep[body] = 0.0f;
  if (awake) {
    r.flags |= B2G_BODY_AWAKE;
  } else {
    r.flags &= ~B2G_BODY_AWAKE;
    r.v[0] = r.v[1] = r.w = 0.0f;
    r.force[0] = r.force[1] = r.torque = 0.0f;
    w.sleepers = true;
  }
  return B2G_OK;
}

B2G_API int b2g_body_set_bullet(b2g_batch* b, int32_t world, int32_t body, int32_t bullet) {
  if (!world_index_ok(b, world) || body < 0 || body >= (int32_t)b->worlds[world].bodies.size())
    return B2G_E_INVALID_ARG;
  if (world < b->NW) TRY(begin_edit(b));
  else b->tail_pack.valid = false;
  b2g_body& r = b->worlds[world].bodies[body];
  if (bullet) r.flags |= B2G_BODY_BULLET;
  else r.flags &= ~B2G_BODY_BULLET;
  return B2G_OK;
}

// b2Body::m_sleepTime of n bodies from `first` (no public getter in the reference; exposed for
// checkpoint tooling and tests).
B2G_API int b2g_bodies_sleep_time_read(b2g_batch* b, int32_t world, int32_t first, int32_t n, float* out) {
  if (!world_index_ok(b, world) || first < 0 || n < 0 || (n > 0 && !out)) return B2G_E_INVALID_ARG;
  if (world < b->NW) TRY(download_state(b));  // a world not on the device yet is its host records
  HostWorld& w = b->worlds[world];
  if (first + n > (int)w.bodies.size()) return B2G_E_INVALID_ARG;
  for (int i = 0; i < n; ++i) out[i] = (size_t)(first + i) < w.body_sleep.size() ? w.body_sleep[first + i] : 0.0f;
  return B2G_OK;
}

B2G_API int b2g_batch_read_states(b2g_batch* b, float* xf4, float* v3, int64_t cap_bodies, int64_t* n_bodies) {
  if (!b) return B2G_E_INVALID_ARG;
  if (b->in_step) return locked(b);
  if (b->structure_dirty) TRY(upload_all(b));
  if (n_bodies) *n_bodies = b->NB;
  int64_t n = std::min<int64_t>(cap_bodies, b->NB);
  if (n <= 0) return B2G_OK;
  cudaSetDevice(b->device);
  if (xf4) CUDA_TRY(b, cudaMemcpyAsync(xf4, b->xf.p, n * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
  if (v3) {
    std::vector<float4> v(n);
    CUDA_TRY(b, cudaMemcpyAsync(v.data(), b->vel.p, n * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(b, cudaStreamSynchronize(b->stream));
    for (int64_t i = 0; i < n; ++i) { v3[3 * i] = v[i].x; v3[3 * i + 1] = v[i].y; v3[3 * i + 2] = v[i].z; }
  }
  CUDA_TRY(b, cudaStreamSynchronize(b->stream));
  return B2G_OK;
}

B2G_API int b2g_step_io(b2g_batch* b, float dt, int32_t vi, int32_t pi, const float* f4, int64_t n_bodies,
                        float* xf4_out, int64_t cap_bodies, int64_t* n_out) {
  if (!b || b->device < 0 || (f4 && n_bodies < 0) || (xf4_out && cap_bodies < 0)) return B2G_E_INVALID_ARG;
  if (b->in_step) return locked(b);
  if (b->structure_dirty) TRY(upload_all(b));
  if (f4 && n_bodies != b->NB) return B2G_E_INVALID_ARG;
  cudaSetDevice(b->device);
  if (f4 && n_bodies) {
    // the previous step is complete (b2g_step_io and b2g_step return after it): nothing reads the
    // forces while they are copied
    CUDA_TRY(b, cudaMemcpyAsync(b->force.p, f4, n_bodies * sizeof(float4), cudaMemcpyHostToDevice, b->io_stream));
    CUDA_TRY(b, cudaEventRecord(b->io_in, b->io_stream));
    b->host_state_stale = true;
  }
  int st = step_begin(b, dt, vi, pi, nullptr);
  if (st != B2G_OK) {
    cudaStreamSynchronize(b->io_stream);
    return st;
  }
  const int64_t n = std::min<int64_t>(cap_bodies, b->NB);
  // after the solve wrote the transforms; the closing broadphase only reads them (a step with
  // continuous collision moves bodies again after it: its transforms are read at the end)
  const bool early = !b->step_ccd;
  if (xf4_out && n > 0 && early) {
    CUDA_TRY(b, cudaStreamWaitEvent(b->io_stream, b->io_solved, 0));
    CUDA_TRY(b, cudaMemcpyAsync(xf4_out, b->xf.p, n * sizeof(float4), cudaMemcpyDeviceToHost, b->io_stream));
  }
  st = step_end(b);
  if (xf4_out && n > 0 && !early && st == B2G_OK) {
    CUDA_TRY(b, cudaMemcpyAsync(xf4_out, b->xf.p, n * sizeof(float4), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(b, cudaStreamSynchronize(b->stream));
  }
  CUDA_TRY(b, cudaStreamSynchronize(b->io_stream));
  if (n_out) *n_out = b->NB;
  return st;
}

B2G_API int b2g_fixtures_read(b2g_batch* b, int32_t world, int32_t first, int32_t n, b2g_fixture* out) {
  if (!world_index_ok(b, world) || first < 0 || n < 0 || (n > 0 && !out)) return B2G_E_INVALID_ARG;
  const HostWorld& w = b->worlds[world];
  if (first + n > (int)w.fixtures.size()) return B2G_E_INVALID_ARG;
  for (int i = 0; i < n; ++i) out[i] = w.fixtures[first + i];
  return B2G_OK;
}

B2G_API int b2g_joints_read(b2g_batch* b, int32_t world, int32_t first, int32_t n, b2g_joint* out) {
  if (!world_index_ok(b, world) || first < 0 || n < 0 || (n > 0 && !out)) return B2G_E_INVALID_ARG;
  if (world < b->NW) TRY(download_state(b));  // a world not on the device yet is its host records
  const HostWorld& w = b->worlds[world];
  if (first + n > (int)w.joints.size()) return B2G_E_INVALID_ARG;
  for (int i = 0; i < n; ++i) out[i] = w.joints[first + i];
  return B2G_OK;
}

B2G_API int b2g_contacts_read(b2g_batch* b, int32_t world, b2g_contact* out, int32_t cap, int32_t* n) {
  if (!world_index_ok(b, world) || !n) return B2G_E_INVALID_ARG;
  if (world < b->NW) TRY(download_state(b));  // a world not on the device yet is its host records
  const HostWorld& w = b->worlds[world];
  *n = (int32_t)w.contacts.size();
  if (out)
    for (int i = 0; i < *n && i < cap; ++i) out[i] = w.contacts[i];
  return B2G_OK;
}

B2G_API int b2g_events_enable(b2g_batch* b, int32_t enable) {
  if (!b) return B2G_E_INVALID_ARG;
  b->events_on = enable != 0;
  b->host_events.clear();
  return B2G_OK;
}

// Delivery order of the step's events: grouped per world; Begin, End, PreSolve, PostSolve; then
// by fixture pair.
static void sort_events(std::vector<b2g_event>& ev) {
  std::stable_sort(ev.begin(), ev.end(), [](const b2g_event& x, const b2g_event& y) {
    if (x.world != y.world) return x.world < y.world;
    if (x.kind != y.kind) return x.kind < y.kind;
    if (x.fixture_a != y.fixture_a) return x.fixture_a < y.fixture_a;
    return x.fixture_b < y.fixture_b;
  });
}

B2G_API int b2g_events_drain(b2g_batch* b, b2g_event* out, int32_t cap, int32_t* n) {
  if (!b || !n) return B2G_E_INVALID_ARG;
  std::vector<b2g_event>& ev = b->host_events;
  sort_events(ev);
  *n = (int32_t)std::min<size_t>(ev.size(), (size_t)std::max(cap, 0));
  if (out)
    for (int i = 0; i < *n; ++i) out[i] = ev[i];
  ev.erase(ev.begin(), ev.begin() + *n);
  return B2G_OK;
}

B2G_API int b2g_events_drain_world(b2g_batch* b, int32_t world, b2g_event* out, int32_t cap, int32_t* n) {
  if (!world_index_ok(b, world) || !n || cap < 0 || (cap > 0 && !out)) return B2G_E_INVALID_ARG;
  std::vector<b2g_event>& ev = b->host_events;
  sort_events(ev);
  auto lo = std::lower_bound(ev.begin(), ev.end(), world, [](const b2g_event& e, int32_t w) { return e.world < w; });
  auto hi = std::upper_bound(lo, ev.end(), world, [](int32_t w, const b2g_event& e) { return w < e.world; });
  const int32_t take = (int32_t)std::min<ptrdiff_t>(hi - lo, cap);
  for (int32_t i = 0; i < take; ++i) out[i] = lo[i];
  ev.erase(lo, lo + take);
  *n = take;
  return B2G_OK;
}

B2G_API int b2g_profile_get(b2g_batch* b, b2g_profile* out) {
  if (!b || !out) return B2G_E_INVALID_ARG;
  *out = b->profile;
  return B2G_OK;
}

B2G_API int b2g_solver_order(b2g_batch* b, int32_t world, int32_t* contact_color, uint32_t* contact_priority,
                             int32_t nc, int32_t* joint_color, uint32_t* joint_priority, int32_t nj) {
  if (!world_index_ok(b, world) || nc < 0 || nj < 0) return B2G_E_INVALID_ARG;
  if (b->device < 0 || b->structure_dirty || world >= b->NW) return B2G_E_INVALID_ARG;
  CUDA_TRY(b, cudaSetDevice(b->device));
  cudaStream_t s = b->stream;
  int w = world;
  // joints: colours and priorities fixed for the layout
  int j0 = b->h_joint_off[w], njw = b->h_joint_off[w + 1] - j0;
  int jn = std::min(nj, njw);
  std::vector<int8_t> jc(std::max(jn, 1));
  if (jn > 0) {
    CUDA_TRY(b, cudaMemcpyAsync(jc.data(), b->jcol.p + j0, jn, cudaMemcpyDeviceToHost, s));
    if (joint_priority) CUDA_TRY(b, cudaMemcpyAsync(joint_priority, b->jprio.p + j0, jn * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  }
  // contacts: the last solve's solver contacts, matched by key into the current contact list
  int info[4] = {0, 0, 0, 0};
  int2 wcw = make_int2(0, 0);
  CUDA_TRY(b, cudaMemcpyAsync(info, b->ncolors.p + 4 * w, sizeof(info), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(b, cudaMemcpyAsync(&wcw, b->wc.p + w, sizeof(int2), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(b, cudaStreamSynchronize(s));
  for (int j = 0; j < jn; ++j)
    if (joint_color) joint_color[j] = jc[j];
  int nsc = b->last_solve_buf < 0 ? 0 : info[2], base = info[3];
  std::vector<int> sl(std::max(nsc, 1));
  std::vector<int8_t> cc(std::max(nsc, 1));
  std::vector<uint32_t> cp(std::max(nsc, 1));
  std::vector<uint64_t> cur_keys(std::max(wcw.y, 1));
  if (nsc > 0) {
    CUDA_TRY(b, cudaMemcpyAsync(sl.data(), b->sc_list.p + base, nsc * sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(cc.data(), b->ccol.p + base, nsc, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaMemcpyAsync(cp.data(), b->cprio.p + base, nsc * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  }
  if (wcw.y > 0)
    CUDA_TRY(b, cudaMemcpyAsync(cur_keys.data(), b->ckey[b->cur].p + wcw.x, wcw.y * sizeof(uint64_t),
                                cudaMemcpyDeviceToHost, s));
  CUDA_TRY(b, cudaStreamSynchronize(s));
  // keys of the solved contacts in the list the solve read (their indices span one world range)
  std::vector<uint64_t> old_keys(std::max(nsc, 1));
  if (nsc > 0) {
    int lo = *std::min_element(sl.begin(), sl.begin() + nsc), hi = *std::max_element(sl.begin(), sl.begin() + nsc);
    std::vector<uint64_t> span(hi - lo + 1);
    CUDA_TRY(b, cudaMemcpyAsync(span.data(), b->ckey[b->last_solve_buf].p + lo, span.size() * sizeof(uint64_t),
                                cudaMemcpyDeviceToHost, s));
    CUDA_TRY(b, cudaStreamSynchronize(s));
    for (int k = 0; k < nsc; ++k) old_keys[k] = span[sl[k] - lo];
  }
  int cn = std::min(nc, wcw.y);
  for (int i = 0; i < cn; ++i) {
    if (contact_color) contact_color[i] = -1;
    if (contact_priority) contact_priority[i] = 0;
  }
  for (int k = 0; k < nsc; ++k) {
    auto it = std::lower_bound(cur_keys.begin(), cur_keys.begin() + wcw.y, old_keys[k]);
    if (it == cur_keys.begin() + wcw.y || *it != old_keys[k]) continue;
    int i = (int)(it - cur_keys.begin());
    if (i >= cn) continue;
    if (contact_color) contact_color[i] = cc[k];
    if (contact_priority) contact_priority[i] = cp[k];
  }
  return B2G_OK;
}

// The per-world trees for queries: pending host edits are uploaded, and when the trees are stale
// (re-layout, compaction) the broadphase rebuilds them without touching the contact list.
static int ensure_query_trees(Batch* b) {
  if (b->device < 0) return B2G_E_INVALID_ARG;
  if (b->in_step) return locked(b);
  CUDA_TRY(b, cudaSetDevice(b->device));
  if (b->structure_dirty) {
    TRY(upload_all(b));
    invalidate_graphs(b);
  } else if ((int)b->worlds.size() > b->NW) {
    TRY(upload_tail(b));  // the appended worlds still get their contacts from the next step
    invalidate_graphs(b);
    b->tree_valid = false;
  }
  if (!b->tree_valid && b->NF > 0) {
    KernelArgs a = step_args(b, 0.0f, 0, 0);
    launch_bp_build(a, b->NF, b->NW, b->cub_tmp.cap, sort_bits(b), b->stream, false);
    CUDA_TRY(b, cudaGetLastError());
    bp_done(b, BP_FULL);
  }
  b->tree_valid = true;
  CUDA_TRY(b, cudaMemsetAsync(b->status.p, 0, sizeof(unsigned int), b->stream));
  return B2G_OK;
}

static int query_status(Batch* b) {
  unsigned int st = 0;
  CUDA_TRY(b, cudaMemcpyAsync(&st, b->status.p, sizeof(st), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(b, cudaStreamSynchronize(b->stream));
  return check_status(b, st);
}

B2G_API int b2g_query_aabb(b2g_batch* b, const int32_t* worlds, const float* boxes, int32_t n, int32_t* counts,
                           int32_t* fixtures, int64_t cap, int64_t* total) {
  if (!b || n < 0 || (n > 0 && (!worlds || !boxes || !counts)) || cap < 0 || (cap > 0 && !fixtures) || !total)
    return B2G_E_INVALID_ARG;
  *total = 0;
  if (n == 0) return B2G_OK;
  NvtxRange range("b2g.query_aabb");
  TRY(ensure_query_trees(b));
  cudaStream_t s = b->stream;
  TRY(ensure(b, b->q_world, n)); TRY(ensure(b, b->q_box, n)); TRY(ensure(b, b->q_counts, n));
  CUDA_TRY(b, cudaMemcpyAsync(b->q_world.p, worlds, n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  CUDA_TRY(b, cudaMemcpyAsync(b->q_box.p, boxes, n * sizeof(float4), cudaMemcpyHostToDevice, s));
  KernelArgs a = step_args(b, 0.0f, 0, 0);
  launch_query_count(a, n, b->q_world.p, b->q_box.p, b->q_counts.p, s);
  CUDA_TRY(b, cudaMemcpyAsync(counts, b->q_counts.p, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  TRY(query_status(b));
  std::vector<int64_t> offs(n);
  int64_t t = 0;
  for (int q = 0; q < n; ++q) {
    offs[q] = t;
    t += counts[q];
  }
  *total = t;
  if (t > cap) {
    set_error(b, "query result larger than the output capacity");
    return B2G_E_CAPACITY;
  }
  if (t == 0) return B2G_OK;
  TRY(upload(b, b->q_offs, offs));
  TRY(ensure(b, b->q_out, (size_t)t));
  launch_query_emit(a, n, b->q_world.p, b->q_box.p, b->q_counts.p, b->q_offs.p, b->q_out.p, s);
  CUDA_TRY(b, cudaMemcpyAsync(fixtures, b->q_out.p, t * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  return query_status(b);
}

B2G_API int b2g_raycast_closest(b2g_batch* b, const int32_t* worlds, const float* rays, int32_t n, b2g_ray_hit* hits) {
  if (!b || n < 0 || (n > 0 && (!worlds || !rays || !hits))) return B2G_E_INVALID_ARG;
  if (n == 0) return B2G_OK;
  NvtxRange range("b2g.raycast");
  TRY(ensure_query_trees(b));
  cudaStream_t s = b->stream;
  TRY(ensure(b, b->q_world, n)); TRY(ensure(b, b->q_box, n)); TRY(ensure(b, b->q_hits, n));
  CUDA_TRY(b, cudaMemcpyAsync(b->q_world.p, worlds, n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  CUDA_TRY(b, cudaMemcpyAsync(b->q_box.p, rays, n * sizeof(float4), cudaMemcpyHostToDevice, s));
  KernelArgs a = step_args(b, 0.0f, 0, 0);
  launch_raycast(a, n, b->q_world.p, b->q_box.p, b->q_hits.p, s);
  CUDA_TRY(b, cudaMemcpyAsync(hits, b->q_hits.p, n * sizeof(b2g_ray_hit), cudaMemcpyDeviceToHost, s));
  return query_status(b);
}

B2G_API int b2g_collide(const b2g_shape* sa, const float* xa, const b2g_shape* sb, const float* xb, int32_t n,
                        b2g_manifold* out, void* stream) {
  if (n < 0 || (n > 0 && (!sa || !xa || !sb || !xb || !out))) return B2G_E_INVALID_ARG;
  launch_collide_pairs(sa, xa, sb, xb, n, out, (cudaStream_t)stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(nullptr, cudaGetErrorString(e));
    return B2G_E_CUDA;
  }
  return B2G_OK;
}

B2G_API int b2g_time_of_impact(const b2g_toi_input* in, int32_t n, b2g_toi_output* out, void* stream) {
  if (n < 0 || (n > 0 && (!in || !out))) return B2G_E_INVALID_ARG;
  launch_time_of_impact(in, n, out, (cudaStream_t)stream);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(nullptr, cudaGetErrorString(e));
    return B2G_E_CUDA;
  }
  return B2G_OK;
}

}  // extern "C"
