// kernels.h - argument block and launchers of the Step kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "engine.h"

namespace b2g {

// Solver contact constraints in colour order, one row per plane and slot; world w owns slots
// [contact_off, contact_off + solver contacts). Split by use so that each phase reads only full,
// coalesced rows: velocity (idx, nf, r0, r1, nmtm, bk, kn, imp) and position (idx, lcs, lnp, lps,
// rad). Body inverse masses are read per body, not per constraint.
struct SolverPlanes {
  int2* idx;     // local body A | pointCount << 24 | pcPointCount << 28, local body B | type << 24
  int* cid;      // live contact index (impulse store, events)
  float4* nf;    // normal.x, normal.y, friction, tangentSpeed
  float4* r0;    // rA.x, rA.y, rB.x, rB.y of point 0
  float4* r1;    // ... of point 1
  float4* nmtm;  // normalMass 0, 1, tangentMass 0, 1
  float4* bk;    // velocityBias 0, 1, K.ex.x, K.ex.y (= K.ey.x)
  float4* kn;    // K.ey.y, normalMass matrix ex.x, ex.y (= ey.x), ey.y
  float4* imp;   // normalImpulse 0, 1, tangentImpulse 0, 1
  float4* lcs;   // localCenterA, localCenterB
  float4* lnp;   // localNormal, localPoint
  float4* lps;   // localPoints 0, 1
  float2* rad;   // radiusA, radiusB
};


// Plain device pointers of one batch, passed by value to every kernel.
struct KernelArgs {
  const int4* wb;
  const int4* wj;
  float4* wg;
  const int* wflags;
  int2* wc;
  uint8_t* wfault;
  // per world, sleep mode: its island graph changed since the last labelling (a solid contact
  // began or stopped touching, a contact was created or destroyed, or the layout changed)
  uint8_t* isl_dirty;
  const int* world_order;

  float4 *xf, *pos, *vel;
  const float4 *massd, *damp;
  float4* force;
  const float2* lc;
  const int *btype, *bworld;
  int2* bstate;        // per body: x flags (B2G_BS_*), y sleep time (float bits)
  uint8_t* bwake;      // per body: woken by a touching change in this step's narrowphase
  int4* sl;            // per body, sleep-mode worlds: x island label (-1 static), y B2G_ISL_* bits,
                       // z last position iteration the island failed, w island minimum sleep time bits

  const b2g_shape* shape;
  const int *fbody, *fgroup, *fsensor, *fworld;
  const float* frad;              // per fixture: shape radius
  const uint32_t* ffilter;
  const float4* fmat;
  float4* aabb;

  JointDev* joints;
  float4* jplanes;  // joint velocity rows (B2G_JV_ROWS planes of jstride slots; solve scratch)
  int jstride;
  const uint64_t* nocollide;
  int n_nocollide;

  // current contact list
  uint64_t* ckey;
  int2* cfix;
  uint32_t* cflags;
  float4* cmat;
  b2g_manifold* cman;
  // both buffers (for the diff)
  uint64_t* ckeyB[2];
  int2* cfixB[2];
  uint32_t* cflagsB[2];
  float4* cmatB[2];
  b2g_manifold* cmanB[2];

  // broadphase
  float4* wbounds;
  uint64_t *mkey, *mkey_sorted;
  int *mval, *mval_sorted;
  int2* nchild;
  int2* nrange;                   // per internal node: its first and last sorted leaf
  int *nparent, *lparent;
  float4* naabb;
  float4* nrec;                   // per internal node, 3 x 16 B: left child box, right child box,
                                  // {left, right, left meta, right meta} (meta: lbvh_meta)
  int* nhi;                       // per internal node: its meta (last leaf of its range, static bit)
  float4* laabb;                  // leaf boxes in sorted order
  int4* lattr;                    // leaf attributes in sorted order (leaf_attr)
  int4* fattr;                    // per fixture: body, group, filter, shape type | body type << 8
  int* nflag;
  int* wroot;
  int* pcount;
  uint32_t* pslots;               // BP_SLOTS partners per fixture from the counting pass
  int bp_f0, bp_w0;               // first fixture and world of a partial broadphase (0: all)
  int* poff;                      // offsets of the pair list being built, per emitter fixture
  const int* poff_old;            // offsets of the live (source) list, or null when unknown
  uint64_t* pairs;
  void* cub_tmp;

  // solver
  int* sc_list;                   // per solver contact: live contact index
  int2* scb;                      // per solver contact: world-local bodies, bit 31 set = static
  float2* srad;                   // per solver contact: the two fixtures' radii (compaction -> prepare)
  int* cslot;                     // per solver contact: its colour-ordered slot
  SolverPlanes sp;
  int8_t* ccol;
  int* corder;
  uint32_t* cprio;
  uint8_t* cready;
  int *inc_cnt, *inc_head;
  unsigned long long* inc_mask;
  int *inc_list, *jinc_list;
  int4 *cwork, *jwork;            // colouring entries and frontiers: 4 per constraint (contacts, joints)
  int2* jcb;
  int8_t* jcol;
  int* jorder;
  int* jranges;                   // per world: 65 joint colour offsets
  int* cranges;                   // per world: 65 contact colour offsets (setup -> iterations)
  uint32_t* jprio;
  uint8_t* jready;
  int* ncolors;                   // per world: contact colours, joint colours, solver contacts, slot base

  // continuous collision (null unless a world runs SolveTOI)
  float4* sweep0;                 // per body: b2Sweep c0.x, c0.y, a0, alpha0 (the solver writes the step's start)
  int* toi_hpos;                  // per contact: its TOI heap node, -1 when not in the heap
  uint8_t* toi_cfl;               // per contact: island and persist flags of the TOI loop
  int4* toi_heap;                 // per world: TOI heap nodes {toi bits, sub-steps, contact, -} from wc.x + 32 w
  uint8_t* toi_bfl;               // per body: island flag of the TOI loop
  int* toi_flags;                 // [0] a TOI island moved bodies, [1] the TOI kernel ran (its pair update had not overflowed)
  // per-body contact and fixture lists of the TOI loop (built at a world's first impact):
  // offsets from b0 + 2 w (nb + 2 per world), lists from 2 c0 (contacts) and f0 (fixtures)
  int *toi_boff, *toi_blist, *toi_foff, *toi_flist;
  VCDev* toi_vc;                  // per world: the TOI island's contact constraints (32)

  // events, status
  EventDev* events;
  int64_t event_cap;
  int events_on;
  int any_sleep;       // some world runs in sleep mode (dead contacts may wake bodies)
  int any_sensor;      // the layout has sensor fixtures (their contacts get an overlap pass)
  unsigned long long* counters;
  unsigned int* status;

  float dt, inv_dt;
  int vi, pi;
  int nf, nw;        // fixture and world counts of the layout
  int64_t ccap;      // contact / pair buffer capacity
};

// device counters (KernelArgs::counters)
#define B2G_CNT_CONTACTS 0   // live contacts
#define B2G_CNT_EVENTS 1     // recorded events
#define B2G_CNT_TOUCHING 2   // solver contacts of the last step
#define B2G_CNT_OVERFLOW 3   // pair capacity needed when the last broadphase overflowed (else 0)
#define B2G_CNT_MAXCOLORS 4  // most constraint colours of any world in the last solve

void launch_collide(const KernelArgs& a, int nw, cudaStream_t s);
// Solver launches per class: class 0 on `s`, the others on side streams forked from and joined
// back to `s` with the given events (classes.size() - 1 streams, classes.size() events).
void launch_solve(const KernelArgs& a, const std::vector<SolveClass>& classes, cudaStream_t s,
                  const cudaStream_t* side, const cudaEvent_t* ev);
void launch_joint_colour(const KernelArgs& a, int w0, int nw, cudaStream_t s);
// Debug check of the last solve's colouring: within every regular colour (0-62) of every active
// world, no two contact constraints and no two joints share a non-static body; a violation
// raises B2G_DEV_COLOUR_CONFLICT. Uses the per-body colour masks as scratch.
void launch_colour_check(const KernelArgs& a, int nw, cudaStream_t s);

// ---- world queries (query.cu)
void launch_query_count(const KernelArgs& a, int n, const int* qw, const float4* qbox, int* counts, cudaStream_t s);
void launch_query_emit(const KernelArgs& a, int n, const int* qw, const float4* qbox, int* counts, const int64_t* offs,
                       int* out, cudaStream_t s);
void launch_raycast(const KernelArgs& a, int n, const int* qw, const float4* rays, b2g_ray_hit* out, cudaStream_t s);

// ---- batch compaction (compact.cu)
struct CompactTables {            // per old world
  const int* wnew;                // new world index, -1 when removed
  const int4* off_old;            // body, fixture, joint offsets in the old layout
  const int4* off_new;            // ... and in the new one
  const int* con_old;             // live contact range start, old and new
  const int* con_new;
};
struct BodyRecs {
  float4 *xf, *pos, *vel, *massd, *damp, *force;
  float2* lc;
  int *btype, *bworld;
  int2* bstate;
};
struct FixRecs {
  b2g_shape* shape;
  int *fbody, *fgroup, *fsensor, *fworld;
  uint32_t* ffilter;
  float4* fmat;
  float* frad;
};
struct ConRecs {
  uint64_t* key;
  int2* fix;
  uint32_t* flags;
  float4* mat;
  b2g_manifold* man;
};
void launch_compact(const CompactTables& t, int nb, const BodyRecs& sb, const BodyRecs& db, int nf, const FixRecs& sf,
                    const FixRecs& df, int nj, const JointDev* sj, JointDev* dj, int64_t nc, const ConRecs& sc,
                    const ConRecs& dc, cudaStream_t s);
void solver_setup();
// Solver launches for worlds listed by body count, largest first, with the given threads per
// CTA for each size class (at most 64, 512, 2048, 8192 and more bodies); a class runs the wide
// build when its worlds fill at most `wide_waves` waves of it.
std::vector<SolveClass> plan_solve_classes(const std::vector<int>& order, const std::vector<int>& bodies,
                                           const int* class_threads, float wide_waves, int cluster_ctas);
// Largest thread-block cluster (CTAs per world) the device runs the cluster solve with: 16 where
// the non-portable size is available, else 8; 0 before solver_setup or when clusters are absent.
int solver_max_cluster_ctas();
bool solver_threads_valid(int t);
void launch_clear_forces(const KernelArgs& a, int nb, cudaStream_t s);
// Broadphase up to the tree (AABBs, Morton sort, LBVH, node boxes); with `pairs` also the pair
// count, its scan and the per-world contact ranges of the list being built.
void launch_bp_build(const KernelArgs& a, int nf, int nw, size_t cub_bytes, int sort_bits, cudaStream_t s,
                     bool pairs = true);
// Broadphase that keeps the per-world trees of fixtures [0, tree_nf) (worlds [0, tree_nw)): their
// leaf boxes are refreshed and the node boxes refit bottom-up, the fixtures appended after them
// get trees of their own, then the pair count, scan and contact ranges as launch_bp_build. Any
// tree yields the same pair set (the partners of a fixture are sorted before emission).
void launch_bp_refit(const KernelArgs& a, int tree_nf, int tree_nw, int nf, int nw, size_t cub_bytes, int sort_bits,
                     cudaStream_t s);
void launch_bp_emit(const KernelArgs& a, int nf, cudaStream_t s);
// Broadphase of the appended fixtures [f0, nf) of worlds [w0, nw) only; their pairs are appended to
// the live list (buffer dst); poff_live (may be null) gets the appended fixtures' offsets.
void launch_bp_tail(const KernelArgs& a, int f0, int nf, int w0, int nw, size_t cub_bytes, int sort_bits, int dst,
                    int* poff_live, cudaStream_t s);
void launch_contact_diff(const KernelArgs& a, int src, int dst, cudaStream_t s);
size_t cub_temp_bytes(int nf);
void launch_time_of_impact(const b2g_toi_input* in, int n, b2g_toi_output* out, cudaStream_t s);
// b2World::SolveTOI for the active worlds flagged B2G_WF_CONTINUOUS, on the live contact list.
void launch_solve_toi(const KernelArgs& a, int nw, cudaStream_t s);
void launch_collide_pairs(const b2g_shape* sa, const float* xa, const b2g_shape* sb, const float* xb, int n,
                          b2g_manifold* out, cudaStream_t s);

}  // namespace b2g
