// engine.h - host side of the GB300 Step engine: a batch of worlds in packed world-major arrays.
//
// Layout (device, one allocation per array, every array world-major and contiguous per world):
//   bodies   : xf float4 (p.x, p.y, q.s, q.c) | pos float4 (c.x, c.y, a, -) | vel float4 (v.x, v.y, w, -)
//              | mass float4 (m, 1/m, I, 1/I) | lc float2 | damp float4 (lin, ang, gravityScale, -)
//              | force float4 (fx, fy, torque, -) | type int | world int
//   fixtures : shape b2g_shape | body int | mat float4 (friction, restitution, threshold, density)
//              | filter uint (category | mask << 16) | group int | sensor int | aabb float4 | world int
//   joints   : JointDev (definition, warm-start impulses, solver temporaries)
//   contacts : double-buffered, sorted by key = global emitter fixture << 32 | global partner
//              fixture; key | (fixture A, fixture B) int2 | flags uint | mat float4 | b2g_manifold
// World w owns bodies [wb.x, wb.x + wb.y), fixtures [wb.z, wb.z + wb.w), joints
// [wj.x, wj.x + wj.y) and, after each broadphase, contacts [wc.x, wc.x + wc.y).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>
#include <string>
#include <vector>

#include "../../include/b2g_capi.h"

namespace b2g {

// Joint record on the device: definition + warm-start state + per-step solver temporaries.
struct JointDev {
  b2g_joint_def d;
  float impulse[3];
  float motorImpulse, lowerImpulse, upperImpulse;
  // temporaries (b2RevoluteJoint / b2PrismaticJoint / b2DistanceJoint members)
  int iA, iB;                 // global body indices
  float lcA[2], lcB[2];
  float mA, mB, invIA, invIB;
  float rA[2], rB[2];
  float K[4];                 // ex.x, ex.y, ey.x, ey.y
  float axialMass, angle;
  float localXAxisA[2], localYAxisA[2], axis[2], perp[2];
  float a1, a2, s1, s2, translation;
  float u[2], currentLength, mass, softMass, gamma, bias;
  float reaction[3];          // force x, y, torque at the last step's inv_dt
  // weld (b2_weld_joint.h:117-125), wheel (b2_wheel_joint.h:178-212), motor (b2_motor_joint.h:
  // 106-122), mouse (b2_mouse_joint.h:110-127) and pulley (b2_pulley_joint.h:125-148) temporaries;
  // the wheel keeps ax/ay in axis/perp and sAx, sBx, sAy, sBy in a1, a2, s1, s2, the motor and
  // friction joints their linear mass in K and angular mass in axialMass, the mouse joint its
  // mass in K, beta in bias and m_C in err, the pulley m_uA in u
  float mass3[9];             // weld m_mass (ex, ey, ez)
  float springMass, motorMass;
  float err[2], angularError;
  float uB[2], constant;
  // gear (b2_gear_joint.h:52-110): bodies C (joint 1's body A) and D (joint 2's body A), the
  // geometry taken from the two joints on upload, and the step temporaries; A and B are d.body_a
  // / d.body_b (the two joints' bodies B). The gear's impulse is impulse[0].
  struct Gear {
    int iC, iD;               // global body indices
    int typeA, typeB;         // B2G_JOINT_REVOLUTE or B2G_JOINT_PRISMATIC (joint 1, joint 2)
    float lA[2], lB[2], lC[2], lD[2];  // local anchors on A, B, C, D
    float axC[2], axD[2];     // joint 1's / joint 2's local axis (prismatic)
    float refA, refB;         // the joints' reference angles
    float lcA[2], lcB[2], lcC[2], lcD[2];
    float mA, mB, mC, mD, iA, iB, iC_, iD_;
    float JvAC[2], JvBD[2], JwA, JwB, JwC, JwD, mass;
  } g;
};

// Per-contact velocity / position constraint (b2ContactVelocityConstraint and
// b2ContactPositionConstraint, src/dynamics/b2_contact_solver.h:51-76 and
// src/dynamics/b2_contact_solver.cpp:36-48), stored once per solver contact.
struct VCDev {
  float rA[2][2], rB[2][2];
  float normalImpulse[2], tangentImpulse[2], normalMass[2], tangentMass[2], velocityBias[2];
  float normal[2];
  float K[4];                 // ex.x, ex.y, ey.x, ey.y
  float NM[4];                // normalMass matrix
  float invMassA, invMassB, invIA, invIB;
  float friction, tangentSpeed;
  int indexA, indexB;         // global body indices
  int pointCount;
  int contact;                // global contact index
  // position part
  float localPoints[2][2];
  float localNormal[2], localPoint[2];
  float localCenterA[2], localCenterB[2];
  float radiusA, radiusB;
  int type, pcPointCount;
};

#define B2G_WF_WARM 1
#define B2G_WF_CLEAR_FORCES 2
#define B2G_WF_ACTIVE 4
#define B2G_WF_NEW_CONTACTS 8
#define B2G_WF_RETIRED 16
#define B2G_WF_FAULTED 32  // produced a non-finite state: frozen (retired) and reported
#define B2G_WF_SLEEPMODE 64     // islands and awake flags are tracked (sleeping allowed or sleepers present)
#define B2G_WF_ALLOW_SLEEP 128  // b2World::SetAllowSleeping(true): island sleep timers run
#define B2G_WF_CONTINUOUS 256  // b2World::SetContinuousPhysics(true) with a bullet or kinematic body: SolveTOI runs

// Body sleep state on the device (bstate.x) and island bits (sl.y).
#define B2G_BS_AWAKE 1        // b2Body::e_awakeFlag
#define B2G_BS_AUTO_SLEEP 2   // b2Body::e_autoSleepFlag
#define B2G_BS_BULLET 4       // b2Body::e_bulletFlag
#define B2G_ISL_AWAKE 1       // (at the island's root) some member was awake: the island is solved
#define B2G_ISL_DONE 2        // (at the root) the island's position constraints were solved
#define B2G_ISL_LINKED 4      // (own entry) the body has a contact or a joint: not an orphan

// b2_common.h:176-182
#define B2G_TIME_TO_SLEEP 0.5f
#define B2G_LINEAR_SLEEP_TOL 0.01f
#define B2G_ANGULAR_SLEEP_TOL (2.0f / 180.0f * 3.14159265359f)

struct HostWorld {
  float gx = 0.0f, gy = -10.0f;
  float inv_dt0 = 0.0f;
  int flags = B2G_WF_WARM | B2G_WF_CLEAR_FORCES;
  bool allow_sleep = false, continuous = false;
  // a bullet or kinematic body is present (1), absent (0), not known since the last upload (-1)
  mutable int toi_bodies = -1;
  bool sleepers = false;  // bodies may be asleep although sleeping is not allowed (created asleep)
  std::vector<b2g_body> bodies;
  std::vector<float> body_sleep;  // b2Body::m_sleepTime per body
  std::vector<uint64_t> body_user;
  std::vector<b2g_fixture> fixtures;
  std::vector<uint64_t> fixture_user;
  std::vector<b2g_joint> joints;
  std::vector<b2g_contact> contacts;  // world-local fixture indices (valid when synced)
  std::vector<std::vector<int>> body_fixtures;  // fixture indices per body, creation order
};

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t cap = 0;
};

struct Batch;

// One solver launch over a contiguous range of the size-sorted world order.
struct SolveClass {
  int first, count, threads, smem;
  int cls;    // size class index
  bool wide;  // the 128-register build (few worlds: latency-bound) rather than the 64-register one
  int ctas;   // CTAs per world: 1, or the thread-block cluster size of the largest class
  int setup_threads, setup_smem;  // the first half's launch (k_setup), for ctas == 1
};
#define B2G_SOLVE_CLASSES 5
#define B2G_JV_ROWS 13  // float4 rows of one joint's solver record (solver_dev.cuh)

// Status word the kernels write instead of trapping (bounded waits and capacity checks).
#define B2G_DEV_OK 0u
#define B2G_DEV_STACK_OVERFLOW 1u
#define B2G_DEV_NONFINITE 2u
#define B2G_DEV_PAIR_OVERFLOW 4u
#define B2G_DEV_COLOR_ROUNDS 8u
#define B2G_DEV_COLOUR_CONFLICT 16u  // debug check: one regular colour holds two constraints of a body
#define B2G_DEV_ISLAND_CHECK 32u     // debug check: a sleep-mode world's island labels are inconsistent

struct EventDev {
  int kind, world, fixtureA, fixtureB, pointCount;
  float normalImpulses[2], tangentImpulses[2];
  b2g_manifold old;
};

// Appended worlds [w0, w1) packed into device layout on the host ahead of the step that uploads
// them (b2g_batch_stage); valid while the layout it was packed against is unchanged.
struct TailPack {
  bool valid = false;
  int w0 = 0, w1 = 0, NB0 = 0, NF0 = 0, NJ0 = 0, NB = 0, NF = 0, NJ = 0;
  std::vector<int> body_off, fix_off, joint_off;  // per packed world
  std::vector<float4> xf, pos, vel, massd, damp, force, fmat;
  std::vector<float2> lc;
  std::vector<int> btype, bworld, fbody, fgroup, fsensor, fworld;
  std::vector<int2> bstate;
  std::vector<float> frad;
  std::vector<b2g_shape> shape;
  std::vector<uint32_t> ffilter;
  std::vector<JointDev> joints;
  std::vector<uint64_t> nocol;
};

struct Batch {
  int device = 0;
  uint64_t budget = 0;
  uint64_t allocated = 0;
  cudaStream_t stream = nullptr;
  std::vector<HostWorld> worlds;
  bool structure_dirty = true;     // host structure changed: full upload before the next step
  bool device_state_valid = false; // device holds the live dynamic state
  bool host_state_stale = false;   // host mirrors are older than the device
  bool events_on = false;
  bool debug_checks = false;       // verify each step's constraint colouring on the device
  std::string error;

  // totals of the current device layout
  int NW = 0, NB = 0, NF = 0, NJ = 0;
  int64_t NC = 0;                 // live contacts
  std::vector<int> h_body_off, h_fix_off, h_joint_off;
  std::vector<uint64_t> h_nocol;  // host copy of the device no-collide list (sorted body pairs)

  // ---- device arrays
  DBuf<int4> wb;                  // body_off, body_cnt, fix_off, fix_cnt
  DBuf<int4> wj;                  // joint_off, joint_cnt, -, -
  DBuf<float4> wg;                // gx, gy, inv_dt0, -
  DBuf<int> wflags;
  DBuf<int2> wc;                  // contact_off, contact_cnt
  DBuf<uint8_t> wfault;           // set by the solver when the world's state became non-finite
  DBuf<uint8_t> isl_dirty;        // per world: its island labels must be recomputed (sleep mode)
  DBuf<int> world_order;          // worlds sorted by work, largest first

  DBuf<float4> xf, pos, vel, massd, damp, force;
  DBuf<float2> lc;
  DBuf<int> btype, bworld;
  DBuf<int2> bstate;              // awake / auto-sleep flags and sleep time per body
  DBuf<uint8_t> bwake;            // narrowphase wake marks (zero between steps)
  DBuf<int4> sl;                  // island scratch of sleep-mode worlds
  bool any_sleep = false;         // some world of the layout runs in sleep mode
  bool any_sensor = false;        // some fixture of the layout is a sensor
  TailPack tail_pack;             // prepared upload of appended worlds
  bool in_step = false;           // between b2g_step_begin and b2g_step_end
  bool step_graph = false;        // the step in flight replays a graph
  bool step_ccd = false;          // the step in flight runs SolveTOI (and a second pair update) in step_end
  // continuous collision scratch (allocated once a world runs SolveTOI)
  DBuf<float4> sweep0;            // per body: b2Sweep c0, a0, alpha0
  DBuf<int> toi_hpos;             // per contact slot: TOI heap node
  DBuf<uint8_t> toi_cfl;          // per contact slot: TOI island / persist flags
  DBuf<int4> toi_heap;            // contact slots + 32 per world: TOI heap nodes
  DBuf<uint8_t> toi_bfl;          // per body: TOI island flag
  DBuf<int> toi_flags;            // [0] some TOI island moved bodies, [1] the TOI kernel ran
  DBuf<int> toi_adj;              // per-body contact and fixture lists of the TOI loop (four sections)
  DBuf<VCDev> toi_vc;             // per world: the TOI island's contact constraints (32)
  bool graph_ccd = false;         // the captured graphs include the TOI stage
  std::chrono::steady_clock::time_point step_t0;  // host time the step in flight began

  DBuf<b2g_shape> shape;
  DBuf<int> fbody, fgroup, fsensor, fworld;
  DBuf<float> frad;
  DBuf<uint32_t> ffilter;
  DBuf<float4> fmat, aabb;

  DBuf<JointDev> joints;
  DBuf<uint64_t> nocollide;       // sorted global body pairs joined by collideConnected=false joints
  int n_nocollide = 0;

  // contacts, double buffered
  DBuf<uint64_t> ckey[2];
  DBuf<int2> cfix[2];
  DBuf<uint32_t> cflags[2];
  DBuf<float4> cmat[2];
  DBuf<b2g_manifold> cman[2];
  int cur = 0;
  int last_solve_buf = -1;        // contact buffer the last solve read (solver order lookups)
  bool tree_valid = false;        // the per-world trees match the current body transforms
  // The broadphase forest kept between steps: trees of fixtures [0, tree_nf) (worlds [0,
  // tree_nw)), refit by the closing broadphase and rebuilt from sorted Morton codes every
  // tree_period broadphases (tree_age counts those since the last full build).
  int tree_nf = 0, tree_nw = 0, tree_age = 0;
  int tree_period = 32;  // broadphases per full build (1: every broadphase builds)

  // world query scratch
  DBuf<int> q_world, q_counts, q_out;
  DBuf<float4> q_box;
  DBuf<int64_t> q_offs;
  DBuf<b2g_ray_hit> q_hits;

  // broadphase scratch
  DBuf<float4> wbounds;
  DBuf<uint64_t> mkey, mkey_sorted;
  DBuf<int> mval, mval_sorted;
  DBuf<int2> nchild;              // internal node children (leaf = index | 0x80000000)
  DBuf<int2> nrange;              // internal node leaf ranges (first, last sorted leaf)
  DBuf<int> nparent, lparent;     // parents of internal nodes and leaves
  DBuf<float4> naabb, nrec, laabb;  // node boxes, node records (3 per node), sorted leaf boxes
  DBuf<int> nhi;                  // node metas (last leaf of the range | static bit)
  DBuf<int4> lattr;               // sorted leaf attributes
  DBuf<int4> fattr;
  DBuf<int> nflag;
  DBuf<int> wroot;                // per world: root node (leaf encoded), -1 if empty
  DBuf<int> pcount;               // per fixture pair count
  DBuf<uint32_t> pslots;          // per fixture: first partners found by the counting pass
  DBuf<int> poffB[2];             // per contact buffer: exclusive scan of pcount (NF + 1 entries)
  bool poff_valid[2] = {false, false};  // offsets describe that buffer's list (built by a broadphase)
  DBuf<uint64_t> pairs;
  DBuf<uint8_t> cub_tmp;
  DBuf<unsigned int> status;      // device status word
  DBuf<unsigned long long> counters;  // [0] pair total, [1] event count

  // solver scratch
  DBuf<int> sc_list;              // per world: compacted solver contact indices (global)
  DBuf<int2> scb;                 // per solver contact: world-local bodies, bit 31 set = static
  DBuf<float2> srad;              // per solver contact: the two fixtures' radii
  DBuf<int> cslot;                // per solver contact: colour-ordered slot
  DBuf<float4> sp_nf, sp_r0, sp_r1, sp_nmtm, sp_bk, sp_kn, sp_imp, sp_lcs, sp_lnp, sp_lps;
  DBuf<int2> sp_idx;
  DBuf<int> sp_cid;
  DBuf<float2> sp_rad;
  DBuf<int8_t> ccol;
  DBuf<int> corder;
  DBuf<uint32_t> cprio;
  DBuf<uint8_t> cready;
  DBuf<int> inc_cnt, inc_head;
  DBuf<unsigned long long> inc_mask;
  DBuf<int> inc_list;             // 2 entries per constraint (contacts), world base 2*contact_off
  DBuf<int> jinc_list;            // 2 entries per joint
  DBuf<int4> cwork, jwork;        // colouring list entries and frontiers, 4 per contact / joint
  DBuf<int2> jcb;
  DBuf<int8_t> jcol;
  DBuf<int> jorder, jranges;
  DBuf<int> cranges;              // per world: 65 contact colour offsets of this step's solve
  DBuf<uint32_t> jprio;
  DBuf<uint8_t> jready;
  DBuf<float4> jplanes;           // joint velocity rows, B2G_JV_ROWS planes of NJ slots (solve scratch)
  DBuf<int> ncolors;              // per world: contact colours, joint colours, solver contacts, slot base
  // compaction targets: swapped with the live arrays by a device compaction, kept for the next
  struct Spare {
    DBuf<float4> xf, pos, vel, massd, damp, force, fmat;
    DBuf<float2> lc;
    DBuf<int> btype, bworld, fbody, fgroup, fsensor, fworld, tables;
    DBuf<int2> bstate;
    DBuf<b2g_shape> shape;
    DBuf<uint32_t> ffilter;
    DBuf<float> frad;
    DBuf<JointDev> joints;
  } spare;

  std::vector<SolveClass> solve_classes;
  std::vector<int> h_world_order;  // worlds by body count, largest first (device world_order)
  int class_threads[B2G_SOLVE_CLASSES] = {64, 128, 256, 512, 1024};
  int cluster_ctas = -1;     // CTAs per world of the largest size class (-1: the device's largest cluster)
  float wide_waves = 1e9f;  // size classes of at most this many waves run the wide solver build (all, by default)
  cudaStream_t side[B2G_SOLVE_CLASSES] = {};
  cudaEvent_t fork_ev[B2G_SOLVE_CLASSES + 1] = {};

  // events
  DBuf<EventDev> events;
  int64_t event_cap = 0;
  std::vector<b2g_event> host_events;

  // profile
  b2g_profile profile{};
  cudaEvent_t ev[8] = {};
  // b2g_step_io: the host copies' stream; io_in is recorded after the forces' copy and waited for
  // before the solve, io_solved is recorded after the solve and waited for by the transforms' copy
  cudaStream_t io_stream = nullptr;
  cudaEvent_t io_in = nullptr, io_solved = nullptr;

  // contact / pair buffer capacity and a version bumped whenever a kernel-visible buffer moves
  int64_t ccap = 0;
  uint64_t layout_version = 1;
  std::vector<int> h_wflags;
  unsigned long long* h_readback = nullptr;  // pinned: device counters + status after each step
  void* h_stage = nullptr;        // pinned staging of appended worlds' records
  size_t h_stage_cap = 0;
  cudaEvent_t stage_ev = nullptr; // recorded after the last staged copies
  float last_dt = 0.0f;
  int last_vi = 0, last_pi = 0;

  // CUDA graphs of one Step (one per parity of the live contact buffer)
  bool use_graphs = true;
  cudaGraphExec_t graph_exec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [broadphase mode][parity]
  uint64_t graph_version = 0;
  float graph_dt = 0;
  int graph_vi = -1, graph_pi = -1;
};

// ---- host functions (engine.cu)
int upload_all(Batch* b);
uint64_t batch_allocated_bytes(const b2g_batch* b);
// Moves a world that is not on the device out of `src` (host records only; the slot is dropped
// when it is the last one, else left retired) and appends it to `dst` as a new world: how a world
// built on another thread's host-only batch joins a device batch without copying its records.
int take_world(b2g_batch* src, int32_t world, HostWorld* out);
int append_world(b2g_batch* dst, HostWorld&& w, int32_t* out_world);
int upload_tail(Batch* b);
int download_state(Batch* b);
int step_batch(Batch* b, float dt, int vi, int pi, const uint8_t* mask, bool sync);
void set_error(Batch* b, const std::string& msg);

// ---- shape processing (shapes.cpp)
int process_fixture_def(const b2g_fixture_def& d, b2g_fixture* out);
void reset_mass_data(HostWorld& w, int body);
void polygon_set(b2g_shape* p, const float* xy, int count);
void polygon_box(b2g_shape* p, float hx, float hy, bool oriented, float cx, float cy, float angle);
void shape_mass(const b2g_shape& s, float density, float* mass, float* cx, float* cy, float* I);

}  // namespace b2g
