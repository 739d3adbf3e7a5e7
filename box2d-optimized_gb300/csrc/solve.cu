// solve.cu - the island solver of one Step for every active world of the batch
// (b2Island::Solve, src/dynamics/b2_island.cpp:253-484; b2ContactSolver,
// src/dynamics/b2_contact_solver.cpp), one CTA per world in two kernels.
//
// Per world, in order; the setup kernel (k_setup, 1024 threads per SM):
//   1. solver contacts: the touching, enabled, non-sensor live contacts (b2_world.cpp:567-599),
//      compacted in list order, with their world-local non-static bodies and priorities;
//   2. deterministic greedy colouring of those contacts in priority order (Jones-Plassmann
//      rounds), in shared memory for what fits; joints keep the colouring computed once per
//      layout by k_joint_colour;
//   3. velocity integration into the global velocity array;
//   4. contact prepare, written straight into colour-ordered constraint planes;
// then the iteration kernel (k_solve):
//   5. warm start, joint InitVelocityConstraints, velocity iterations (joints then contacts) on
//      the body state in shared memory when the world fits, StoreImpulses, position
//      integration, position iterations (contacts then joints) with the world's early exit,
//      transforms.
// Constraints of one colour share no non-static body, so a colour runs in parallel; colours
// run in order with a CTA barrier between them, which reproduces the sequential Gauss-Seidel
// sweep in colour order. Worlds are launched in size classes (threads and shared memory per
// class) on forked streams so that small and large worlds run side by side.
#include "solve_world.cuh"

namespace b2g {

// Joint colouring of worlds [w0, w0 + gridDim.x), once per layout: joints and the static flags
// of their bodies change only through structural edits, which re-upload the layout.
template <int T>
__global__ void __launch_bounds__(T) k_joint_colour(KernelArgs a, int w0) {
  __shared__ int jr[65];
  const int w = w0 + blockIdx.x;
  const int4 wb = a.wb[w];
  const int b0 = wb.x, nb = wb.y;
  const int4 wj = a.wj[w];
  const int j0 = wj.x, nj = wj.y;
  if (nj == 0) {
    if (threadIdx.x == 0) a.ncolors[4 * w + 1] = 0;
    return;
  }
  for (int k = threadIdx.x; k < nj; k += T) {
    const JointDev& J = a.joints[j0 + k];
    int ia = J.d.body_a, ib = J.d.body_b;
    a.jcb[j0 + k] = J.d.type == B2G_JOINT_GEAR
                        ? make_int2(B2G_CB_SERIAL, B2G_CB_SERIAL)
                        : make_int2((ia - b0) | (a.btype[ia] == B2G_STATIC ? (int)0x80000000 : 0),
                                    (ib - b0) | (a.btype[ib] == B2G_STATIC ? (int)0x80000000 : 0));
    a.jprio[j0 + k] = jointPriority((uint32_t)k);
  }
  __syncthreads();
  ColourMem m;
  m.cnt = a.inc_cnt + b0;
  m.head = a.inc_head + b0;
  m.mask = a.inc_mask + b0;
  m.list = a.jinc_list + 2 * (int64_t)j0;
  m.cb = a.jcb + j0;
  m.col = a.jcol + j0;
  m.rdy = a.jready + j0;
  m.ent = a.jwork + 4 * (int64_t)j0;
  m.wl0 = m.ent + 2 * (int64_t)nj;
  m.wl1 = m.wl0 + nj;
  CtaTeam<T> tm;
  int njc = colour_constraints(tm, nj, nb, m, a.jprio + j0, a.jorder + j0, nullptr, jr, a.status);
  for (int c = threadIdx.x; c <= njc; c += T) a.jranges[65 * (int64_t)w + c] = jr[c];
  if (threadIdx.x == 0) a.ncolors[4 * w + 1] = njc;
}

// One block per world: each constraint of a regular colour sets its colour's bit in the masks of
// its non-static bodies; a bit found already set is a conflict. Contacts first, then (masks
// cleared) joints, since the two sets are solved in separate sweeps.
__device__ __forceinline__ void colour_mark(unsigned long long* mask, int2 cb, int col, unsigned int* status) {
  if (col < 0 || col >= 63) return;  // the serial colour is solved by one thread
  const unsigned long long bit = 1ull << col;
  const int ends[2] = {cb.x, cb.y};
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    if (ends[e] < 0) continue;  // static body (bit 31 set)
    if (atomicOr(&mask[ends[e]], bit) & bit) atomicOr(status, B2G_DEV_COLOUR_CONFLICT);
  }
}

__global__ void __launch_bounds__(256) k_colour_check(KernelArgs a) {
  const int w = blockIdx.x;
  if ((a.wflags[w] & B2G_WF_ACTIVE) == 0) return;
  const int4 wb = a.wb[w];
  const int b0 = wb.x, nb = wb.y;
  unsigned long long* mask = a.inc_mask + b0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) mask[i] = 0ull;
  __syncthreads();
  const int nsc = a.ncolors[4 * w + 2], c0 = a.ncolors[4 * w + 3];
  for (int k = threadIdx.x; k < nsc; k += blockDim.x) colour_mark(mask, a.scb[c0 + k], a.ccol[c0 + k], a.status);
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += blockDim.x) mask[i] = 0ull;
  __syncthreads();
  const int4 wj = a.wj[w];
  const int j0 = wj.x, nj = wj.y;
  for (int k = threadIdx.x; k < nj; k += blockDim.x) colour_mark(mask, a.jcb[j0 + k], a.jcol[j0 + k], a.status);
  if (!(a.wflags[w] & B2G_WF_SLEEPMODE)) return;
  // the step's islands: every label is a root no larger than its body, and solid contacts and
  // joints join bodies of one label
  int4* SL = a.sl + b0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    const int r = isl_label(SL, i);
    if (r >= 0 && (r > i || isl_label(SL, r) != r)) atomicOr(a.status, B2G_DEV_ISLAND_CHECK);
  }
  const int2 wc = a.wc[w];
  for (int k = threadIdx.x; k < wc.y; k += blockDim.x) {
    const int2 f = a.cfix[wc.x + k];
    const uint32_t fl = a.cflags[wc.x + k];
    if (!(fl & B2G_CONTACT_TOUCHING) || !(fl & B2G_CONTACT_ENABLED) || a.fsensor[f.x] || a.fsensor[f.y]) continue;
    const int la = isl_label(SL, a.fbody[f.x] - b0), lb = isl_label(SL, a.fbody[f.y] - b0);
    if (la >= 0 && lb >= 0 && la != lb) atomicOr(a.status, B2G_DEV_ISLAND_CHECK);
  }
  for (int k = threadIdx.x; k < nj; k += blockDim.x) {
    const JointDev& J = a.joints[j0 + k];
    const int la = isl_label(SL, J.d.body_a - b0), lb = isl_label(SL, J.d.body_b - b0);
    if (la >= 0 && lb >= 0 && la != lb) atomicOr(a.status, B2G_DEV_ISLAND_CHECK);
  }
}

void launch_colour_check(const KernelArgs& a, int nw, cudaStream_t s) {
  if (nw > 0) k_colour_check<<<nw, 256, 0, s>>>(a);
}

// ---- launch planning
// Class by world body count: threads per CTA and the dynamic shared memory that holds the
// world's body state and inverse masses (24 B/body) and, room permitting, its colouring arrays
// (16 B/body + 26 B per contact, about 68 B/body at two contacts per body).
static const int kClassMaxBodies[B2G_SOLVE_CLASSES] = {64, 512, 2048, 8192, 1 << 30};
// Shared-memory allowance by threads per CTA (64, 128, 256, 512, 1024) of the occupancy and the
// wide builds: the SM holds kSolveBlocks<T, WIDE> such CTAs, and the allowance keeps that many
// resident.
static const int kSmemCapByThreads[2][B2G_SOLVE_CLASSES] = {{16 << 10, 24 << 10, 56 << 10, 110 << 10, 200 << 10},
                                                            {27 << 10, 54 << 10, 110 << 10, 220 << 10, 220 << 10}};
static int g_num_sms = 0;
// The setup kernel (k_setup): at most 512 threads per world, 1024 threads per SM; its dynamic
// shared memory (for the colouring) by threads per CTA (64, 128, 256, 512), so that 1024 / T
// CTAs stay resident.
static const int kSetupMaxThreads = 512;
static const int kSetupSmemCap[4] = {12 << 10, 24 << 10, 48 << 10, 100 << 10};

static int threads_index(int t) {
  int k = 0;
  while (k + 1 < B2G_SOLVE_CLASSES && (64 << k) < t) ++k;
  return k;
}

bool solver_threads_valid(int t) { return t == 64 || t == 128 || t == 256 || t == 512 || t == 1024; }

std::vector<SolveClass> plan_solve_classes(const std::vector<int>& order, const std::vector<int>& bodies,
                                           const int* class_threads, float wide_waves, int cluster_ctas) {
  // `order` lists worlds by body count, largest first: each class is a contiguous range
  std::vector<SolveClass> out;
  int n = (int)order.size();
  int i = 0;
  for (int c = B2G_SOLVE_CLASSES - 1; c >= 0 && i < n; --c) {
    int lo = c > 0 ? kClassMaxBodies[c - 1] : -1;
    int start = i;
    int nbmax = 0;
    while (i < n && bodies[order[i]] > lo) {
      nbmax = nbmax > bodies[order[i]] ? nbmax : bodies[order[i]];
      ++i;
    }
    if (i == start) continue;
    // the iterations hold the bodies' state and inverse masses (24 B per body); the setup as
    // much of the colouring as fits (at two contacts per body: 16 + 2 x 26 B per body)
    int64_t need = 24ll * nbmax + 16;
    need = (need + 15) & ~15ll;
    const int64_t setup_need = ((68ll * nbmax) + 15) & ~15ll;
    int t = class_threads[c];
    int ti = threads_index(t);
    // the wide build unless the class holds more than wide_waves waves of it
    bool wide = g_num_sms > 0 && (double)(i - start) * t <= (double)wide_waves * 512.0 * g_num_sms;
    int cap = kSmemCapByThreads[wide ? 1 : 0][ti];
    int smem = (int)(need < cap ? need : cap);
    // the largest class: a thread-block cluster per world when the device runs one
    if (c == B2G_SOLVE_CLASSES - 1 && cluster_ctas > 1) {
      out.push_back({start, i - start, kClusterThreads, 0, c, true, cluster_ctas, 0, 0});
      continue;
    }
    const int st = t < kSetupMaxThreads ? t : kSetupMaxThreads;
    const int scap = kSetupSmemCap[threads_index(st)];
    out.push_back({start, i - start, t, smem, c, wide, 1, st, (int)(setup_need < scap ? setup_need : scap)});
  }
  return out;
}

template <int T>
static void set_smem_attr(int c) {
  cudaFuncSetAttribute(k_solve<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemCapByThreads[0][c]);
}

template <int T>
static void set_setup_smem_attr(int c) {
  cudaFuncSetAttribute(k_setup<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSetupSmemCap[c]);
}

void solver_setup() {
  // the setup kernel's dynamic allowance comes on top of its static shared memory
  set_setup_smem_attr<64>(0);
  set_setup_smem_attr<128>(1);
  set_setup_smem_attr<256>(2);
  set_setup_smem_attr<512>(3);
  set_smem_attr<64>(0);
  set_smem_attr<128>(1);
  set_smem_attr<256>(2);
  set_smem_attr<512>(3);
  set_smem_attr<1024>(4);
  solve_wide_setup(kSmemCapByThreads[1]);
  solve_cluster_setup();
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
}

static void launch_class(const KernelArgs& a, const SolveClass& c, cudaStream_t s) {
  if (c.ctas > 1) {
    launch_solve_class_cluster(a, c, s);
    return;
  }
  switch (c.setup_threads) {
    case 64: k_setup<64><<<c.count, 64, c.setup_smem, s>>>(a, c.first, c.setup_smem); break;
    case 128: k_setup<128><<<c.count, 128, c.setup_smem, s>>>(a, c.first, c.setup_smem); break;
    case 256: k_setup<256><<<c.count, 256, c.setup_smem, s>>>(a, c.first, c.setup_smem); break;
    default: k_setup<512><<<c.count, 512, c.setup_smem, s>>>(a, c.first, c.setup_smem); break;
  }
  if (c.wide) {
    launch_solve_class_wide(a, c, s);
    return;
  }
  switch (c.threads) {
    case 64: k_solve<64, false><<<c.count, 64, c.smem, s>>>(a, c.first, c.smem); break;
    case 128: k_solve<128, false><<<c.count, 128, c.smem, s>>>(a, c.first, c.smem); break;
    case 256: k_solve<256, false><<<c.count, 256, c.smem, s>>>(a, c.first, c.smem); break;
    case 512: k_solve<512, false><<<c.count, 512, c.smem, s>>>(a, c.first, c.smem); break;
    default: k_solve<1024, false><<<c.count, 1024, c.smem, s>>>(a, c.first, c.smem); break;
  }
}

void launch_solve(const KernelArgs& a, const std::vector<SolveClass>& classes, cudaStream_t s, const cudaStream_t* side,
                  const cudaEvent_t* ev) {
  if (classes.empty()) return;
  if (classes.size() == 1) {
    launch_class(a, classes[0], s);
    return;
  }
  cudaEventRecord(ev[0], s);
  for (size_t i = 1; i < classes.size(); ++i) {
    cudaStreamWaitEvent(side[i - 1], ev[0], 0);
    launch_class(a, classes[i], side[i - 1]);
    cudaEventRecord(ev[i], side[i - 1]);
  }
  launch_class(a, classes[0], s);
  for (size_t i = 1; i < classes.size(); ++i) cudaStreamWaitEvent(s, ev[i], 0);
}

void launch_joint_colour(const KernelArgs& a, int w0, int nw, cudaStream_t s) {
  if (nw > 0) k_joint_colour<256><<<nw, 256, 0, s>>>(a, w0);
}

}  // namespace b2g
