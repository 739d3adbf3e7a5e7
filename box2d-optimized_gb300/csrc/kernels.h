// kernels.h - argument block and launchers of the Step kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

namespace b2g {

#define SOLVER_THREADS 256

// Plain device pointers of one batch, passed by value to every kernel.
struct KernelArgs {
  const int4* wb;
  const int4* wj;
  float4* wg;
  const int* wflags;
  int2* wc;
  const int* world_order;

  float4 *xf, *pos, *vel;
  const float4 *massd, *damp;
  float4* force;
  const float2* lc;
  const int *btype, *bworld;

  const b2g_shape* shape;
  const int *fbody, *fgroup, *fsensor, *fworld;
  const uint32_t* ffilter;
  const float4* fmat;
  float4* aabb;

  JointDev* joints;
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
  int *nparent, *lparent;
  float4* naabb;
  int* nflag;
  int* wroot;
  int* pcount;
  int* poff;
  uint64_t* pairs;
  void* cub_tmp;

  // solver
  int* sc_list;
  VCDev* vc;
  int *ccolor, *corder;
  uint32_t* cprio;
  uint8_t* cready;
  int *inc_cnt, *inc_off, *inc_head;
  unsigned long long* inc_mask;
  int *inc_list, *jinc_list;
  int *jcolor, *jorder;
  uint32_t* jprio;
  uint8_t* jready;
  int* ncolors;

  // events, status
  EventDev* events;
  int64_t event_cap;
  int events_on;
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

void launch_collide(const KernelArgs& a, cudaStream_t s);
void launch_solve(const KernelArgs& a, int nw, cudaStream_t s);
void launch_clear_forces(const KernelArgs& a, int nb, cudaStream_t s);
void launch_bp_build(const KernelArgs& a, int nf, int nw, size_t cub_bytes, int sort_bits, cudaStream_t s);
void launch_bp_emit(const KernelArgs& a, int nf, cudaStream_t s);
void launch_contact_diff(const KernelArgs& a, int src, int dst, cudaStream_t s);
size_t cub_temp_bytes(int nf);
void launch_collide_pairs(const b2g_shape* sa, const float* xa, const b2g_shape* sb, const float* xb, int n,
                          b2g_manifold* out, cudaStream_t s);

}  // namespace b2g
