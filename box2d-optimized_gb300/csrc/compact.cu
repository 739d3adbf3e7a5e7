// compact.cu - device-side compaction of a batch: the worlds that are kept move down to close
// the gaps left by retired ones, in every body, fixture, joint and live-contact array, with their
// global indices (bodies of fixtures and joints, fixtures of contact keys) remapped. World order
// is preserved, so every array stays world-major and the contact list stays sorted by key.
#include "dev_common.cuh"
#include "kernels.h"

namespace b2g {

static inline unsigned cgrid(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

__global__ void k_compact_bodies(CompactTables t, int n, BodyRecs s, BodyRecs d) {
  int ob = blockIdx.x * blockDim.x + threadIdx.x;
  if (ob >= n) return;
  int w = s.bworld[ob];
  int nw = t.wnew[w];
  if (nw < 0) return;
  int nb = t.off_new[w].x + (ob - t.off_old[w].x);
  d.xf[nb] = s.xf[ob];
  d.pos[nb] = s.pos[ob];
  d.vel[nb] = s.vel[ob];
  d.massd[nb] = s.massd[ob];
  d.damp[nb] = s.damp[ob];
  d.force[nb] = s.force[ob];
  d.lc[nb] = s.lc[ob];
  d.btype[nb] = s.btype[ob];
  d.bstate[nb] = s.bstate[ob];
  d.bworld[nb] = nw;
}

__global__ void k_compact_fixtures(CompactTables t, int n, FixRecs s, FixRecs d) {
  int of = blockIdx.x * blockDim.x + threadIdx.x;
  if (of >= n) return;
  int w = s.fworld[of];
  int nw = t.wnew[w];
  if (nw < 0) return;
  int4 oo = t.off_old[w], on = t.off_new[w];
  int nf = on.y + (of - oo.y);
  d.shape[nf] = s.shape[of];
  d.fbody[nf] = s.fbody[of] - oo.x + on.x;
  d.fgroup[nf] = s.fgroup[of];
  d.fsensor[nf] = s.fsensor[of];
  d.fworld[nf] = nw;
  d.ffilter[nf] = s.ffilter[of];
  d.fmat[nf] = s.fmat[of];
  d.frad[nf] = s.frad[of];
}

__global__ void k_compact_joints(CompactTables t, int n, const JointDev* s, const int* bworld_old, JointDev* d) {
  int oj = blockIdx.x * blockDim.x + threadIdx.x;
  if (oj >= n) return;
  JointDev J = s[oj];
  int w = bworld_old[J.d.body_a];
  if (t.wnew[w] < 0) return;
  int4 oo = t.off_old[w], on = t.off_new[w];
  int db = on.x - oo.x;
  J.d.body_a += db;
  J.d.body_b += db;
  J.iA += db;
  J.iB += db;
  if (J.d.type == B2G_JOINT_GEAR) {
    J.g.iC += db;
    J.g.iD += db;
  }
  d[on.z + (oj - oo.z)] = J;
}

__global__ void k_compact_contacts(CompactTables t, int64_t n, ConRecs s, const int* fworld_old, ConRecs d) {
  int64_t oc = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (oc >= n) return;
  int2 fx = s.fix[oc];
  int w = fworld_old[fx.x];
  if (t.wnew[w] < 0) return;
  int df = t.off_new[w].y - t.off_old[w].y;
  int64_t nc = t.con_new[w] + (oc - t.con_old[w]);
  uint64_t key = s.key[oc];
  uint32_t e = (uint32_t)(key >> 32) + (uint32_t)df, p = (uint32_t)key + (uint32_t)df;
  d.key[nc] = ((uint64_t)e << 32) | p;
  d.fix[nc] = make_int2(fx.x + df, fx.y + df);
  d.flags[nc] = s.flags[oc];
  d.mat[nc] = s.mat[oc];
  copy_manifold(&d.man[nc], &s.man[oc]);
}

void launch_compact(const CompactTables& t, int nb, const BodyRecs& sb, const BodyRecs& db, int nf, const FixRecs& sf,
                    const FixRecs& df, int nj, const JointDev* sj, JointDev* dj, int64_t nc, const ConRecs& sc,
                    const ConRecs& dc, cudaStream_t s) {
  // joints and contacts read the old body / fixture world arrays: all kernels read only sources
  if (nj > 0) k_compact_joints<<<cgrid(nj, 128), 128, 0, s>>>(t, nj, sj, sb.bworld, dj);
  if (nc > 0) k_compact_contacts<<<cgrid(nc, 256), 256, 0, s>>>(t, nc, sc, sf.fworld, dc);
  if (nb > 0) k_compact_bodies<<<cgrid(nb, 256), 256, 0, s>>>(t, nb, sb, db);
  if (nf > 0) k_compact_fixtures<<<cgrid(nf, 128), 128, 0, s>>>(t, nf, sf, df);
}

}  // namespace b2g
