// solve_world.cuh - the per-world island solve and its device helpers: the setup half (k_setup:
// islands, solver contacts, colouring, velocity integration, constraint preparation) and the
// iteration half (k_solve, in two builds that differ only in their register budget: the
// occupancy build in solve.cu and the wide build in solve_wide.cu), and the thread-block cluster
// kernel that runs both halves for the largest worlds (solve_cluster.cu).
#pragma once
#include <cuda/atomic>

#include "b2g_math.cuh"
#include "dev_common.cuh"
#include "engine.h"
#include "kernels.h"
#include "solver_dev.cuh"

namespace b2g {

#define FULL_MASK 0xffffffffu

// ---- teams: the threads that solve one world together
//
// CtaTeam<T>: one CTA of T threads; its barrier is __syncthreads.
// ClusterTeam<T, CS>: a thread-block cluster of CS CTAs of T threads each, one world per
// cluster, for worlds too large for one SM. Its barrier is the cluster barrier with release /
// acquire semantics at cluster scope, which orders the team's global-memory and shared-memory
// accesses across the cluster's SMs the way __syncthreads orders a CTA's. Team-wide counters
// live in the shared memory of the cluster's first CTA (rank 0), which the other CTAs reach
// through distributed shared memory.
//
// Every function below is written once against this interface: tid() numbers the team's
// threads 0..kThreads-1, sync() is the team barrier, any() / all() are team-wide votes, lead(p)
// maps a __shared__ object to the team's copy (rank 0's), rank() is the CTA's rank.

__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// Generic address of `p` (a __shared__ object of this CTA) in the shared memory of CTA `rank` of
// the cluster.
template <class X>
__device__ __forceinline__ X* cluster_map(X* p, unsigned rank) {
  uint64_t out;
  asm volatile("mapa.u64 %0, %1, %2;" : "=l"(out) : "l"((uint64_t)p), "r"(rank));
  return reinterpret_cast<X*>(out);
}

template <int T>
struct CtaTeam {
  static constexpr int kThreads = T;
  static constexpr int kCtas = 1;
  static constexpr cuda::thread_scope kScope = cuda::thread_scope_block;
  __device__ __forceinline__ int tid() const { return threadIdx.x; }
  __device__ __forceinline__ int rank() const { return 0; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  __device__ __forceinline__ int any(int p) { return __syncthreads_or(p); }
  __device__ __forceinline__ int all(int p) { return __syncthreads_and(p); }
  template <class X>
  __device__ __forceinline__ X* lead(X* p) const { return p; }
  __device__ __forceinline__ int next_phase() { return 0; }
};

template <int T, int CS>
struct ClusterTeam {
  static constexpr int kThreads = T * CS;
  static constexpr int kCtas = CS;
  static constexpr cuda::thread_scope kScope = cuda::thread_scope_device;
  int r;         // this CTA's rank in the cluster
  int* votes;    // rank 0's three vote words (team copies)
  int vphase;    // the vote word of the next any()
  int sphase;    // parity of the next double-buffered team scratch
  __device__ __forceinline__ int tid() const { return r * T + (int)threadIdx.x; }
  __device__ __forceinline__ int rank() const { return r; }
  __device__ __forceinline__ void sync() const { cluster_barrier(); }
  // CTA vote, then one word on rank 0: the word of a call is cleared two calls before its use
  // (every reader of its previous use has passed a team barrier since), so one team barrier per vote
  __device__ int any(int p) {
    const int local = __syncthreads_or(p);
    int* v = votes + vphase;
    if (threadIdx.x == 0) {
      if (r == 0) votes[vphase == 2 ? 0 : vphase + 1] = 0;
      if (local) atomicOr(v, 1);
    }
    cluster_barrier();
    const int res = *(volatile int*)v;
    vphase = vphase == 2 ? 0 : vphase + 1;
    return res;
  }
  __device__ __forceinline__ int all(int p) { return !any(!p); }
  template <class X>
  __device__ __forceinline__ X* lead(X* p) const { return cluster_map(p, 0); }
  __device__ __forceinline__ int next_phase() {
    const int s = sphase;
    sphase ^= 1;
    return s;
  }
};

// Exclusive prefix of one value per warp of the team (`v`, as given by the warp's lane 0) in team
// warp order: returns the warp's base in every lane and the team total in *total. One CTA barrier
// pair, and in a cluster one team barrier between them: each CTA scans its own warps, rank 0
// collects the CTA sums (double-buffered by call parity, so that a fast CTA's next call does not
// overwrite sums that a slow one still reads).
template <class Team>
__device__ __forceinline__ int team_warp_scan(Team& tm, int v, int* total) {
  constexpr int NW = (Team::kThreads / Team::kCtas) / 32;
  __shared__ int wbase[NW + 1];
  __shared__ int csum[2][Team::kCtas > 1 ? Team::kCtas : 1];
  __shared__ int cbase[2];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) wbase[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int w = 0; w < NW; ++w) {
      const int c = wbase[w];
      wbase[w] = acc;
      acc += c;
    }
    wbase[NW] = acc;
  }
  if constexpr (Team::kCtas == 1) {
    __syncthreads();
    const int base = wbase[wid];
    *total = wbase[NW];
    __syncthreads();  // wbase is reused by the next call
    return base;
  } else {
    const int ph = tm.next_phase();
    if (threadIdx.x == 0) tm.lead(&csum[ph][0])[tm.rank()] = wbase[NW];
    tm.sync();
    if (threadIdx.x == 0) {
      const int* cs = tm.lead(&csum[ph][0]);
      int before = 0, all = 0;
      for (int q = 0; q < Team::kCtas; ++q) {
        const int c = cs[q];
        if (q < tm.rank()) before += c;
        all += c;
      }
      cbase[0] = before;
      cbase[1] = all;
    }
    __syncthreads();
    const int base = cbase[0] + wbase[wid];
    *total = cbase[1];
    __syncthreads();  // wbase and cbase are reused by the next call
    return base;
  }
}

// Stable compaction of [0, n) with kThreads / 32 warp-owned segments (multiples of 32 items, in
// list order): `flag(k)` is evaluated twice, once to count each warp's kept items by ballots and
// once to place them, and kept item k is handed to `emit(k, rank)` with its rank in list order.
// Returns the number kept (in every thread).
// The counting pass keeps each chunk's ballot in shared memory (up to kCompactChunks chunks per
// warp), so the placing pass reads it back instead of evaluating flag() again.
constexpr int kCompactChunks = 64;
template <class Team, class Flag, class Emit>
__device__ __forceinline__ int block_compact(Team& tm, int n, Flag flag, Emit emit) {
  constexpr int NWARP = Team::kThreads / 32;
  constexpr int CW = Team::kThreads / Team::kCtas / 32;  // warps of one CTA
  __shared__ unsigned ballots[CW][kCompactChunks];
  const int lane = threadIdx.x & 31, wid = tm.tid() >> 5, lw = threadIdx.x >> 5;
  const int seg = (((n + NWARP - 1) / NWARP) + 31) & ~31;
  const int s0 = min(n, wid * seg), s1 = min(n, s0 + seg);
  const bool keep = seg / 32 <= kCompactChunks;  // the same for every warp of the team
  int cnt = 0;
  for (int k0 = s0, c = 0; k0 < s1; k0 += 32, ++c) {
    const int k = k0 + lane;
    const unsigned b = __ballot_sync(FULL_MASK, k < s1 && flag(k));
    if (keep && lane == 0) ballots[lw][c] = b;
    cnt += __popc(b);
  }
  __syncwarp();
  int total;
  int base = team_warp_scan(tm, cnt, &total);
  const unsigned lt = (1u << lane) - 1u;
  for (int k0 = s0, c = 0; k0 < s1; k0 += 32, ++c) {
    const int k = k0 + lane;
    const unsigned b = keep ? ballots[lw][c] : __ballot_sync(FULL_MASK, k < s1 && flag(k));
    if ((b >> lane) & 1u) emit(k, base + __popc(b & lt));
    base += __popc(b);
  }
  tm.sync();  // every emit() is visible, and flag()'s inputs may change, after the call
  return total;
}

// Exclusive prefix sums of get(i) over [0, n) in index order, handed to put(i, prefix), with
// warp-owned segments: each warp sums its segment, the warp sums are scanned across the team,
// each warp scans its segment on top. Returns the total (in every thread).
template <class Team, class Get, class Put>
__device__ __forceinline__ int block_exclusive_scan(Team& tm, int n, Get get, Put put) {
  constexpr int NWARP = Team::kThreads / 32;
  const int lane = threadIdx.x & 31, wid = tm.tid() >> 5;
  const int seg = (((n + NWARP - 1) / NWARP) + 31) & ~31;
  const int s0 = min(n, wid * seg), s1 = min(n, s0 + seg);
  int sum = 0;
  for (int k = s0 + lane; k < s1; k += 32) sum += get(k);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(FULL_MASK, sum, o);
  int total;
  int base = team_warp_scan(tm, sum, &total);
  for (int k0 = s0; k0 < s1; k0 += 32) {
    const int k = k0 + lane;
    const int v = k < s1 ? get(k) : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL_MASK, x, o);
      if (lane >= o) x += y;
    }
    if (k < s1) put(k, base + x - v);
    base += __shfl_sync(FULL_MASK, x, 31);
  }
  tm.sync();  // every put() is visible, and get()'s inputs may change, after the call
  return total;
}

// Constraint bodies (ColourMem::cb) of a constraint that is always solved serially (colour 63):
// a gear joint, which moves four bodies. Bits 31 and 30: no world-local body index has bit 30 set.
#define B2G_CB_SERIAL ((int)0xC0000000)

// Working arrays of one colouring, each in shared or global memory (generic pointers).
struct ColourMem {
  int* cnt;                  // per body: incidence count, then fill counter
  int* head;                 // per body: list offset, then first uncoloured entry
  unsigned long long* mask;  // per body: colours taken
  int* list;                 // 2 per constraint: per-body incidence lists
  const int2* cb;            // per constraint: world-local bodies, negative (bit 31 set) = static
  int8_t* col;               // per constraint: colour, -1 until coloured
  uint8_t* rdy;              // per constraint: claimed for a round's frontier
  int4* ent;                 // 2 per constraint, global: list entries {k, body x, body y, slot of
                             // k in the list of its other body (-1: none)}
  int4* wl0;                 // frontiers of entries (n each, global)
  int4* wl1;
};

// Greedy colouring in priority order, computed in parallel rounds (Jones-Plassmann with
// smallest-free-colour choice): a constraint is coloured once it is the first uncoloured entry
// of the priority-sorted incidence list of each of its non-static bodies; it then takes the
// lowest colour not used at those bodies. The result equals the sequential greedy pass in
// (priority, index) order. Colours 0..62 are regular; 63 is the overflow colour, solved
// serially in priority order. Buckets the constraints by colour into `order` (and its inverse
// into `slot` when given) and writes the colour offsets to `ranges` (ncol + 1 entries). Returns
// the number of colours (max + 1).
template <class Team>
__device__ int colour_constraints(Team& tm, int n, int nb, const ColourMem m, const uint32_t* prio, int* order,
                                  int* slot, int* ranges, unsigned int* status) {
  constexpr int NT = Team::kThreads;
  const int tid = tm.tid();
  for (int i = tid; i < nb; i += NT) {
    m.cnt[i] = 0;
    m.mask[i] = 0ull;
  }
  for (int k = tid; k < n; k += NT) m.col[k] = -1;
  tm.sync();
  for (int k = tid; k < n; k += NT) {
    int2 b = m.cb[k];
    if (b.x >= 0) atomicAdd(&m.cnt[b.x], 1);
    if (b.y >= 0) atomicAdd(&m.cnt[b.y], 1);
  }
  tm.sync();
  const int nslots = block_exclusive_scan(tm, nb, [&](int i) { return m.cnt[i]; }, [&](int i, int p) { m.head[i] = p; });
  for (int i = tid; i < nb; i += NT) m.cnt[i] = 0;
  tm.sync();
  for (int k = tid; k < n; k += NT) {
    int2 b = m.cb[k];
    if (b.x >= 0) m.list[m.head[b.x] + atomicAdd(&m.cnt[b.x], 1)] = k;
    if (b.y >= 0) m.list[m.head[b.y] + atomicAdd(&m.cnt[b.y], 1)] = k;
  }
  tm.sync();
  // each body's list in (priority, index) order: lists of up to 8 entries sorted in registers
  // (their priorities read together), longer ones by insertion; cnt becomes the list's end
  for (int i = tid; i < nb; i += NT) {
    const int off = m.head[i], cnt = m.cnt[i];
    if (cnt <= 8) {
      uint64_t key[8];
#pragma unroll
      for (int x = 0; x < 8; ++x) {
        const int kx = x < cnt ? m.list[off + x] : 0;
        key[x] = x < cnt ? (((uint64_t)prio[kx] << 32) | (uint32_t)kx) : ~0ull;
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
#pragma unroll
        for (int x = r & 1; x + 1 < 8; x += 2) {
          const uint64_t u = key[x], v = key[x + 1];
          key[x] = u < v ? u : v;
          key[x + 1] = u < v ? v : u;
        }
      }
#pragma unroll
      for (int x = 0; x < 8; ++x)
        if (x < cnt) m.list[off + x] = (int)(uint32_t)key[x];
    } else {
      for (int x = 1; x < cnt; ++x) {
        int kx = m.list[off + x];
        uint32_t px = prio[kx];
        int y = x - 1;
        while (y >= 0) {
          int ky = m.list[off + y];
          uint32_t py = prio[ky];
          if (py < px || (py == px && ky < kx)) break;
          m.list[off + y + 1] = ky;
          --y;
        }
        m.list[off + y + 1] = kx;
      }
    }
    m.cnt[i] = off + cnt;
  }
  // each list slot's entry: the constraint, its bodies and its slot in the list of its other
  // body, so that one load of an entry tells whether its constraint heads both its lists. The
  // constraints' slots per body go to the second frontier's space first (unused until a round).
  // A thread per slot: the slot's body is the constraint's body whose list range holds it (the
  // lists lie one after another in body order, heads still at their starts).
  tm.sync();
  int2* posk = reinterpret_cast<int2*>(m.wl1);
  auto on_x = [&](int s2, int2 c) { return c.x >= 0 && s2 >= m.head[c.x] && s2 < m.cnt[c.x]; };
  for (int s2 = tid; s2 < nslots; s2 += NT) {
    const int k = m.list[s2];
    if (on_x(s2, m.cb[k])) posk[k].x = s2;
    else posk[k].y = s2;
  }
  tm.sync();
  for (int s2 = tid; s2 < nslots; s2 += NT) {
    const int k = m.list[s2];
    const int2 c = m.cb[k];
    const bool onX = on_x(s2, c);
    const int other = onX ? c.y : c.x;
    m.ent[s2] = make_int4(k, c.x, c.y, other < 0 ? -1 : (onX ? posk[k].y : posk[k].x));
  }
  // rounds: a round colours every constraint that heads the priority lists of all its
  // non-static bodies (at least the uncoloured one of lowest (priority, index)). The frontier of
  // a round holds exactly those: at the start, the constraints that head all their lists; after
  // a round, the new heads of the lists its constraints left, where they head all their lists
  // (claimed once through their rdy byte: two lists may hand over the same constraint). Each
  // constraint is looked at a bounded number of times, whatever the number of rounds. Frontier
  // sizes alternate between two team counters: a round reads one and fills the other, which it
  // clears before its first barrier (every thread read it two barriers ago).
  __shared__ int s_cnt_own[2];
  int* s_cnt = tm.lead(s_cnt_own);
  if (tid == 0) {
    s_cnt[0] = 0;
    s_cnt[1] = 0;
  }
  for (int k = tid; k < n; k += NT) m.rdy[k] = 0;
  tm.sync();
  int4* wl = m.wl0;
  int4* wn = m.wl1;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  // pushes the flagged entries of a warp onto frontier `dst` (team counter `ctr`)
  auto push = [&](bool f, int4 e, int4* dst, int* ctr) {
    const unsigned bal = __ballot_sync(FULL_MASK, f);
    int base = 0;
    if (lane == 0 && bal) base = atomicAdd(ctr, __popc(bal));
    base = __shfl_sync(FULL_MASK, base, 0);
    if (f) dst[base + __popc(bal & lt)] = e;
  };
  // whether the entry at the head of body bb's list heads its other body's list too
  auto heads_other = [&](int bb, int4 e) {
    const int other = e.y == bb ? e.z : e.y;
    return other < 0 || m.head[other] == e.w;
  };
  // the first frontier: list heads that head both their lists (pushed from the x body's list when
  // both bodies have one), and the constraints without a non-static body
  for (int i0 = 0; i0 < nb; i0 += NT) {  // team-uniform trip counts: whole warps reach the ballots
    const int i = i0 + tid;
    int4 e = make_int4(0, 0, 0, 0);
    bool f = false;
    if (i < nb && m.head[i] < m.cnt[i]) {
      e = m.ent[m.head[i]];
      f = heads_other(i, e) && (e.y == i || e.y < 0);
    }
    push(f, e, wl, &s_cnt[0]);
  }
  for (int i0 = 0; i0 < n; i0 += NT) {
    const int k = i0 + tid;
    int2 c = make_int2(0, 0);
    if (k < n) c = m.cb[k];
    push(k < n && c.x < 0 && c.y < 0, make_int4(k, c.x, c.y, -1), wl, &s_cnt[0]);
  }
  tm.sync();
  int coloured = 0;
  bool done = (n == 0);
  for (int round = 0; round <= n && !done; ++round) {
    const int cur = round & 1;
    const int cnt = *(volatile int*)&s_cnt[cur];
    if (cnt == 0) break;  // every thread reads the same count
    if (round > 0 && tid == 0) s_cnt[cur ^ 1] = 0;
    for (int i = tid; i < cnt; i += NT) {
      const int4 e = wl[i];
      const int k = e.x;
      const int2 b = make_int2(e.y, e.z);
      const unsigned long long used = (b.x >= 0 ? m.mask[b.x] : 0ull) | (b.y >= 0 ? m.mask[b.y] : 0ull);
      const unsigned long long freeBits = ~used & ((1ull << 63) - 1ull);
      int c;
      if (freeBits == 0ull || b.x == B2G_CB_SERIAL) {
        c = 63;
      } else {
        c = __ffsll((long long)freeBits) - 1;
        if (b.x >= 0) m.mask[b.x] |= 1ull << c;
        if (b.y >= 0) m.mask[b.y] |= 1ull << c;
      }
      m.col[k] = (int8_t)c;
      if (b.x >= 0) m.head[b.x] += 1;
      if (b.y >= 0) m.head[b.y] += 1;
    }
    coloured += cnt;
    tm.sync();
    for (int i0 = 0; i0 < cnt; i0 += NT) {
      const int i = i0 + tid;
      int4 cand[2] = {make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0)};
      bool has[2] = {false, false};
      if (i < cnt) {
        const int4 e = wl[i];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int bb = q ? e.z : e.y;
          if (bb < 0) continue;
          const int h = m.head[bb];
          if (h >= m.cnt[bb]) continue;  // the list is done
          const int4 e2 = m.ent[h];
          if (!heads_other(bb, e2)) continue;
          // claim the constraint: set its rdy byte through the aligned word that holds it
          const uintptr_t addr = reinterpret_cast<uintptr_t>(&m.rdy[e2.x]);
          const unsigned sh = (unsigned)(addr & 3u) * 8u;
          const unsigned old = atomicOr(reinterpret_cast<unsigned*>(addr & ~(uintptr_t)3u), 1u << sh);
          if (!((old >> sh) & 1u)) {
            cand[q] = e2;
            has[q] = true;
          }
        }
      }
      push(has[0], cand[0], wn, &s_cnt[cur ^ 1]);
      push(has[1], cand[1], wn, &s_cnt[cur ^ 1]);
    }
    tm.sync();
    int4* t = wl;
    wl = wn;
    wn = t;
  }
  done = (coloured == n);
  if (!done && tid == 0) atomicOr(status, B2G_DEV_COLOR_ROUNDS);
  // bucket by colour: each CTA counts its constraints per colour; a colour's slots go to the CTAs
  // in rank order (the order inside a colour does not matter), so CTA r places its constraints of
  // colour c from off[c] = start of c + counts of c in the CTAs before it
  __shared__ int col_cnt[64];       // this CTA's count per colour, then its fill counter
  __shared__ int col_off[65];       // global start of each colour, then this CTA's offset
  __shared__ int col_tot[65];       // team total per colour, then the colour offsets
  __shared__ int cta_cnt[Team::kCtas > 1 ? 2 : 1][Team::kCtas > 1 ? Team::kCtas * 64 : 1];
  if (threadIdx.x < 64) col_cnt[threadIdx.x] = 0;
  __syncthreads();
  for (int k = tid; k < n; k += NT) {
    int c = m.col[k];
    if (c < 0) c = 63;  // only after a failed colouring (status raised)
    atomicAdd(&col_cnt[c], 1);
  }
  __syncthreads();
  if constexpr (Team::kCtas == 1) {
    if (threadIdx.x < 64) col_tot[threadIdx.x] = col_cnt[threadIdx.x];
  } else {
    const int ph = tm.next_phase();
    int* all = tm.lead(&cta_cnt[ph][0]);
    if (threadIdx.x < 64) all[tm.rank() * 64 + threadIdx.x] = col_cnt[threadIdx.x];
    tm.sync();
    if (threadIdx.x < 64) {
      int before = 0, tot = 0;
      for (int q = 0; q < Team::kCtas; ++q) {
        const int v = all[q * 64 + threadIdx.x];
        if (q < tm.rank()) before += v;
        tot += v;
      }
      col_tot[threadIdx.x] = tot;
      col_off[threadIdx.x] = before;  // added to the colour's start below
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0, mx = -1;
    for (int c = 0; c < 64; ++c) {
      const int t = col_tot[c];
      if (t > 0) mx = c;
      col_tot[c] = s;
      s += t;
    }
    col_tot[64] = s;
    col_off[64] = mx + 1;  // the number of colours
  }
  __syncthreads();
  const int ncol = col_off[64];
  if (threadIdx.x < 64) {
    col_off[threadIdx.x] = col_tot[threadIdx.x] + (Team::kCtas == 1 ? 0 : col_off[threadIdx.x]);
    col_cnt[threadIdx.x] = 0;
  }
  __syncthreads();
  for (int k = tid; k < n; k += NT) {
    int c = m.col[k];
    if (c < 0) c = 63;
    int pos = col_off[c] + atomicAdd(&col_cnt[c], 1);
    order[pos] = k;
    if (slot) slot[k] = pos;
  }
  tm.sync();
  const int n63 = col_tot[64] - col_tot[63];
  if (tid == 0 && n63 > 1) {
    int off = col_tot[63], cnt = n63;
    for (int x = 1; x < cnt; ++x) {
      int kx = order[off + x];
      uint32_t px = prio[kx];
      int y = x - 1;
      while (y >= 0) {
        int ky = order[off + y];
        uint32_t py = prio[ky];
        if (py < px || (py == px && ky < kx)) break;
        order[off + y + 1] = ky;
        --y;
      }
      order[off + y + 1] = kx;
    }
    if (slot)
      for (int x = 0; x < cnt; ++x) slot[order[off + x]] = off + x;
  }
  for (int c = threadIdx.x; c <= ncol; c += Team::kThreads / Team::kCtas) ranges[c] = col_tot[c];
  tm.sync();
  return ncol;
}

// ---- constraint planes <-> the per-constraint register record
__device__ __forceinline__ void store_planes(const SolverPlanes& P, int s, const VCDev& vc) {
  P.idx[s] = make_int2(vc.indexA | (vc.pointCount << 24) | (vc.pcPointCount << 28), vc.indexB | (vc.type << 24));
  P.cid[s] = vc.contact;
  P.nf[s] = make_float4(vc.normal[0], vc.normal[1], vc.friction, vc.tangentSpeed);
  P.r0[s] = make_float4(vc.rA[0][0], vc.rA[0][1], vc.rB[0][0], vc.rB[0][1]);
  P.r1[s] = make_float4(vc.rA[1][0], vc.rA[1][1], vc.rB[1][0], vc.rB[1][1]);
  P.nmtm[s] = make_float4(vc.normalMass[0], vc.normalMass[1], vc.tangentMass[0], vc.tangentMass[1]);
  P.bk[s] = make_float4(vc.velocityBias[0], vc.velocityBias[1], vc.K[0], vc.K[1]);
  P.kn[s] = make_float4(vc.K[3], vc.NM[0], vc.NM[1], vc.NM[3]);
  P.imp[s] = make_float4(vc.normalImpulse[0], vc.normalImpulse[1], vc.tangentImpulse[0], vc.tangentImpulse[1]);
  P.lcs[s] = make_float4(vc.localCenterA[0], vc.localCenterA[1], vc.localCenterB[0], vc.localCenterB[1]);
  P.lnp[s] = make_float4(vc.localNormal[0], vc.localNormal[1], vc.localPoint[0], vc.localPoint[1]);
  P.lps[s] = make_float4(vc.localPoints[0][0], vc.localPoints[0][1], vc.localPoints[1][0], vc.localPoints[1][1]);
  P.rad[s] = make_float2(vc.radiusA, vc.radiusB);
}

// Inverse mass and inertia per world-local body: (1/m, 1/I) pairs in shared memory, or the
// global mass records (m, 1/m, I, 1/I) of the world.
struct Masses {
  const float2* sm;
  const float4* g;
  __device__ __forceinline__ float2 get(int i) const {
    if (sm) return sm[i];
    float4 m = g[i];
    return make_float2(m.y, m.w);
  }
};

// The rows of one constraint read by the velocity phase (warm start, velocity iterations) and by
// the position iterations; all loads are issued together (none waits for another).
struct VelRows {
  int2 id;
  float4 nf, r0, r1, nmtm, bk, kn, imp;
};
struct PosRows {
  int2 id;
  float4 lcs, lnp, lps;
  float2 rad;
};

__device__ __forceinline__ void fetch_vel(const SolverPlanes& P, int s, VelRows& r) {
  r.id = P.idx[s];
  r.nf = P.nf[s];
  r.r0 = P.r0[s];
  r.r1 = P.r1[s];
  r.nmtm = P.nmtm[s];
  r.bk = P.bk[s];
  r.kn = P.kn[s];
  r.imp = P.imp[s];
}

// L1 prefetch of a constraint's velocity rows (no registers held).
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
__device__ __forceinline__ void hint_vel(const SolverPlanes& P, int s) {
  prefetch_l1(P.idx + s);
  prefetch_l1(P.nf + s);
  prefetch_l1(P.r0 + s);
  prefetch_l1(P.r1 + s);
  prefetch_l1(P.nmtm + s);
  prefetch_l1(P.bk + s);
  prefetch_l1(P.kn + s);
  prefetch_l1(P.imp + s);
}

// L1 prefetch of a constraint's position rows (no registers held).
__device__ __forceinline__ void hint_pos(const SolverPlanes& P, int s) {
  prefetch_l1(P.idx + s);
  prefetch_l1(P.lcs + s);
  prefetch_l1(P.lnp + s);
  prefetch_l1(P.lps + s);
  prefetch_l1(P.rad + s);
}
__device__ __forceinline__ void fetch_pos(const SolverPlanes& P, int s, PosRows& r) {
  r.id = P.idx[s];
  r.lcs = P.lcs[s];
  r.lnp = P.lnp[s];
  r.lps = P.lps[s];
  r.rad = P.rad[s];
}

__device__ __forceinline__ void unpack_common(int2 id, VCDev& vc, const Masses& M) {
  vc.indexA = id.x & 0xffffff;
  vc.indexB = id.y & 0xffffff;
  vc.pointCount = (id.x >> 24) & 15;
  vc.pcPointCount = (id.x >> 28) & 15;
  vc.type = id.y >> 24;
  float2 ma = M.get(vc.indexA), mb = M.get(vc.indexB);
  vc.invMassA = ma.x; vc.invIA = ma.y; vc.invMassB = mb.x; vc.invIB = mb.y;
}

// Fields read by warmStartContact / solveContactVelocity (1-point rows of the second point and
// the block solver hold zeros and are not used).
__device__ __forceinline__ void unpack_vel(const VelRows& r, VCDev& vc, const Masses& M) {
  unpack_common(r.id, vc, M);
  vc.normal[0] = r.nf.x; vc.normal[1] = r.nf.y; vc.friction = r.nf.z; vc.tangentSpeed = r.nf.w;
  vc.rA[0][0] = r.r0.x; vc.rA[0][1] = r.r0.y; vc.rB[0][0] = r.r0.z; vc.rB[0][1] = r.r0.w;
  vc.rA[1][0] = r.r1.x; vc.rA[1][1] = r.r1.y; vc.rB[1][0] = r.r1.z; vc.rB[1][1] = r.r1.w;
  vc.normalImpulse[0] = r.imp.x; vc.normalImpulse[1] = r.imp.y;
  vc.tangentImpulse[0] = r.imp.z; vc.tangentImpulse[1] = r.imp.w;
  vc.normalMass[0] = r.nmtm.x; vc.normalMass[1] = r.nmtm.y; vc.tangentMass[0] = r.nmtm.z; vc.tangentMass[1] = r.nmtm.w;
  vc.velocityBias[0] = r.bk.x; vc.velocityBias[1] = r.bk.y;
  vc.K[0] = r.bk.z; vc.K[1] = r.bk.w; vc.K[2] = r.bk.w; vc.K[3] = r.kn.x;
  vc.NM[0] = r.kn.y; vc.NM[1] = r.kn.z; vc.NM[2] = r.kn.z; vc.NM[3] = r.kn.w;
}

// Fields read by solveContactPosition.
__device__ __forceinline__ void unpack_pos(const PosRows& r, VCDev& vc, const Masses& M) {
  unpack_common(r.id, vc, M);
  vc.localCenterA[0] = r.lcs.x; vc.localCenterA[1] = r.lcs.y; vc.localCenterB[0] = r.lcs.z; vc.localCenterB[1] = r.lcs.w;
  vc.localNormal[0] = r.lnp.x; vc.localNormal[1] = r.lnp.y; vc.localPoint[0] = r.lnp.z; vc.localPoint[1] = r.lnp.w;
  vc.localPoints[0][0] = r.lps.x; vc.localPoints[0][1] = r.lps.y;
  vc.localPoints[1][0] = r.lps.z; vc.localPoints[1][1] = r.lps.w;
  vc.radiusA = r.rad.x; vc.radiusB = r.rad.y;
}

// One pass over the contact colours: colour by colour, a team barrier after each; colour 63 (the
// overflow colour) is solved serially by thread 0 in priority order. With PREFETCH each thread
// reads the rows of its first constraint of the next regular colour before the barrier, so that
// their round trip overlaps the wait, and within a colour the rows of its next constraint before
// it solves the current one: rows do not change while a colour is solved (a constraint's impulses
// are written only by its own solve, once per pass), only the bodies do, and those are read after.
// PIPE (with PREFETCH): 1 = the rows of the thread's next constraint of the colour are read into
// registers before the current one is solved; 2 = they are only prefetched into L1 (`hint`), for
// rows too large to hold twice in registers.
template <class Team, class Rows, bool PREFETCH, int PIPE, class Fetch, class Solve, class Hint>
__device__ __forceinline__ void colour_sweep(Team& tm, const int* ranges, int ncol, int c0, Fetch fetch, Solve solve,
                                             Hint hint) {
  constexpr int NT = Team::kThreads;
  const int tid = tm.tid();
  Rows pre;
  bool have = false;  // pre holds the rows of this thread's first constraint of colour c
  if (PREFETCH && ncol > 0 && ranges[0] + tid < ranges[1]) {
    fetch(c0 + ranges[0] + tid, pre);
    have = true;
  }
  for (int c = 0; c < ncol; ++c) {
    int s = ranges[c], e = ranges[c + 1];
    if (c == 63) {
      if (tid == 0)
        for (int i = s; i < e; ++i) {
          Rows r;
          fetch(c0 + i, r);
          solve(c0 + i, r);
        }
    } else if (PREFETCH && PIPE == 2) {
      int i = s + tid;
      if (have) {
        if (i + NT < e) hint(c0 + i + NT);
        solve(c0 + i, pre);
        i += NT;
      }
      for (; i < e; i += NT) {
        Rows r;
        fetch(c0 + i, r);
        if (i + NT < e) hint(c0 + i + NT);
        solve(c0 + i, r);
      }
    } else if (PREFETCH && PIPE == 1) {
      // a thread with several constraints in the colour reads the next one's rows before it
      // solves the current one, so that their round trip overlaps the solve
      int i = s + tid;
      Rows cur;
      bool hc = have;
      if (hc) cur = pre;
      else if (i < e) {
        fetch(c0 + i, cur);
        hc = true;
      }
      while (hc) {
        Rows nxt;
        const int j = i + NT;
        const bool hn = j < e;
        if (hn) fetch(c0 + j, nxt);
        solve(c0 + i, cur);
        i = j;
        cur = nxt;
        hc = hn;
      }
    } else {
      for (int i = s + tid; i < e; i += NT) {
        Rows r;
        fetch(c0 + i, r);
        solve(c0 + i, r);
      }
    }
    have = false;
    if (PREFETCH && c + 1 < ncol && c + 1 != 63 && ranges[c + 1] + tid < ranges[c + 2]) {
      fetch(c0 + ranges[c + 1] + tid, pre);
      have = true;
    }
    tm.sync();
  }
}

// Carves 16-byte aligned pieces out of the CTA's dynamic shared memory.
struct SmemCarver {
  unsigned char* p;
  size_t left;
  __device__ void* take(size_t bytes) {
    bytes = (bytes + 15) & ~(size_t)15;
    if (bytes > left) return nullptr;
    void* r = p;
    p += bytes;
    left -= bytes;
    return r;
  }
};

// ---- islands of sleep-mode worlds (b2World::Solve's depth-first search, src/dynamics/b2_world.cpp:520-650)
// Connected components over solid contacts (touching, enabled, no sensor) and joints between
// non-static bodies, as a lock-free union-find that always hooks the larger root under the
// smaller: every component's root is its lowest body index, whatever the order of the unions.
// A world's island records are touched by its CTA alone: every access is a CTA-scope atomic
// (loads included, so that none is served from a line older than an atomic), and the CTA barrier
// orders the phases.
template <cuda::thread_scope S = cuda::thread_scope_block>
__device__ __forceinline__ int isl_load(int* p) {
  return cuda::atomic_ref<int, S>(*p).load(cuda::memory_order_relaxed);
}
template <cuda::thread_scope S = cuda::thread_scope_block>
__device__ __forceinline__ void isl_store(int* p, int v) {
  cuda::atomic_ref<int, S>(*p).store(v, cuda::memory_order_relaxed);
}
template <cuda::thread_scope S = cuda::thread_scope_block>
__device__ __forceinline__ void isl_or(int* p, int v) {
  cuda::atomic_ref<int, S>(*p).fetch_or(v, cuda::memory_order_relaxed);
}
template <cuda::thread_scope S = cuda::thread_scope_block>
__device__ __forceinline__ int isl_label(int4* SL, int i) { return isl_load<S>(&SL[i].x); }
template <cuda::thread_scope S = cuda::thread_scope_block>
__device__ __forceinline__ int isl_bits(int4* SL, int i) { return isl_load<S>(&SL[i].y); }

// Root of x. With `halve`, path halving shortens the walk (x is no root, so no hook targets it);
// halving stores only during the unions: a late halving store could otherwise overwrite a final
// label with an intermediate ancestor.
template <cuda::thread_scope S = cuda::thread_scope_block>
__device__ inline int isl_find(int4* SL, int x, bool halve, unsigned int* status) {
  for (int guard = 0; guard < (1 << 24); ++guard) {
    int p = isl_load<S>(&SL[x].x);
    if (p == x) return x;
    int g = isl_load<S>(&SL[p].x);
    if (halve && g != p) isl_store<S>(&SL[x].x, g);
    x = g;
  }
  raise_status(status, B2G_DEV_STACK_OVERFLOW);
  return x;
}

template <cuda::thread_scope S = cuda::thread_scope_block>
__device__ inline void isl_unite(int4* SL, int x, int y, unsigned int* status) {
  for (int guard = 0; guard < (1 << 20); ++guard) {
    x = isl_find<S>(SL, x, true, status);
    y = isl_find<S>(SL, y, true, status);
    if (x == y) return;
    if (x < y) {
      int t = x;
      x = y;
      y = t;
    }
    int expect = x;  // x was hooked meanwhile when this fails: retry from its root
    if (cuda::atomic_ref<int, S>(SL[x].x)
            .compare_exchange_strong(expect, y, cuda::memory_order_relaxed))
      return;
  }
  raise_status(status, B2G_DEV_STACK_OVERFLOW);
}

// Applies this step's narrowphase wakes (b2Contact::Update's SetAwake(true) on a touching change,
// src/dynamics/b2_contact.cpp:183-188), labels the islands, and wakes every member of an island
// that holds an awake body (the search marks the bodies it reaches awake without resetting their
// sleep timers, b2_world.cpp:565-566). Sleeping islands are neither integrated nor solved.
// The labels are kept between steps: a world whose island graph did not change since its last
// labelling (no solid contact began or stopped touching, no contact was created or destroyed,
// same layout: the world's isl_dirty flag is clear) reuses them and only redoes the awake marks.
// Relabelling in shared memory (a CTA team whose shared memory holds 6 bytes per body): the labels
// (int), linked marks and awake marks (a byte each) are worked on there with block-scope
// atomics, and the island records are written once at the end. Same result as the global path.
template <class Team>
__device__ void relabel_islands_smem(Team& tm, const KernelArgs& a, int b0, int nb, int c0, int ncAll, int j0,
                                     int nj, unsigned char* smem) {
  constexpr int T = Team::kThreads;
  const int tid = tm.tid();
  int* lab = reinterpret_cast<int*>(smem);
  uint8_t* lnk = smem + 4 * (size_t)nb;
  uint8_t* awk = lnk + nb;
  int4* SL = a.sl + b0;
  int2* BS = a.bstate + b0;
  // the same union-find as the global path (lock-free, the larger root hooked under the smaller)
  for (int i = tid; i < nb; i += T) {
    lab[i] = a.btype[b0 + i] == B2G_STATIC ? -1 : i;
    lnk[i] = 0;
    awk[i] = 0;
  }
  tm.sync();
  auto find = [&](int x, bool halve) {
    for (int guard = 0; guard < (1 << 24); ++guard) {
      const int p = cuda::atomic_ref<int, cuda::thread_scope_block>(lab[x]).load(cuda::memory_order_relaxed);
      if (p == x) return x;
      const int g = cuda::atomic_ref<int, cuda::thread_scope_block>(lab[p]).load(cuda::memory_order_relaxed);
      if (halve && g != p) cuda::atomic_ref<int, cuda::thread_scope_block>(lab[x]).store(g, cuda::memory_order_relaxed);
      x = g;
    }
    raise_status(a.status, B2G_DEV_STACK_OVERFLOW);
    return x;
  };
  auto unite = [&](int x, int y) {
    for (int guard = 0; guard < (1 << 20); ++guard) {
      x = find(x, true);
      y = find(y, true);
      if (x == y) return;
      if (x < y) {
        const int t = x;
        x = y;
        y = t;
      }
      int expect = x;  // x was hooked meanwhile when this fails: retry from its root
      if (cuda::atomic_ref<int, cuda::thread_scope_block>(lab[x])
              .compare_exchange_strong(expect, y, cuda::memory_order_relaxed))
        return;
    }
    raise_status(a.status, B2G_DEV_STACK_OVERFLOW);
  };
  for (int k = tid; k < ncAll; k += T) {
    const int2 f = a.cfix[c0 + k];
    const int ia = a.fbody[f.x] - b0, ib = a.fbody[f.y] - b0;
    lnk[ia] = 1;
    lnk[ib] = 1;
    const uint32_t fl = a.cflags[c0 + k];
    if ((fl & B2G_CONTACT_TOUCHING) && (fl & B2G_CONTACT_ENABLED) && (!a.any_sensor || (!a.fsensor[f.x] && !a.fsensor[f.y])) &&
        lab[ia] >= 0 && lab[ib] >= 0)
      unite(ia, ib);
  }
  for (int k = tid; k < nj; k += T) {
    const JointDev& J = a.joints[j0 + k];
    const int ia = J.d.body_a - b0, ib = J.d.body_b - b0;
    lnk[ia] = 1;
    lnk[ib] = 1;
    if (lab[ia] >= 0 && lab[ib] >= 0) unite(ia, ib);
  }
  tm.sync();
  // labels (roots no longer change), and the awake mark of every island with an awake member
  for (int i = tid; i < nb; i += T) {
    if (lab[i] < 0) continue;
    const int r = find(i, false);
    if (BS[i].x & B2G_BS_AWAKE) awk[r] = 1;
  }
  tm.sync();
  for (int i = tid; i < nb; i += T) {
    const int l = lab[i];
    const int r = l < 0 ? -1 : find(i, false);
    if (r >= 0 && awk[r]) BS[i].x |= B2G_BS_AWAKE;
    SL[i] = make_int4(r, (lnk[i] ? B2G_ISL_LINKED : 0) | (r == i && awk[i] ? B2G_ISL_AWAKE : 0), 0, 0x7f7fffff);
  }
  tm.sync();
}

template <class Team>
__device__ void build_islands(Team& tm, const KernelArgs& a, int w, int b0, int nb, int c0, int ncAll, int j0,
                              int nj, unsigned char* smem = nullptr, int smem_bytes = 0) {
  constexpr cuda::thread_scope S = Team::kScope;
  constexpr int T = Team::kThreads;
  const int tid = tm.tid();
  int4* SL = a.sl + b0;
  int2* BS = a.bstate + b0;
  const bool relabel = a.isl_dirty[w] != 0;
  if (relabel && Team::kCtas == 1 && smem && 6 * (size_t)nb <= (size_t)smem_bytes) {
    // this step's narrowphase wakes first, as below
    for (int i = tid; i < nb; i += T) {
      const int bi = b0 + i;
      if (a.bwake[bi]) {
        a.bwake[bi] = 0;
        if (a.btype[bi] != B2G_STATIC) {
          int2 st = BS[i];
          st.x |= B2G_BS_AWAKE;
          st.y = 0;
          BS[i] = st;
        }
      }
    }
    tm.sync();
    relabel_islands_smem(tm, a, b0, nb, c0, ncAll, j0, nj, smem);
    if (tid == 0) a.isl_dirty[w] = 0;  // every thread read the flag before the first barrier
    tm.sync();
    return;
  }
  for (int i = tid; i < nb; i += T) {
    const int bi = b0 + i;
    const bool stat = a.btype[bi] == B2G_STATIC;
    if (a.bwake[bi]) {
      a.bwake[bi] = 0;
      if (!stat) {
        int2 st = BS[i];
        st.x |= B2G_BS_AWAKE;
        st.y = 0;
        BS[i] = st;
      }
    }
    if (relabel) {
      isl_store<S>(&SL[i].x, stat ? -1 : i);
      isl_store<S>(&SL[i].y, 0);
    } else {  // the label and the body's LINKED bit stand; the island bits start over
      isl_store<S>(&SL[i].y, isl_load<S>(&SL[i].y) & B2G_ISL_LINKED);
    }
    isl_store<S>(&SL[i].z, 0);
    isl_store<S>(&SL[i].w, 0x7f7fffff);  // FLT_MAX: no member timed yet
  }
  tm.sync();
  if (relabel) {
    for (int k = tid; k < ncAll; k += T) {
      const int2 f = a.cfix[c0 + k];
      const int ia = a.fbody[f.x] - b0, ib = a.fbody[f.y] - b0;
      if (!(isl_bits<S>(SL, ia) & B2G_ISL_LINKED)) isl_or<S>(&SL[ia].y, B2G_ISL_LINKED);
      if (!(isl_bits<S>(SL, ib) & B2G_ISL_LINKED)) isl_or<S>(&SL[ib].y, B2G_ISL_LINKED);
      const uint32_t fl = a.cflags[c0 + k];
      if ((fl & B2G_CONTACT_TOUCHING) && (fl & B2G_CONTACT_ENABLED) && (!a.any_sensor || (!a.fsensor[f.x] && !a.fsensor[f.y])) &&
          isl_load<S>(&SL[ia].x) >= 0 && isl_load<S>(&SL[ib].x) >= 0)
        isl_unite<S>(SL, ia, ib, a.status);
    }
    for (int k = tid; k < nj; k += T) {
      const JointDev& J = a.joints[j0 + k];
      const int ia = J.d.body_a - b0, ib = J.d.body_b - b0;
      isl_or<S>(&SL[ia].y, B2G_ISL_LINKED);
      isl_or<S>(&SL[ib].y, B2G_ISL_LINKED);
      if (isl_load<S>(&SL[ia].x) >= 0 && isl_load<S>(&SL[ib].x) >= 0) isl_unite<S>(SL, ia, ib, a.status);
    }
    tm.sync();
  }
  // labels, and the awake mark of every island with an awake member (roots no longer change)
  for (int i = tid; i < nb; i += T) {
    if (isl_load<S>(&SL[i].x) < 0) continue;
    int r;
    if (relabel) {
      r = isl_find<S>(SL, i, false, a.status);
      isl_store<S>(&SL[i].x, r);
    } else {
      r = isl_load<S>(&SL[i].x);
    }
    if (BS[i].x & B2G_BS_AWAKE) isl_or<S>(&SL[r].y, B2G_ISL_AWAKE);
  }
  tm.sync();
  for (int i = tid; i < nb; i += T) {
    const int r = isl_label<S>(SL, i);
    if (r >= 0 && (isl_bits<S>(SL, r) & B2G_ISL_AWAKE)) BS[i].x |= B2G_BS_AWAKE;
  }
  if (tid == 0 && relabel) a.isl_dirty[w] = 0;  // every thread read the flag before the first barrier
  tm.sync();
}

// Island root of a contact or joint between world-local bodies la and lb (one is non-static).
template <cuda::thread_scope S = cuda::thread_scope_block>
__device__ __forceinline__ int isl_root(int4* SL, int la, int lb) {
  const int r = isl_label<S>(SL, la);
  return r >= 0 ? r : isl_label<S>(SL, lb);
}

__device__ __forceinline__ bool joint_awake(const KernelArgs& a, const JointDev& J) {
  return ((a.bstate[J.d.body_a].x | a.bstate[J.d.body_b].x) & B2G_BS_AWAKE) != 0;
}

// Sleep timers of the bodies solved this step, then islands whose every member has rested for
// b2_timeToSleep and whose position constraints were solved go to sleep (SetAwake(false): flags,
// timer, velocities, force and torque cleared; include/box2d/b2_body.h:719-740). A body with no
// contact and no joint is an orphan: it times itself, and when its timer runs out its velocity and
// force are cleared but it stays awake (b2World::Solve marks orphans awake after solving them,
// b2_world.cpp:545-549).
template <class Team>
__device__ void sleep_islands(Team& tm, const KernelArgs& a, int b0, int nb) {
  constexpr cuda::thread_scope S = Team::kScope;
  constexpr int T = Team::kThreads;
  const int tid = tm.tid();
  int4* SL = a.sl + b0;
  int2* BS = a.bstate + b0;
  const float linTolSqr = B2G_LINEAR_SLEEP_TOL * B2G_LINEAR_SLEEP_TOL;
  const float angTolSqr = B2G_ANGULAR_SLEEP_TOL * B2G_ANGULAR_SLEEP_TOL;
  const float h = a.dt;
  for (int i = tid; i < nb; i += T) {
    const int ex = isl_label<S>(SL, i), ey = isl_bits<S>(SL, i);
    int2 st = BS[i];
    if (ex < 0 || !(st.x & B2G_BS_AWAKE)) continue;
    const int bi = b0 + i;
    const float4 v4 = a.vel[bi];
    const bool orphan = !(ey & B2G_ISL_LINKED);
    float t = 0.0f;
    if ((st.x & B2G_BS_AUTO_SLEEP) == 0 || v4.z * v4.z > angTolSqr || v4.x * v4.x + v4.y * v4.y > linTolSqr) {
      st.y = 0;
    } else {
      t = __int_as_float(st.y) + h;
      st.y = __float_as_int(t);
    }
    if (orphan) {
      if (t >= B2G_TIME_TO_SLEEP) {
        st.y = 0;
        a.vel[bi] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        a.force[bi] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
    } else {
      // t >= 0: the bit patterns order as the floats
      cuda::atomic_ref<int, S>(SL[ex].w).fetch_min(__float_as_int(t), cuda::memory_order_relaxed);
    }
    BS[i] = st;
  }
  tm.sync();
  for (int i = tid; i < nb; i += T) {
    const int ex = isl_label<S>(SL, i);
    if (ex < 0 || !(isl_bits<S>(SL, i) & B2G_ISL_LINKED) || !(BS[i].x & B2G_BS_AWAKE)) continue;
    const float rmin = __int_as_float(isl_load<S>(&SL[ex].w));
    if (!(rmin >= B2G_TIME_TO_SLEEP) || !(isl_bits<S>(SL, ex) & B2G_ISL_DONE)) continue;
    const int bi = b0 + i;
    BS[i] = make_int2(BS[i].x & ~B2G_BS_AWAKE, 0);
    a.vel[bi] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    a.force[bi] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
}

// Resident CTAs per SM the solve kernel is built for. The occupancy build holds 1024 threads per
// SM at up to 64 registers a thread; the wide build holds 512 threads per SM at up to 128
// registers, where the joint and contact solvers run unspilled and each thread can read its next
// colour's rows before the barrier. The wide build is faster on every measured workload and is
// the default for every size class; the occupancy build stays for b2g_batch_set_solver_waves.
// (At 1024 threads per CTA the register file allows 64 registers either way.)
template <int T, bool WIDE>
constexpr int kSolveBlocks = WIDE ? (T >= 512 ? 1 : 512 / T) : 1024 / T;

// The first half of the island solve of world w by team tm: islands (sleep-mode worlds), the
// solver contacts and their colouring, velocity integration and the contact constraints. Its
// results are in global memory (the world's colour ranges in a.cranges, the integrated
// velocities in a.vel, the constraint planes), so that the second half (iterate_world) can run
// in another kernel. smem / smem_bytes: the CTA's dynamic shared memory, for whatever part of the
// colouring's working arrays fits (a cluster team passes none).
template <class Team>
__device__ __forceinline__ void setup_world(Team& tm, const KernelArgs& a, int w, unsigned char* smem, int smem_bytes) {
  constexpr cuda::thread_scope S = Team::kScope;
  constexpr int NT = Team::kThreads;            // threads of the team
  constexpr int TC = NT / Team::kCtas;          // threads of one CTA
  const int tid = tm.tid();
  __shared__ int cranges[65];
  const int4 wb = a.wb[w];
  const int b0 = wb.x, nb = wb.y, fo = wb.z;
  const int2 wc = a.wc[w];
  const int c0 = wc.x, ncAll = wc.y;
  const int4 wj = a.wj[w];
  const int j0 = wj.x, nj = wj.y;
  const float4 wg = a.wg[w];
  const float h = a.dt;
  const float dtRatio = wg.z * a.dt;
  const int wfl = a.wflags[w];
  const bool warm = (wfl & B2G_WF_WARM) != 0;
  const bool sleepMode = (wfl & B2G_WF_SLEEPMODE) != 0;
  const V2 gravity = mk(wg.x, wg.y);
  const SolverPlanes P = a.sp;
  int4* const SL = a.sl + b0;
  int2* const BS = a.bstate + b0;

  // 0. sleep-mode worlds: wakes, islands, awake islands
  if (sleepMode) build_islands(tm, a, w, b0, nb, c0, ncAll, j0, nj, smem, smem_bytes);

  // 1. solver contacts in list order, with local bodies (static = -1) and colouring priorities
  const int nsc = block_compact(tm, 
      ncAll,
      [&](int k) {
        const uint32_t fl = a.cflags[c0 + k];
        const int2 f = a.cfix[c0 + k];
        bool flag = (fl & B2G_CONTACT_TOUCHING) && (fl & B2G_CONTACT_ENABLED) && (!a.any_sensor || (!a.fsensor[f.x] && !a.fsensor[f.y]));
        // contacts of sleeping islands are not solved: after the labelling every member of an awake
        // island is awake and no member of a sleeping one is (static bodies never are), so the
        // island's mark is its bodies' flag, one read instead of a walk to the root
        if (flag && sleepMode) flag = ((BS[a.fbody[f.x] - b0].x | BS[a.fbody[f.y] - b0].x) & B2G_BS_AWAKE) != 0;
        return flag;
      },
      [&](int k, int r) {
        const int s = c0 + r;
        const int2 f = a.cfix[c0 + k];
        a.sc_list[s] = c0 + k;
        const int ia = a.fbody[f.x], ib = a.fbody[f.y];
        a.scb[s] = make_int2((ia - b0) | (a.btype[ia] == B2G_STATIC ? (int)0x80000000 : 0),
                             (ib - b0) | (a.btype[ib] == B2G_STATIC ? (int)0x80000000 : 0));
        a.srad[s] = make_float2(a.frad[f.x], a.frad[f.y]);
        const uint64_t key = a.ckey[c0 + k];
        a.cprio[s] = contactPriority((uint32_t)(key >> 32) - (uint32_t)fo, (uint32_t)key - (uint32_t)fo);
      });

  // 2. colour the solver contacts (shared memory for whatever fits)
  int ncc = 0;
  if (nsc > 0) {
    SmemCarver sc{smem, (size_t)smem_bytes};
    ColourMem m;
    m.mask = (unsigned long long*)sc.take(8 * (size_t)nb);
    m.cnt = (int*)sc.take(4 * (size_t)nb);
    m.head = (int*)sc.take(4 * (size_t)nb);
    bool bodySm = m.mask && m.cnt && m.head;
    if (!bodySm) {
      m.mask = a.inc_mask + b0;
      m.cnt = a.inc_cnt + b0;
      m.head = a.inc_head + b0;
    }
    int* list = bodySm ? (int*)sc.take(8 * (size_t)nsc) : nullptr;
    int2* cb = bodySm ? (int2*)sc.take(8 * (size_t)nsc) : nullptr;
    int8_t* col = bodySm ? (int8_t*)sc.take((size_t)nsc) : nullptr;
    uint8_t* rdy = bodySm ? (uint8_t*)sc.take((size_t)nsc) : nullptr;
    bool conSm = list && cb && col && rdy;
    if (conSm) {
      for (int k = tid; k < nsc; k += NT) cb[k] = a.scb[c0 + k];
      tm.sync();
      m.list = list; m.cb = cb; m.col = col; m.rdy = rdy;
    } else {
      m.list = a.inc_list + 2 * (int64_t)c0;
      m.cb = a.scb + c0;
      m.col = a.ccol + c0;
      m.rdy = a.cready + c0;
    }
    m.ent = a.cwork + 4 * (int64_t)c0;
    m.wl0 = m.ent + 2 * (int64_t)nsc;
    m.wl1 = m.wl0 + nsc;
    ncc = colour_constraints(tm, nsc, nb, m, a.cprio + c0, a.corder + c0, a.cslot + c0, cranges, a.status);
    if (conSm) {
      for (int k = tid; k < nsc; k += NT) a.ccol[c0 + k] = col[k];
      tm.sync();
    }
  }
  // the colour ranges for the iterations (joints: colours fixed per layout)
  for (int c = tid; c <= ncc; c += NT) a.cranges[65 * (int64_t)w + c] = cranges[c];
  const int njc = nj > 0 ? a.ncolors[4 * w + 1] : 0;
  if (tid == 0) {
    a.ncolors[4 * w] = ncc;
    a.ncolors[4 * w + 2] = nsc;
    a.ncolors[4 * w + 3] = c0;
    atomicAdd(&a.counters[B2G_CNT_TOUCHING], (unsigned long long)nsc);
    atomicMax(&a.counters[B2G_CNT_MAXCOLORS], (unsigned long long)(ncc > njc ? ncc : njc));
  }

  // 3. velocity integration (b2_island.cpp:256-293, SolveOrphan :187-206) into the global
  //    velocity array
  for (int i = tid; i < nb; i += NT) {
    int bi = b0 + i;
    if (a.btype[bi] == B2G_DYNAMIC && (!sleepMode || (BS[i].x & B2G_BS_AWAKE))) {
      float4 v4 = a.vel[bi];
      float4 md = a.massd[bi];
      float4 dmp = a.damp[bi];
      float4 fr = a.force[bi];
      V2 v = mk(v4.x, v4.y);
      float wv = v4.z;
      addTo(v, (h * md.y) * (dmp.z * md.x * gravity + mk(fr.x, fr.y)));
      wv += h * md.w * fr.z;
      v.x /= (1.0f + h * dmp.x);
      v.y /= (1.0f + h * dmp.x);
      wv /= (1.0f + h * dmp.y);
      a.vel[bi] = make_float4(v.x, v.y, wv, 0.0f);
    }
  }
  tm.sync();
  const float4* bs = a.vel + b0;

  // 4. prepare (b2ContactSolver::Initialize + InitializeVelocityConstraints) in list order, each
  //    constraint written to its colour-ordered slot; each turn reads the next contact's index
  //    rows up front and, after preparing the current one, prefetches the next one's gathers
  //    (manifold, material, both bodies) into L2
  for (int k = tid; k < nsc; k += NT) {
    const bool more = k + NT < nsc;
    const int cin = more ? a.sc_list[c0 + k + NT] : 0;
    const int2 lbn = more ? a.scb[c0 + k + NT] : make_int2(0, 0);
    int ci = a.sc_list[c0 + k];
    int p = a.cslot[c0 + k];
    int2 lb = a.scb[c0 + k];
    const float2 rad = a.srad[c0 + k];
    int la = lb.x & 0x7fffffff, lbb = lb.y & 0x7fffffff;
    int ia = b0 + la, ib = b0 + lbb;
    b2g_manifold m = ld_manifold(&a.cman[ci]);
    VCDev vc;
    for (int q = 0; q < 4; ++q) vc.K[q] = vc.NM[q] = 0.0f;
    prepareContact(vc, m, a.cmat[ci], rad.x, rad.y, la, lbb, a.massd[ia], a.massd[ib], a.lc[ia], a.lc[ib],
                   a.pos[ia], bs[la], a.pos[ib], bs[lbb], dtRatio, warm, ci);
    store_planes(P, c0 + p, vc);
    if (more) {
      auto l2 = [](const void* q) { asm volatile("prefetch.global.L2 [%0];" ::"l"(q)); };  // no registers held
      const int na = b0 + (lbn.x & 0x7fffffff), nb2 = b0 + (lbn.y & 0x7fffffff);
      l2(&a.cman[cin]);
      l2(reinterpret_cast<const char*>(&a.cman[cin]) + 32);
      l2(&a.cmat[cin]);
      l2(&a.massd[na]); l2(&a.massd[nb2]);
      l2(&a.lc[na]); l2(&a.lc[nb2]);
      l2(&a.pos[na]); l2(&a.pos[nb2]);
      l2(&bs[na - b0]); l2(&bs[nb2 - b0]);
    }
  }
}

// The second half of the island solve of world w by team tm, after setup_world: warm start,
// velocity iterations, position integration and iterations, transforms and sleep timers.
// smem / smem_bytes: the CTA's dynamic shared memory, which holds the world's body state and
// inverse masses when they fit (a cluster team passes none: its world's arrays stay in global
// memory). PREFETCH: each thread reads its next colour's rows before the colour barrier (the
// 128-register builds).
template <class Team, bool PREFETCH>
__device__ __forceinline__ void iterate_world(Team& tm, const KernelArgs& a, int w, unsigned char* smem, int smem_bytes) {
  constexpr cuda::thread_scope S = Team::kScope;
  constexpr int NT = Team::kThreads;            // threads of the team
  constexpr int TC = NT / Team::kCtas;          // threads of one CTA
  const int tid = tm.tid();
  __shared__ int cranges[65];
  __shared__ int jranges[65];
  const int4 wb = a.wb[w];
  const int b0 = wb.x, nb = wb.y, fo = wb.z;
  const int2 wc = a.wc[w];
  const int c0 = wc.x, ncAll = wc.y;
  const int4 wj = a.wj[w];
  const int j0 = wj.x, nj = wj.y;
  const float4 wg = a.wg[w];
  const float h = a.dt;
  const float dtRatio = wg.z * a.dt;
  const int wfl = a.wflags[w];
  const bool warm = (wfl & B2G_WF_WARM) != 0;
  const bool sleepMode = (wfl & B2G_WF_SLEEPMODE) != 0;
  const V2 gravity = mk(wg.x, wg.y);
  const SolverPlanes P = a.sp;
  int4* const SL = a.sl + b0;
  int2* const BS = a.bstate + b0;

  const int ncc = a.ncolors[4 * w];
  const int nsc = a.ncolors[4 * w + 2];
  const int njc = nj > 0 ? a.ncolors[4 * w + 1] : 0;
  for (int c = threadIdx.x; c <= ncc; c += TC) cranges[c] = a.cranges[65 * (int64_t)w + c];
  for (int c = threadIdx.x; c <= njc; c += TC) jranges[c] = a.jranges[65 * (int64_t)w + c];
  // the body-state buffer: shared memory (with the bodies' inverse masses) when the world's
  // bodies fit, else the global velocity array
  const bool bsm = (size_t)nb * (sizeof(float4) + sizeof(float2)) <= (size_t)smem_bytes;
  float4* bs = bsm ? reinterpret_cast<float4*>(smem) : a.vel + b0;
  float2* msm = bsm ? reinterpret_cast<float2*>(smem + sizeof(float4) * (size_t)nb) : nullptr;
  const Masses M{msm, a.massd + b0};
  if (bsm)
    for (int i = tid; i < nb; i += NT) {
      const float4 md = a.massd[b0 + i];
      bs[i] = a.vel[b0 + i];
      msm[i] = make_float2(md.y, md.w);
    }
  tm.sync();
  float4* jb = bs - b0;  // joints address bodies by global index

  // 5. warm start contacts, then joint InitVelocityConstraints, colour by colour
  auto fetchV = [&](int slot, VelRows& r) { fetch_vel(P, slot, r); };
  auto fetchP = [&](int slot, PosRows& r) { fetch_pos(P, slot, r); };
  auto hintV = [&](int slot) { hint_vel(P, slot); };
  if (warm) {
    colour_sweep<Team, VelRows, PREFETCH, 2>(tm, cranges, ncc, c0, fetchV, [&](int slot, const VelRows& r) {
      VCDev vc;
      unpack_vel(r, vc, M);
      warmStartContact(vc, bs);
    }, hintV);
  }
  for (int c = 0; c < njc; ++c) {
    int s = jranges[c], e = jranges[c + 1];
    const int step = c == 63 ? 1 : NT, i0 = c == 63 ? s : s + tid;
    if (c != 63 || tid == 0)
      for (int i = i0; i < e; i += step) {
        JointDev& J = a.joints[j0 + a.jorder[j0 + i]];
        if (sleepMode && !joint_awake(a, J)) {
          jointPackAsleep(a.jplanes, j0 + i);
          continue;
        }
        if (c == 63 && J.d.type == B2G_JOINT_GEAR) {  // gears are coloured 63: one thread, on the record
          gearInit(J, a.massd, a.lc, a.pos, jb, warm);
          jointPackGear(a.jplanes, j0 + i, J.d.body_a, J.d.body_b);
          continue;
        }
        jointInitSlot(J, a.jplanes, a.jstride, j0 + i, a.massd, a.lc, a.pos, jb, a.dt, dtRatio, warm);
      }
    tm.sync();
  }

  // 6. velocity iterations: joints, then contacts (b2_island.cpp:327-346)
  for (int it = 0; it < a.vi; ++it) {
    for (int c = 0; c < njc; ++c) {
      int s = jranges[c], e = jranges[c + 1];
      const int step = c == 63 ? 1 : NT, i0 = c == 63 ? s : s + tid;
      if (c != 63 || tid == 0)
        for (int i = i0; i < e; i += step) {
          if (PREFETCH && i + step < e)  // the rows this thread's next joint of the colour reads
            for (int k = 0; k < 9; ++k) prefetch_l1(a.jplanes + (int64_t)k * a.jstride + j0 + i + step);
          if (c == 63 && jointSlotIsGear(a.jplanes, j0 + i)) gearSolveVelocity(a.joints[j0 + a.jorder[j0 + i]], jb);
          else jointSolveVelocitySlot(a.jplanes, a.jstride, j0 + i, jb, a.dt, a.inv_dt);
        }
      tm.sync();
    }
    colour_sweep<Team, VelRows, PREFETCH, 2>(tm, cranges, ncc, c0, fetchV, [&](int slot, const VelRows& r) {
      VCDev vc;
      unpack_vel(r, vc, M);
      solveContactVelocity(vc, bs);
      P.imp[slot] = make_float4(vc.normalImpulse[0], vc.normalImpulse[1], vc.tangentImpulse[0], vc.tangentImpulse[1]);
    }, hintV);
  }

  // 7. StoreImpulses (b2_contact_solver.cpp:641-657); the joints' impulses back into their records
  for (int i = tid; i < nj; i += NT)  // a gear's impulse is already on its record
    if (!jointSlotIsGear(a.jplanes, j0 + i)) jointStoreImpulses(a.jplanes, a.jstride, j0 + i, a.joints[j0 + a.jorder[j0 + i]]);
  for (int p = tid; p < nsc; p += NT) {
    int pc = (P.idx[c0 + p].x >> 24) & 15;
    float4 im = P.imp[c0 + p];
    b2g_manifold* m = &a.cman[P.cid[c0 + p]];
    if (pc > 0) { m->points[0].normal_impulse = im.x; m->points[0].tangent_impulse = im.z; }
    if (pc > 1) { m->points[1].normal_impulse = im.y; m->points[1].tangent_impulse = im.w; }
  }

  // 8. integrate positions (b2_island.cpp:349-385); the buffer switches to positions. Worlds with
  //    continuous collision keep every body's position at the step's start (b2Sweep c0, a0)
  const bool sweeps = a.sweep0 != nullptr && (wfl & B2G_WF_CONTINUOUS);
  for (int i = tid; i < nb; i += NT) {
    int bi = b0 + i;
    float4 p4 = a.pos[bi];
    if (sweeps) a.sweep0[bi] = make_float4(p4.x, p4.y, p4.z, 0.0f);
    if (a.btype[bi] == B2G_STATIC || (sleepMode && !(BS[i].x & B2G_BS_AWAKE))) {
      if (bsm) bs[i] = p4;
      continue;
    }
    float4 v4 = bs[i];
    V2 c = mk(p4.x, p4.y);
    float an = p4.z;
    V2 v = mk(v4.x, v4.y);
    float wv = v4.z;
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
    a.vel[bi] = make_float4(v.x, v.y, wv, 0.0f);
    if (bsm) bs[i] = make_float4(c.x, c.y, an, 0.0f);
    else a.pos[bi] = make_float4(c.x, c.y, an, 0.0f);
  }
  tm.sync();
  float4* ps = bsm ? bs : a.pos + b0;
  float4* jp = ps - b0;

  // 9. position iterations: contacts then joints (b2_island.cpp:387-428). Early exit for the
  //    world; in sleep-mode worlds per island, as the reference's island loop: an island whose
  //    constraints were all okay in an iteration is done and no longer iterated.
  for (int it = 0; it < a.pi; ++it) {
    int okay = 1;
    auto hintP = [&](int slot) { hint_pos(P, slot); };
    colour_sweep<Team, PosRows, PREFETCH, 2>(tm, cranges, ncc, c0, fetchP, [&](int slot, const PosRows& r) {
      VCDev vc;
      unpack_pos(r, vc, M);
      int root = 0;
      if (sleepMode) {
        root = isl_root<S>(SL, vc.indexA, vc.indexB);
        if (isl_bits<S>(SL, root) & B2G_ISL_DONE) return;
      }
      if (!(solveContactPosition(vc, ps) >= -3.0f * B2G_LINEAR_SLOP)) {
        okay = 0;
        if (sleepMode) isl_store<S>(&SL[root].z, it + 1);
      }
    }, hintP);
    for (int c = 0; c < njc; ++c) {
      int s = jranges[c], e = jranges[c + 1];
      const int step = c == 63 ? 1 : NT, i0 = c == 63 ? s : s + tid;
      if (c != 63 || tid == 0)
        for (int i = i0; i < e; i += step) {
          int root = 0;
          if (sleepMode) {
            const float4 h = a.jplanes[j0 + i];
            if (__float_as_int(h.w) & B2G_JV_ASLEEP) continue;
            root = isl_root<S>(SL, __float_as_int(h.x) - b0, __float_as_int(h.y) - b0);
            if (isl_bits<S>(SL, root) & B2G_ISL_DONE) continue;
          }
          const bool ok = (c == 63 && jointSlotIsGear(a.jplanes, j0 + i))
                              ? gearSolvePosition(a.joints[j0 + a.jorder[j0 + i]], jp)
                              : jointSolvePositionSlot(a.jplanes, a.jstride, j0 + i, jp);
          if (!ok) {
            okay = 0;
            if (sleepMode) isl_store<S>(&SL[root].z, it + 1);
          }
        }
      tm.sync();
    }
    if (sleepMode) {
      tm.sync();
      int pending = 0;
      for (int i = tid; i < nb; i += NT) {
        const int ey = isl_bits<S>(SL, i);
        if (isl_label<S>(SL, i) != i || !(ey & B2G_ISL_AWAKE) || (ey & B2G_ISL_DONE)) continue;
        if (isl_load<S>(&SL[i].z) == it + 1) pending = 1;
        else isl_or<S>(&SL[i].y, B2G_ISL_DONE);
      }
      if (!tm.any(pending)) break;
    } else if (tm.all(okay)) {
      break;
    }
  }

  // 10. transforms (b2Body::SynchronizeTransform, include/box2d/b2_body.h:957-961), finite check
  int bad = 0;
  for (int i = tid; i < nb; i += NT) {
    int bi = b0 + i;
    if (a.btype[bi] == B2G_STATIC || (sleepMode && !(BS[i].x & B2G_BS_AWAKE))) continue;
    float4 p4 = ps[i];
    if (bsm) a.pos[bi] = p4;
    Rot q = rotOf(p4.z);
    float2 l = a.lc[bi];
    V2 p = mk(p4.x, p4.y) - mul(q, mk(l.x, l.y));
    a.xf[bi] = make_float4(p.x, p.y, q.s, q.c);
    float4 v4 = a.vel[bi];
    if (!isfinite(p4.x) || !isfinite(p4.y) || !isfinite(p4.z) || !isfinite(v4.x) || !isfinite(v4.y) || !isfinite(v4.z))
      bad = 1;
  }
  if (tm.any(bad) && tid == 0) {  // the host freezes this world; the others go on
    a.wfault[w] = 1;
    atomicOr(a.status, B2G_DEV_NONFINITE);
  }

  // 11. sleep timers (b2_island.cpp:444-483; orphans b2Island::SolveOrphan :230-249)
  if (wfl & B2G_WF_ALLOW_SLEEP) sleep_islands(tm, a, b0, nb);
  if (a.events_on) {
    for (int p = tid; p < nsc; p += NT) {
      int pc = (P.idx[c0 + p].x >> 24) & 15;
      float4 im = P.imp[c0 + p];
      int2 f = a.cfix[P.cid[c0 + p]];
      float ni[2] = {im.x, im.y}, ti[2] = {im.z, im.w};
      record_event(a, B2G_EVENT_POSTSOLVE, w, f.x - fo, f.y - fo, pc, ni, ti, 0);
    }
  }
  if (tid == 0 && a.dt > 0.0f) a.wg[w].z = a.inv_dt;
}

// The first half of the solve for the size classes of the batch, one CTA per world; T is at most
// 512 and the launch keeps 1024 threads per SM resident (64 registers a thread).
template <int T>
constexpr int kSetupBlocks = 1024 / T;
template <int T>
__global__ void __launch_bounds__(T, kSetupBlocks<T>) k_setup(KernelArgs a, int first, int smem_bytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = a.world_order[first + blockIdx.x];
  if ((a.wflags[w] & B2G_WF_ACTIVE) == 0) return;
  CtaTeam<T> tm;
  setup_world(tm, a, w, smem, smem_bytes);
}

// The second half for the size classes, one CTA per world.
template <int T, bool WIDE>
__global__ void __launch_bounds__(T, kSolveBlocks<T, WIDE>) k_solve(KernelArgs a, int first, int smem_bytes) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = a.world_order[first + blockIdx.x];
  if ((a.wflags[w] & B2G_WF_ACTIVE) == 0) return;
  CtaTeam<T> tm;
  iterate_world<CtaTeam<T>, (WIDE && T <= 512)>(tm, a, w, smem, smem_bytes);
}

// One thread-block cluster of CS CTAs per world: the worlds above the largest CTA class. The
// world's arrays stay in global memory; every colour barrier is a cluster barrier.
template <int T, int CS>
__global__ void __launch_bounds__(T, 1) k_solve_cluster(KernelArgs a, int first) {
  __shared__ int votes[3];
  ClusterTeam<T, CS> tm;
  tm.r = (int)cluster_rank();
  tm.vphase = 0;
  tm.sphase = 0;
  if (threadIdx.x < 3) votes[threadIdx.x] = 0;
  tm.votes = cluster_map(votes, 0);
  cluster_barrier();  // every CTA runs, and rank 0's votes are clear, before any remote access
  const int w = a.world_order[first + (int)(blockIdx.x / CS)];
  if ((a.wflags[w] & B2G_WF_ACTIVE) != 0) {
    setup_world(tm, a, w, nullptr, 0);
    tm.sync();  // the setup's global results are visible across the cluster
    iterate_world<ClusterTeam<T, CS>, (T <= 512)>(tm, a, w, nullptr, 0);
  }
  cluster_barrier();  // rank 0's shared memory outlives every remote access to it
}

// The wide build's launches and setup (solve_wide.cu).
void launch_solve_class_wide(const KernelArgs& a, const SolveClass& c, cudaStream_t s);
void solve_wide_setup(const int* smem_caps);
// The cluster build (solve_cluster.cu): kClusterThreads threads per CTA, c.ctas CTAs per world.
constexpr int kClusterThreads = 512;
void launch_solve_class_cluster(const KernelArgs& a, const SolveClass& c, cudaStream_t s);
void solve_cluster_setup();

}  // namespace b2g
