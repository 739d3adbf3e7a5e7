// pairs.cu - standalone broadphase over caller AABBs (b2g_pairs).
//
// Every pair (i < j) of n AABBs that overlap under the reference's inclusive test
// (include/box2d/b2_collision.h:270-276), i.e. the pair set b2BroadPhase::UpdateAndQuery reports
// (include/box2d/b2_broad_phase.h:252-343), as a sorted list of i << 32 | j. Built like the batch
// broadphase: 30-bit Morton codes of the AABB centres, radix sort, Karras LBVH, bottom-up bounds,
// a counting traversal, an exclusive scan and an emitting traversal that sorts each segment.
#include <cub/cub.cuh>

#include "../../include/b2g_capi.h"
#include "pairs.h"

namespace b2g {

#define PLEAF 0x80000000u

__device__ __forceinline__ uint32_t p_expand15(uint32_t v) {
  v &= 0x7fffu;
  v = (v | (v << 8)) & 0x00ff00ffu;
  v = (v | (v << 4)) & 0x0f0f0f0fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}

__global__ void kp_bounds(const float4* aabb, int n, float4* out) {
  float mnx = 3.4e38f, mny = 3.4e38f, mxx = -3.4e38f, mxy = -3.4e38f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    float4 b = aabb[i];
    float cx = b.x + b.z, cy = b.y + b.w;
    mnx = fminf(mnx, cx); mny = fminf(mny, cy); mxx = fmaxf(mxx, cx); mxy = fmaxf(mxy, cy);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
    mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
    mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
    mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
  }
  __shared__ float s[4][32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { s[0][wid] = mnx; s[1][wid] = mny; s[2][wid] = mxx; s[3][wid] = mxy; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x + 31) / 32; ++k) {
      mnx = fminf(mnx, s[0][k]); mny = fminf(mny, s[1][k]); mxx = fmaxf(mxx, s[2][k]); mxy = fmaxf(mxy, s[3][k]);
    }
    *out = make_float4(mnx, mny, mxx, mxy);
  }
}

__global__ void kp_morton(const float4* aabb, int n, const float4* bnd, uint32_t* key, int* val) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 w = *bnd;
  float4 b = aabb[i];
  float ex = fmaxf(w.z - w.x, 1e-30f), ey = fmaxf(w.w - w.y, 1e-30f);
  float ux = fminf(fmaxf((b.x + b.z - w.x) / ex, 0.0f), 1.0f);
  float uy = fminf(fmaxf((b.y + b.w - w.y) / ey, 0.0f), 1.0f);
  uint32_t qx = (uint32_t)fminf(ux * 32768.0f, 32767.0f), qy = (uint32_t)fminf(uy * 32768.0f, 32767.0f);
  key[i] = (p_expand15(qx) << 1) | p_expand15(qy);
  val[i] = i;
}

__device__ __forceinline__ int p_delta(const uint32_t* k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  uint32_t x = k[i], y = k[j];
  if (x == y) return 32 + __clz((unsigned)(i ^ j));
  return __clz(x ^ y);
}

__global__ void kp_internal(const uint32_t* k, int n, int2* child, int* nparent, int* lparent) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int d = (p_delta(k, n, i, i + 1) - p_delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = p_delta(k, n, i, i - d);
  int lmax = 2;
  while (p_delta(k, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (p_delta(k, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = p_delta(k, n, i, j);
  int s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (p_delta(k, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  int g = i + s * d + min(d, 0);
  int lo = min(i, j), hi = max(i, j);
  child[i] = make_int2(lo == g ? (int)(g | PLEAF) : g, hi == g + 1 ? (int)((g + 1) | PLEAF) : g + 1);
  if (lo == g) lparent[g] = i; else nparent[g] = i;
  if (hi == g + 1) lparent[g + 1] = i; else nparent[g + 1] = i;
  if (i == 0) nparent[0] = -1;
}

__global__ void kp_init(int n, int* lparent, int* flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) lparent[i] = -1;
  if (i < n - 1) flag[i] = 0;
}

// Status bits of a pair search (PairsScratch::status): any of them fails the call with
// B2G_E_CAPACITY instead of returning an incomplete pair set.
#define P_ST_STACK 1u  // a traversal outgrew its stack or its visit bound
#define P_ST_DEPTH 2u  // a bottom-up walk passed the depth bound (node bounds left unwritten)

__global__ void kp_node_bounds(const float4* aabb, const int* val, int n, const int2* child, const int* nparent,
                               const int* lparent, float4* naabb, int* flag, unsigned int* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int p = lparent[i];
  int guard = 0;
  while (p >= 0) {
    if (++guard > 256) {  // malformed tree: stop instead of looping, and fail the call
      atomicOr(status, P_ST_DEPTH);
      return;
    }
    __threadfence();
    if (atomicAdd(&flag[p], 1) == 0) return;
    __threadfence();
    int2 ch = child[p];
    float4 l = (ch.x & PLEAF) ? aabb[val[ch.x & ~PLEAF]] : __ldcg(&naabb[ch.x]);
    float4 r = (ch.y & PLEAF) ? aabb[val[ch.y & ~PLEAF]] : __ldcg(&naabb[ch.y]);
    __stcg(&naabb[p], make_float4(fminf(l.x, r.x), fminf(l.y, r.y), fmaxf(l.z, r.z), fmaxf(l.w, r.w)));
    p = nparent[p];
  }
}

__device__ __forceinline__ bool p_overlap(float4 a, float4 b) {
  return (a.z >= b.x) & (a.x <= b.z) & (a.w >= b.y) & (a.y <= b.w);
}

// Counting pass (EMIT = false): counts[f] = partners g > f of box f. Emitting pass: `counts` is
// the 64-bit exclusive scan of the counts, and box f writes its partners to [counts[f],
// counts[f + 1]) of `pairs` in (f, g) order. A segment outside [0, cap) is never written.
template <bool EMIT>
__global__ void kp_traverse(const float4* aabb, const int* val, int n, const int2* child, const float4* naabb,
                            int64_t* counts, uint64_t* pairs, int64_t cap, unsigned int* status) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n) return;
  int64_t cnt = 0;
  int64_t off = 0;
  if (EMIT) {
    off = counts[f];
    const int64_t end = counts[f + 1];
    if (end == off) return;
    if (off < 0 || end > cap || end < off) return;
  }
  if (n > 1) {
    float4 box = aabb[f];
    int stack[96];
    int sp = 0;
    stack[sp++] = 0;
    int visits = 0;
    while (sp > 0) {
      if (++visits > 2 * n + 8) {  // each internal node at most once
        atomicOr(status, P_ST_STACK);
        break;
      }
      int node = stack[--sp];
      int2 ch = child[node];
      int kids[2] = {ch.x, ch.y};
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        int c = kids[q];
        if (c & PLEAF) {
          int g = val[c & ~PLEAF];
          if (g > f && p_overlap(box, aabb[g])) {
            if (EMIT) pairs[off + cnt] = ((uint64_t)(uint32_t)f << 32) | (uint32_t)g;
            ++cnt;
          }
        } else if (p_overlap(box, naabb[c])) {
          if (sp < 96) stack[sp++] = c;
          else atomicOr(status, P_ST_STACK);
        }
      }
    }
  }
  if (!EMIT) {
    counts[f] = cnt;
  } else {
    uint64_t* seg = pairs + off;
    for (int x = 1; x < cnt; ++x) {
      uint64_t v = seg[x];
      int y = x - 1;
      while (y >= 0 && seg[y] > v) { seg[y + 1] = seg[y]; --y; }
      seg[y + 1] = v;
    }
  }
}

size_t pairs_scratch_bytes(int n) {
  size_t cub_sort = 0, cub_scan = 0;
  cub::DeviceRadixSort::SortPairs((void*)nullptr, cub_sort, (uint32_t*)nullptr, (uint32_t*)nullptr, (int*)nullptr,
                                  (int*)nullptr, n, 0, 30);
  cub::DeviceScan::ExclusiveSum((void*)nullptr, cub_scan, (int64_t*)nullptr, (int64_t*)nullptr, n + 1);
  PairsScratch s = pairs_scratch_layout(nullptr, n, cub_sort > cub_scan ? cub_sort : cub_scan);
  return s.total_bytes;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

PairsScratch pairs_scratch_layout(void* base, int n, size_t cub_bytes) {
  PairsScratch s;
  size_t o = 0;
  size_t un = (size_t)(n > 1 ? n : 1);
  char* b = (char*)base;
  auto take = [&](size_t bytes) { void* p = b ? (void*)(b + o) : nullptr; o = align256(o + bytes); return p; };
  s.bounds = (float4*)take(sizeof(float4));
  s.key = (uint32_t*)take(un * 4);
  s.key_sorted = (uint32_t*)take(un * 4);
  s.val = (int*)take(un * 4);
  s.val_sorted = (int*)take(un * 4);
  s.child = (int2*)take(un * 8);
  s.nparent = (int*)take(un * 4);
  s.lparent = (int*)take(un * 4);
  s.naabb = (float4*)take(un * 16);
  s.flag = (int*)take(un * 4);
  s.counts = (int64_t*)take((un + 1) * 8);
  s.offsets = (int64_t*)take((un + 1) * 8);
  s.status = (unsigned int*)take(16);
  s.cub = take(cub_bytes);
  s.cub_bytes = cub_bytes;
  s.total_bytes = o;
  return s;
}

static inline unsigned pgrid(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// Runs the whole pair search with the scratch laid out in `s`; the pair total is left in
// s.counts[n] (device). The emit pass is skipped (and B2G_E_CAPACITY returned by the caller)
// when the total exceeds cap.
int pairs_run(const float4* aabb, int n, uint64_t* pairs, int64_t cap, int64_t* n_pairs, const PairsScratch& s,
              cudaStream_t st) {
  if (n <= 0) {
    if (n_pairs) *n_pairs = 0;
    return B2G_OK;
  }
  cudaMemsetAsync(s.status, 0, sizeof(unsigned int), st);
  kp_bounds<<<1, 1024, 0, st>>>(aabb, n, s.bounds);
  kp_morton<<<pgrid(n, 256), 256, 0, st>>>(aabb, n, s.bounds, s.key, s.val);
  size_t bytes = s.cub_bytes;
  cub::DeviceRadixSort::SortPairs(s.cub, bytes, s.key, s.key_sorted, s.val, s.val_sorted, n, 0, 30, st);
  kp_init<<<pgrid(n, 256), 256, 0, st>>>(n, s.lparent, s.flag);
  if (n > 1) {
    kp_internal<<<pgrid(n - 1, 256), 256, 0, st>>>(s.key_sorted, n, s.child, s.nparent, s.lparent);
    kp_node_bounds<<<pgrid(n, 256), 256, 0, st>>>(aabb, s.val_sorted, n, s.child, s.nparent, s.lparent, s.naabb,
                                                  s.flag, s.status);
  }
  kp_traverse<false><<<pgrid(n, 128), 128, 0, st>>>(aabb, s.val_sorted, n, s.child, s.naabb, s.counts, pairs, cap,
                                                     s.status);
  cudaMemsetAsync(s.counts + n, 0, sizeof(int64_t), st);
  bytes = s.cub_bytes;
  cub::DeviceScan::ExclusiveSum(s.cub, bytes, s.counts, s.offsets, n + 1, st);  // 64-bit sums
  int64_t total = 0;
  unsigned int status = 0;
  cudaMemcpyAsync(&total, s.offsets + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&status, s.status, sizeof(unsigned int), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return B2G_E_CUDA;
  if (n_pairs) *n_pairs = total;
  if (status) return B2G_E_CAPACITY;
  if (total > cap) return B2G_E_CAPACITY;
  kp_traverse<true><<<pgrid(n, 128), 128, 0, st>>>(aabb, s.val_sorted, n, s.child, s.naabb, s.offsets, pairs, cap,
                                                    s.status);
  if (cudaStreamSynchronize(st) != cudaSuccess) return B2G_E_CUDA;
  return cudaGetLastError() == cudaSuccess ? B2G_OK : B2G_E_CUDA;
}

}  // namespace b2g

extern "C" B2G_API int b2g_pairs(const float* d_aabbs, int32_t n, uint64_t* d_pairs, int64_t cap, int64_t* n_pairs,
                                 void* stream) {
  if (n < 0 || cap < 0 || (n > 0 && !d_aabbs) || (cap > 0 && !d_pairs)) return B2G_E_INVALID_ARG;
  if (n == 0) {
    if (n_pairs) *n_pairs = 0;
    return B2G_OK;
  }
  size_t bytes = b2g::pairs_scratch_bytes(n);
  void* base = nullptr;
  if (cudaMalloc(&base, bytes) != cudaSuccess) {
    cudaGetLastError();  // clear the failed allocation's error; the context stays usable
    return B2G_E_OUT_OF_MEMORY;
  }
  size_t cub_bytes = 0, cub_scan = 0;
  cub::DeviceRadixSort::SortPairs((void*)nullptr, cub_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (int*)nullptr,
                                  (int*)nullptr, n, 0, 30);
  cub::DeviceScan::ExclusiveSum((void*)nullptr, cub_scan, (int64_t*)nullptr, (int64_t*)nullptr, n + 1);
  b2g::PairsScratch s = b2g::pairs_scratch_layout(base, n, cub_bytes > cub_scan ? cub_bytes : cub_scan);
  int st = b2g::pairs_run((const float4*)d_aabbs, n, d_pairs, cap, n_pairs, s, (cudaStream_t)stream);
  cudaStreamSynchronize((cudaStream_t)stream);
  cudaFree(base);
  return st;
}

// ------------------------------------------------------------------------------------------
// Allocation-free variant of b2g_pairs.
//
// Its scratch is one file-scope device array, so a call allocates nothing. Every GPU that loads
// the library holds this array (B2G_PAIRS_STATIC_SCRATCH_BYTES) until the process exits, and
// every call shares it: calls that overlap on the GPU (different streams, or host threads)
// race on it and must be serialised by the caller. Each call re-initialises the parts that must
// start at zero (status word, arrival counters, the count terminator) before using them.
#include <mutex>

namespace b2g {

#define B2G_PAIRS_STATIC_SCRATCH_BYTES (16u << 20)
static __device__ __align__(256) unsigned char g_pairs_static_scratch[B2G_PAIRS_STATIC_SCRATCH_BYTES];

// Device address of the array, looked up once per device with that device current (the array's
// name on the host is only a stand-in, not a device address). The first call on a device does
// this set-up.
static std::mutex g_static_mutex;
static void* g_static_ptr[64] = {};

static int static_scratch_for_current_device(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return B2G_E_CUDA;
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_pairs_static_scratch);
    if (e != cudaSuccess || !p) return B2G_E_CUDA;
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return B2G_OK;
}

}  // namespace b2g

extern "C" B2G_API int b2g_pairs_static(const float* d_aabbs, int32_t n, uint64_t* d_pairs, int64_t cap,
                                        int64_t* n_pairs, void* stream) {
  if (n < 0 || cap < 0 || (n > 0 && !d_aabbs) || (cap > 0 && !d_pairs)) return B2G_E_INVALID_ARG;
  if (n > B2G_PAIRS_STATIC_MAX) return B2G_E_CAPACITY;
  if (n == 0) {
    if (n_pairs) *n_pairs = 0;
    return B2G_OK;
  }
  void* base = nullptr;
  int st = b2g::static_scratch_for_current_device(&base);
  if (st != B2G_OK) return st;
  size_t cub_bytes = 0, cub_scan = 0;
  cub::DeviceRadixSort::SortPairs((void*)nullptr, cub_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr, (int*)nullptr,
                                  (int*)nullptr, n, 0, 30);
  cub::DeviceScan::ExclusiveSum((void*)nullptr, cub_scan, (int64_t*)nullptr, (int64_t*)nullptr, n + 1);
  b2g::PairsScratch s = b2g::pairs_scratch_layout(base, n, cub_bytes > cub_scan ? cub_bytes : cub_scan);
  if (s.total_bytes > B2G_PAIRS_STATIC_SCRATCH_BYTES) return B2G_E_CAPACITY;
  return b2g::pairs_run((const float4*)d_aabbs, n, d_pairs, cap, n_pairs, s, (cudaStream_t)stream);
}
