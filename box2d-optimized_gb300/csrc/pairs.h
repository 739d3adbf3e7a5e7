// pairs.h - scratch layout of the standalone broadphase (pairs.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace b2g {

// Device scratch of one pair search over n AABBs, carved out of one block of memory.
struct PairsScratch {
  float4* bounds;
  uint32_t *key, *key_sorted;
  int *val, *val_sorted;
  int2* child;
  int *nparent, *lparent;
  float4* naabb;
  int* flag;
  int64_t* counts;      // n + 1 entries: pairs per AABB (up to n - 1 each)
  int64_t* offsets;     // n + 1 entries: exclusive scan of counts; offsets[n] = number of pairs,
                        // which passes 2^31 for dense overlap from about 65 536 boxes
  unsigned int* status; // non-zero: traversal stack overflow or a malformed tree
  void* cub;
  size_t cub_bytes;
  size_t total_bytes;
};

// Lays the scratch out from `base` (pass nullptr to only compute total_bytes).
PairsScratch pairs_scratch_layout(void* base, int n, size_t cub_bytes);
size_t pairs_scratch_bytes(int n);
int pairs_run(const float4* aabb, int n, uint64_t* pairs, int64_t cap, int64_t* n_pairs, const PairsScratch& s,
              cudaStream_t st);

}  // namespace b2g
