// toi.cu - continuous collision kernels: batched time of impact of swept shape pairs.
#include <cuda_runtime.h>

#include "b2g_math.cuh"
#include "kernels.h"
#include "toi.cuh"

namespace b2g {

__device__ __forceinline__ Sweep sweepOf(const b2g_sweep& s) {
  Sweep o;
  o.lc = mk(s.local_center[0], s.local_center[1]);
  o.c0 = mk(s.c0[0], s.c0[1]);
  o.c = mk(s.c[0], s.c[1]);
  o.a0 = s.a0;
  o.a = s.a;
  o.alpha0 = s.alpha0;
  return o;
}

// One thread per input pair.
__global__ void k_time_of_impact(const b2g_toi_input* in, int n, b2g_toi_output* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const b2g_toi_input& q = in[i];
  float t;
  int state = timeOfImpact(q.shape_a, q.shape_b, sweepOf(q.sweep_a), sweepOf(q.sweep_b), q.t_max, &t);
  b2g_toi_output r;
  r.state = state;
  r.t = t;
  out[i] = r;
}

void launch_time_of_impact(const b2g_toi_input* in, int n, b2g_toi_output* out, cudaStream_t s) {
  if (n > 0) k_time_of_impact<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(in, n, out);
}

}  // namespace b2g
