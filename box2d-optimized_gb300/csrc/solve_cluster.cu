// solve_cluster.cu - the island solve of the largest worlds (more bodies than the largest CTA
// class holds: single large scenes of tens of thousands of bodies) on a thread-block cluster per
// world. The same solve as the per-CTA kernel (solve_world.cuh, written against a team of
// threads), with the team's barrier the cluster barrier, so the world's colours are solved by
// CS SMs at once instead of one. Results do not depend on the team: a colour's constraints share
// no non-static body, and everything else is order-independent or computed by one thread.
#include "solve_world.cuh"

namespace b2g {

static int g_cluster_ctas = 0;

int solver_max_cluster_ctas() { return g_cluster_ctas; }

// Whether the device can keep one cluster of `cs` CTAs of the cluster kernel resident.
template <int CS>
static bool cluster_runs(cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CS);
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_solve_cluster<kClusterThreads, CS>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n > 0;
}

void solve_cluster_setup() {
  g_cluster_ctas = 0;
  if (cudaFuncSetAttribute(k_solve_cluster<kClusterThreads, 16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
          cudaSuccess &&
      cluster_runs<16>(0)) {
    g_cluster_ctas = 16;
    return;
  }
  cudaGetLastError();
  if (cluster_runs<8>(0)) g_cluster_ctas = 8;
}

template <int CS>
static void launch_cluster(const KernelArgs& a, const SolveClass& c, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(c.count * CS));
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_solve_cluster<kClusterThreads, CS>, a, c.first);
}

void launch_solve_class_cluster(const KernelArgs& a, const SolveClass& c, cudaStream_t s) {
  if (c.ctas >= 16) launch_cluster<16>(a, c, s);
  else if (c.ctas >= 8) launch_cluster<8>(a, c, s);
  else if (c.ctas >= 4) launch_cluster<4>(a, c, s);
  else launch_cluster<2>(a, c, s);
}

}  // namespace b2g
