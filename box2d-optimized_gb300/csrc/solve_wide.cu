// solve_wide.cu - the wide build of the per-world solve kernel: 512 threads per SM at up to 128
// registers a thread, so the joint and contact solvers run unspilled and each thread reads its
// next colour's rows before the barrier; the default for every size class. A translation unit of
// its own so that the two builds compile in parallel.
#include "solve_world.cuh"

namespace b2g {

void solve_wide_setup(const int* smem_caps) {
  cudaFuncSetAttribute(k_solve<64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_caps[0]);
  cudaFuncSetAttribute(k_solve<128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_caps[1]);
  cudaFuncSetAttribute(k_solve<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_caps[2]);
  cudaFuncSetAttribute(k_solve<512, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_caps[3]);
  cudaFuncSetAttribute(k_solve<1024, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_caps[4]);
}

void launch_solve_class_wide(const KernelArgs& a, const SolveClass& c, cudaStream_t s) {
  switch (c.threads) {
    case 64: k_solve<64, true><<<c.count, 64, c.smem, s>>>(a, c.first, c.smem); break;
    case 128: k_solve<128, true><<<c.count, 128, c.smem, s>>>(a, c.first, c.smem); break;
    case 256: k_solve<256, true><<<c.count, 256, c.smem, s>>>(a, c.first, c.smem); break;
    case 512: k_solve<512, true><<<c.count, 512, c.smem, s>>>(a, c.first, c.smem); break;
    default: k_solve<1024, true><<<c.count, 1024, c.smem, s>>>(a, c.first, c.smem); break;
  }
}

}  // namespace b2g
