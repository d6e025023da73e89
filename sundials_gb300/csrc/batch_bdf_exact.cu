// batch_bdf_exact.cu -- instantiates the batched BDF kernel for the
// FP64_EXACT mode.  This translation unit is compiled with -fmad=false (see
// sundials_gb300/build.py), so no product and sum is fused: every operation
// rounds like the reference compiled for x86-64.
#include "batch_bdf_kernel.cuh"

namespace bdf {

cudaError_t launch_exact(const Params& P, int grid, cudaStream_t stream)
{
  k_batch_bdf<SUNBATCHBDF_FP64_EXACT><<<grid, WARPS * 32, 0, stream>>>(P);
  return cudaGetLastError();
}

cudaError_t occupancy_exact(int* blocks_per_sm)
{
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
    blocks_per_sm, k_batch_bdf<SUNBATCHBDF_FP64_EXACT>, WARPS * 32, 0);
}

}  // namespace bdf
