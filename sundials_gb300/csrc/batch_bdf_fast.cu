// batch_bdf_fast.cu -- instantiates the batched BDF kernel for the FP64 (FMA)
// and MIXED (FP32 factorisation + FP64 refinement) modes.
#include "batch_bdf_kernel.cuh"

namespace bdf {

cudaError_t launch_fast(const Params& P, int mode, int grid, cudaStream_t stream)
{
  if (mode == SUNBATCHBDF_MIXED)
    k_batch_bdf<SUNBATCHBDF_MIXED><<<grid, WARPS * 32, 0, stream>>>(P);
  else
    k_batch_bdf<SUNBATCHBDF_FP64><<<grid, WARPS * 32, 0, stream>>>(P);
  return cudaGetLastError();
}

cudaError_t occupancy_fast(int mode, int* blocks_per_sm)
{
  if (mode == SUNBATCHBDF_MIXED)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      blocks_per_sm, k_batch_bdf<SUNBATCHBDF_MIXED>, WARPS * 32, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm,
                                                       k_batch_bdf<SUNBATCHBDF_FP64>,
                                                       WARPS * 32, 0);
}

}  // namespace bdf
