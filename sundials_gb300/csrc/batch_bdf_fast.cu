// batch_bdf_fast.cu -- instantiates the batched BDF kernel for the FP64 (FMA)
// and MIXED (FP32 inverse + FP64 refinement) modes, all three size buckets,
// without the learned-predictor code (batch_bdf_learn.cu has it).
#include "batch_bdf_kernel.cuh"

namespace bdf {

cudaError_t launch_fast(const Params& P, int mode, int nb, int grid, cudaStream_t stream,
                        const int32_t* order, int64_t count, unsigned int* next)
{
  return fast_launch<false>(P, mode, nb, grid, stream, order, count, next);
}

cudaError_t occupancy_fast(int mode, int nb, int* per_sm)
{
  return fast_occupancy<false>(mode, nb, per_sm);
}

}  // namespace bdf
