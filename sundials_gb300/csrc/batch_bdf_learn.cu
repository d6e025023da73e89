// batch_bdf_learn.cu -- the fast modes' batched BDF kernels with the learned
// Newton predictor and the training-data recorder compiled in; launched only
// while a predictor or a recorder is attached (SetPredictor / SetRecorder).
#include "batch_bdf_kernel.cuh"

namespace bdf {

cudaError_t launch_fast_learn(const Params& P, int mode, int nb, int grid, cudaStream_t stream,
                              const int32_t* order, int64_t count, unsigned int* next)
{
  return fast_launch<true>(P, mode, nb, grid, stream, order, count, next);
}

cudaError_t occupancy_fast_learn(int mode, int nb, int* per_sm)
{
  return fast_occupancy<true>(mode, nb, per_sm);
}

}  // namespace bdf
