// batch_bdf_fast.cu -- instantiates the batched BDF kernel for the FP64 (FMA)
// and MIXED (FP32 inverse + FP64 refinement) modes, all three size buckets.
#include "batch_bdf_kernel.cuh"

namespace bdf {

// (the kernel's shared-memory limit was set by occ_one at creation)
template <int MODE, int NB>
static cudaError_t launch_one(const Params& P, int grid, cudaStream_t stream, const int32_t* order,
                              int64_t count, unsigned int* next)
{
  const size_t smem = Layout<MODE, NB>::warp_bytes;
  k_batch_bdf<MODE, NB><<<grid, 32, smem, stream>>>(P, order, count, next);
  return cudaGetLastError();
}

template <int MODE, int NB>
static cudaError_t occ_one(int* per_sm)
{
  const size_t smem = Layout<MODE, NB>::warp_bytes;
  cudaFuncSetAttribute(k_batch_bdf<MODE, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch_bdf<MODE, NB>, 32, smem);
}

cudaError_t launch_fast(const Params& P, int mode, int nb, int grid, cudaStream_t stream,
                        const int32_t* order, int64_t count, unsigned int* next)
{
  if (mode == SUNBATCHBDF_MIXED)
    return nb <= 32   ? launch_one<SUNBATCHBDF_MIXED, 32>(P, grid, stream, order, count, next)
           : nb <= 48 ? launch_one<SUNBATCHBDF_MIXED, 48>(P, grid, stream, order, count, next)
                      : launch_one<SUNBATCHBDF_MIXED, 64>(P, grid, stream, order, count, next);
  return nb <= 32   ? launch_one<SUNBATCHBDF_FP64, 32>(P, grid, stream, order, count, next)
         : nb <= 48 ? launch_one<SUNBATCHBDF_FP64, 48>(P, grid, stream, order, count, next)
                    : launch_one<SUNBATCHBDF_FP64, 64>(P, grid, stream, order, count, next);
}

cudaError_t occupancy_fast(int mode, int nb, int* per_sm)
{
  if (mode == SUNBATCHBDF_MIXED)
    return nb <= 32   ? occ_one<SUNBATCHBDF_MIXED, 32>(per_sm)
           : nb <= 48 ? occ_one<SUNBATCHBDF_MIXED, 48>(per_sm)
                      : occ_one<SUNBATCHBDF_MIXED, 64>(per_sm);
  return nb <= 32   ? occ_one<SUNBATCHBDF_FP64, 32>(per_sm)
         : nb <= 48 ? occ_one<SUNBATCHBDF_FP64, 48>(per_sm)
                    : occ_one<SUNBATCHBDF_FP64, 64>(per_sm);
}

}  // namespace bdf
