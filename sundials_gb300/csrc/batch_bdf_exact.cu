// batch_bdf_exact.cu -- instantiates the batched BDF kernel for the
// FP64_EXACT mode.  This translation unit is compiled with -fmad=false (see
// sundials_gb300/build.py), so no product and sum is fused: every operation
// rounds like the reference compiled for x86-64.
#include "batch_bdf_kernel.cuh"

namespace bdf {

// (the kernel's shared-memory limit was set by occ_one at creation)
template <int NB>
static cudaError_t launch_one(const Params& P, int grid, cudaStream_t stream, const int32_t* order,
                              int64_t count, unsigned int* next)
{
  const size_t smem = Layout<SUNBATCHBDF_FP64_EXACT, NB>::warp_bytes;
  k_batch_bdf<SUNBATCHBDF_FP64_EXACT, NB><<<grid, 32, smem, stream>>>(P, order, count, next);
  return cudaGetLastError();
}

template <int NB>
static cudaError_t occ_one(int* per_sm)
{
  const size_t smem = Layout<SUNBATCHBDF_FP64_EXACT, NB>::warp_bytes;
  cudaFuncSetAttribute(k_batch_bdf<SUNBATCHBDF_FP64_EXACT, NB>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch_bdf<SUNBATCHBDF_FP64_EXACT, NB>,
                                                       32, smem);
}

cudaError_t launch_exact(const Params& P, int nb, int grid, cudaStream_t stream,
                         const int32_t* order, int64_t count, unsigned int* next)
{
  return nb <= 32   ? launch_one<32>(P, grid, stream, order, count, next)
         : nb <= 48 ? launch_one<48>(P, grid, stream, order, count, next)
                    : launch_one<64>(P, grid, stream, order, count, next);
}

cudaError_t occupancy_exact(int nb, int* per_sm)
{
  return nb <= 32 ? occ_one<32>(per_sm) : nb <= 48 ? occ_one<48>(per_sm) : occ_one<64>(per_sm);
}

}  // namespace bdf
