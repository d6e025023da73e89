// gb300_common.cuh -- shared device helpers for the sm_103a kernels:
// launch shapes sized to the SM count, deterministic fixed-order block and
// grid reductions (no floating-point atomics), and the library's error state.
//
// The reference reduces with warp shuffles and then one double atomicAdd per
// block (sundials_cuda_kernels.cuh:248-424), whose order depends on block
// scheduling.  Here every level has a fixed order: a thread sums its own
// grid-stride elements in index order, a warp combines lanes with a fixed
// butterfly, a block combines warps in index order, and the last block to
// finish combines the per-block partials in block-index order.  The result is
// therefore the same bits on every run for a given length and launch shape.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sundials_gb300_abi.h"

namespace gb300 {

constexpr int kBlock = 256;          // threads per block for vector kernels
constexpr int kWarps = kBlock / 32;  // warps per block
constexpr int kMaxRedBlocks = 1024;  // upper bound on blocks of a reduction
constexpr int kMaxRedVals = 8;       // values reduced together in one launch

// ---------------------------------------------------------------- errors
void set_error(int code, const char* msg);
bool check_cuda(cudaError_t err, const char* what);
void count_launch();
int num_sms();

// --------------------------------------------------------- launch shapes
// Elementwise kernels: one element pair per thread per trip, a grid-stride
// loop, at most 8 resident 256-thread blocks per SM.
inline int stream_grid(int64_t items)
{
  int64_t need = (items + kBlock - 1) / kBlock;
  int64_t cap  = (int64_t)num_sms() * 8;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

// Reductions: enough blocks to fill the GPU, each block reading at least 4
// element pairs per thread; up to 8,192 pairs one block does it all (its
// result is written directly: no last-block ticket, no fence, no second
// block to schedule -- latency is all that counts at that size).  The launch
// shape depends only on the length.
inline int reduce_grid(int64_t items)
{
  if (items <= 8192) return 1;
  int64_t need = (items + 4 * kBlock - 1) / (4 * kBlock);
  int64_t cap  = (int64_t)num_sms() * 4;
  if (cap > kMaxRedBlocks) cap = kMaxRedBlocks;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

// ------------------------------------------------------ combine functors
struct SumOp
{
  __host__ __device__ static double identity() { return 0.0; }
  __host__ __device__ static double combine(double a, double b) { return a + b; }
};
struct MaxOp
{
  __host__ __device__ static double identity() { return 0.0; }  // used on |x| only
  __host__ __device__ static double combine(double a, double b) { return a > b ? a : b; }
};
struct MinOp
{
  __host__ __device__ static double identity() { return 1.7976931348623157e308; }
  __host__ __device__ static double combine(double a, double b) { return a < b ? a : b; }
};

// Fixed butterfly within a warp: every lane ends with the same value.
template <class Op>
__device__ __forceinline__ double warp_reduce(double v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    v = Op::combine(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

// Block reduction of NV values per thread; thread 0 receives the results.
// `scratch` must hold kWarps * NV doubles.
template <class Op, int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], double* scratch)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_reduce<Op>(v[k]);
  if (lane == 0)
  {
#pragma unroll
    for (int k = 0; k < NV; ++k) scratch[k * kWarps + warp] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
#pragma unroll
    for (int k = 0; k < NV; ++k)
    {
      double acc = scratch[k * kWarps];
      for (int w = 1; w < kWarps; ++w) acc = Op::combine(acc, scratch[k * kWarps + w]);
      v[k] = acc;
    }
  }
  __syncthreads();
}

// Grid completion: block results go to partials[k * nblocks + b]; the last
// block to arrive (atomic ticket, no spinning) combines them in block order
// with a fixed tree and returns true on thread 0 with the totals in v.
// `counter` is reset to zero by that block for the next launch.
template <class Op, int NV>
__device__ __forceinline__ bool grid_finish(double (&v)[NV], double* partials,
                                            unsigned int* counter, int nblocks,
                                            int bid, double* scratch)
{
  __shared__ bool is_last;
  if (threadIdx.x == 0)
  {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * nblocks + bid] = v[k];
    __threadfence();
    unsigned int ticket = atomicAdd(counter, 1u);
    is_last = (ticket == (unsigned int)(nblocks - 1));
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  // Each thread folds blocks t, t+256, ... in order; then the block tree.
#pragma unroll
  for (int k = 0; k < NV; ++k)
  {
    double acc = Op::identity();
    bool first = true;
    for (int b = threadIdx.x; b < nblocks; b += kBlock)
    {
      double p = __ldcg(&partials[k * nblocks + b]);
      acc = first ? p : Op::combine(acc, p);
      first = false;
    }
    v[k] = acc;
  }
  block_reduce<Op, NV>(v, scratch);
  if (threadIdx.x == 0) *counter = 0u;
  return threadIdx.x == 0;
}

}  // namespace gb300
