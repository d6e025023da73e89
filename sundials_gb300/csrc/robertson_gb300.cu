// robertson_gb300.cu -- user functions of a batch of Robertson kinetics
// cells (include/robertson_gb300.h) as sm_103a kernels over NVECTOR_GB300,
// with the exact block-Jacobi preconditioner on SUNLinSol_BlockLU_GB300.
//
// One thread per cell: the 3 species of a cell are 24 contiguous bytes, so a
// warp reads 768 contiguous bytes per vector; the Jacobian blocks (9 doubles
// per cell, column-major) are one block of the block-diagonal matrix each.
// Compiled without contraction: every product and sum is rounded separately,
// in the order stated in the header.
#include <cuda_runtime.h>
#include <stdlib.h>

#include <vector>

#include "../../include/nvector_gb300.h"
#include "../../include/robertson_gb300.h"
#include "../../include/sunlinsol_blocklu_gb300.h"
#include "gb300_common.cuh"

using namespace gb300;

struct SUNRoberts_GB300_
{
  int64_t ncells;
  double* d_k;   // k1, k2, k3 per cell
  double* d_J;   // saved Jacobian blocks, 9 per cell, column-major
  SUNMatrix P;   // I - gamma J, 3x3 blocks
  SUNLinearSolver LS;
};

namespace {

__global__ void __launch_bounds__(kBlock)
  k_rob_rhs(int64_t ncells, const double* __restrict__ k, const double* __restrict__ y,
            double* __restrict__ ydot)
{
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += stride)
  {
    const double k1 = k[3 * c], k2 = k[3 * c + 1], k3 = k[3 * c + 2];
    const double y1 = y[3 * c], y2 = y[3 * c + 1], y3 = y[3 * c + 2];
    const double yd1 = (-k1) * y1 + (k3 * y2) * y3;
    const double yd3 = (k2 * y2) * y2;
    ydot[3 * c]     = yd1;
    ydot[3 * c + 1] = -yd1 - yd3;
    ydot[3 * c + 2] = yd3;
  }
}

// Jacobian entries of cell c at y (row i, column j -> e[j*3 + i])
__device__ __forceinline__ void rob_jac(double k1, double k2, double k3, double y2, double y3,
                                        double (&e)[9])
{
  e[0] = -k1;
  e[1] = k1;
  e[2] = 0.0;
  e[3] = k3 * y3;
  e[4] = (-k3 * y3) - ((2.0 * k2) * y2);
  e[5] = (2.0 * k2) * y2;
  e[6] = k3 * y2;
  e[7] = -k3 * y2;
  e[8] = 0.0;
}

__global__ void __launch_bounds__(kBlock)
  k_rob_jtimes(int64_t ncells, const double* __restrict__ k, const double* __restrict__ y,
               const double* __restrict__ v, double* __restrict__ jv)
{
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += stride)
  {
    double e[9];
    rob_jac(k[3 * c], k[3 * c + 1], k[3 * c + 2], y[3 * c + 1], y[3 * c + 2], e);
    const double v1 = v[3 * c], v2 = v[3 * c + 1], v3 = v[3 * c + 2];
    jv[3 * c]     = (e[0] * v1 + e[3] * v2) + e[6] * v3;
    jv[3 * c + 1] = (e[1] * v1 + e[4] * v2) + e[7] * v3;
    jv[3 * c + 2] = (e[2] * v1 + e[5] * v2) + e[8] * v3;
  }
}

__global__ void __launch_bounds__(kBlock)
  k_rob_jac(int64_t ncells, const double* __restrict__ k, const double* __restrict__ y,
            double* __restrict__ J)
{
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += stride)
  {
    double e[9];
    rob_jac(k[3 * c], k[3 * c + 1], k[3 * c + 2], y[3 * c + 1], y[3 * c + 2], e);
#pragma unroll
    for (int q = 0; q < 9; q++) J[9 * c + q] = e[q];
  }
}

// P = (-gamma) J, then P_ii += 1 (SUNDlsMat_denseScale, denseAddIdentity)
__global__ void __launch_bounds__(kBlock)
  k_rob_newton_matrix(int64_t ncells, const double* __restrict__ J, double* __restrict__ P,
                      double mgamma)
{
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < 9 * ncells; e += stride)
  {
    const int q = (int)(e % 9);
    double a    = mgamma * J[e];
    if (q == 0 || q == 4 || q == 8) a = a + 1.0;
    P[e] = a;
  }
}

bool same_length(SUNRoberts_GB300 p, N_Vector v)
{
  return p && v && N_VGetLength_GB300(v) == 3 * p->ncells;
}

}  // namespace

extern "C" {

SUNRoberts_GB300 SUNRoberts_GB300_Create(sunindextype ncells, const sunrealtype* k, N_Vector tmpl,
                                         int lu_precision, SUNContext sunctx)
{
  if (ncells < 1 || !k || !tmpl || N_VGetLength_GB300(tmpl) != 3 * ncells)
  {
    set_error(SUN_ERR_ARG_INCOMPATIBLE, "SUNRoberts_GB300_Create: bad arguments");
    return nullptr;
  }
  SUNRoberts_GB300 p = (SUNRoberts_GB300)calloc(1, sizeof(*p));
  if (!p) return nullptr;
  p->ncells = ncells;
  if (!check_cuda(cudaMalloc(&p->d_k, sizeof(double) * 3 * ncells), "cudaMalloc") ||
      !check_cuda(cudaMalloc(&p->d_J, sizeof(double) * 9 * ncells), "cudaMalloc") ||
      !check_cuda(cudaMemcpy(p->d_k, k, sizeof(double) * 3 * ncells, cudaMemcpyHostToDevice),
                  "cudaMemcpy") ||
      !check_cuda(cudaMemset(p->d_J, 0, sizeof(double) * 9 * ncells), "cudaMemset"))
  {
    SUNRoberts_GB300_Free(p);
    return nullptr;
  }
  std::vector<sunindextype> off(ncells + 1);
  for (int64_t c = 0; c <= ncells; c++) off[c] = 3 * c;
  p->P = SUNMatrix_BlockDiag_GB300(ncells, off.data(), sunctx);
  p->LS = p->P ? SUNLinSol_BlockLU_GB300(tmpl, p->P, lu_precision, sunctx) : nullptr;
  if (!p->P || !p->LS || SUNLinSolInitialize_BlockLU_GB300(p->LS) != SUN_SUCCESS)
  {
    SUNRoberts_GB300_Free(p);
    return nullptr;
  }
  return p;
}

void SUNRoberts_GB300_Free(SUNRoberts_GB300 p)
{
  if (!p) return;
  if (p->LS) SUNLinSolFree_BlockLU_GB300(p->LS);
  if (p->P) SUNMatDestroy_BlockDiag_GB300(p->P);
  cudaFree(p->d_k);
  cudaFree(p->d_J);
  free(p);
}

int SUNRoberts_GB300_RHS(sunrealtype, N_Vector y, N_Vector ydot, void* pv)
{
  SUNRoberts_GB300 p = (SUNRoberts_GB300)pv;
  if (!same_length(p, y) || !same_length(p, ydot)) return -1;
  cudaStream_t s = (cudaStream_t)N_VGetStream_GB300(ydot);
  k_rob_rhs<<<stream_grid(p->ncells), kBlock, 0, s>>>(
    p->ncells, p->d_k, N_VGetDeviceArrayPointer_GB300(y), N_VGetDeviceArrayPointer_GB300(ydot));
  count_launch();
  return check_cuda(cudaGetLastError(), "robertson rhs launch") ? 0 : -1;
}

int SUNRoberts_GB300_JTimes(N_Vector v, N_Vector Jv, sunrealtype, N_Vector y, N_Vector, void* pv,
                            N_Vector)
{
  SUNRoberts_GB300 p = (SUNRoberts_GB300)pv;
  if (!same_length(p, v) || !same_length(p, Jv) || !same_length(p, y) || v == Jv) return -1;
  cudaStream_t s = (cudaStream_t)N_VGetStream_GB300(Jv);
  k_rob_jtimes<<<stream_grid(p->ncells), kBlock, 0, s>>>(
    p->ncells, p->d_k, N_VGetDeviceArrayPointer_GB300(y), N_VGetDeviceArrayPointer_GB300(v),
    N_VGetDeviceArrayPointer_GB300(Jv));
  count_launch();
  return check_cuda(cudaGetLastError(), "robertson jtimes launch") ? 0 : -1;
}

int SUNRoberts_GB300_Jac(sunrealtype, N_Vector y, N_Vector, SUNMatrix J, void* pv, N_Vector,
                         N_Vector, N_Vector)
{
  SUNRoberts_GB300 p = (SUNRoberts_GB300)pv;
  if (!same_length(p, y) || !J || SUNMatrix_BlockDiag_GB300_Rows(J) != 3 * p->ncells ||
      SUNMatrix_BlockDiag_GB300_NNZ(J) != 9 * p->ncells)
    return -1;
  cudaStream_t s = (cudaStream_t)N_VGetStream_GB300(y);
  k_rob_jac<<<stream_grid(p->ncells), kBlock, 0, s>>>(p->ncells, p->d_k,
                                                      N_VGetDeviceArrayPointer_GB300(y),
                                                      SUNMatrix_BlockDiag_GB300_Data(J));
  count_launch();
  return check_cuda(cudaGetLastError(), "robertson jac launch") ? 0 : -1;
}

int SUNRoberts_GB300_CVPSetup(sunrealtype, N_Vector y, N_Vector, sunbooleantype jok,
                              sunbooleantype* jcurPtr, sunrealtype gamma, void* pv)
{
  SUNRoberts_GB300 p = (SUNRoberts_GB300)pv;
  if (!same_length(p, y) || !jcurPtr) return -1;
  // the vectors' stream, on which the block LU (built on tmpl) works too
  cudaStream_t s = (cudaStream_t)N_VGetStream_GB300(y);
  if (!jok)
  {
    k_rob_jac<<<stream_grid(p->ncells), kBlock, 0, s>>>(p->ncells, p->d_k,
                                                        N_VGetDeviceArrayPointer_GB300(y), p->d_J);
    count_launch();
    *jcurPtr = SUNTRUE;
  }
  else *jcurPtr = SUNFALSE;
  k_rob_newton_matrix<<<stream_grid(9 * p->ncells), kBlock, 0, s>>>(
    p->ncells, p->d_J, SUNMatrix_BlockDiag_GB300_Data(p->P), -gamma);
  count_launch();
  if (!check_cuda(cudaGetLastError(), "robertson psetup launch")) return -1;
  const int flag = SUNLinSolSetup_BlockLU_GB300(p->LS, p->P);
  if (flag == 0) return 0;
  return flag > 0 ? 1 : -1;
}

int SUNRoberts_GB300_CVPSolve(sunrealtype, N_Vector, N_Vector, N_Vector r, N_Vector z,
                              sunrealtype, sunrealtype, int, void* pv)
{
  SUNRoberts_GB300 p = (SUNRoberts_GB300)pv;
  if (!same_length(p, r) || !same_length(p, z)) return -1;
  const int flag = SUNLinSolSolve_BlockLU_GB300(p->LS, p->P, z, r, 0.0);
  return flag == 0 ? 0 : (flag > 0 ? 1 : -1);
}

}  // extern "C"
