// bruss3d_gb300.cu -- the 3-D advection-reaction benchmark's user functions
// (include/bruss3d_gb300.h) as sm_103a kernels over NVECTOR_GB300.
//
// One thread per cell (its 3 species are 24 contiguous bytes, so a warp's
// loads of the cell and of its z neighbour are contiguous; the y and x
// neighbours are one row / one plane away and come from L2 after the first
// read).  Compiled without contraction: every product and sum is rounded
// separately, in the order of the reference's C expressions.
#include <cuda_runtime.h>
#include <stdlib.h>

#include "../../include/bruss3d_gb300.h"
#include "../../include/nvector_gb300.h"
#include "gb300_common.cuh"

using namespace gb300;

struct SUNBruss3D_GB300_
{
  int64_t nx, ny, nz;
  double A, B, k1, k2, k3, k4, k5, k6, c;
  double cx, cy, cz;  // -c / dx, -c / dy, -c / dz
};

namespace {

struct Coef
{
  int64_t nx, ny, nz;
  double A, B, k1, k2, k3, k4, k5, k6, c, cx, cy, cz;
};

Coef coef(const SUNBruss3D_GB300_* p)
{
  return Coef{p->nx, p->ny, p->nz, p->A,  p->B,  p->k1, p->k2, p->k3,
              p->k4, p->k5, p->k6, p->c, p->cx, p->cy, p->cz};
}

// the advection of species l at cell (i, j, k), c != 0
__device__ __forceinline__ double advect(const Coef& q, const double* __restrict__ y, int64_t i,
                                         int64_t j, int64_t k, int l)
{
  const int64_t cell = (i * q.ny + j) * q.nz + k;
  const double yc    = y[3 * cell + l];
  if (q.c > 0.0)
  {
    const int64_t im = i > 0 ? i - 1 : q.nx - 1, jm = j > 0 ? j - 1 : q.ny - 1,
                  km = k > 0 ? k - 1 : q.nz - 1;
    const double yx = y[3 * ((im * q.ny + j) * q.nz + k) + l];
    const double yy = y[3 * ((i * q.ny + jm) * q.nz + k) + l];
    const double yz = y[3 * ((i * q.ny + j) * q.nz + km) + l];
    double d;
    if (i > 0 && j > 0 && k > 0)
    {  // interior kernel: z, y, x
      d = q.cz * (yc - yz);
      d = d + q.cy * (yc - yy);
      d = d + q.cx * (yc - yx);
    }
    else
    {  // face kernels: x, y, z
      d = q.cx * (yc - yx);
      d = d + q.cy * (yc - yy);
      d = d + q.cz * (yc - yz);
    }
    return d;
  }
  const int64_t ip = i + 1 < q.nx ? i + 1 : 0, jp = j + 1 < q.ny ? j + 1 : 0,
                kp = k + 1 < q.nz ? k + 1 : 0;
  const double yx = y[3 * ((ip * q.ny + j) * q.nz + k) + l];
  const double yy = y[3 * ((i * q.ny + jp) * q.nz + k) + l];
  const double yz = y[3 * ((i * q.ny + j) * q.nz + kp) + l];
  double d;
  if (i + 1 < q.nx && j + 1 < q.ny && k + 1 < q.nz)
  {
    d = q.cz * (yz - yc);
    d = d + q.cy * (yy - yc);
    d = d + q.cx * (yx - yc);
  }
  else
  {
    d = q.cx * (yx - yc);
    d = d + q.cy * (yy - yc);
    d = d + q.cz * (yz - yc);
  }
  return d;
}

// MODE 0: advection; 1: reaction alone (0 + g); 2: advection + reaction
template <int MODE>
__global__ void __launch_bounds__(kBlock)
  k_bruss_rhs(Coef q, const double* __restrict__ y, double* __restrict__ ydot)
{
  const int64_t ncell  = q.nx * q.ny * q.nz;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; cell < ncell;
       cell += stride)
  {
    const int64_t k = cell % q.nz, j = (cell / q.nz) % q.ny, i = cell / (q.nz * q.ny);
    double d0 = 0.0, d1 = 0.0, d2 = 0.0;
    if (MODE != 1 && q.c != 0.0)
    {
      d0 = advect(q, y, i, j, k, 0);
      d1 = advect(q, y, i, j, k, 1);
      d2 = advect(q, y, i, j, k, 2);
    }
    if (MODE != 0)
    {
      const double u = y[3 * cell], v = y[3 * cell + 1], w = y[3 * cell + 2];
      d0 = d0 + ((((q.k1 * q.A) - ((q.k2 * w) * u)) + (((q.k3 * u) * u) * v)) - (q.k4 * u));
      d1 = d1 + (((q.k2 * w) * u) - (((q.k3 * u) * u) * v));
      d2 = d2 + (((((-q.k2) * w) * u) + (q.k5 * q.B)) - (q.k6 * w));
    }
    ydot[3 * cell]     = d0;
    ydot[3 * cell + 1] = d1;
    ydot[3 * cell + 2] = d2;
  }
}

// x = (I - gamma dg/dy)^{-1} b per cell, the reference's closed form
__global__ void __launch_bounds__(kBlock)
  k_bruss_solve(Coef q, const double* __restrict__ y, const double* __restrict__ b,
                double* __restrict__ x, double gamma)
{
  const int64_t ncell  = q.nx * q.ny * q.nz;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t cell = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; cell < ncell;
       cell += stride)
  {
    const double u = y[3 * cell], v = y[3 * cell + 1], w = y[3 * cell + 2];
    const double b0 = b[3 * cell], b1 = b[3 * cell + 1], b2 = b[3 * cell + 2];
    const double k2 = q.k2, k3 = q.k3, k4 = q.k4, k6 = q.k6;
    // J = dg/dy
    double A0 = (((-k2) * w) + (((2.0 * k3) * u) * v)) - k4;
    double A1 = (k3 * u) * u;
    double A2 = (-k2) * u;
    double A3 = (k2 * w) - (((2.0 * k3) * u) * v);
    double A4 = ((-k3) * u) * u;
    double A5 = k2 * u;
    double A6 = (-k2) * w;
    double A7 = 0.0;
    double A8 = ((-k2) * u) - k6;
    // A = I - gamma J
    A0 = 1. - (gamma * A0);
    A1 = (-gamma) * A1;
    A2 = (-gamma) * A2;
    A3 = (-gamma) * A3;
    A4 = 1. - (gamma * A4);
    A5 = (-gamma) * A5;
    A6 = (-gamma) * A6;
    A7 = (-gamma) * A7;
    A8 = 1. - (gamma * A8);
    const double s0  = A4 * A8;
    const double s1  = A1 * A5;
    const double s2  = A2 * A7;
    const double s3  = A5 * A7;
    const double s4  = A1 * A8;
    const double s5  = A2 * A4;
    const double s6  = 1.0 / (((((A0 * s0 - A0 * s3) + A3 * s2) - A3 * s4) + A6 * s1) - A6 * s5);
    const double s7  = A2 * A3;
    const double s8  = A6 * b0;
    const double s9  = A2 * A6;
    const double s10 = A3 * b0;
    const double s11 = 1.0 / A0;
    const double s12 = A1 * s11;
    const double s13 = ((-A6) * s12 + A7) / ((-A3) * s12 + A4);
    x[3 * cell]     = s6 * ((b0 * (s0 - s3) + b1 * (s2 - s4)) + b2 * (s1 - s5));
    x[3 * cell + 1] = s6 * (((b2 * (s7 - A0 * A5) + b1 * (A0 * A8 - s9)) + A5 * s8) - A8 * s10);
    x[3 * cell + 2] = (((-b2) + s11 * s8) + s13 * (b1 - s10 * s11)) /
                      (((-A8) + s11 * s9) + s13 * (A5 - s11 * s7));
  }
}

bool fits(const SUNBruss3D_GB300_* p, N_Vector v)
{
  return p && v && N_VGetLength_GB300(v) == 3 * p->nx * p->ny * p->nz;
}

template <int MODE>
int rhs(void* pv, N_Vector y, N_Vector ydot)
{
  SUNBruss3D_GB300 p = (SUNBruss3D_GB300)pv;
  if (!fits(p, y) || !fits(p, ydot) || y == ydot) return -1;
  cudaStream_t s = (cudaStream_t)N_VGetStream_GB300(ydot);
  k_bruss_rhs<MODE><<<stream_grid(p->nx * p->ny * p->nz), kBlock, 0, s>>>(
    coef(p), N_VGetDeviceArrayPointer_GB300(y), N_VGetDeviceArrayPointer_GB300(ydot));
  count_launch();
  return check_cuda(cudaGetLastError(), "bruss3d rhs launch") ? 0 : -1;
}

}  // namespace

extern "C" {

SUNBruss3D_GB300 SUNBruss3D_GB300_Create(sunindextype nx, sunindextype ny, sunindextype nz,
                                         sunrealtype xmax, sunrealtype A, sunrealtype B,
                                         const sunrealtype* k, sunrealtype c)
{
  if (nx < 1 || ny < 1 || nz < 1 || !k || !(xmax > 0.0))
  {
    set_error(SUN_ERR_ARG_OUTOFRANGE, "SUNBruss3D_GB300_Create: bad arguments");
    return nullptr;
  }
  SUNBruss3D_GB300 p = (SUNBruss3D_GB300)calloc(1, sizeof(*p));
  if (!p) return nullptr;
  p->nx = nx;
  p->ny = ny;
  p->nz = nz;
  p->A  = A;
  p->B  = B;
  p->k1 = k[0];
  p->k2 = k[1];
  p->k3 = k[2];
  p->k4 = k[3];
  p->k5 = k[4];
  p->k6 = k[5];
  p->c  = c;
  // ParallelGrid: dx = (bx - ax) / nx on [0, xmax); cx = -c / dx
  const double dx = (xmax - 0.0) / (double)nx, dy = (xmax - 0.0) / (double)ny,
               dz = (xmax - 0.0) / (double)nz;
  p->cx = -c / dx;
  p->cy = -c / dy;
  p->cz = -c / dz;
  return p;
}

void SUNBruss3D_GB300_Free(SUNBruss3D_GB300 p) { free(p); }

int SUNBruss3D_GB300_Advection(sunrealtype, N_Vector y, N_Vector ydot, void* p)
{
  return rhs<0>(p, y, ydot);
}

int SUNBruss3D_GB300_Reaction(sunrealtype, N_Vector y, N_Vector ydot, void* p)
{
  return rhs<1>(p, y, ydot);
}

int SUNBruss3D_GB300_RHS(sunrealtype, N_Vector y, N_Vector ydot, void* p)
{
  return rhs<2>(p, y, ydot);
}

int SUNBruss3D_GB300_SolveReaction(N_Vector y, N_Vector x, N_Vector b, sunrealtype gamma,
                                   void* pv)
{
  SUNBruss3D_GB300 p = (SUNBruss3D_GB300)pv;
  if (!fits(p, y) || !fits(p, x) || !fits(p, b)) return -1;
  cudaStream_t s = (cudaStream_t)N_VGetStream_GB300(x);
  k_bruss_solve<<<stream_grid(p->nx * p->ny * p->nz), kBlock, 0, s>>>(
    coef(p), N_VGetDeviceArrayPointer_GB300(y), N_VGetDeviceArrayPointer_GB300(b),
    N_VGetDeviceArrayPointer_GB300(x), gamma);
  count_launch();
  return check_cuda(cudaGetLastError(), "bruss3d reaction solve launch") ? 0 : -1;
}

int SUNBruss3D_GB300_CVPSolve(sunrealtype, N_Vector y, N_Vector, N_Vector r, N_Vector z,
                              sunrealtype gamma, sunrealtype, int, void* p)
{
  return SUNBruss3D_GB300_SolveReaction(y, z, r, gamma, p);
}

}  // extern "C"
