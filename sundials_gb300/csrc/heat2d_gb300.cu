// heat2d_gb300.cu -- 5-point heat-equation user functions (right-hand side,
// J v, z = v - gamma J v, Jacobi preconditioner) as sm_103a kernels over
// NVECTOR_GB300 vectors.  The stencil follows examples/cvode/CXX_serial/
// cv_heat2D.cpp:305-367 without its manufactured forcing term, on the interior
// points only (the reference stores the boundary ring and keeps it at zero).
//
// One thread per pair of neighbouring x points (16-byte loads and stores when
// nx is even); the rows above and below are re-read from L2, so DRAM sees one
// read and one write per point.  The file is compiled without contraction:
// every product and sum is rounded separately in the reference's order.
#include <cuda_runtime.h>
#include <stdlib.h>

#include "../../include/heat2d_gb300.h"
#include "../../include/nvector_gb300.h"
#include "gb300_common.cuh"

using namespace gb300;

struct SUNHeat2D_GB300_
{
  int64_t nx, ny;
  double kx, ky, cx, cy, cc;
  double gamma, d;  // Newton-matrix gamma and Jacobi factor 1/(1 - gamma cc)
};

namespace {

__device__ __forceinline__ double stencil(double c, double w, double e, double s, double n,
                                          double cx, double cy, double cc)
{
  return (cc * c + cx * (w + e)) + cy * (s + n);
}

// mode 0: out = J v;  mode 1: out = v + (-gamma) J v
template <int MODE>
__global__ void __launch_bounds__(kBlock)
  k_heat_apply(int64_t nx, int64_t ny, const double* __restrict__ v, double* __restrict__ out,
               double cx, double cy, double cc, double mgamma, int vec)
{
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (vec)
  {
    const int64_t hx    = nx >> 1;
    const int64_t total = hx * ny;
    for (int64_t p = tid; p < total; p += stride)
    {
      const int64_t j = p / hx, i = (p - j * hx) * 2;
      const int64_t c = j * nx + i;
      const double2 vc = *(const double2*)(v + c);
      const double2 vs = j > 0 ? *(const double2*)(v + c - nx) : make_double2(0.0, 0.0);
      const double2 vn = j + 1 < ny ? *(const double2*)(v + c + nx) : make_double2(0.0, 0.0);
      const double w0  = i > 0 ? v[c - 1] : 0.0;
      const double e1  = i + 2 < nx ? v[c + 2] : 0.0;
      double r0 = stencil(vc.x, w0, vc.y, vs.x, vn.x, cx, cy, cc);
      double r1 = stencil(vc.y, vc.x, e1, vs.y, vn.y, cx, cy, cc);
      if (MODE == 1)
      {
        r0 = vc.x + mgamma * r0;
        r1 = vc.y + mgamma * r1;
      }
      *(double2*)(out + c) = make_double2(r0, r1);
    }
    return;
  }
  const int64_t total = nx * ny;
  for (int64_t c = tid; c < total; c += stride)
  {
    const int64_t j = c / nx, i = c - j * nx;
    const double vc = v[c];
    const double w  = i > 0 ? v[c - 1] : 0.0;
    const double e  = i + 1 < nx ? v[c + 1] : 0.0;
    const double s  = j > 0 ? v[c - nx] : 0.0;
    const double n  = j + 1 < ny ? v[c + nx] : 0.0;
    double r        = stencil(vc, w, e, s, n, cx, cy, cc);
    if (MODE == 1) r = vc + mgamma * r;
    out[c] = r;
  }
}

int apply(SUNHeat2D_GB300 p, N_Vector v, N_Vector out, int mode)
{
  if (!p || N_VGetLength_GB300(v) != p->nx * p->ny || N_VGetLength_GB300(out) != p->nx * p->ny)
    return -1;
  const double* dv = N_VGetDeviceArrayPointer_GB300(v);
  double* dz       = N_VGetDeviceArrayPointer_GB300(out);
  if (dv == dz) return -1;  // the stencil needs distinct input and output
  cudaStream_t s = (cudaStream_t)N_VGetStream_GB300(out);
  int vec = (p->nx % 2 == 0) && (((uintptr_t)dv | (uintptr_t)dz) & 15u) == 0;
  int64_t items = vec ? (p->nx / 2) * p->ny : p->nx * p->ny;
  int grid      = stream_grid(items);
  if (mode == 0)
    k_heat_apply<0><<<grid, kBlock, 0, s>>>(p->nx, p->ny, dv, dz, p->cx, p->cy, p->cc, 0.0, vec);
  else
    k_heat_apply<1><<<grid, kBlock, 0, s>>>(p->nx, p->ny, dv, dz, p->cx, p->cy, p->cc,
                                            -p->gamma, vec);
  count_launch();
  return check_cuda(cudaGetLastError(), "heat2d stencil launch") ? 0 : -1;
}

}  // namespace

extern "C" {

SUNHeat2D_GB300 SUNHeat2D_GB300_Create(sunindextype nx, sunindextype ny, sunrealtype kx,
                                       sunrealtype ky)
{
  if (nx < 1 || ny < 1) return nullptr;
  SUNHeat2D_GB300 p = (SUNHeat2D_GB300)calloc(1, sizeof(*p));
  p->nx = nx;
  p->ny = ny;
  p->kx = kx;
  p->ky = ky;
  const double dx = 1.0 / (double)(nx + 1), dy = 1.0 / (double)(ny + 1);
  p->cx    = kx / (dx * dx);
  p->cy    = ky / (dy * dy);
  p->cc    = -2.0 * (p->cx + p->cy);
  p->gamma = 0.0;
  p->d     = 1.0;
  return p;
}

void SUNHeat2D_GB300_Free(SUNHeat2D_GB300 p) { free(p); }

SUNErrCode SUNHeat2D_GB300_SetGamma(SUNHeat2D_GB300 p, sunrealtype gamma)
{
  if (!p) return SUN_ERR_ARG_CORRUPT;
  p->gamma = gamma;
  return SUN_SUCCESS;
}

int SUNHeat2D_GB300_RHS(sunrealtype, N_Vector u, N_Vector f, void* p)
{
  return apply((SUNHeat2D_GB300)p, u, f, 0);
}

int SUNHeat2D_GB300_JTimes(N_Vector v, N_Vector Jv, sunrealtype, N_Vector, N_Vector, void* p,
                           N_Vector)
{
  return apply((SUNHeat2D_GB300)p, v, Jv, 0);
}

int SUNHeat2D_GB300_ATimes(void* p, N_Vector v, N_Vector z)
{
  return apply((SUNHeat2D_GB300)p, v, z, 1);
}

int SUNHeat2D_GB300_PSetup(void* pv)
{
  SUNHeat2D_GB300 p = (SUNHeat2D_GB300)pv;
  if (!p) return -1;
  p->d = 1.0 / (1.0 - p->gamma * p->cc);
  return 0;
}

int SUNHeat2D_GB300_PSolve(void* pv, N_Vector r, N_Vector z, sunrealtype, int)
{
  SUNHeat2D_GB300 p = (SUNHeat2D_GB300)pv;
  if (!p) return -1;
  N_VScale_GB300(p->d, r, z);
  return 0;
}

// Like the reference example's PSetup, *jcurPtr is left as the integrator set it.
int SUNHeat2D_GB300_CVPSetup(sunrealtype, N_Vector, N_Vector, sunbooleantype, sunbooleantype*,
                             sunrealtype gamma, void* pv)
{
  SUNHeat2D_GB300 p = (SUNHeat2D_GB300)pv;
  if (!p) return -1;
  p->gamma = gamma;
  return SUNHeat2D_GB300_PSetup(p);
}

int SUNHeat2D_GB300_CVPSolve(sunrealtype, N_Vector, N_Vector, N_Vector r, N_Vector z,
                             sunrealtype, sunrealtype, int, void* pv)
{
  return SUNHeat2D_GB300_PSolve(pv, r, z, 0.0, 0);
}

}  // extern "C"
