/* cvode_heat2d_gb300.c -- what a SUNDIALS user writes to integrate the 2-D
 * heat problem of examples/cvode/CXX_serial/cv_heat2D.cpp with the GB300
 * modules plugged into the unchanged CVODE: every vector an NVECTOR_GB300,
 * SUNLinSol_SPGMR_GB300 as the linear solver, and the device user functions
 * of include/heat2d_gb300.h.  Compiled against the reference's headers
 * (SUNGB300_WITH_SUNDIALS makes the GB300 headers defer to them) and linked
 * against the reference's CVODE and libsundials_gb300.so; needs a GB300 to run.
 *
 *   usage: cvode_heat2d_gb300 [nx] [ny]
 */
#define SUNGB300_WITH_SUNDIALS
#include <cvode/cvode.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <sundials/sundials_core.h>

#include "heat2d_gb300.h"
#include "nvector_gb300.h"
#include "sunlinsol_spgmr_gb300.h"

static int check(int flag, const char* what)
{
  if (flag < 0) fprintf(stderr, "%s failed: %d\n", what, flag);
  return flag < 0;
}

int main(int argc, char** argv)
{
  const sunindextype nx = argc > 1 ? atol(argv[1]) : 64, ny = argc > 2 ? atol(argv[2]) : 64;
  const sunrealtype rtol = 1e-6, atol = 1e-10, tf = 0.1;
  SUNContext ctx;
  if (check(SUNContext_Create(SUN_COMM_NULL, &ctx), "SUNContext_Create")) return 1;

  /* u0 = sin(pi x) sin(pi y) on the interior points, row by row */
  N_Vector u = N_VNew_GB300(nx * ny, ctx);
  if (!u) return 1;
  sunrealtype* uh = N_VGetHostArrayPointer_GB300(u);
  for (sunindextype j = 0; j < ny; j++)
    for (sunindextype i = 0; i < nx; i++)
      uh[j * nx + i] = sin(M_PI * (i + 1) / (nx + 1)) * sin(M_PI * (j + 1) / (ny + 1));
  N_VCopyToDevice_GB300(u);

  SUNHeat2D_GB300 heat = SUNHeat2D_GB300_Create(nx, ny, 1.0, 1.0);
  void* cvode_mem      = CVodeCreate(CV_BDF, ctx);
  if (check(CVodeInit(cvode_mem, SUNHeat2D_GB300_RHS, 0.0, u), "CVodeInit")) return 1;
  if (check(CVodeSetUserData(cvode_mem, heat), "CVodeSetUserData")) return 1;
  if (check(CVodeSStolerances(cvode_mem, rtol, atol), "CVodeSStolerances")) return 1;

  SUNLinearSolver LS = SUNLinSol_SPGMR_GB300(u, SUN_PREC_LEFT, 5, ctx);
  if (check(CVodeSetLinearSolver(cvode_mem, LS, NULL), "CVodeSetLinearSolver")) return 1;
  if (check(CVodeSetJacTimes(cvode_mem, NULL, SUNHeat2D_GB300_JTimes), "CVodeSetJacTimes"))
    return 1;
  if (check(CVodeSetPreconditioner(cvode_mem, SUNHeat2D_GB300_CVPSetup,
                                   SUNHeat2D_GB300_CVPSolve),
            "CVodeSetPreconditioner"))
    return 1;

  sunrealtype t = 0.0;
  if (check(CVode(cvode_mem, tf, u, &t, CV_NORMAL), "CVode")) return 1;
  N_VCopyFromDevice_GB300(u);
  printf("t = %g, u(center) = %.10e\n", t, N_VGetHostArrayPointer_GB300(u)[(ny / 2) * nx + nx / 2]);
  CVodePrintAllStats(cvode_mem, stdout, SUN_OUTPUTFORMAT_TABLE);

  CVodeFree(&cvode_mem);
  SUNLinSolFree(LS);
  SUNHeat2D_GB300_Free(heat);
  N_VDestroy(u);
  SUNContext_Free(&ctx);
  return 0;
}
