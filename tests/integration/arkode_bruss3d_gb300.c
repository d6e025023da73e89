/* arkode_bruss3d_gb300.c -- what a SUNDIALS user writes to run the 3-D
 * advection-reaction benchmark's ARKODE configurations
 * (benchmarks/advection_reaction_3D/raja/arkode_driver.cpp: ARK-DIRK, its
 * default, and ARK-IMEX) with the GB300 modules plugged into the unchanged
 * ARKODE: every vector an NVECTOR_GB300, SUNLinSol_SPGMR_GB300 as the linear
 * solver, the device user functions of include/bruss3d_gb300.h.  Compiled
 * against the reference's headers (SUNGB300_WITH_SUNDIALS makes the GB300
 * headers defer to them) and linked against the reference's ARKODE and
 * libsundials_gb300.so; needs a GB300 to run.
 *
 *   usage: arkode_bruss3d_gb300 [n] [imex]
 */
#define SUNGB300_WITH_SUNDIALS
#include <arkode/arkode.h>
#include <arkode/arkode_arkstep.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <sundials/sundials_core.h>
#include <sunnonlinsol/sunnonlinsol_newton.h>

#include "bruss3d_gb300.h"
#include "nvector_gb300.h"
#include "sunlinsol_spgmr_gb300.h"

static int check(int flag, const char* what)
{
  if (flag < 0) fprintf(stderr, "%s failed: %d\n", what, flag);
  return flag < 0;
}

int main(int argc, char** argv)
{
  const sunindextype n = argc > 1 ? atol(argv[1]) : 64;
  const int imex       = argc > 2 ? atoi(argv[2]) : 0;
  const sunrealtype xmax = 1.0, A = 1.0, B = 3.5, c = 0.01, rtol = 1e-6, atol = 1e-9;
  const sunrealtype k[6] = {1.0, 1.0, 1.0, 1.0, 1.0 / 5.0e-6, 1.0 / 5.0e-6};
  SUNContext ctx;
  if (check(SUNContext_Create(SUN_COMM_NULL, &ctx), "SUNContext_Create")) return 1;

  /* steady state plus a Gaussian bump (advection_reaction_3D.cpp:566-637) */
  N_Vector y = N_VNew_GB300(3 * n * n * n, ctx);
  if (!y) return 1;
  sunrealtype* yh       = N_VGetHostArrayPointer_GB300(y);
  const sunrealtype mu = xmax / 2.0, sigma = xmax / 4.0, dx = xmax / n;
  const sunrealtype denom = 2.0 * sqrt(sigma * sigma * sigma * pow(2.0 * M_PI, 3.0));
  for (sunindextype i = 0; i < n; i++)
    for (sunindextype j = 0; j < n; j++)
      for (sunindextype l = 0; l < n; l++)
      {
        const sunrealtype x[3] = {i * dx, j * dx, l * dx};
        sunrealtype p          = 0.0;
        for (int a = 0; a < 3; a++) p += 0.1 * exp(-((x[a] - mu) * (x[a] - mu) / sigma) / denom);
        const sunindextype cell = (i * n + j) * n + l;
        yh[3 * cell]     = k[0] * A / k[3] + p;
        yh[3 * cell + 1] = k[1] * k[3] * B / (k[0] * k[2] * A) + p;
        yh[3 * cell + 2] = 3.0 + p;
      }
  N_VCopyToDevice_GB300(y);

  SUNBruss3D_GB300 prob = SUNBruss3D_GB300_Create(n, n, n, xmax, A, B, k, c);
  void* arkode_mem = imex ? ARKStepCreate(SUNBruss3D_GB300_Advection, SUNBruss3D_GB300_Reaction,
                                          0.0, y, ctx)
                          : ARKStepCreate(NULL, SUNBruss3D_GB300_RHS, 0.0, y, ctx);
  if (!arkode_mem) return 1;
  if (check(ARKodeSetOrder(arkode_mem, 3), "ARKodeSetOrder")) return 1;
  if (check(ARKodeSetUserData(arkode_mem, prob), "ARKodeSetUserData")) return 1;
  if (check(ARKodeSStolerances(arkode_mem, rtol, atol), "ARKodeSStolerances")) return 1;
  if (check(ARKodeSetMaxNumSteps(arkode_mem, 100000), "ARKodeSetMaxNumSteps")) return 1;
  SUNNonlinearSolver NLS = SUNNonlinSol_Newton(y, ctx);
  if (check(ARKodeSetNonlinearSolver(arkode_mem, NLS), "ARKodeSetNonlinearSolver")) return 1;
  SUNLinearSolver LS = SUNLinSol_SPGMR_GB300(y, SUN_PREC_LEFT, 0, ctx);
  if (check(ARKodeSetLinearSolver(arkode_mem, LS, NULL), "ARKodeSetLinearSolver")) return 1;
  if (check(ARKodeSetPreconditioner(arkode_mem, NULL, SUNBruss3D_GB300_CVPSolve),
            "ARKodeSetPreconditioner"))
    return 1;

  sunrealtype t = 0.0;
  for (int iout = 1; iout <= 10; iout++)
    if (check(ARKodeEvolve(arkode_mem, iout * 1.0, y, &t, ARK_NORMAL), "ARKodeEvolve")) return 1;
  N_VCopyFromDevice_GB300(y);
  printf("t = %g, u(0) = %.10e\n", t, N_VGetHostArrayPointer_GB300(y)[0]);
  ARKodePrintAllStats(arkode_mem, stdout, SUN_OUTPUTFORMAT_TABLE);

  ARKodeFree(&arkode_mem);
  SUNNonlinSolFree(NLS);
  SUNLinSolFree(LS);
  SUNBruss3D_GB300_Free(prob);
  N_VDestroy(y);
  SUNContext_Free(&ctx);
  return 0;
}
