/* ---------------------------------------------------------------------------
 * heat2d_gb300.h -- device user functions for the 2D heat equation
 * u_t = kx u_xx + ky u_yy on the unit square with zero Dirichlet boundaries,
 * discretised by the 5-point stencil on an nx x ny interior grid
 * (dx = 1/(nx+1), dy = 1/(ny+1)), over NVECTOR_GB300 vectors laid out row by
 * row (x fastest).  These are the user-side callbacks a CVODE + SPGMR run of
 * this problem needs -- right-hand side, Jacobian-times-vector, Jacobi
 * preconditioner -- as sm_103a kernels, with the integrators' own callback
 * signatures, plus the SUNATimesFn / SUNPSolveFn forms that drive an SPGMR
 * solve of (I - gamma J) x = b directly.
 *
 * Restates (reference, file:line):
 *   f (stencil part; the reference adds a manufactured forcing term)
 *                            examples/cvode/CXX_serial/cv_heat2D.cpp:305-367
 *   PSetup / PSolve (Jacobi, d = 1/(1 - gamma cc))
 *                            examples/cvode/CXX_serial/cv_heat2D.cpp:371-408
 *   Jv of the same stencil   benchmarks/diffusion_2D/diffusion_2D.cpp
 *   cvLsATimes z = v - gamma J v   src/cvode/cvode_ls.c:895-918
 * Stencil sums are rounded in the reference's order:
 *   (cc u_c + cx (u_w + u_e)) + cy (u_s + u_n),
 * and z = v + (-gamma) Jv, each operation rounded separately.
 * ------------------------------------------------------------------------- */
#ifndef HEAT2D_GB300_H
#define HEAT2D_GB300_H

#include "sundials_gb300_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct SUNHeat2D_GB300_* SUNHeat2D_GB300;

SUNGB300_EXPORT SUNHeat2D_GB300 SUNHeat2D_GB300_Create(sunindextype nx, sunindextype ny,
                                                       sunrealtype kx, sunrealtype ky);
SUNGB300_EXPORT void SUNHeat2D_GB300_Free(SUNHeat2D_GB300 p);
/* gamma of the Newton matrix I - gamma J used by ATimes / PSetup / PSolve. */
SUNGB300_EXPORT SUNErrCode SUNHeat2D_GB300_SetGamma(SUNHeat2D_GB300 p, sunrealtype gamma);

/* CVRhsFn: f = J u (the problem is linear and autonomous). */
SUNGB300_EXPORT int SUNHeat2D_GB300_RHS(sunrealtype t, N_Vector u, N_Vector f, void* p);
/* CVLsJacTimesVecFn: Jv = J v. */
SUNGB300_EXPORT int SUNHeat2D_GB300_JTimes(N_Vector v, N_Vector Jv, sunrealtype t, N_Vector y,
                                           N_Vector fy, void* p, N_Vector tmp);
/* CVLsPrecSetupFn / CVLsPrecSolveFn: Jacobi preconditioner of I - gamma J. */
SUNGB300_EXPORT int SUNHeat2D_GB300_CVPSetup(sunrealtype t, N_Vector y, N_Vector fy,
                                             sunbooleantype jok, sunbooleantype* jcurPtr,
                                             sunrealtype gamma, void* p);
SUNGB300_EXPORT int SUNHeat2D_GB300_CVPSolve(sunrealtype t, N_Vector y, N_Vector fy, N_Vector r,
                                             N_Vector z, sunrealtype gamma, sunrealtype delta,
                                             int lr, void* p);
/* SUNATimesFn: z = v - gamma J v in one pass.  SUNPSetupFn / SUNPSolveFn:
 * z = d r with d = 1 / (1 - gamma cc), cc = -2 (kx/dx^2 + ky/dy^2). */
SUNGB300_EXPORT int SUNHeat2D_GB300_ATimes(void* p, N_Vector v, N_Vector z);
SUNGB300_EXPORT int SUNHeat2D_GB300_PSetup(void* p);
SUNGB300_EXPORT int SUNHeat2D_GB300_PSolve(void* p, N_Vector r, N_Vector z, sunrealtype tol,
                                           int lr);

#ifdef __cplusplus
}
#endif

#endif /* HEAT2D_GB300_H */
