/* ---------------------------------------------------------------------------
 * bruss3d_gb300.h -- device user functions of the 3-D advection-reaction
 * benchmark (Brusselator chemistry, upwind advection on a periodic grid) over
 * one NVECTOR_GB300 vector: the fields u, v, w of cell (i, j, k) at
 * ((i*ny + j)*nz + k)*3 + {0, 1, 2} (x slowest, the 3 species fastest), the
 * grid [0, xmax)^3 with dx = xmax/nx, dy = xmax/ny, dz = xmax/nz.
 *
 *   u_t = -c grad.u + k1 A - k2 w u + k3 u^2 v - k4 u
 *   v_t = -c grad.v + k2 w u - k3 u^2 v
 *   w_t = -c grad.w - k2 w u + k5 B - k6 w
 *
 * Restates (reference, file:line):
 *   Advection (first-order upwind in the direction of c; one process, so
 *     the periodic neighbours of the faces are the grid's own opposite
 *     faces)          benchmarks/advection_reaction_3D/raja/rhs3D.hpp:30-320
 *   Reaction          rhs3D.hpp:322-383 (added to the advection, or alone)
 *   AdvectionReaction rhs3D.hpp:386-406 (the CVODE right-hand side)
 *   SolveReactionLinSys: the 3x3 system (I - gamma dg/dy) x = b of every
 *     cell, in closed form  rhs3D.hpp:441-552; PSolve rhs3D.hpp:672-686
 * Rounding follows those sources operation for operation with no
 * contraction: interior cells sum the upwind differences in the order z, y,
 * x, cells on an upwind face (i, j or k = 0 for c > 0; = n-1 for c < 0) in
 * the order x, y, z, as the reference's interior and face kernels do.
 * ------------------------------------------------------------------------- */
#ifndef BRUSS3D_GB300_H
#define BRUSS3D_GB300_H

#include "sundials_gb300_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct SUNBruss3D_GB300_* SUNBruss3D_GB300;

/* k: k1..k6 (6 values); the benchmark's defaults are xmax = 1, A = 1,
 * B = 3.5, k1 = k2 = k3 = k4 = 1, k5 = k6 = 1/5e-6, c = 0.01. */
SUNGB300_EXPORT SUNBruss3D_GB300 SUNBruss3D_GB300_Create(sunindextype nx, sunindextype ny,
                                                         sunindextype nz, sunrealtype xmax,
                                                         sunrealtype A, sunrealtype B,
                                                         const sunrealtype* k, sunrealtype c);
SUNGB300_EXPORT void SUNBruss3D_GB300_Free(SUNBruss3D_GB300 p);

/* ARKRhsFn / CVRhsFn forms: the explicit (advection), implicit (reaction)
 * and full (advection + reaction) right-hand sides. */
SUNGB300_EXPORT int SUNBruss3D_GB300_Advection(sunrealtype t, N_Vector y, N_Vector ydot, void* p);
SUNGB300_EXPORT int SUNBruss3D_GB300_Reaction(sunrealtype t, N_Vector y, N_Vector ydot, void* p);
SUNGB300_EXPORT int SUNBruss3D_GB300_RHS(sunrealtype t, N_Vector y, N_Vector ydot, void* p);
/* x = (I - gamma dg/dy)^{-1} b per cell, at the state y; x may be b (the
 * in-place linear solve of the benchmark's task-local Newton,
 * arkode_driver.cpp:580-596). */
SUNGB300_EXPORT int SUNBruss3D_GB300_SolveReaction(N_Vector y, N_Vector x, N_Vector b,
                                                   sunrealtype gamma, void* p);
/* CVLsPrecSolveFn / ARKLsPrecSolveFn (same signature): z = (I - gamma
 * dg/dy)^{-1} r, the benchmark's PSolve for its CVODE and ARK-DIRK drivers
 * (cvode_driver.cpp:96-102, arkode_driver.cpp:117-130). */
SUNGB300_EXPORT int SUNBruss3D_GB300_CVPSolve(sunrealtype t, N_Vector y, N_Vector fy,
                                              N_Vector r, N_Vector z, sunrealtype gamma,
                                              sunrealtype delta, int lr, void* p);

#ifdef __cplusplus
}
#endif

#endif /* BRUSS3D_GB300_H */
