/* ---------------------------------------------------------------------------
 * robertson_gb300.h -- device user functions for a batch of independent
 * Robertson chemical-kinetics cells (3 species each, y1 y2 y3 of cell c at
 * 3c, 3c+1, 3c+2 of one NVECTOR_GB300 vector), with per-cell rate constants:
 *   y1' = -k1 y1 + k3 y2 y3,   y3' = k2 y2^2,   y2' = -y1' - y3'.
 * These are the callbacks a CVODE or ARKODE (ARKStep, implicit right-hand
 * side) + SPGMR run of the batch needs (the two packages' callback types
 * have the same signatures): right-hand side, Jacobian-times-vector, and
 * the exact block-Jacobi
 * preconditioner P = I - gamma J_c per cell, factored and applied by
 * SUNLinSol_BlockLU_GB300 on a SUNMatrix_BlockDiag_GB300 of 3x3 blocks.
 *
 * Restates (reference, file:line):
 *   f and the Jacobian blocks   examples/cvode/cuda/cvRoberts_block_cusolversp_batchqr.cu:316-333, 409-440
 *                               (rate constants per cell instead of 0.04, 3e7, 1e4)
 *   preconditioner setup/solve  examples/cvode/serial/cvDiurnal_kry.c:714-845
 *                               (jok: reuse the saved Jacobian blocks, else
 *                               recompute them and set *jcurPtr; P = -gamma J,
 *                               P += I, denseGETRF per block; solve = GETRS)
 * Rounding: f as the reference kernel ((-k1) y1 + (k3 y2) y3, (k2 y2) y2);
 * J v row by row left to right with the Jacobian entries of the reference
 * kernel (row 2, column 2: (-k3 y3) - (2 k2) y2); every operation rounded
 * separately (no contraction).
 * ------------------------------------------------------------------------- */
#ifndef ROBERTSON_GB300_H
#define ROBERTSON_GB300_H

#include "sundials_gb300_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct SUNRoberts_GB300_* SUNRoberts_GB300;

/* ncells cells; k (host, 3*ncells): k1, k2, k3 of each cell; tmpl: an
 * NVECTOR_GB300 of length 3*ncells (the preconditioner's solver is built on
 * it); lu_precision: SUNBLOCKLU_FP64 or SUNBLOCKLU_MIXED. */
SUNGB300_EXPORT SUNRoberts_GB300 SUNRoberts_GB300_Create(sunindextype ncells,
                                                         const sunrealtype* k, N_Vector tmpl,
                                                         int lu_precision, SUNContext sunctx);
SUNGB300_EXPORT void SUNRoberts_GB300_Free(SUNRoberts_GB300 p);

/* CVRhsFn / ARKRhsFn */
SUNGB300_EXPORT int SUNRoberts_GB300_RHS(sunrealtype t, N_Vector y, N_Vector ydot, void* p);
/* CVLsJacTimesVecFn / ARKLsJacTimesVecFn: Jv = J(y) v */
SUNGB300_EXPORT int SUNRoberts_GB300_JTimes(N_Vector v, N_Vector Jv, sunrealtype t, N_Vector y,
                                            N_Vector fy, void* p, N_Vector tmp);
/* CVLsJacFn / ARKLsJacFn: J(y) into a SUNMatrix_BlockDiag_GB300 of ncells
 * 3x3 blocks, for CVodeSetLinearSolver(cvode_mem, SUNLinSol_BlockLU_GB300(y,
 * J, ...), J) + CVodeSetJacFn (or the ARKode* equivalents) -- the reference
 * example's direct block solve
 * (cvRoberts_block_cusolversp_batchqr.cu:196-223, there on cuSolverSp). */
SUNGB300_EXPORT int SUNRoberts_GB300_Jac(sunrealtype t, N_Vector y, N_Vector fy, SUNMatrix J,
                                         void* p, N_Vector tmp1, N_Vector tmp2, N_Vector tmp3);
/* CVLsPrecSetupFn / CVLsPrecSolveFn (ARKLsPrecSetupFn / ARKLsPrecSolveFn):
 * exact block-Jacobi preconditioner.
 * Setup returns 1 (recoverable) if a block is singular. */
SUNGB300_EXPORT int SUNRoberts_GB300_CVPSetup(sunrealtype t, N_Vector y, N_Vector fy,
                                              sunbooleantype jok, sunbooleantype* jcurPtr,
                                              sunrealtype gamma, void* p);
SUNGB300_EXPORT int SUNRoberts_GB300_CVPSolve(sunrealtype t, N_Vector y, N_Vector fy,
                                              N_Vector r, N_Vector z, sunrealtype gamma,
                                              sunrealtype delta, int lr, void* p);

#ifdef __cplusplus
}
#endif

#endif /* ROBERTSON_GB300_H */
