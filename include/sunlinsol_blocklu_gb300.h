/* ---------------------------------------------------------------------------
 * sunlinsol_blocklu_gb300.h -- a block-diagonal SUNMatrix with ragged dense
 * blocks in GB300 HBM, and a direct SUNLinearSolver that factors and solves
 * all blocks in batched sm_103a kernels.
 *
 * Replaces (reference interface, file:line):
 *   SUNMatrix_MagmaDenseBlock / SUNLinSol_MagmaDense
 *     src/sunmatrix/magmadense/sunmatrix_magmadense.cpp:84,
 *     src/sunlinsol/magmadense/sunlinsol_magmadense.cpp:314-454 (uniform
 *     blocks, MAGMA getrf/getrs_batched);
 *   SUNLinSol_Dense per block: setup = SUNDlsMat_denseGETRF, solve =
 *     SUNDlsMat_denseGETRS (src/sunlinsol/dense/sunlinsol_dense.c:128-180,
 *     src/sundials/sundials_dense.c:85-193);
 *   SUNMatScaleAddI / Copy / Zero / Matvec of SUNMATRIX_DENSE
 *     (src/sunmatrix/dense/sunmatrix_dense.c:265-330).
 * Both objects plug into CVODE / ARKODE unchanged through
 * CVodeSetLinearSolver(cvode_mem, LS, A) (src/cvode/cvode_ls.c:56) or
 * ARKodeSetLinearSolver (src/arkode/arkode_ls.c:50): the solver is
 * SUNLINEARSOLVER_DIRECT and the matrix implements zero, copy, scaleadd,
 * scaleaddi and matvec (what cvLsLinSys, cvode_ls.c:1311-1400, calls).
 *
 * Layout: block b covers rows/columns off[b] .. off[b+1]-1 of the global
 * matrix and is stored column-major, contiguously, at data + boff[b] with
 * boff[b] = sum_{c<b} n_c^2 (n_b = off[b+1]-off[b], 1 <= n_b <= 64).
 *
 * Arithmetic:
 *   SUNBLOCKLU_FP64   the reference's GETRF/GETRS, operation for operation,
 *                     with no fused multiply-add: every block's factors and
 *                     solution are bit-identical to SUNLINSOL_DENSE's;
 *   SUNBLOCKLU_MIXED  FP32 inverse of each block (Gauss-Jordan with partial
 *                     pivoting), applied in FP32 and refined once in FP64
 *                     against the FP64 matrix, which setup leaves intact.
 *                     Setup probes each inverse X with two vectors v
 *                     (|v - X A v|_inf <= 1/4, i.e. the refinement contracts);
 *                     a block that fails the probe, or meets a zero pivot in
 *                     FP32, is factored by the FP64 path instead (a copy of
 *                     it, in storage allocated on first need) and solved
 *                     exactly as SUNBLOCKLU_FP64 solves it.
 * Setup returns SUNLS_LUFACT_FAIL (recoverable) if any block has a zero
 * pivot in FP64; SUNLinSolLastFlag then gives 1 + the global column of the
 * first one.
 * ------------------------------------------------------------------------- */
#ifndef SUNLINSOL_BLOCKLU_GB300_H
#define SUNLINSOL_BLOCKLU_GB300_H

#include "sundials_gb300_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SUNBLOCKLU_FP64  0
#define SUNBLOCKLU_MIXED 1

/* ---- matrix ------------------------------------------------------------- */

/* nblocks blocks; off (host, nblocks+1 entries, off[0] = 0) gives the block
 * boundaries.  Entries are zero-initialised on the device. */
SUNGB300_EXPORT SUNMatrix SUNMatrix_BlockDiag_GB300(sunindextype nblocks,
                                                   const sunindextype* off,
                                                   SUNContext sunctx);
SUNGB300_EXPORT sunindextype SUNMatrix_BlockDiag_GB300_NumBlocks(SUNMatrix A);
SUNGB300_EXPORT sunindextype SUNMatrix_BlockDiag_GB300_Rows(SUNMatrix A);
SUNGB300_EXPORT sunindextype SUNMatrix_BlockDiag_GB300_NNZ(SUNMatrix A);
/* Device pointer to all blocks (boff layout) and to block b. */
SUNGB300_EXPORT sunrealtype* SUNMatrix_BlockDiag_GB300_Data(SUNMatrix A);
SUNGB300_EXPORT sunrealtype* SUNMatrix_BlockDiag_GB300_BlockData(SUNMatrix A,
                                                                 sunindextype b);
/* Copy all entries from / to a host array in the boff layout. */
SUNGB300_EXPORT SUNErrCode SUNMatrix_BlockDiag_GB300_CopyToDevice(SUNMatrix A,
                                                                  const sunrealtype* h);
SUNGB300_EXPORT SUNErrCode SUNMatrix_BlockDiag_GB300_CopyFromDevice(SUNMatrix A,
                                                                    sunrealtype* h);

SUNGB300_EXPORT SUNMatrix_ID SUNMatGetID_BlockDiag_GB300(SUNMatrix A);
SUNGB300_EXPORT SUNMatrix SUNMatClone_BlockDiag_GB300(SUNMatrix A);
SUNGB300_EXPORT void SUNMatDestroy_BlockDiag_GB300(SUNMatrix A);
SUNGB300_EXPORT SUNErrCode SUNMatZero_BlockDiag_GB300(SUNMatrix A);
SUNGB300_EXPORT SUNErrCode SUNMatCopy_BlockDiag_GB300(SUNMatrix A, SUNMatrix B);
SUNGB300_EXPORT SUNErrCode SUNMatScaleAdd_BlockDiag_GB300(sunrealtype c, SUNMatrix A,
                                                          SUNMatrix B);
SUNGB300_EXPORT SUNErrCode SUNMatScaleAddI_BlockDiag_GB300(sunrealtype c, SUNMatrix A);
SUNGB300_EXPORT SUNErrCode SUNMatMatvec_BlockDiag_GB300(SUNMatrix A, N_Vector x,
                                                        N_Vector y);

/* ---- linear solver -------------------------------------------------------- */

SUNGB300_EXPORT SUNLinearSolver SUNLinSol_BlockLU_GB300(N_Vector y, SUNMatrix A,
                                                       int precision,
                                                       SUNContext sunctx);
SUNGB300_EXPORT SUNLinearSolver_Type SUNLinSolGetType_BlockLU_GB300(SUNLinearSolver S);
SUNGB300_EXPORT SUNLinearSolver_ID SUNLinSolGetID_BlockLU_GB300(SUNLinearSolver S);
SUNGB300_EXPORT SUNErrCode SUNLinSolInitialize_BlockLU_GB300(SUNLinearSolver S);
SUNGB300_EXPORT int SUNLinSolSetup_BlockLU_GB300(SUNLinearSolver S, SUNMatrix A);
SUNGB300_EXPORT int SUNLinSolSolve_BlockLU_GB300(SUNLinearSolver S, SUNMatrix A,
                                                 N_Vector x, N_Vector b,
                                                 sunrealtype tol);
SUNGB300_EXPORT sunindextype SUNLinSolLastFlag_BlockLU_GB300(SUNLinearSolver S);
SUNGB300_EXPORT SUNErrCode SUNLinSolFree_BlockLU_GB300(SUNLinearSolver S);

#ifdef __cplusplus
}
#endif

#endif /* SUNLINSOL_BLOCKLU_GB300_H */
