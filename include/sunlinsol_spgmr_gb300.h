/* ---------------------------------------------------------------------------
 * sunlinsol_spgmr_gb300.h -- restarted GMRES (SPGMR) over NVECTOR_GB300 whose
 * Gram-Schmidt orthogonalisation runs as fused sm_103a kernels.
 *
 * Replaces (reference interface, file:line):
 *   SUNLinSol_SPGMR and its operations       src/sunlinsol/spgmr/sunlinsol_spgmr.c:70-990
 *     (constructor :70, SetPrecType :253, SetGSType :270, SetMaxRestarts :286,
 *      Initialize :312, SetATimes :395, SetPreconditioner :405,
 *      SetScalingVectors :417, SetZeroGuess :427, Setup :434, Solve :461-932,
 *      NumIters/ResNorm/Resid/LastFlag/Space/Free :934-990)
 *   SUNModifiedGS / SUNClassicalGS           src/sundials/sundials_iterative.c:45-170
 *   SUNQRfact / SUNQRsol (restated, host)    src/sundials/sundials_iterative.c:181-329
 * Plugged in unchanged through CVodeSetLinearSolver(cvode_mem, LS, NULL)
 * (src/cvode/cvode_ls.c:56) or ARKodeSetLinearSolver (src/arkode/arkode_ls.c:50):
 * the solver is SUNLINEARSOLVER_ITERATIVE with ID SUNLINEARSOLVER_SPGMR, and
 * ATimes / Psetup / Psolve are the integrator's host callbacks operating on
 * N_Vectors (src/sundials/sundials_iterative.h:100-140).
 *
 * The algorithm, its options, defaults (maxl 5, no restarts, modified
 * Gram-Schmidt), return codes and counters are the reference's.  What differs
 * is how the Arnoldi step reaches the GPU:
 *   classical GS   two kernels per pass over the basis -- all dot products of
 *                  the new vector (and its norm) in one read of V, then the
 *                  update fused with the new norm -- and the Hessenberg column
 *                  lands in pinned host memory;
 *   modified GS    one kernel per basis vector, each applying the previous
 *                  projection and computing the next dot product, with the
 *                  coefficients passed on in device memory (no host round
 *                  trip between them);
 *   both           one stream synchronisation per Arnoldi step (a second only
 *                  when the reorthogonalisation test fires); the 1/h
 *                  normalisation of the new basis vector is fused into the next
 *                  step's first pass over it; copies between the basis and the
 *                  work vector are replaced by exchanging vector handles.
 * All dot products are the library's deterministic fixed-order reductions,
 * so the solve is bitwise reproducible run to run; relative to the reference
 * on NVECTOR_SERIAL they differ only in the summation order (and in fused
 * multiply-adds, unless the vectors are in N_VSetFMA_GB300(v, SUNFALSE) mode).
 *
 * Requirements: y, the scaling vectors and every vector handed to Solve are
 * NVECTOR_GB300 vectors of the same length on the same stream; ATimes and
 * Psolve must order their work on that stream (the legacy default stream for
 * vectors made by N_VNew_GB300).  The solver's work vector (returned by
 * SUNLinSolResid) and basis vectors are scratch between calls: a Solve may
 * exchange their handles.
 * ------------------------------------------------------------------------- */
#ifndef SUNLINSOL_SPGMR_GB300_H
#define SUNLINSOL_SPGMR_GB300_H

#include "sundials_gb300_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SUNSPGMR_GB300_MAXL_DEFAULT  5
#define SUNSPGMR_GB300_MAXRS_DEFAULT 0

SUNGB300_EXPORT SUNLinearSolver SUNLinSol_SPGMR_GB300(N_Vector y, int pretype, int maxl,
                                                     SUNContext sunctx);
SUNGB300_EXPORT SUNErrCode SUNLinSol_SPGMR_GB300SetPrecType(SUNLinearSolver S, int pretype);
SUNGB300_EXPORT SUNErrCode SUNLinSol_SPGMR_GB300SetGSType(SUNLinearSolver S, int gstype);
SUNGB300_EXPORT SUNErrCode SUNLinSol_SPGMR_GB300SetMaxRestarts(SUNLinearSolver S, int maxrs);
/* SUNTRUE (default): the fused Gram-Schmidt kernels above.  SUNFALSE: the
 * reference's sequence of separate N_Vector operations (N_VDotProdMulti,
 * N_VLinearCombination, N_VDotProd, N_VScale and copies; one synchronisation
 * per reduction), kept for A/B measurement.  No counterpart in the reference. */
SUNGB300_EXPORT SUNErrCode SUNLinSol_SPGMR_GB300SetFusedGS(SUNLinearSolver S,
                                                           sunbooleantype onoff);
/* Number of stream synchronisations made by the last Solve.  No counterpart
 * in the reference. */
SUNGB300_EXPORT long int SUNLinSol_SPGMR_GB300NumSyncs(SUNLinearSolver S);

SUNGB300_EXPORT SUNLinearSolver_Type SUNLinSolGetType_SPGMR_GB300(SUNLinearSolver S);
SUNGB300_EXPORT SUNLinearSolver_ID SUNLinSolGetID_SPGMR_GB300(SUNLinearSolver S);
SUNGB300_EXPORT SUNErrCode SUNLinSolInitialize_SPGMR_GB300(SUNLinearSolver S);
SUNGB300_EXPORT SUNErrCode SUNLinSolSetATimes_SPGMR_GB300(SUNLinearSolver S, void* ATdata,
                                                          SUNATimesFn ATimes);
SUNGB300_EXPORT SUNErrCode SUNLinSolSetPreconditioner_SPGMR_GB300(SUNLinearSolver S,
                                                                  void* Pdata,
                                                                  SUNPSetupFn Pset,
                                                                  SUNPSolveFn Psol);
SUNGB300_EXPORT SUNErrCode SUNLinSolSetScalingVectors_SPGMR_GB300(SUNLinearSolver S,
                                                                  N_Vector s1, N_Vector s2);
SUNGB300_EXPORT SUNErrCode SUNLinSolSetZeroGuess_SPGMR_GB300(SUNLinearSolver S,
                                                             sunbooleantype onoff);
SUNGB300_EXPORT int SUNLinSolSetup_SPGMR_GB300(SUNLinearSolver S, SUNMatrix A);
SUNGB300_EXPORT int SUNLinSolSolve_SPGMR_GB300(SUNLinearSolver S, SUNMatrix A, N_Vector x,
                                               N_Vector b, sunrealtype tol);
SUNGB300_EXPORT int SUNLinSolNumIters_SPGMR_GB300(SUNLinearSolver S);
SUNGB300_EXPORT sunrealtype SUNLinSolResNorm_SPGMR_GB300(SUNLinearSolver S);
SUNGB300_EXPORT N_Vector SUNLinSolResid_SPGMR_GB300(SUNLinearSolver S);
SUNGB300_EXPORT sunindextype SUNLinSolLastFlag_SPGMR_GB300(SUNLinearSolver S);
SUNGB300_EXPORT SUNErrCode SUNLinSolSpace_SPGMR_GB300(SUNLinearSolver S, long int* lenrwLS,
                                                      long int* leniwLS);
SUNGB300_EXPORT SUNErrCode SUNLinSolFree_SPGMR_GB300(SUNLinearSolver S);

#ifdef __cplusplus
}
#endif

#endif /* SUNLINSOL_SPGMR_GB300_H */
