/* ---------------------------------------------------------------------------
 * cvode_fused_gb300.h -- CVODE's integrator-specific fused kernels over
 * NVECTOR_GB300 vectors, with the reference's own symbol names, so a CVODE
 * built with SUNDIALS_BUILD_PACKAGE_FUSED_KERNELS and
 * CVodeSetUseIntegratorFusedKernels(cvode_mem, SUNTRUE) (src/cvode/cvode_io.c)
 * runs them on GB300 by linking this library in place of the reference's
 * sundials_cvode_fused_cuda (src/cvode/CMakeLists.txt).
 *
 * Replaces (reference, file:line):
 *   declarations          src/cvode/cvode_impl.h:639-665
 *   CUDA implementations  src/cvode/cvode_fused_gpu.cpp:62-413
 *   serial semantics      src/cvode/cvode_fused_stubs.c:30-160
 * Each call is one sm_103a kernel over the vectors (cvEwtSet*_fused with
 * atolmin0 also reduces min(tempv) in the same pass and synchronises once).
 * Arithmetic follows the output vector's mode: in N_VSetFMA_GB300(v, SUNFALSE)
 * mode every element is the bit-for-bit result of the stub's N_Vector
 * sequence on NVECTOR_SERIAL; in the default FMA mode products are contracted
 * into the adds as an nvcc build of the CUDA kernels does.  The comparison in
 * cvDiagSetup_buildM is the stub's |y_i| >= uround (N_VCompare).
 * All vectors must be NVECTOR_GB300 of one length; a mismatch returns -1.
 * ------------------------------------------------------------------------- */
#ifndef CVODE_FUSED_GB300_H
#define CVODE_FUSED_GB300_H

#include "sundials_gb300_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

SUNGB300_EXPORT int cvEwtSetSS_fused(const sunbooleantype atolmin0, const sunrealtype reltol,
                                     const sunrealtype Sabstol, const N_Vector ycur,
                                     N_Vector tempv, N_Vector weight);
SUNGB300_EXPORT int cvEwtSetSV_fused(const sunbooleantype atolmin0, const sunrealtype reltol,
                                     const N_Vector Vabstol, const N_Vector ycur,
                                     N_Vector tempv, N_Vector weight);
SUNGB300_EXPORT int cvCheckConstraints_fused(const N_Vector c, const N_Vector ewt,
                                             const N_Vector y, const N_Vector mm,
                                             N_Vector tempv);
SUNGB300_EXPORT int cvNlsResid_fused(const sunrealtype rl1, const sunrealtype ngamma,
                                     const N_Vector zn1, const N_Vector ycor,
                                     const N_Vector ftemp, N_Vector res);
SUNGB300_EXPORT int cvDiagSetup_formY(const sunrealtype h, const sunrealtype r,
                                      const N_Vector fpred, const N_Vector zn1,
                                      const N_Vector ypred, N_Vector ftemp, N_Vector y);
SUNGB300_EXPORT int cvDiagSetup_buildM(const sunrealtype fract, const sunrealtype uround,
                                       const sunrealtype h, const N_Vector ftemp,
                                       const N_Vector fpred, const N_Vector ewt, N_Vector bit,
                                       N_Vector bitcomp, N_Vector y, N_Vector M);
SUNGB300_EXPORT int cvDiagSolve_updateM(const sunrealtype r, N_Vector M);

#ifdef __cplusplus
}
#endif

#endif /* CVODE_FUSED_GB300_H */
