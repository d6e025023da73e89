/* ---------------------------------------------------------------------------
 * nvector_gb300.h -- NVECTOR_GB300: an N_Vector whose data live in GB300 HBM
 * and whose every operation is a hand-written sm_103a kernel.
 *
 * It is a drop-in for the reference's NVECTOR_CUDA / NVECTOR_SERIAL
 * constructors: the vector is a standard SUNDIALS N_Vector (ID
 * SUNDIALS_NVEC_CUSTOM) whose ops table is filled completely, so CVODE, ARKODE,
 * SPGMR and the Newton solver call it through the generic N_V* dispatch
 * (sundials_nvector.c:383-835) without any change.
 *
 * Replaces (reference interface, file:line):
 *   N_VNew_Cuda / N_VNewManaged_Cuda / N_VMake_Cuda   nvector_cuda.cu:131-330
 *   N_VNew_Serial / N_VMake_Serial                    nvector_serial.c:80-215
 *   N_VCopyToDevice_Cuda / N_VCopyFromDevice_Cuda     nvector_cuda.cu:553-597
 *   N_VEnableFusedOps_Cuda and the per-op Enable*     nvector_cuda.cu:2089-2260
 *   every N_V*_Cuda / N_V*_Serial operation           nvector_serial.c:387-1600
 *
 * Semantics that differ from NVECTOR_CUDA on purpose:
 *   - fused and vector-array operations are ENABLED by default;
 *   - reductions are bitwise deterministic (fixed-order trees, no float
 *     atomics), so a rerun reproduces every CVODE counter;
 *   - coefficient / pointer arrays of fused ops travel as kernel parameters
 *     (no host-to-device staging copy and no extra stream synchronisation);
 *   - arithmetic: by default a*x+y terms are fused multiply-adds, as in the
 *     reference's NVECTOR_CUDA kernels compiled by nvcc (at most one rounding
 *     per term away from NVECTOR_SERIAL); N_VSetFMA_GB300(v, SUNFALSE)
 *     selects separately rounded products and sums in NVECTOR_SERIAL's order,
 *     which makes every streaming and fused op bit-identical to the serial
 *     vector (and costs up to 1.8x more FP64 instructions on GB300).
 *
 * Memory: the device array is cudaMalloc'd; a pinned host mirror is created
 * on first use of N_VGetArrayPointer / N_VCopyFromDevice.  Host <-> device
 * copies are explicit, as with NVECTOR_CUDA.  All work of a vector and its
 * clones is ordered on one CUDA stream; a reduction synchronises that stream
 * only.
 * ------------------------------------------------------------------------- */
#ifndef NVECTOR_GB300_H
#define NVECTOR_GB300_H

#include "sundials_gb300_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- constructors --------------------------------------------------------*/

/* New vector of length `length`; device data allocated, host mirror lazy. */
SUNGB300_EXPORT N_Vector N_VNew_GB300(sunindextype length, SUNContext sunctx);

/* Same, with all work ordered on the given cudaStream_t (passed as void*). */
SUNGB300_EXPORT N_Vector N_VNewWithStream_GB300(sunindextype length,
                                                void* cuda_stream,
                                                SUNContext sunctx);

/* Vector object with ops and no data (nvector_serial.c:80 N_VNewEmpty_Serial). */
SUNGB300_EXPORT N_Vector N_VNewEmpty_GB300(SUNContext sunctx);

/* Wrap caller-owned arrays (either may be NULL); nvector_cuda.cu:283 N_VMake_Cuda. */
SUNGB300_EXPORT N_Vector N_VMake_GB300(sunindextype length, sunrealtype* h_vdata,
                                       sunrealtype* d_vdata, SUNContext sunctx);

/* ---- data movement and accessors ----------------------------------------*/

SUNGB300_EXPORT void N_VCopyToDevice_GB300(N_Vector v);
SUNGB300_EXPORT void N_VCopyFromDevice_GB300(N_Vector v);
SUNGB300_EXPORT sunrealtype* N_VGetHostArrayPointer_GB300(N_Vector v);
SUNGB300_EXPORT sunrealtype* N_VGetDeviceArrayPointer_GB300(N_Vector v);
SUNGB300_EXPORT void N_VSetDeviceArrayPointer_GB300(sunrealtype* d_vdata,
                                                    N_Vector v);
SUNGB300_EXPORT void* N_VGetStream_GB300(N_Vector v);
SUNGB300_EXPORT sunbooleantype N_VIsManagedMemory_GB300(N_Vector v);

/* ---- configuration --------------------------------------------------------*/

SUNGB300_EXPORT SUNErrCode N_VEnableFusedOps_GB300(N_Vector v, sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableLinearCombination_GB300(N_Vector v,
                                                            sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableScaleAddMulti_GB300(N_Vector v,
                                                        sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableDotProdMulti_GB300(N_Vector v,
                                                       sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableLinearSumVectorArray_GB300(N_Vector v,
                                                               sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableScaleVectorArray_GB300(N_Vector v,
                                                           sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableConstVectorArray_GB300(N_Vector v,
                                                           sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableWrmsNormVectorArray_GB300(N_Vector v,
                                                              sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableWrmsNormMaskVectorArray_GB300(N_Vector v,
                                                                  sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableScaleAddMultiVectorArray_GB300(N_Vector v,
                                                                   sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableLinearCombinationVectorArray_GB300(
  N_Vector v, sunbooleantype tf);
SUNGB300_EXPORT SUNErrCode N_VEnableDotProdMultiLocal_GB300(N_Vector v,
                                                            sunbooleantype tf);

/* SUNTRUE (default): fused multiply-add.  SUNFALSE: separately rounded
 * products and sums in NVECTOR_SERIAL's order.  Inherited by clones; an
 * operation uses the mode of its output vector (of x for reductions). */
SUNGB300_EXPORT SUNErrCode N_VSetFMA_GB300(N_Vector v, sunbooleantype use_fma);
/* The mode set above (SUNTRUE for a vector that is not an NVECTOR_GB300). */
SUNGB300_EXPORT sunbooleantype N_VGetFMA_GB300(N_Vector v);

/* Last CUDA / argument error seen by this library on the calling thread
 * (0 = none); reading it clears it.  Errors are also reported to the
 * SUNContext when the library is linked with libsundials_core. */
SUNGB300_EXPORT int SUNGB300_GetLastError(void);
SUNGB300_EXPORT const char* SUNGB300_GetLastErrorMessage(void);

/* Number of kernels this library has launched in this process. */
SUNGB300_EXPORT long long SUNGB300_KernelLaunchCount(void);

/* ---- operations (the ops table entries; same meaning as N_V*_Serial) ----*/

SUNGB300_EXPORT N_Vector_ID N_VGetVectorID_GB300(N_Vector v);
SUNGB300_EXPORT N_Vector N_VCloneEmpty_GB300(N_Vector w);
SUNGB300_EXPORT N_Vector N_VClone_GB300(N_Vector w);
SUNGB300_EXPORT void N_VDestroy_GB300(N_Vector v);
SUNGB300_EXPORT void N_VSpace_GB300(N_Vector v, sunindextype* lrw,
                                    sunindextype* liw);
SUNGB300_EXPORT sunrealtype* N_VGetArrayPointer_GB300(N_Vector v);
SUNGB300_EXPORT void N_VSetArrayPointer_GB300(sunrealtype* v_data, N_Vector v);
SUNGB300_EXPORT SUNComm N_VGetCommunicator_GB300(N_Vector v);
SUNGB300_EXPORT sunindextype N_VGetLength_GB300(N_Vector v);

SUNGB300_EXPORT void N_VLinearSum_GB300(sunrealtype a, N_Vector x, sunrealtype b,
                                        N_Vector y, N_Vector z);
SUNGB300_EXPORT void N_VConst_GB300(sunrealtype c, N_Vector z);
SUNGB300_EXPORT void N_VProd_GB300(N_Vector x, N_Vector y, N_Vector z);
SUNGB300_EXPORT void N_VDiv_GB300(N_Vector x, N_Vector y, N_Vector z);
SUNGB300_EXPORT void N_VScale_GB300(sunrealtype c, N_Vector x, N_Vector z);
SUNGB300_EXPORT void N_VAbs_GB300(N_Vector x, N_Vector z);
SUNGB300_EXPORT void N_VInv_GB300(N_Vector x, N_Vector z);
SUNGB300_EXPORT void N_VAddConst_GB300(N_Vector x, sunrealtype b, N_Vector z);
SUNGB300_EXPORT sunrealtype N_VDotProd_GB300(N_Vector x, N_Vector y);
SUNGB300_EXPORT sunrealtype N_VMaxNorm_GB300(N_Vector x);
SUNGB300_EXPORT sunrealtype N_VWrmsNorm_GB300(N_Vector x, N_Vector w);
SUNGB300_EXPORT sunrealtype N_VWrmsNormMask_GB300(N_Vector x, N_Vector w,
                                                  N_Vector id);
SUNGB300_EXPORT sunrealtype N_VMin_GB300(N_Vector x);
SUNGB300_EXPORT sunrealtype N_VWL2Norm_GB300(N_Vector x, N_Vector w);
SUNGB300_EXPORT sunrealtype N_VL1Norm_GB300(N_Vector x);
SUNGB300_EXPORT void N_VCompare_GB300(sunrealtype c, N_Vector x, N_Vector z);
SUNGB300_EXPORT sunbooleantype N_VInvTest_GB300(N_Vector x, N_Vector z);
SUNGB300_EXPORT sunbooleantype N_VConstrMask_GB300(N_Vector c, N_Vector x,
                                                   N_Vector m);
SUNGB300_EXPORT sunrealtype N_VMinQuotient_GB300(N_Vector num, N_Vector denom);

SUNGB300_EXPORT SUNErrCode N_VLinearCombination_GB300(int nvec, sunrealtype* c,
                                                      N_Vector* X, N_Vector z);
SUNGB300_EXPORT SUNErrCode N_VScaleAddMulti_GB300(int nvec, sunrealtype* a,
                                                  N_Vector x, N_Vector* Y,
                                                  N_Vector* Z);
SUNGB300_EXPORT SUNErrCode N_VDotProdMulti_GB300(int nvec, N_Vector x,
                                                 N_Vector* Y,
                                                 sunrealtype* dotprods);

SUNGB300_EXPORT SUNErrCode N_VLinearSumVectorArray_GB300(int nvec, sunrealtype a,
                                                         N_Vector* X,
                                                         sunrealtype b,
                                                         N_Vector* Y,
                                                         N_Vector* Z);
SUNGB300_EXPORT SUNErrCode N_VScaleVectorArray_GB300(int nvec, sunrealtype* c,
                                                     N_Vector* X, N_Vector* Z);
SUNGB300_EXPORT SUNErrCode N_VConstVectorArray_GB300(int nvec, sunrealtype c,
                                                     N_Vector* Z);
SUNGB300_EXPORT SUNErrCode N_VWrmsNormVectorArray_GB300(int nvec, N_Vector* X,
                                                        N_Vector* W,
                                                        sunrealtype* nrm);
SUNGB300_EXPORT SUNErrCode N_VWrmsNormMaskVectorArray_GB300(int nvec,
                                                            N_Vector* X,
                                                            N_Vector* W,
                                                            N_Vector id,
                                                            sunrealtype* nrm);
SUNGB300_EXPORT SUNErrCode N_VScaleAddMultiVectorArray_GB300(
  int nvec, int nsum, sunrealtype* a, N_Vector* X, N_Vector** Y, N_Vector** Z);
SUNGB300_EXPORT SUNErrCode N_VLinearCombinationVectorArray_GB300(
  int nvec, int nsum, sunrealtype* c, N_Vector** X, N_Vector* Z);

SUNGB300_EXPORT sunrealtype N_VWSqrSumLocal_GB300(N_Vector x, N_Vector w);
SUNGB300_EXPORT sunrealtype N_VWSqrSumMaskLocal_GB300(N_Vector x, N_Vector w,
                                                      N_Vector id);
SUNGB300_EXPORT SUNErrCode N_VDotProdMultiLocal_GB300(int nvec, N_Vector x,
                                                      N_Vector* Y,
                                                      sunrealtype* dotprods);
SUNGB300_EXPORT SUNErrCode N_VDotProdMultiAllReduce_GB300(int nvec, N_Vector x,
                                                          sunrealtype* sum);

/* Allocation-free dot products, for callers that cannot let the library
 * allocate device memory (an application whose own pool owns the GPU's
 * memory after start-up, or a service that must not call cudaMalloc, which
 * synchronises the device, in its steady state).  This entry point has no
 * counterpart in the reference.
 *
 * d_out[k] = x . Y[k] for k < nvec, with x, the nvec pointers in Y and d_out
 * device arrays (Y itself is a host array of device pointers), length n,
 * enqueued on cuda_stream (NULL: the legacy default stream).  Same bits as
 * N_VDotProdMulti_GB300 on the same data.  nvec must be 1..8
 * (SUNGB300_NOALLOC_MAXVEC): the reduction's scratch is one static device
 * array of 8 x 1024 partial sums (64 KB plus a counter) that every GPU
 * holds from library load to process exit; larger nvec returns
 * SUN_ERR_ARG_OUTOFRANGE without launching.  The first call on a device
 * looks up that array's address (make it before any stream capture).
 * Calls share the array: calls that overlap on the GPU race.  Nothing is
 * allocated and nothing is freed. */
#define SUNGB300_NOALLOC_MAXVEC 8
SUNGB300_EXPORT SUNErrCode N_VDotProdMultiNoAlloc_GB300(int nvec, const sunrealtype* x,
                                                        const sunrealtype* const* Y,
                                                        sunindextype n, sunrealtype* d_out,
                                                        void* cuda_stream);

SUNGB300_EXPORT SUNErrCode N_VBufSize_GB300(N_Vector x, sunindextype* size);
SUNGB300_EXPORT SUNErrCode N_VBufPack_GB300(N_Vector x, void* buf);
SUNGB300_EXPORT SUNErrCode N_VBufUnpack_GB300(N_Vector x, void* buf);

SUNGB300_EXPORT void N_VPrint_GB300(N_Vector v);
SUNGB300_EXPORT void N_VPrintFile_GB300(N_Vector v, FILE* outfile);

#ifdef __cplusplus
}
#endif

#endif /* NVECTOR_GB300_H */
