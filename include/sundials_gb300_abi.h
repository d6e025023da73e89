/* ---------------------------------------------------------------------------
 * sundials_gb300_abi.h -- the SUNDIALS v7.5.0 types that the GB300 modules
 * exchange with CVODE / ARKODE, declared so the library builds without a
 * SUNDIALS installation.
 *
 * The GB300 N_Vector, SUNMatrix and SUNLinearSolver are plugged into the
 * unchanged integrators through the reference's own object model: a struct of
 * function pointers ("ops") plus an opaque content pointer.  For that to work
 * the layouts below must be identical, field for field, to
 *   include/sundials/sundials_nvector.h:101-205       (N_Vector, ops table)
 *   include/sundials/sundials_matrix.h:89-116         (SUNMatrix)
 *   include/sundials/sundials_linearsolver.h:117-150  (SUNLinearSolver)
 *   include/sundials/sundials_iterative.h:61-140      (callback types)
 *   include/sundials/sundials_types.h                 (scalar types)
 * with SUNDIALS' default configuration: sunrealtype = double,
 * sunindextype = int64_t, no MPI (SUNComm = int).
 *
 * When the reference's headers are available, define SUNGB300_WITH_SUNDIALS
 * (or include <sundials/sundials_core.h> first) and this file defers to them.
 * ------------------------------------------------------------------------- */
#ifndef SUNDIALS_GB300_ABI_H
#define SUNDIALS_GB300_ABI_H

#include <stdint.h>
#include <stdio.h>

#if defined(SUNGB300_WITH_SUNDIALS)
#include <sundials/sundials_core.h>
#include <sundials/sundials_iterative.h>
#include <sundials/sundials_linearsolver.h>
#include <sundials/sundials_matrix.h>
#include <sundials/sundials_nvector.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define SUNGB300_EXPORT __attribute__((visibility("default")))

#if !defined(_SUNDIALS_TYPES_H)
/* sundials_types.h: double precision, 64-bit indices, no MPI. */
typedef double sunrealtype;
typedef int64_t sunindextype;
typedef int sunbooleantype;
typedef long int suncountertype;
typedef int SUNErrCode;
typedef int SUNComm;
typedef struct SUNContext_* SUNContext;
#define SUNTRUE 1
#define SUNFALSE 0
#define SUN_COMM_NULL 0
#endif

#if !defined(_SUNDIALS_ERRORS_H)
/* sundials_errors.h: the codes returned by this library (same values). */
enum
{
  SUN_SUCCESS              = 0,
  SUN_ERR_ARG_CORRUPT      = -9999,
  SUN_ERR_ARG_INCOMPATIBLE = -9998,
  SUN_ERR_ARG_OUTOFRANGE   = -9997,
  SUN_ERR_GENERIC          = -9994,
  SUN_ERR_OP_FAIL          = -9990,
  SUN_ERR_MEM_FAIL         = -9989,
  SUN_ERR_MALLOC_FAIL      = -9988,
  SUN_ERR_EXT_FAIL         = -9987,
  SUN_ERR_NOT_IMPLEMENTED  = -9985
};
#endif

#if !defined(_NVECTOR_H)
typedef enum
{
  SUNDIALS_NVEC_SERIAL,
  SUNDIALS_NVEC_PARALLEL,
  SUNDIALS_NVEC_OPENMP,
  SUNDIALS_NVEC_PTHREADS,
  SUNDIALS_NVEC_PARHYP,
  SUNDIALS_NVEC_PETSC,
  SUNDIALS_NVEC_CUDA,
  SUNDIALS_NVEC_HIP,
  SUNDIALS_NVEC_SYCL,
  SUNDIALS_NVEC_RAJA,
  SUNDIALS_NVEC_KOKKOS,
  SUNDIALS_NVEC_OPENMPDEV,
  SUNDIALS_NVEC_TRILINOS,
  SUNDIALS_NVEC_MANYVECTOR,
  SUNDIALS_NVEC_MPIMANYVECTOR,
  SUNDIALS_NVEC_MPIPLUSX,
  SUNDIALS_NVEC_CUSTOM
} N_Vector_ID;

typedef struct _generic_N_Vector_Ops* N_Vector_Ops;
typedef struct _generic_N_Vector* N_Vector;
typedef N_Vector* N_Vector_S;

/* Field order is the ABI: sundials_nvector.h:101-195. */
struct _generic_N_Vector_Ops
{
  N_Vector_ID (*nvgetvectorid)(N_Vector);
  N_Vector (*nvclone)(N_Vector);
  N_Vector (*nvcloneempty)(N_Vector);
  void (*nvdestroy)(N_Vector);
  void (*nvspace)(N_Vector, sunindextype*, sunindextype*);
  sunrealtype* (*nvgetarraypointer)(N_Vector);
  sunrealtype* (*nvgetdevicearraypointer)(N_Vector);
  void (*nvsetarraypointer)(sunrealtype*, N_Vector);
  SUNComm (*nvgetcommunicator)(N_Vector);
  sunindextype (*nvgetlength)(N_Vector);
  sunindextype (*nvgetlocallength)(N_Vector);
  void (*nvlinearsum)(sunrealtype, N_Vector, sunrealtype, N_Vector, N_Vector);
  void (*nvconst)(sunrealtype, N_Vector);
  void (*nvprod)(N_Vector, N_Vector, N_Vector);
  void (*nvdiv)(N_Vector, N_Vector, N_Vector);
  void (*nvscale)(sunrealtype, N_Vector, N_Vector);
  void (*nvabs)(N_Vector, N_Vector);
  void (*nvinv)(N_Vector, N_Vector);
  void (*nvaddconst)(N_Vector, sunrealtype, N_Vector);
  sunrealtype (*nvdotprod)(N_Vector, N_Vector);
  sunrealtype (*nvmaxnorm)(N_Vector);
  sunrealtype (*nvwrmsnorm)(N_Vector, N_Vector);
  sunrealtype (*nvwrmsnormmask)(N_Vector, N_Vector, N_Vector);
  sunrealtype (*nvmin)(N_Vector);
  sunrealtype (*nvwl2norm)(N_Vector, N_Vector);
  sunrealtype (*nvl1norm)(N_Vector);
  void (*nvcompare)(sunrealtype, N_Vector, N_Vector);
  sunbooleantype (*nvinvtest)(N_Vector, N_Vector);
  sunbooleantype (*nvconstrmask)(N_Vector, N_Vector, N_Vector);
  sunrealtype (*nvminquotient)(N_Vector, N_Vector);
  SUNErrCode (*nvlinearcombination)(int, sunrealtype*, N_Vector*, N_Vector);
  SUNErrCode (*nvscaleaddmulti)(int, sunrealtype*, N_Vector, N_Vector*,
                                N_Vector*);
  SUNErrCode (*nvdotprodmulti)(int, N_Vector, N_Vector*, sunrealtype*);
  SUNErrCode (*nvlinearsumvectorarray)(int, sunrealtype, N_Vector*, sunrealtype,
                                       N_Vector*, N_Vector*);
  SUNErrCode (*nvscalevectorarray)(int, sunrealtype*, N_Vector*, N_Vector*);
  SUNErrCode (*nvconstvectorarray)(int, sunrealtype, N_Vector*);
  SUNErrCode (*nvwrmsnormvectorarray)(int, N_Vector*, N_Vector*, sunrealtype*);
  SUNErrCode (*nvwrmsnormmaskvectorarray)(int, N_Vector*, N_Vector*, N_Vector,
                                          sunrealtype*);
  SUNErrCode (*nvscaleaddmultivectorarray)(int, int, sunrealtype*, N_Vector*,
                                           N_Vector**, N_Vector**);
  SUNErrCode (*nvlinearcombinationvectorarray)(int, int, sunrealtype*,
                                               N_Vector**, N_Vector*);
  sunrealtype (*nvdotprodlocal)(N_Vector, N_Vector);
  sunrealtype (*nvmaxnormlocal)(N_Vector);
  sunrealtype (*nvminlocal)(N_Vector);
  sunrealtype (*nvl1normlocal)(N_Vector);
  sunbooleantype (*nvinvtestlocal)(N_Vector, N_Vector);
  sunbooleantype (*nvconstrmasklocal)(N_Vector, N_Vector, N_Vector);
  sunrealtype (*nvminquotientlocal)(N_Vector, N_Vector);
  sunrealtype (*nvwsqrsumlocal)(N_Vector, N_Vector);
  sunrealtype (*nvwsqrsummasklocal)(N_Vector, N_Vector, N_Vector);
  SUNErrCode (*nvdotprodmultilocal)(int, N_Vector, N_Vector*, sunrealtype*);
  SUNErrCode (*nvdotprodmultiallreduce)(int, N_Vector, sunrealtype*);
  SUNErrCode (*nvbufsize)(N_Vector, sunindextype*);
  SUNErrCode (*nvbufpack)(N_Vector, void*);
  SUNErrCode (*nvbufunpack)(N_Vector, void*);
  void (*nvprint)(N_Vector);
  void (*nvprintfile)(N_Vector, FILE*);
};

struct _generic_N_Vector
{
  void* content;
  N_Vector_Ops ops;
  SUNContext sunctx;
};
#endif /* _NVECTOR_H */

#if !defined(_SUNMATRIX_H)
typedef enum
{
  SUNMATRIX_DENSE,
  SUNMATRIX_MAGMADENSE,
  SUNMATRIX_ONEMKLDENSE,
  SUNMATRIX_BAND,
  SUNMATRIX_SPARSE,
  SUNMATRIX_SLUNRLOC,
  SUNMATRIX_CUSPARSE,
  SUNMATRIX_GINKGO,
  SUNMATRIX_GINKGOBATCH,
  SUNMATRIX_KOKKOSDENSE,
  SUNMATRIX_CUSTOM
} SUNMatrix_ID;

typedef struct _generic_SUNMatrix_Ops* SUNMatrix_Ops;
typedef struct _generic_SUNMatrix* SUNMatrix;

/* Field order is the ABI: sundials_matrix.h:89-102. */
struct _generic_SUNMatrix_Ops
{
  SUNMatrix_ID (*getid)(SUNMatrix);
  SUNMatrix (*clone)(SUNMatrix);
  void (*destroy)(SUNMatrix);
  SUNErrCode (*zero)(SUNMatrix);
  SUNErrCode (*copy)(SUNMatrix, SUNMatrix);
  SUNErrCode (*scaleadd)(sunrealtype, SUNMatrix, SUNMatrix);
  SUNErrCode (*scaleaddi)(sunrealtype, SUNMatrix);
  SUNErrCode (*matvecsetup)(SUNMatrix);
  SUNErrCode (*matvec)(SUNMatrix, N_Vector, N_Vector);
  SUNErrCode (*mathermitiantransposevec)(SUNMatrix, N_Vector, N_Vector);
  SUNErrCode (*space)(SUNMatrix, long int*, long int*);
};

struct _generic_SUNMatrix
{
  void* content;
  SUNMatrix_Ops ops;
  SUNContext sunctx;
};
#endif /* _SUNMATRIX_H */

#if !defined(_SUNDIALS_ITERATIVE_H)
enum
{
  SUN_PREC_NONE,
  SUN_PREC_LEFT,
  SUN_PREC_RIGHT,
  SUN_PREC_BOTH
};
enum
{
  SUN_MODIFIED_GS  = 1,
  SUN_CLASSICAL_GS = 2
};
typedef int (*SUNATimesFn)(void* A_data, N_Vector v, N_Vector z);
typedef int (*SUNPSetupFn)(void* P_data);
typedef int (*SUNPSolveFn)(void* P_data, N_Vector r, N_Vector z,
                           sunrealtype tol, int lr);
#endif

#if !defined(_SUNLINEARSOLVER_H)
typedef enum
{
  SUNLINEARSOLVER_DIRECT,
  SUNLINEARSOLVER_ITERATIVE,
  SUNLINEARSOLVER_MATRIX_ITERATIVE,
  SUNLINEARSOLVER_MATRIX_EMBEDDED
} SUNLinearSolver_Type;

typedef enum
{
  SUNLINEARSOLVER_BAND,
  SUNLINEARSOLVER_DENSE,
  SUNLINEARSOLVER_KLU,
  SUNLINEARSOLVER_LAPACKBAND,
  SUNLINEARSOLVER_LAPACKDENSE,
  SUNLINEARSOLVER_PCG,
  SUNLINEARSOLVER_SPBCGS,
  SUNLINEARSOLVER_SPFGMR,
  SUNLINEARSOLVER_SPGMR,
  SUNLINEARSOLVER_SPTFQMR,
  SUNLINEARSOLVER_SUPERLUDIST,
  SUNLINEARSOLVER_SUPERLUMT,
  SUNLINEARSOLVER_CUSOLVERSP_BATCHQR,
  SUNLINEARSOLVER_MAGMADENSE,
  SUNLINEARSOLVER_ONEMKLDENSE,
  SUNLINEARSOLVER_GINKGO,
  SUNLINEARSOLVER_GINKGOBATCH,
  SUNLINEARSOLVER_KOKKOSDENSE,
  SUNLINEARSOLVER_CUSTOM
} SUNLinearSolver_ID;

typedef struct _generic_SUNLinearSolver_Ops* SUNLinearSolver_Ops;
typedef struct _generic_SUNLinearSolver* SUNLinearSolver;

/* Field order is the ABI: sundials_linearsolver.h:117-142. */
struct _generic_SUNLinearSolver_Ops
{
  SUNLinearSolver_Type (*gettype)(SUNLinearSolver);
  SUNLinearSolver_ID (*getid)(SUNLinearSolver);
  SUNErrCode (*setatimes)(SUNLinearSolver, void*, SUNATimesFn);
  SUNErrCode (*setpreconditioner)(SUNLinearSolver, void*, SUNPSetupFn,
                                  SUNPSolveFn);
  SUNErrCode (*setscalingvectors)(SUNLinearSolver, N_Vector, N_Vector);
  SUNErrCode (*setoptions)(SUNLinearSolver, const char* LSid,
                           const char* file_name, int argc, char* argv[]);
  SUNErrCode (*setzeroguess)(SUNLinearSolver, sunbooleantype);
  SUNErrCode (*initialize)(SUNLinearSolver);
  int (*setup)(SUNLinearSolver, SUNMatrix);
  int (*solve)(SUNLinearSolver, SUNMatrix, N_Vector, N_Vector, sunrealtype);
  int (*numiters)(SUNLinearSolver);
  sunrealtype (*resnorm)(SUNLinearSolver);
  sunindextype (*lastflag)(SUNLinearSolver);
  SUNErrCode (*space)(SUNLinearSolver, long int*, long int*);
  N_Vector (*resid)(SUNLinearSolver);
  SUNErrCode (*free)(SUNLinearSolver);
};

struct _generic_SUNLinearSolver
{
  void* content;
  SUNLinearSolver_Ops ops;
  SUNContext sunctx;
};

/* sundials_linearsolver.h:229-248 */
#define SUNLS_ATIMES_NULL       -804
#define SUNLS_ATIMES_FAIL_UNREC -805
#define SUNLS_PSET_FAIL_UNREC   -806
#define SUNLS_PSOLVE_NULL       -807
#define SUNLS_PSOLVE_FAIL_UNREC -808
#define SUNLS_GS_FAIL           -810
#define SUNLS_QRSOL_FAIL        -811
#define SUNLS_RECOV_FAILURE     800
#define SUNLS_RES_REDUCED       801
#define SUNLS_CONV_FAIL         802
#define SUNLS_ATIMES_FAIL_REC   803
#define SUNLS_PSET_FAIL_REC     804
#define SUNLS_PSOLVE_FAIL_REC   805
#define SUNLS_PACKAGE_FAIL_REC  806
#define SUNLS_QRFACT_FAIL       807
#define SUNLS_LUFACT_FAIL       808
#endif /* _SUNLINEARSOLVER_H */

#ifdef __cplusplus
}
#endif

#endif /* SUNDIALS_GB300_ABI_H */
