/* Hand-written configuration header for compiling the reference's serial
 * CVODE / ARKODE / NVECTOR_SERIAL / dense / SPGMR sources directly with gcc
 * (no CMake).  It fixes the reference's defaults: double precision, 64-bit
 * indices, no MPI, no profiling, logging level 2 (warnings).  Test oracle
 * infrastructure only. */
#ifndef _SUNDIALS_CONFIG_H
#define _SUNDIALS_CONFIG_H
#include "sundials/sundials_export.h"
#if defined(__cplusplus)
#define SUNDIALS_NOEXCEPT noexcept
#else
#define SUNDIALS_NOEXCEPT
#endif
#ifndef SUNDIALS_DEPRECATED_MSG
#define SUNDIALS_DEPRECATED_MSG(msg) __attribute__((__deprecated__(msg)))
#endif
#ifndef SUNDIALS_DEPRECATED_EXPORT_MSG
#define SUNDIALS_DEPRECATED_EXPORT_MSG(msg) SUNDIALS_EXPORT SUNDIALS_DEPRECATED_MSG(msg)
#endif
#ifndef SUNDIALS_DEPRECATED_NO_EXPORT_MSG
#define SUNDIALS_DEPRECATED_NO_EXPORT_MSG(msg) SUNDIALS_NO_EXPORT SUNDIALS_DEPRECATED_MSG(msg)
#endif
#define SUNDIALS_VERSION "7.5.0"
#define SUNDIALS_VERSION_MAJOR 7
#define SUNDIALS_VERSION_MINOR 5
#define SUNDIALS_VERSION_PATCH 0
#define SUNDIALS_VERSION_LABEL ""
#define SUNDIALS_GIT_VERSION ""
#define SUNDIALS_C_COMPILER_HAS_BUILTIN_EXPECT
#define SUNDIALS_C_COMPILER_HAS_ATTRIBUTE_UNUSED
#define SUNDIALS_DOUBLE_PRECISION 1
#define SUNDIALS_INT64_T 1
#define SUNDIALS_INDEX_TYPE int64_t
#define SUNDIALS_COUNTER_TYPE long int
#define SUNDIALS_HAVE_POSIX_TIMERS
#define SUNDIALS_LOGGING_LEVEL 2
#define SUN_C_COMPILER "GNU"
#define SUN_C_COMPILER_VERSION ""
#define SUN_C_COMPILER_FLAGS ""
#define SUN_CXX_COMPILER ""
#define SUN_CXX_COMPILER_VERSION ""
#define SUN_CXX_COMPILER_FLAGS ""
#define SUN_FORTRAN_COMPILER ""
#define SUN_FORTRAN_COMPILER_VERSION ""
#define SUN_FORTRAN_COMPILER_FLAGS ""
#define SUN_BUILD_TYPE "Release"
#define SUN_JOB_ID ""
#define SUN_JOB_START_TIME ""
#define SUN_TPL_LIST ""
#define SUN_TPL_LIST_SIZE ""
#define SUNDIALS_SPACK_VERSION ""
#define SUN_MPI_C_COMPILER ""
#define SUN_MPI_C_VERSION ""
#define SUN_MPI_CXX_COMPILER ""
#define SUN_MPI_CXX_VERSION ""
#define SUN_MPI_FORTRAN_COMPILER ""
#define SUN_MPI_FORTRAN_VERSION ""
#define SUNDIALS_MPI_ENABLED 0
#endif
