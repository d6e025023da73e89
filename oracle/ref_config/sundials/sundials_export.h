/* Hand-written stand-in for the export header that the reference's CMake
 * build would generate (GenerateExportHeader).  Used only to compile the
 * reference's serial sources into the test oracle library oracle/_ref. */
#ifndef ORACLE_SUNDIALS_EXPORT_H
#define ORACLE_SUNDIALS_EXPORT_H
#define SUNDIALS_EXPORT __attribute__((visibility("default")))
#define SUNDIALS_NO_EXPORT __attribute__((visibility("hidden")))
#define SUNDIALS_DEPRECATED __attribute__((__deprecated__))
#define SUNDIALS_DEPRECATED_EXPORT SUNDIALS_EXPORT SUNDIALS_DEPRECATED
#define SUNDIALS_DEPRECATED_NO_EXPORT SUNDIALS_NO_EXPORT SUNDIALS_DEPRECATED
#endif
