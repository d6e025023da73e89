/* fixedpoint_port.h -- TEST ORACLE (checker only): the reference's
 * SUNNonlinSol_FixedPoint (Anderson acceleration) restated over the generic
 * vector ops table, shared by the CVODE and ARKStep restatements. */
#ifndef ORACLE_FIXEDPOINT_PORT_H
#define ORACLE_FIXEDPOINT_PORT_H

#include "../include/sundials_gb300_abi.h"

typedef struct FPPort FPPort;
/* the integrator's fixed-point function g(ycor) and convergence test */
typedef int (*FPSysFn)(void* mem, N_Vector ycor, N_Vector g);
typedef int (*FPCTestFn)(void* mem, N_Vector ycor, N_Vector del, double tol, int curiter);

FPPort* fp_port_create(N_Vector tmpl, int m); /* maxiters 3, no damping */
void fp_port_free(FPPort* fp);
int fp_port_solve(FPPort* fp, N_Vector ycor, double tol, FPSysFn sys, FPCTestFn ctest,
                  void* mem);
void fp_port_set_maxiters(FPPort* fp, int maxiters);
long fp_port_niters(const FPPort* fp);
long fp_port_nconvfails(const FPPort* fp);

#endif
