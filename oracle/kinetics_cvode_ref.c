/* kinetics_cvode_ref.c -- TEST ORACLE: integrates every system of a kinetics
 * problem file with the reference's own, unmodified CVODE (BDF, Newton,
 * NVECTOR_SERIAL, SUNMATRIX_DENSE + SUNLINSOL_DENSE, analytic Jacobian) and
 * writes per-system counters and y(tout).  Built by oracle/Makefile against
 * oracle/_ref/libsundials_ref.so, only where the reference sources exist; its
 * outputs become the golden fixtures in tests/golden/.
 *
 * usage: kinetics_cvode_ref problem.bin out.bin rtol atol tout [first count]
 * Output: for each system, one KinStats record followed by n doubles. */
#include <cvode/cvode.h>
#include <nvector/nvector_serial.h>
#include <stdio.h>
#include <stdlib.h>
#include <sundials/sundials_context.h>
#include <sunlinsol/sunlinsol_dense.h>
#include <sunmatrix/sunmatrix_dense.h>

#include "kinetics_model.h"

static int f_cb(sunrealtype t, N_Vector y, N_Vector ydot, void* ud)
{
  (void)t;
  kin_rhs((const KinSys*)ud, N_VGetArrayPointer(y), N_VGetArrayPointer(ydot));
  return 0;
}

static int jac_cb(sunrealtype t, N_Vector y, N_Vector fy, SUNMatrix J, void* ud,
                  N_Vector t1, N_Vector t2, N_Vector t3)
{
  (void)t; (void)fy; (void)t1; (void)t2; (void)t3;
  kin_jac((const KinSys*)ud, N_VGetArrayPointer(y), SUNDenseMatrix_Data(J));
  return 0;
}

static void* rd(FILE* f, size_t bytes)
{
  void* p = malloc(bytes ? bytes : 1);
  if (bytes && fread(p, 1, bytes, f) != bytes) { fprintf(stderr, "short read\n"); exit(2); }
  return p;
}

int main(int argc, char** argv)
{
  if (argc < 6) { fprintf(stderr, "usage: %s problem.bin out.bin rtol atol tout [first count]\n", argv[0]); return 2; }
  double rtol = atof(argv[3]), atol = atof(argv[4]), tout = atof(argv[5]);
  FILE* fp = fopen(argv[1], "rb");
  if (!fp) { perror("open problem"); return 2; }
  int64_t hdr[3];
  if (fread(hdr, 8, 3, fp) != 3) return 2;
  int64_t nsys = hdr[0], Y = hdr[1], R = hdr[2];
  int32_t* n     = rd(fp, 4 * nsys);
  int64_t* y_off = rd(fp, 8 * (nsys + 1));
  int64_t* r_off = rd(fp, 8 * (nsys + 1));
  int32_t* rt = rd(fp, 4 * R);
  int32_t* ra = rd(fp, 4 * R);
  int32_t* rb = rd(fp, 4 * R);
  int32_t* rc = rd(fp, 4 * R);
  double* rk  = rd(fp, 8 * R);
  double* y0  = rd(fp, 8 * Y);
  fclose(fp);
  int64_t first = argc > 6 ? atoll(argv[6]) : 0;
  int64_t count = argc > 7 ? atoll(argv[7]) : nsys - first;

  KinStats* st = calloc(count, sizeof(KinStats));
  double* yout = calloc(Y, sizeof(double));

#pragma omp parallel
  {
    SUNContext ctx;
    SUNContext_Create(SUN_COMM_NULL, &ctx);
#pragma omp for schedule(dynamic, 4)
    for (int64_t s = first; s < first + count; s++)
    {
      KinSys sys = {n[s], (int)(r_off[s + 1] - r_off[s]), rt + r_off[s], ra + r_off[s],
                    rb + r_off[s], rc + r_off[s], rk + r_off[s]};
      N_Vector y = N_VNew_Serial(n[s], ctx);
      for (int i = 0; i < n[s]; i++) NV_Ith_S(y, i) = y0[y_off[s] + i];
      void* cv = CVodeCreate(CV_BDF, ctx);
      CVodeInit(cv, f_cb, 0.0, y);
      CVodeSStolerances(cv, rtol, atol);
      CVodeSetUserData(cv, &sys);
      SUNMatrix A       = SUNDenseMatrix(n[s], n[s], ctx);
      SUNLinearSolver L = SUNLinSol_Dense(y, A, ctx);
      CVodeSetLinearSolver(cv, L, A);
      CVodeSetJacFn(cv, jac_cb);
      CVodeSetMaxNumSteps(cv, 1000000);
      double t  = 0.0;
      int flag  = CVode(cv, tout, y, &t, CV_NORMAL);
      KinStats* o = &st[s - first];
      long v;
      CVodeGetNumSteps(cv, &v); o->nst = v;
      CVodeGetNumRhsEvals(cv, &v); o->nfe = v;
      CVodeGetNumLinSolvSetups(cv, &v); o->nsetups = v;
      CVodeGetNumJacEvals(cv, &v); o->nje = v;
      CVodeGetNumNonlinSolvIters(cv, &v); o->nni = v;
      CVodeGetNumStepSolveFails(cv, &v); o->ncfn = v;
      CVodeGetNumErrTestFails(cv, &v); o->netf = v;
      CVodeGetNumNonlinSolvConvFails(cv, &v); o->nnf = v;
      int q; CVodeGetLastOrder(cv, &q); o->qu = q;
      CVodeGetLastStep(cv, &o->hu);
      CVodeGetCurrentTime(cv, &o->tn);
      o->flag = flag;
      for (int i = 0; i < n[s]; i++) yout[y_off[s] + i] = NV_Ith_S(y, i);
      SUNLinSolFree(L);
      SUNMatDestroy(A);
      N_VDestroy(y);
      CVodeFree(&cv);
    }
    SUNContext_Free(&ctx);
  }
  FILE* fo = fopen(argv[2], "wb");
  for (int64_t s = first; s < first + count; s++)
  {
    fwrite(&st[s - first], sizeof(KinStats), 1, fo);
    fwrite(yout + y_off[s], 8, n[s], fo);
  }
  fclose(fo);
  return 0;
}
