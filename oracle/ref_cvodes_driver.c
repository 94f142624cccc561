/*
 * The reference's own CVODES behind the oracle's integrator interface —
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile.ref from the vendored
 * SUNDIALS sources of the reference (ThirdParty/sundials) into oracle/_ref/;
 * used to generate golden vectors and to pin the restated integrator.
 *
 * Sets CVODES up the way amici::CVodeSolver does for an ODE model
 * (src/solver.cpp:193-264, src/solver_cvodes.cpp:130-187,280-460):
 * CVodeCreate(BDF), CVodeInit(xdot), scalar tolerances, dense linear solver
 * with the analytic Jacobian (AMICI's LinearSolver::dense), Newton, staggered
 * sensitivities with CVodeSensInit1 + explicit sensitivity tolerances +
 * CVodeSetSensErrCon(true) (solver.cpp:641-656), max nonlinear iterations and
 * convergence failures, stability-limit detection as requested, and before
 * every output CVodeSetStopTime(tout) plus the remaining step budget
 * (solver.cpp:107-160).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cvodes/cvodes.h>
#include <nvector/nvector_serial.h>
#include <sundials/sundials_context.h>
#include <sunlinsol/sunlinsol_dense.h>
#include <sunmatrix/sunmatrix_dense.h>

#include "oracle_integrator.h"

typedef struct {
    const oracle_model* m;
    const double *p, *k;
    int n, ns;
    const int32_t* plist;
    SUNContext ctx;
    void* cvode_mem;
    N_Vector y;
    N_Vector* yS;
    SUNMatrix A;
    SUNLinearSolver LS;
    double* Jtmp;
    double* dfdp;
    double* xS; /* contiguous copy of the sensitivities [ns*n] */
    int64_t nst;
} refmem;

static int f_xdot(sunrealtype t, N_Vector y, N_Vector ydot, void* ud) {
    refmem* r = (refmem*)ud;
    r->m->xdot(N_VGetArrayPointer(ydot), t, N_VGetArrayPointer(y), r->p, r->k);
    return 0;
}

static int f_jac(sunrealtype t, N_Vector y, N_Vector fy, SUNMatrix J, void* ud, N_Vector t1,
                 N_Vector t2, N_Vector t3) {
    (void)fy; (void)t1; (void)t2; (void)t3;
    refmem* r = (refmem*)ud;
    r->m->jac(SUNDenseMatrix_Data(J), t, N_VGetArrayPointer(y), r->p, r->k);
    return 0;
}

/* Model_ODE::fsxdot (src/model_ode.cpp:419-450) */
static int f_sxdot(int Ns, sunrealtype t, N_Vector y, N_Vector ydot, int iS, N_Vector yS,
                   N_Vector ySdot, void* ud, N_Vector t1, N_Vector t2) {
    (void)Ns; (void)ydot; (void)t1; (void)t2;
    refmem* r = (refmem*)ud;
    const int n = r->n;
    const double* x = N_VGetArrayPointer(y);
    if (iS == 0) {
        r->m->jac(r->Jtmp, t, x, r->p, r->k);
        r->m->dxdotdp(r->dfdp, t, x, r->p, r->k);
    }
    const double* s = N_VGetArrayPointer(yS);
    double* out = N_VGetArrayPointer(ySdot);
    const double* col = r->dfdp + (size_t)r->plist[iS] * n;
    for (int i = 0; i < n; i++) out[i] = col[i];
    for (int j = 0; j < n; j++) {
        double sj = s[j];
        if (sj == 0.0) continue;
        const double* Jc = r->Jtmp + (size_t)j * n;
        for (int i = 0; i < n; i++) out[i] += Jc[i] * sj;
    }
    return 0;
}

static void* ref_create(const oracle_model* m, const oracle_options* o, const double* p,
                        const double* k, int ns, const int32_t* plist, const double* x0,
                        const double* sx0) {
    refmem* r = (refmem*)calloc(1, sizeof(refmem));
    const int n = m->nx;
    r->m = m; r->p = p; r->k = k; r->n = n; r->ns = ns; r->plist = plist;
    SUNContext_Create(SUN_COMM_NULL, &r->ctx);
    r->y = N_VNew_Serial(n, r->ctx);
    memcpy(N_VGetArrayPointer(r->y), x0, sizeof(double) * n);
    r->cvode_mem = CVodeCreate(CV_BDF, r->ctx);
    CVodeInit(r->cvode_mem, f_xdot, 0.0, r->y);
    CVodeSStolerances(r->cvode_mem, o->rtol, o->atol);
    CVodeSetUserData(r->cvode_mem, r);
    CVodeSetStabLimDet(r->cvode_mem, o->stldet ? SUNTRUE : SUNFALSE);
    r->A = SUNDenseMatrix(n, n, r->ctx);
    r->LS = SUNLinSol_Dense(r->y, r->A, r->ctx);
    CVodeSetLinearSolver(r->cvode_mem, r->LS, r->A);
    CVodeSetJacFn(r->cvode_mem, f_jac);
    r->Jtmp = (double*)calloc((size_t)n * n + 1, sizeof(double));
    r->dfdp = (double*)calloc((size_t)m->np * n + 1, sizeof(double));
    r->xS = (double*)calloc((size_t)n * (ns > 0 ? ns : 1), sizeof(double));
    if (ns > 0) {
        r->yS = N_VCloneVectorArray(ns, r->y);
        for (int is = 0; is < ns; is++)
            memcpy(N_VGetArrayPointer(r->yS[is]), sx0 + (size_t)is * n, sizeof(double) * n);
        CVodeSensInit1(r->cvode_mem, ns, CV_STAGGERED, f_sxdot, r->yS);
        double* pbar = (double*)malloc(sizeof(double) * ns);
        int* pl = (int*)malloc(sizeof(int) * ns);
        for (int is = 0; is < ns; is++) { pbar[is] = 1.0; pl[is] = plist[is]; }
        CVodeSetSensParams(r->cvode_mem, (sunrealtype*)p, pbar, pl);
        free(pbar); free(pl);
        double rtolS = isnan(o->rtol_fsa) ? o->rtol : o->rtol_fsa;
        double atolS = isnan(o->atol_fsa) ? o->atol : o->atol_fsa;
        double* atols = (double*)malloc(sizeof(double) * ns);
        for (int is = 0; is < ns; is++) atols[is] = atolS;
        CVodeSensSStolerances(r->cvode_mem, rtolS, atols);
        free(atols);
        CVodeSetSensErrCon(r->cvode_mem, SUNTRUE);
    }
    CVodeSetMaxNonlinIters(r->cvode_mem, o->max_nonlin_iters > 0 ? o->max_nonlin_iters : 3);
    CVodeSetMaxConvFails(r->cvode_mem, o->max_conv_fails > 0 ? o->max_conv_fails : 10);
    if (o->max_step_size > 0.0 && isfinite(o->max_step_size))
        CVodeSetMaxStep(r->cvode_mem, o->max_step_size);
    memcpy(r->xS, sx0, sizeof(double) * n * (ns > 0 ? ns : 0));
    return r;
}

static int ref_solve(void* h, double tout, int64_t mxstep, double* tret) {
    refmem* r = (refmem*)h;
    CVodeSetStopTime(r->cvode_mem, tout);
    CVodeSetMaxNumSteps(r->cvode_mem, (long)mxstep);
    int flag = CVode(r->cvode_mem, tout, r->y, tret, CV_NORMAL);
    long nst = 0;
    CVodeGetNumSteps(r->cvode_mem, &nst);
    r->nst = nst;
    if (flag >= 0 && r->ns > 0) {
        double t;
        CVodeGetSens(r->cvode_mem, &t, r->yS);
        for (int is = 0; is < r->ns; is++)
            memcpy(r->xS + (size_t)is * r->n, N_VGetArrayPointer(r->yS[is]), sizeof(double) * r->n);
    }
    return flag;
}

static const double* ref_x(void* h) { return N_VGetArrayPointer(((refmem*)h)->y); }
static const double* ref_sx(void* h) { return ((refmem*)h)->xS; }
static int64_t ref_nst(void* h) { return ((refmem*)h)->nst; }

static void ref_destroy(void* h) {
    refmem* r = (refmem*)h;
    if (r->ns > 0) N_VDestroyVectorArray(r->yS, r->ns);
    CVodeFree(&r->cvode_mem);
    SUNLinSolFree(r->LS);
    SUNMatDestroy(r->A);
    N_VDestroy(r->y);
    SUNContext_Free(&r->ctx);
    free(r->Jtmp); free(r->dfdp); free(r->xS); free(r);
}

const oracle_integrator oracle_integrator_impl = {ref_create, ref_solve, ref_x, ref_sx, ref_nst,
                                                  ref_destroy};
