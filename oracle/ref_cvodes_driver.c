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

#include "cvodes_impl.h"
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
    int force_reinit, called; /* force_reinit_postprocess_F_, solver_was_called_F_ */
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

/* the trigger functions (solver_cvodes.cpp:1140-1160 froot) */
static int f_root(sunrealtype t, N_Vector y, sunrealtype* g, void* ud) {
    refmem* r = (refmem*)ud;
    r->m->root(g, t, N_VGetArrayPointer(y), r->p, r->k);
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
    if (m->nroot > 0) CVodeRootInit(r->cvode_mem, m->nroot, f_root); /* solver_cvodes.cpp:227 */
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

/* CVodeSolver::reInit_post_process (solver_cvodes.cpp:531-583) */
static int ref_reinit_post_process(refmem* r, double tout, double* tret) {
    CVodeMem cv_mem = (CVodeMem)r->cvode_mem;
    long nst_tmp = cv_mem->cv_nst;
    cv_mem->cv_nst = 0;
    CVodeSetStopTime(cv_mem, tout);
    int status = CVode(cv_mem, tout, r->y, tret, CV_ONE_STEP);
    if (status != CV_SUCCESS) return -99; /* a CvodeException (a root return included): AMICI_ERROR */
    cv_mem->cv_nst = nst_tmp + 1;
    r->force_reinit = 0;
    return 0;
}

static int ref_solve(void* h, double tout, int64_t mxstep, double* tret) {
    refmem* r = (refmem*)h;
    CVodeSetStopTime(r->cvode_mem, tout);
    CVodeSetMaxNumSteps(r->cvode_mem, (long)mxstep);
    if (r->force_reinit) {
        int s = ref_reinit_post_process(r, tout, tret);
        if (s) {
            long nst = 0;
            CVodeGetNumSteps(r->cvode_mem, &nst);
            r->nst = nst;
            return s;
        }
    }
    r->called = 1;
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

/* Solver::step: CVode(tout, ONE_STEP) without a stop time (solver.cpp:162-178) */
static int ref_one_step(void* h, double tout, double* tret) {
    refmem* r = (refmem*)h;
    int flag = CVode(r->cvode_mem, tout, r->y, tret, CV_ONE_STEP);
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

/* CVodeSolver::reinit + reset_state and sens_reinit (solver_cvodes.cpp:
 * 471-505,586-616) */
static void ref_reset_state(CVodeMem cv_mem, N_Vector y0) {
    cv_mem->cv_q = 1;
    cv_mem->cv_L = 2;
    cv_mem->cv_qwait = cv_mem->cv_L;
    cv_mem->cv_qu = 0;
    cv_mem->cv_hu = 0.0;
    cv_mem->cv_tolsf = 1.0;
    cv_mem->cv_h0u = 0.0;
    cv_mem->cv_next_h = 0.0;
    cv_mem->cv_next_q = 0;
    N_VScale(1.0, y0, cv_mem->cv_zn[0]);
}

static void ref_reinit(void* h, double t, const double* x, const double* sx) {
    refmem* r = (refmem*)h;
    CVodeMem cv_mem = (CVodeMem)r->cvode_mem;
    cv_mem->cv_tn = t;
    if (r->called) r->force_reinit = 1;
    memcpy(N_VGetArrayPointer(r->y), x, sizeof(double) * r->n);
    ref_reset_state(cv_mem, r->y);
    if (r->ns > 0 && sx) {
        for (int is = 0; is < r->ns; is++) {
            memcpy(N_VGetArrayPointer(r->yS[is]), sx + (size_t)is * r->n, sizeof(double) * r->n);
            N_VScale(1.0, r->yS[is], cv_mem->cv_znS[0][is]);
        }
        memcpy(r->xS, sx, sizeof(double) * r->n * r->ns);
    }
}

static void ref_root_info(void* h, int* iroots) { CVodeGetRootInfo(((refmem*)h)->cvode_mem, iroots); }

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

const oracle_integrator oracle_integrator_impl = {ref_create, ref_solve, ref_one_step, ref_x, ref_sx,
                                                  ref_nst, ref_destroy, ref_reinit, ref_root_info};

/* ======================================================================== */
/* Adjoint sensitivities with the reference's CVODES, set up and driven the  */
/* way amici::CVodeSolver does for an ODE model:                             */
/*   CVodeAdjInit(maxsteps + 1, CV_POLYNOMIAL) (solver_cvodes.cpp:726-739),  */
/*   CVodeF with a stop time at every output (solver.cpp:141-160),           */
/*   CVodeCreateB / CVodeInitB / CVodeQuadInitB, dense linear solver with    */
/*   the backward Jacobian, CVodeSStolerancesB, CVodeQuadSStolerancesB,      */
/*   CVodeSetQuadErrConB (solver.cpp:267-298,658-691), CVodeB per output and */
/*   AMICI's reinitialisation after every adjoint jump: reset_state and the  */
/*   one-step reInit_post_process (solver_cvodes.cpp:470-560,618-648,830-845).*/
/* ======================================================================== */
#include <cvodes/cvodes_ls.h>

#include "oracle_adjoint.h"

typedef struct {
    refmem f;
    const int32_t* plist;
    int nplist;
    int which;
    N_Vector yB, qB, ytmpB;
    SUNMatrix AB;
    SUNLinearSolver LSB;
    double *J, *dfdp;
    double rtolB, atolB, rtolQ, atolQ;
    int errconQ, force_reinit, called_b, stldet;
    int64_t maxsteps;
} refadj;

static int fB_xBdot(sunrealtype t, N_Vector y, N_Vector yB, N_Vector yBdot, void* ud) {
    refadj* r = (refadj*)ud;
    oracle_fxBdot(r->f.m, r->f.p, r->f.k, r->J, t, N_VGetArrayPointer(y), N_VGetArrayPointer(yB),
                  N_VGetArrayPointer(yBdot));
    return 0;
}

static int fB_jac(sunrealtype t, N_Vector y, N_Vector yB, N_Vector fyB, SUNMatrix JB, void* ud,
                  N_Vector t1, N_Vector t2, N_Vector t3) {
    (void)yB; (void)fyB; (void)t1; (void)t2; (void)t3;
    refadj* r = (refadj*)ud;
    oracle_fJB(r->f.m, r->f.p, r->f.k, r->J, t, N_VGetArrayPointer(y), SUNDenseMatrix_Data(JB));
    return 0;
}

static int fB_qBdot(sunrealtype t, N_Vector y, N_Vector yB, N_Vector qBdot, void* ud) {
    refadj* r = (refadj*)ud;
    oracle_fqBdot(r->f.m, r->f.p, r->f.k, r->dfdp, r->nplist, r->plist, t, N_VGetArrayPointer(y),
                  N_VGetArrayPointer(yB), N_VGetArrayPointer(qBdot));
    return 0;
}

static void* refadj_create(const oracle_model* m, const oracle_options* o, const double* p,
                           const double* k, int nplist, const int32_t* plist, const double* x0) {
    refadj* r = (refadj*)calloc(1, sizeof(refadj));
    refmem* f = (refmem*)ref_create(m, o, p, k, 0, NULL, x0, NULL);
    r->f = *f;
    free(f);
    CVodeSetUserData(r->f.cvode_mem, r);
    r->plist = plist;
    r->nplist = nplist;
    r->maxsteps = o->maxsteps;
    CVodeAdjInit(r->f.cvode_mem, (long)(o->maxsteps + 1), CV_POLYNOMIAL);
    r->J = (double*)calloc((size_t)m->nx * m->nx + 1, sizeof(double));
    r->dfdp = (double*)calloc((size_t)m->np * m->nx + 1, sizeof(double));
    r->rtolB = isnan(o->rtol_b) ? o->rtol : o->rtol_b;
    r->atolB = isnan(o->atol_b) ? o->atol : o->atol_b;
    r->rtolQ = isnan(o->rtol_quad) ? o->rtol : o->rtol_quad;
    r->atolQ = isnan(o->atol_quad) ? o->atol : o->atol_quad;
    r->errconQ = !isinf(r->atolQ) && !isinf(r->rtolQ);
    r->stldet = o->stldet;  /* Solver::setup_b: set_stab_lim_det_b(which, stldet_), solver.cpp:297 */
    return r;
}

/* user data of the forward callbacks is the refmem at the start of refadj */
static int refadj_solve_f(void* h, double tout, int64_t mxstep, double* tret) {
    refadj* r = (refadj*)h;
    int ncheck = 0;
    CVodeSetStopTime(r->f.cvode_mem, tout);
    CVodeSetMaxNumSteps(r->f.cvode_mem, (long)mxstep);
    int flag = CVodeF(r->f.cvode_mem, tout, r->f.y, tret, CV_NORMAL, &ncheck);
    long nst = 0;
    CVodeGetNumSteps(r->f.cvode_mem, &nst);
    r->f.nst = nst;
    return flag;
}
static const double* refadj_x(void* h) { return N_VGetArrayPointer(((refadj*)h)->f.y); }
static int64_t refadj_nst(void* h) { return ((refadj*)h)->f.nst; }

static int refadj_setup_b(void* h, double tB0, const double* xB0, const double* xQB0) {
    refadj* r = (refadj*)h;
    const int n = r->f.n;
    void* mem = r->f.cvode_mem;
    r->yB = N_VNew_Serial(n, r->f.ctx);
    memcpy(N_VGetArrayPointer(r->yB), xB0, sizeof(double) * n);
    r->qB = N_VNew_Serial(r->nplist, r->f.ctx);
    memcpy(N_VGetArrayPointer(r->qB), xQB0, sizeof(double) * r->nplist);
    r->ytmpB = N_VNew_Serial(n, r->f.ctx);
    CVodeCreateB(mem, CV_BDF, &r->which);
    CVodeInitB(mem, r->which, fB_xBdot, tB0, r->yB);
    CVodeSetUserDataB(mem, r->which, r);
    r->AB = SUNDenseMatrix(n, n, r->f.ctx);
    r->LSB = SUNLinSol_Dense(r->yB, r->AB, r->f.ctx);
    CVodeSetLinearSolverB(mem, r->which, r->LSB, r->AB);
    CVodeSetJacFnB(mem, r->which, fB_jac);
    CVodeQuadInitB(mem, r->which, fB_qBdot, r->qB);
    CVodeSStolerancesB(mem, r->which, r->rtolB, r->atolB);
    CVodeSetQuadErrConB(mem, r->which, r->errconQ ? SUNTRUE : SUNFALSE);
    CVodeQuadSStolerancesB(mem, r->which, r->rtolQ, r->atolQ);
    CVodeSetStabLimDetB(mem, r->which, r->stldet ? SUNTRUE : SUNFALSE);
    return 0;
}

/* CVodeSolver::reset_state (solver_cvodes.cpp:471-505) */
static void refadj_reset_state(CVodeMem cv_mem, N_Vector y0) {
    cv_mem->cv_q = 1;
    cv_mem->cv_L = 2;
    cv_mem->cv_qwait = cv_mem->cv_L;
    cv_mem->cv_qu = 0;
    cv_mem->cv_hu = 0.0;
    cv_mem->cv_tolsf = 1.0;
    cv_mem->cv_h0u = 0.0;
    cv_mem->cv_next_h = 0.0;
    cv_mem->cv_next_q = 0;
    N_VScale(1.0, y0, cv_mem->cv_zn[0]);
}

/* CVodeSolver::reinit_post_process_b / reInit_post_process (solver_cvodes.cpp:512-560) */
static int refadj_reinit_post_process(refadj* r, double tnext) {
    CVodeMem cv_mem = (CVodeMem)r->f.cvode_mem;
    CVadjMem ca_mem = cv_mem->cv_adj_mem;
    CVodeBMem cvB_mem = ca_mem->cvB_mem;
    ca_mem->ca_bckpbCrt = cvB_mem;
    CVodeMem bm = cvB_mem->cv_mem;
    long nst_tmp = bm->cv_nst;
    bm->cv_nst = 0;
    CVodeSetStopTime(bm, tnext);
    double tret;
    int status = CVode(bm, tnext, r->ytmpB, &tret, CV_ONE_STEP);
    if (status != CV_SUCCESS) return -99; /* a CvodeException: AMICI_ERROR */
    bm->cv_nst = nst_tmp + 1;
    cvB_mem->cv_tout = tret;
    r->force_reinit = 0;
    return 0;
}

static int refadj_run_b(void* h, double tBout, int64_t mxstepsB) {
    refadj* r = (refadj*)h;
    CVodeSetMaxNumStepsB(r->f.cvode_mem, r->which, (long)mxstepsB);
    if (r->force_reinit) {
        int s = refadj_reinit_post_process(r, tBout);
        if (s) return s;
    }
    int flag = CVodeB(r->f.cvode_mem, tBout, CV_NORMAL);
    r->called_b = 1;
    return flag < 0 ? flag : 0;
}

static void refadj_get_b(void* h, double* xB, double* xQB) {
    refadj* r = (refadj*)h;
    double t;
    CVodeGetB(r->f.cvode_mem, r->which, &t, r->yB);
    CVodeGetQuadB(r->f.cvode_mem, r->which, &t, r->qB);
    memcpy(xB, N_VGetArrayPointer(r->yB), sizeof(double) * r->f.n);
    memcpy(xQB, N_VGetArrayPointer(r->qB), sizeof(double) * r->nplist);
}

/* CVodeSolver::reinit_b + reinit_quad_b (solver_cvodes.cpp:618-648) */
static void refadj_reinit_b(void* h, double t, const double* xB, const double* xQB) {
    refadj* r = (refadj*)h;
    CVodeMem bm = (CVodeMem)CVodeGetAdjCVodeBmem(r->f.cvode_mem, r->which);
    if (r->called_b) r->force_reinit = 1;
    bm->cv_tn = t;
    memcpy(N_VGetArrayPointer(r->ytmpB), xB, sizeof(double) * r->f.n);
    refadj_reset_state(bm, r->ytmpB);
    memcpy(N_VGetArrayPointer(bm->cv_znQ[0]), xQB, sizeof(double) * r->nplist);
}

static int64_t refadj_nst_b(void* h) {
    refadj* r = (refadj*)h;
    if (!r->yB) return 0;
    long nst = 0;
    CVodeGetNumSteps(CVodeGetAdjCVodeBmem(r->f.cvode_mem, r->which), &nst);
    return nst;
}

static void refadj_destroy(void* h) {
    refadj* r = (refadj*)h;
    if (r->yB) {
        N_VDestroy(r->yB);
        N_VDestroy(r->qB);
        N_VDestroy(r->ytmpB);
    }
    CVodeFree(&r->f.cvode_mem); /* also releases the adjoint and backward memories */
    if (r->LSB) SUNLinSolFree(r->LSB);
    if (r->AB) SUNMatDestroy(r->AB);
    SUNLinSolFree(r->f.LS);
    SUNMatDestroy(r->f.A);
    N_VDestroy(r->f.y);
    SUNContext_Free(&r->f.ctx);
    free(r->f.Jtmp); free(r->f.dfdp); free(r->f.xS);
    free(r->J);
    free(r->dfdp);
    free(r);
}

const oracle_adjoint_ops oracle_adjoint_impl = {refadj_create, refadj_solve_f, refadj_x, refadj_nst,
                                                refadj_setup_b, refadj_run_b, refadj_get_b,
                                                refadj_reinit_b, refadj_nst_b, refadj_destroy};
