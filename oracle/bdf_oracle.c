/*
 * CPU oracle for the batched stiff-ODE path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's forward simulation path for ODE
 * models: AMICI's output loop with a stop time at every output
 * (src/forwardproblem.cpp:53-151, src/solver.cpp:141-160) around CVODES'
 * variable-order BDF integrator (ThirdParty/sundials/src/cvodes/cvodes.c),
 * modified Newton with a dense LU of M = I - gamma*J
 * (sunnonlinsol/newton/sunnonlinsol_newton.c:176-335, cvodes/cvodes_nls.c,
 * cvodes/cvodes_ls.c:1611-1860, sundials/sundials_dense.c:82-175), staggered
 * forward sensitivities (cvodes.c:7167-7218, cvodes/cvodes_nls_stg.c) and the
 * Gaussian log-likelihood of ReturnData (amici_glue.c).
 *
 * Used by the tests, the smoke check and the CPU-baseline leg of the
 * benchmark to check results; the product path never calls it.  Its parity is
 * pinned by golden vectors produced by the reference's own CVODES (compiled
 * from the reference sources by oracle/Makefile.ref) on the same inputs.
 *
 * Not restated (not exercised by the workloads): root finding/events, Adams
 * methods, constraints, projection.
 */
#include "bdf_oracle.h"
#include "oracle_adjoint.h"
#include "oracle_integrator.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants: cvodes_impl.h:55-135,178-204; cvodes.c:280-305 ---------- */
#define QMAX 5
#define LMAX (QMAX + 1)
#define ETA_MIN_FX 0.0
#define ETA_MAX_FX 1.5
#define ETA_MAX_FS 10000.0
#define ETA_MAX_ES 10.0
#define ETA_MAX_GS 10.0
#define ETA_MIN 0.1
#define ETA_MAX_EF 0.2
#define ETA_MIN_EF 0.1
#define ETA_CF 0.25
#define SMALL_NST 10
#define SMALL_NEF 2
#define ONEPSM 1.000001
#define ADDON 0.000001
#define BIAS1 6.0
#define BIAS2 6.0
#define BIAS3 10.0
#define LONG_WAIT 10
#define MXNEF 7
#define MXNEF1 3
#define CRDOWN 0.3
#define RDIV 2.0
#define FUZZ_FACTOR 100.0
#define HLB_FACTOR 100.0
#define HUB_FACTOR 0.1
#define H_BIAS 0.5
#define MAX_ITERS 4
#define CORTES 0.1
#define MSBP 20
#define DGMAX_LSETUP 0.3
#define MSBJ 51         /* cvodes_ls_impl.h:40 */
#define DGMAX_JBAD 0.2  /* cvodes_ls_impl.h:41 */
#define UROUND DBL_EPSILON

/* return codes (cvodes.h / cvodes_impl.h) */
#define CV_SUCCESS 0
#define CV_TSTOP_RETURN 1
#define CV_TOO_MUCH_WORK (-1)
#define CV_TOO_MUCH_ACC (-2)
#define CV_ERR_FAILURE (-3)
#define CV_CONV_FAILURE (-4)
#define CV_LSETUP_FAIL (-6)
#define CV_ILL_INPUT (-22)
#define CV_ROOT_RETURN 2
/* cvRcheck* results (cvodes.c:227-238) */
#define RTFOUND 1
#define CLOSERT 3
#define CV_TOO_CLOSE (-27)
#define DO_ERROR_TEST 2
#define PREDICT_AGAIN 3
#define TRY_AGAIN 5
#define FIRST_CALL 6
#define PREV_CONV_FAIL 7
#define PREV_ERR_FAIL 9
#define NLS_CONV_RECVR 901
#define NLS_CONTINUE 902
#define CV_NO_FAILURES 0
#define CV_FAIL_BAD_J 1
#define CV_FAIL_OTHER 2

typedef struct {
    const oracle_model* m;
    const double *p, *k;
    int n, ns;
    const int32_t* plist;
    double rtol, atol, rtolS, atolS;
    int maxcor, maxncf, lu_f32;
    double hmin, hmax_inv;
    /* Nordsieck history and work vectors */
    double* zn[LMAX];
    double *ewt, *acor, *tempv, *ftemp, *y;
    /* sensitivities: znS[j][is*n + i] */
    double* znS[LMAX];
    double *ewtS, *acorS, *tempvS, *ftempS, *yS;
    double *savedJ, *M, *Jtmp, *dfdp;
    float* Mf;
    int* piv;
    /* scalars */
    double tn, h, hprime, hscale, eta, etamax, hu, h0u;
    double tau[LMAX + 1], l[LMAX], tq[6];
    double rl1, gamma, gammap, gamrat, crate, crateS, delp, acnrm, acnrmS;
    double saved_tq5, etaqm1, etaq, etaqp1, tstop;
    int q, qprime, qwait, L, indx_acor, convfail, jcur, tstopset;
    int jcur_nls, jcur_stg; /* NEWTON_CONTENT(NLS)->jcur of the state / staggered solvers */
    int64_t nst, nstlp, nstlj, nscon;
    /* stability-limit detection (CVodeSetStabLimDet): scaled derivative
     * norms of the last five steps, ssdat[i][k] with i = 1 the newest and
     * k = 1, 2, 3 for the orders q-1, q, q+1 (cvodes_impl.h cv_ssdat) */
    int sldeton;
    double ssdat[6][4];
    int64_t nor;
    oracle_stats st;
    double* buf;
    /* quadratures (the backward problem's xQB): znQ[j][nq] */
    int nq, errconQ, qu;
    double rtolQ, atolQ, acnrmQ, tretlast;
    double* znQ[LMAX];
    double *ewtQ, *acorQ, *tempvQ, *yQ;
    /* adjoint: the backward problem evaluates its right-hand sides at the
     * forward solution interpolated from the stored steps */
    struct asa_mem* adj;
    /* forward run with adjoint storage: called after every step */
    void (*store)(struct asa_mem* a, const double* y, double t, int order);
    struct asa_mem* store_into;
    /* a reinitialisation after an event (CVodeSolver::reinit/sens_reinit,
     * solver_cvodes.cpp:586-616): the next solve first takes the one step of
     * reInit_post_process; called = solver_was_called_F_ */
    int force_reinit, called;
    double* sxret; /* the sensitivities of the last return */
    /* root finding (CVodeRootInit, cvodes.c:2674): nrtfn trigger functions
     * and the search state of cvRcheck1-3 / cvRootfind; taskc 1 = ONE_STEP */
    int nrtfn, irfnd, taskc;
    double *glo, *ghi, *grout, *yret;
    int *iroots, *gactive;
    double tlo, thi, trout, ttol, toutc;
} cvmem;

/* Interpolation data of the forward run (cvodea.c: dt_mem with
 * CVpolynomialDataMem, CVAfindIndex :2548, CVApolynomialGetY :3270) and the
 * context of the backward right-hand sides. */
typedef struct asa_mem {
    const oracle_model* m;
    const double *p, *k;
    const int32_t* plist;
    int n, nplist;
    int64_t np, cap;       /* stored points, capacity */
    double* t;             /* [cap] */
    double* y;             /* [cap * n] */
    int* order;            /* [cap] */
    int64_t ilast;
    int newdata;
    double T[LMAX];
    double* Y;             /* [LMAX * n] divided differences */
    double *xt, *J, *dfdp; /* interpolated state, Jacobian and dxdot/dp work */
} asa_mem;

static void asa_get_y(asa_mem* a, double t, double* y);

/* SUNRpowerR / SUNRpowerI (sundials_math.c:25-51) */
static double powr(double base, double e) { return base <= 0.0 ? 0.0 : pow(base, e); }
static double powi(double base, int e) {
    double prod = 1.0;
    for (int i = 1; i <= e; i++) prod *= base;
    return prod;
}

/* ---- vector helpers (nvector_serial semantics) ------------------------- */
static double wrms(int n, const double* v, const double* w) {
    double s = 0.0;
    for (int i = 0; i < n; i++) { double t = v[i] * w[i]; s += t * t; }
    return sqrt(s / n);
}

/* cvSensNorm: maximum over sensitivity WRMS norms (cvodes.c cvSensNorm) */
static double sens_norm(const cvmem* c, const double* vS, const double* wS) {
    double nrm = 0.0;
    for (int is = 0; is < c->ns; is++) {
        double v = wrms(c->n, vS + (size_t)is * c->n, wS + (size_t)is * c->n);
        if (is == 0 || v > nrm) nrm = v;
    }
    return nrm;
}

/* cvEwtSetSS (cvodes.c:9118): w = 1/(rtol*|y| + atol) */
static int ewt_set(int n, double rtol, double atol, const double* y, double* w) {
    for (int i = 0; i < n; i++) {
        double t = rtol * fabs(y[i]) + atol;
        if (t <= 0.0) return -1;
        w[i] = 1.0 / t;
    }
    return 0;
}

static int sens_ewt_set(cvmem* c, const double* yS, double* wS) {
    for (int is = 0; is < c->ns; is++)
        if (ewt_set(c->n, c->rtolS, c->atolS, yS + (size_t)is * c->n, wS + (size_t)is * c->n))
            return -1;
    return 0;
}

static void rhs(cvmem* c, double t, const double* y, double* f) {
    if (c->adj) { /* CVArhs (cvodea.c:3430): forward state by interpolation */
        asa_mem* a = c->adj;
        asa_get_y(a, t, a->xt);
        oracle_fxBdot(a->m, a->p, a->k, a->J, t, a->xt, y, f);
    } else {
        c->m->xdot(f, t, y, c->p, c->k);
    }
    c->st.nfe++;
}

/* quadrature right-hand side (CVArhsQ, cvodea.c:3481) */
static void rhsQ(cvmem* c, double t, const double* y, double* fq) {
    asa_mem* a = c->adj;
    asa_get_y(a, t, a->xt);
    oracle_fqBdot(a->m, a->p, a->k, a->dfdp, a->nplist, a->plist, t, a->xt, y, fq);
}

/* cvQuadUpdateNorm (cvodes.c:9360): the larger of the two, NaN-propagating like the reference */
static double upd_norm(double old_nrm, double nrm) { return (old_nrm > nrm) ? old_nrm : nrm; }

/* cvQuadEwtSetSS (cvodes.c:9177) */
static int quad_ewt_set(cvmem* c, const double* q, double* w) {
    for (int i = 0; i < c->nq; i++) {
        double t = c->rtolQ * fabs(q[i]) + c->atolQ;
        if (c->atolQ == 0.0 && t <= 0.0) return -1;
        w[i] = 1.0 / t;
    }
    return 0;
}

/* Sensitivity RHS, Model_ODE::fsxdot (src/model_ode.cpp:419-450):
 * sxdot_is = J(y) sx_is + dxdot/dp_{plist[is]} */
static void sens_rhs(cvmem* c, double t, const double* y, const double* yS, double* fS) {
    const int n = c->n;
    c->m->jac(c->Jtmp, t, y, c->p, c->k);
    c->m->dxdotdp(c->dfdp, t, y, c->p, c->k);
    for (int is = 0; is < c->ns; is++) {
        const double* s = yS + (size_t)is * n;
        double* out = fS + (size_t)is * n;
        const double* col = c->dfdp + (size_t)c->plist[is] * n;
        for (int i = 0; i < n; i++) out[i] = col[i];
        for (int j = 0; j < n; j++) {
            double sj = s[j];
            if (sj == 0.0) continue;
            const double* Jc = c->Jtmp + (size_t)j * n;
            for (int i = 0; i < n; i++) out[i] += Jc[i] * sj;
        }
    }
}

/* ---- dense LU: SUNDlsMat_denseGETRF / GETRS (sundials_dense.c:82-175) -- */
static int dense_getrf(double* a, int n, int* p) {
    for (int k = 0; k < n; k++) {
        double* colk = a + (size_t)k * n;
        int l = k;
        for (int i = k + 1; i < n; i++)
            if (fabs(colk[i]) > fabs(colk[l])) l = i;
        p[k] = l;
        if (colk[l] == 0.0) return k + 1;
        if (l != k)
            for (int i = 0; i < n; i++) {
                double t = a[(size_t)i * n + l];
                a[(size_t)i * n + l] = a[(size_t)i * n + k];
                a[(size_t)i * n + k] = t;
            }
        double mult = 1.0 / colk[k];
        for (int i = k + 1; i < n; i++) colk[i] *= mult;
        for (int j = k + 1; j < n; j++) {
            double* colj = a + (size_t)j * n;
            double akj = colj[k];
            if (akj != 0.0)
                for (int i = k + 1; i < n; i++) colj[i] -= akj * colk[i];
        }
    }
    return 0;
}

static void dense_getrs(const double* a, int n, const int* p, double* b) {
    for (int k = 0; k < n; k++) {
        int pk = p[k];
        if (pk != k) { double t = b[k]; b[k] = b[pk]; b[pk] = t; }
    }
    for (int k = 0; k < n - 1; k++) {
        const double* colk = a + (size_t)k * n;
        for (int i = k + 1; i < n; i++) b[i] -= colk[i] * b[k];
    }
    for (int k = n - 1; k > 0; k--) {
        const double* colk = a + (size_t)k * n;
        b[k] /= colk[k];
        for (int i = 0; i < k; i++) b[i] -= colk[i] * b[k];
    }
    b[0] /= a[0];
}

/* Single-precision variant: the iteration matrix factorised in float, the
 * right-hand side and the correction kept in double. */
static int dense_getrf_f(float* a, int n, int* p) {
    for (int k = 0; k < n; k++) {
        float* colk = a + (size_t)k * n;
        int l = k;
        for (int i = k + 1; i < n; i++)
            if (fabsf(colk[i]) > fabsf(colk[l])) l = i;
        p[k] = l;
        if (colk[l] == 0.0f) return k + 1;
        if (l != k)
            for (int i = 0; i < n; i++) {
                float t = a[(size_t)i * n + l];
                a[(size_t)i * n + l] = a[(size_t)i * n + k];
                a[(size_t)i * n + k] = t;
            }
        float mult = 1.0f / colk[k];
        for (int i = k + 1; i < n; i++) colk[i] *= mult;
        for (int j = k + 1; j < n; j++) {
            float* colj = a + (size_t)j * n;
            float akj = colj[k];
            if (akj != 0.0f)
                for (int i = k + 1; i < n; i++) colj[i] -= akj * colk[i];
        }
    }
    return 0;
}

static void dense_getrs_f(const float* a, int n, const int* p, double* b) {
    for (int k = 0; k < n; k++) {
        int pk = p[k];
        if (pk != k) { double t = b[k]; b[k] = b[pk]; b[pk] = t; }
    }
    for (int k = 0; k < n - 1; k++) {
        const float* colk = a + (size_t)k * n;
        for (int i = k + 1; i < n; i++) b[i] -= (double)colk[i] * b[k];
    }
    for (int k = n - 1; k > 0; k--) {
        const float* colk = a + (size_t)k * n;
        b[k] /= (double)colk[k];
        for (int i = 0; i < k; i++) b[i] -= (double)colk[i] * b[k];
    }
    b[0] /= (double)a[0];
}

/* ---- linear solver interface: cvLsSetup / cvLsSolve (cvodes_ls.c) ------ */
/* Returns 0, or 1 (recoverable: singular M).  ypred = c->y. */
static int lsetup(cvmem* c) {
    const int n = c->n;
    double dgamma = fabs(c->gamma / c->gammap - 1.0);
    int jbad = (c->nst == 0) || (c->nst >= c->nstlj + MSBJ) ||
               ((c->convfail == CV_FAIL_BAD_J) && (dgamma < DGMAX_JBAD)) ||
               (c->convfail == CV_FAIL_OTHER);
    /* cvLsLinSys (cvodes_ls.c:1386): reuse the saved Jacobian if jok */
    if (!jbad) {
        c->jcur = 0;
    } else {
        if (c->adj) { /* backward Jacobian -J^T at the interpolated forward state */
            asa_mem* a = c->adj;
            asa_get_y(a, c->tn, a->xt);
            oracle_fJB(a->m, a->p, a->k, a->J, c->tn, a->xt, c->savedJ);
        } else {
            c->m->jac(c->savedJ, c->tn, c->y, c->p, c->k);
        }
        c->st.nje++;
        c->jcur = 1;
        c->nstlj = c->nst;
    }
    int ret;
    if (c->lu_f32) {
        for (size_t e = 0; e < (size_t)n * n; e++) c->Mf[e] = (float)(-c->gamma * c->savedJ[e]);
        for (int i = 0; i < n; i++) c->Mf[(size_t)i * n + i] += 1.0f;
        ret = dense_getrf_f(c->Mf, n, c->piv);
    } else {
        for (size_t e = 0; e < (size_t)n * n; e++) c->M[e] = -c->gamma * c->savedJ[e];
        for (int i = 0; i < n; i++) c->M[(size_t)i * n + i] += 1.0;
        ret = dense_getrf(c->M, n, c->piv);
    }
    /* cvNlsLSetup (cvodes_nls.c:244-275) bookkeeping */
    c->st.nsetups++;
    c->gamrat = 1.0;
    c->gammap = c->gamma;
    c->crate = 1.0;
    c->crateS = 1.0;
    c->nstlp = c->nst;
    return ret > 0 ? 1 : 0;
}

static void lsolve(cvmem* c, double* b) {
    if (c->lu_f32) dense_getrs_f(c->Mf, c->n, c->piv, b);
    else dense_getrs(c->M, c->n, c->piv, b);
    if (c->gamrat != 1.0) { /* cvodes_ls.c:1851-1853 */
        double s = 2.0 / (1.0 + c->gamrat);
        for (int i = 0; i < c->n; i++) b[i] *= s;
    }
}

/* ---- BDF coefficient management (cvodes.c:6112-6894) ------------------ */
static void rescale(cvmem* c) {
    const int n = c->n;
    double f = c->eta;
    for (int j = 1; j <= c->q; j++, f *= c->eta) {
        for (int i = 0; i < n; i++) c->zn[j][i] *= f;
        for (int e = 0; e < n * c->ns; e++) c->znS[j][e] *= f;
        for (int e = 0; e < c->nq; e++) c->znQ[j][e] *= f;
    }
    c->h = c->hscale * c->eta;
    c->hscale = c->h;
    c->nscon = 0;
}

static void increase_bdf(cvmem* c) {
    const int n = c->n;
    double alpha0, alpha1, prod, xi, xiold, hsum, A1;
    for (int i = 0; i <= QMAX; i++) c->l[i] = 0.0;
    c->l[2] = alpha1 = prod = xiold = 1.0;
    alpha0 = -1.0;
    hsum = c->hscale;
    if (c->q > 1) {
        for (int j = 1; j < c->q; j++) {
            hsum += c->tau[j + 1];
            xi = hsum / c->hscale;
            prod *= xi;
            alpha0 -= 1.0 / (j + 1);
            alpha1 += 1.0 / xi;
            for (int i = j + 2; i >= 2; i--) c->l[i] = c->l[i] * xiold + c->l[i - 1];
            xiold = xi;
        }
    }
    A1 = (-alpha0 - alpha1) / prod;
    const int L = c->L;
    for (int i = 0; i < n; i++) c->zn[L][i] = A1 * c->zn[c->indx_acor][i];
    for (int e = 0; e < n * c->ns; e++) c->znS[L][e] = A1 * c->znS[c->indx_acor][e];
    for (int e = 0; e < c->nq; e++) c->znQ[L][e] = A1 * c->znQ[c->indx_acor][e];
    for (int j = 2; j <= c->q; j++) {
        for (int i = 0; i < n; i++) c->zn[j][i] += c->l[j] * c->zn[L][i];
        for (int e = 0; e < n * c->ns; e++) c->znS[j][e] += c->l[j] * c->znS[L][e];
        for (int e = 0; e < c->nq; e++) c->znQ[j][e] += c->l[j] * c->znQ[L][e];
    }
}

static void decrease_bdf(cvmem* c) {
    const int n = c->n;
    double hsum, xi;
    for (int i = 0; i <= QMAX; i++) c->l[i] = 0.0;
    c->l[2] = 1.0;
    hsum = 0.0;
    for (int j = 1; j <= c->q - 2; j++) {
        hsum += c->tau[j];
        xi = hsum / c->hscale;
        for (int i = j + 2; i >= 2; i--) c->l[i] = c->l[i] * xi + c->l[i - 1];
    }
    for (int j = 2; j < c->q; j++) {
        for (int i = 0; i < n; i++) c->zn[j][i] += -c->l[j] * c->zn[c->q][i];
        for (int e = 0; e < n * c->ns; e++) c->znS[j][e] += -c->l[j] * c->znS[c->q][e];
        for (int e = 0; e < c->nq; e++) c->znQ[j][e] += -c->l[j] * c->znQ[c->q][e];
    }
}

static void adjust_order(cvmem* c, int dq) {
    if (c->q == 2 && dq != 1) return; /* cvAdjustOrder (cvodes.c:6134) */
    if (dq == 1) increase_bdf(c);
    else if (dq == -1) decrease_bdf(c);
}

static void adjust_params(cvmem* c) {
    if (c->qprime != c->q) {
        adjust_order(c, c->qprime - c->q);
        c->q = c->qprime;
        c->L = c->q + 1;
        c->qwait = c->L;
    }
    rescale(c);
}

static void predict(cvmem* c) {
    const int n = c->n;
    c->tn += c->h;
    if (c->tstopset && (c->tn - c->tstop) * c->h > 0.0) c->tn = c->tstop;
    for (int k = 1; k <= c->q; k++)
        for (int j = c->q; j >= k; j--) {
            for (int i = 0; i < n; i++) c->zn[j - 1][i] += c->zn[j][i];
            for (int e = 0; e < n * c->ns; e++) c->znS[j - 1][e] += c->znS[j][e];
            for (int e = 0; e < c->nq; e++) c->znQ[j - 1][e] += c->znQ[j][e];
        }
}

static void restore(cvmem* c, double saved_t) {
    const int n = c->n;
    c->tn = saved_t;
    for (int k = 1; k <= c->q; k++)
        for (int j = c->q; j >= k; j--) {
            for (int i = 0; i < n; i++) c->zn[j - 1][i] -= c->zn[j][i];
            for (int e = 0; e < n * c->ns; e++) c->znS[j - 1][e] -= c->znS[j][e];
            for (int e = 0; e < c->nq; e++) c->znQ[j - 1][e] -= c->znQ[j][e];
        }
}

static void set_bdf(cvmem* c) {
    double alpha0, alpha0_hat, xi_inv, xistar_inv, hsum;
    c->l[0] = c->l[1] = xi_inv = xistar_inv = 1.0;
    for (int i = 2; i <= c->q; i++) c->l[i] = 0.0;
    alpha0 = alpha0_hat = -1.0;
    hsum = c->h;
    if (c->q > 1) {
        for (int j = 2; j < c->q; j++) {
            hsum += c->tau[j - 1];
            xi_inv = c->h / hsum;
            alpha0 -= 1.0 / j;
            for (int i = j; i >= 1; i--) c->l[i] += c->l[i - 1] * xi_inv;
        }
        alpha0 -= 1.0 / c->q;
        xistar_inv = -c->l[1] - alpha0;
        hsum += c->tau[c->q - 1];
        xi_inv = c->h / hsum;
        alpha0_hat = -c->l[1] - xi_inv;
        for (int i = c->q; i >= 1; i--) c->l[i] += c->l[i - 1] * xistar_inv;
    }
    /* cvSetTqBDF (cvodes.c:6848) */
    double A1 = 1.0 - alpha0_hat + alpha0;
    double A2 = 1.0 + c->q * A1;
    c->tq[2] = fabs(A1 / (alpha0 * A2));
    c->tq[5] = fabs(A2 * xistar_inv / (c->l[c->q] * xi_inv));
    if (c->qwait == 1) {
        if (c->q > 1) {
            double C = xistar_inv / c->l[c->q];
            double A3 = alpha0 + 1.0 / c->q;
            double A4 = alpha0_hat + xi_inv;
            double Cpinv = (1.0 - A4 + A3) / A3;
            c->tq[1] = fabs(C * Cpinv);
        } else {
            c->tq[1] = 1.0;
        }
        hsum += c->tau[c->q];
        xi_inv = c->h / hsum;
        double A5 = alpha0 - (1.0 / (c->q + 1));
        double A6 = alpha0_hat - xi_inv;
        double Cppinv = (1.0 - A6 + A5) / A2;
        c->tq[3] = fabs(Cppinv / (xi_inv * (c->q + 2) * A5));
    }
    c->tq[4] = CORTES / c->tq[2];
}

static void cv_set(cvmem* c) { /* cvSet (cvodes.c:6617) */
    set_bdf(c);
    c->rl1 = 1.0 / c->l[1];
    c->gamma = c->h * c->rl1;
    if (c->nst == 0) c->gammap = c->gamma;
    c->gamrat = (c->nst > 0) ? c->gamma / c->gammap : 1.0;
}

/* ---- nonlinear solves -------------------------------------------------- */
/* state residual cvNlsResidual (cvodes_nls.c:353): res = rl1*zn1 + ycor - gamma*f(zn0+ycor) */
static void nls_residual(cvmem* c, const double* ycor, double* res) {
    for (int i = 0; i < c->n; i++) c->y[i] = c->zn[0][i] + ycor[i];
    rhs(c, c->tn, c->y, c->ftemp);
    for (int i = 0; i < c->n; i++)
        res[i] = (c->rl1 * c->zn[1][i] + ycor[i]) + (-c->gamma) * c->ftemp[i];
}

/* cvNlsConvTest (cvodes_nls.c:303-350) */
static int nls_convtest(cvmem* c, int m, const double* ycor, const double* delta) {
    double del = wrms(c->n, delta, c->ewt);
    if (m > 0) c->crate = fmax(CRDOWN * c->crate, del / c->delp);
    double dcon = del * fmin(1.0, c->crate) / c->tq[4];
    if (dcon <= 1.0) {
        c->acnrm = (m == 0) ? del : wrms(c->n, ycor, c->ewt);
        return CV_SUCCESS;
    }
    if (m >= 1 && del > RDIV * c->delp) return NLS_CONV_RECVR;
    c->delp = del;
    return NLS_CONTINUE;
}

/* cvNls + SUNNonlinSolSolve_Newton for the state (acor is the correction). */
static int cv_nls(cvmem* c, int nflag) {
    const int n = c->n;
    c->convfail = ((nflag == FIRST_CALL) || (nflag == PREV_ERR_FAIL)) ? CV_NO_FAILURES : CV_FAIL_OTHER;
    int callSetup = (nflag == PREV_CONV_FAIL) || (nflag == PREV_ERR_FAIL) || (c->nst == 0) ||
                    (c->nst >= c->nstlp + MSBP) || (fabs(c->gamrat - 1.0) > DGMAX_LSETUP);
    double* ycor = c->acor;
    double* delta = c->tempv;
    memset(ycor, 0, sizeof(double) * n);
    int jbad = 0, retval;
    for (;;) {
        int curiter = 0;
        nls_residual(c, ycor, delta);
        if (callSetup) {
            if (jbad) c->convfail = CV_FAIL_BAD_J;
            retval = lsetup(c);
            c->jcur_nls = c->jcur;
            if (retval != 0) return NLS_CONV_RECVR; /* newton.c:231-233 */
        }
        for (;;) {
            c->st.nni++;
            for (int i = 0; i < n; i++) delta[i] = -delta[i];
            lsolve(c, delta);
            for (int i = 0; i < n; i++) ycor[i] += delta[i];
            retval = nls_convtest(c, curiter, ycor, delta);
            curiter++;
            if (retval == CV_SUCCESS) {
                /* cvNls tail (cvodes.c:6985-7001) */
                for (int i = 0; i < n; i++) c->y[i] = c->zn[0][i] + ycor[i];
                c->jcur = 0;
                c->jcur_nls = 0;
                return CV_SUCCESS;
            }
            if (retval != NLS_CONTINUE) break;
            if (curiter >= c->maxcor) { retval = NLS_CONV_RECVR; break; }
            nls_residual(c, ycor, delta);
        }
        if (retval == NLS_CONV_RECVR && !c->jcur_nls) {
            callSetup = 1;
            jbad = 1;
            memset(ycor, 0, sizeof(double) * n);
            continue;
        }
        break;
    }
    return retval;
}

/* staggered sensitivity residual cvNlsResidualSensStg (cvodes_nls_stg.c:376) */
static void stg_residual(cvmem* c, const double* ycorS, double* resS) {
    const int n = c->n, ne = c->n * c->ns;
    for (int e = 0; e < ne; e++) c->yS[e] = c->znS[0][e] + ycorS[e];
    sens_rhs(c, c->tn, c->y, c->yS, c->ftempS);
    for (int e = 0; e < ne; e++)
        resS[e] = c->rl1 * c->znS[1][e] + ycorS[e] + (-c->gamma) * c->ftempS[e];
    (void)n;
}

/* cvNlsConvTestSensStg (cvodes_nls_stg.c:332-372) */
static int stg_convtest(cvmem* c, int m, const double* ycorS, const double* deltaS) {
    double Del = sens_norm(c, deltaS, c->ewtS);
    if (m > 0) c->crateS = fmax(CRDOWN * c->crateS, Del / c->delp);
    double dcon = Del * fmin(1.0, c->crateS) / c->tq[4];
    if (dcon <= 1.0) {
        c->acnrmS = (m == 0) ? Del : sens_norm(c, ycorS, c->ewtS);
        return CV_SUCCESS;
    }
    if (m >= 1 && Del > RDIV * c->delp) return NLS_CONV_RECVR;
    c->delp = Del;
    return NLS_CONTINUE;
}

/* cvStgrNls (cvodes.c:7167-7218) with the Newton driver; callSetup = false */
static int stgr_nls(cvmem* c) {
    const int n = c->n, ne = c->n * c->ns;
    double* ycorS = c->acorS;
    double* deltaS = c->tempvS;
    memset(ycorS, 0, sizeof(double) * ne);
    int callSetup = 0, jbad = 0, retval;
    for (;;) {
        int curiter = 0;
        stg_residual(c, ycorS, deltaS);
        if (callSetup) {
            if (jbad) c->convfail = CV_FAIL_BAD_J;
            retval = lsetup(c);
            c->jcur_stg = c->jcur;
            if (retval != 0) return NLS_CONV_RECVR;
        }
        for (;;) {
            for (int e = 0; e < ne; e++) deltaS[e] = -deltaS[e];
            for (int is = 0; is < c->ns; is++) lsolve(c, deltaS + (size_t)is * n);
            for (int e = 0; e < ne; e++) ycorS[e] += deltaS[e];
            retval = stg_convtest(c, curiter, ycorS, deltaS);
            curiter++;
            if (retval == CV_SUCCESS) {
                for (int e = 0; e < ne; e++) c->yS[e] = c->znS[0][e] + ycorS[e];
                c->jcur = 0;
                c->jcur_stg = 0;
                return CV_SUCCESS;
            }
            if (retval != NLS_CONTINUE) break;
            if (curiter >= c->maxcor) { retval = NLS_CONV_RECVR; break; }
            stg_residual(c, ycorS, deltaS);
        }
        if (retval == NLS_CONV_RECVR && !c->jcur_stg) {
            callSetup = 1;
            jbad = 1;
            memset(ycorS, 0, sizeof(double) * ne);
            continue;
        }
        break;
    }
    return retval;
}

/* cvHandleNFlag (cvodes.c:7309-7371) */
static int handle_nflag(cvmem* c, int* nflag, double saved_t, int* ncf, int64_t* ncfn) {
    if (*nflag == CV_SUCCESS) return DO_ERROR_TEST;
    (*ncfn)++;
    restore(c, saved_t);
    (*ncf)++;
    c->etamax = 1.0;
    if (fabs(c->h) <= c->hmin * ONEPSM || *ncf == c->maxncf) return CV_CONV_FAILURE;
    c->eta = fmax(ETA_CF, c->hmin / fabs(c->h));
    *nflag = PREV_CONV_FAIL;
    rescale(c);
    return PREDICT_AGAIN;
}

/* cvDoErrorTest (cvodes.c:7461-7632) */
static int do_error_test(cvmem* c, int* nflag, double saved_t, double acor_nrm, int* nef,
                         int64_t* netf, double* dsmp) {
    const int n = c->n;
    double dsm = acor_nrm * c->tq[2];
    *dsmp = dsm;
    if (dsm <= 1.0) return CV_SUCCESS;
    (*nef)++;
    (*netf)++;
    *nflag = PREV_ERR_FAIL;
    restore(c, saved_t);
    if (fabs(c->h) <= c->hmin * ONEPSM || *nef == MXNEF) return CV_ERR_FAILURE;
    c->etamax = 1.0;
    if (*nef <= MXNEF1) {
        c->eta = 1.0 / (powr(BIAS2 * dsm, 1.0 / c->L) + ADDON);
        c->eta = fmax(ETA_MIN_EF, fmax(c->eta, c->hmin / fabs(c->h)));
        if (*nef >= SMALL_NEF) c->eta = fmin(c->eta, ETA_MAX_EF);
        rescale(c);
        return TRY_AGAIN;
    }
    if (c->q > 1) {
        c->eta = fmax(ETA_MIN_EF, c->hmin / fabs(c->h));
        adjust_order(c, -1);
        c->L = c->q;
        c->q--;
        c->qwait = c->L;
        rescale(c);
        return TRY_AGAIN;
    }
    c->eta = fmax(ETA_MIN_EF, c->hmin / fabs(c->h));
    c->h *= c->eta;
    c->hscale = c->h;
    c->qwait = LONG_WAIT;
    c->nscon = 0;
    rhs(c, c->tn, c->zn[0], c->tempv);
    for (int i = 0; i < n; i++) c->zn[1][i] = c->h * c->tempv[i];
    if (c->nq) { /* cvodes.c:7559-7568 */
        rhsQ(c, c->tn, c->zn[0], c->tempvQ);
        for (int e = 0; e < c->nq; e++) c->znQ[1][e] = c->h * c->tempvQ[e];
    }
    if (c->ns > 0) {
        sens_rhs(c, c->tn, c->zn[0], c->znS[0], c->tempvS);
        for (int e = 0; e < n * c->ns; e++) c->znS[1][e] = c->h * c->tempvS[e];
    }
    return TRY_AGAIN;
}

/* cvCompleteStep (cvodes.c:7634-7745) */
static void complete_step(cvmem* c) {
    const int n = c->n, ne = c->n * c->ns;
    c->nst++;
    c->nscon++;
    c->hu = c->h;
    c->qu = c->q;
    for (int i = c->q; i >= 2; i--) c->tau[i] = c->tau[i - 1];
    if (c->q == 1 && c->nst > 1) c->tau[2] = c->tau[1];
    c->tau[1] = c->h;
    for (int j = 0; j <= c->q; j++) {
        for (int i = 0; i < n; i++) c->zn[j][i] += c->l[j] * c->acor[i];
        for (int e = 0; e < ne; e++) c->znS[j][e] += c->l[j] * c->acorS[e];
        for (int e = 0; e < c->nq; e++) c->znQ[j][e] += c->l[j] * c->acorQ[e];
    }
    c->qwait--;
    if (c->qwait == 1 && c->q != QMAX) {
        memcpy(c->zn[QMAX], c->acor, sizeof(double) * n);
        if (c->nq) memcpy(c->znQ[QMAX], c->acorQ, sizeof(double) * c->nq);
        if (ne) memcpy(c->znS[QMAX], c->acorS, sizeof(double) * ne);
        c->saved_tq5 = c->tq[5];
        c->indx_acor = QMAX;
    }
}

static void set_eta(cvmem* c) { /* cvSetEta (cvodes.c:7798) */
    if (c->eta > ETA_MIN_FX && c->eta < ETA_MAX_FX) {
        c->eta = 1.0;
        c->hprime = c->h;
    } else {
        if (c->eta >= ETA_MAX_FX) {
            c->eta = fmin(c->eta, c->etamax);
            c->eta /= fmax(1.0, fabs(c->h) * c->hmax_inv * c->eta);
        } else {
            c->eta = fmax(c->eta, ETA_MIN);
            c->eta = fmax(c->eta, c->hmin / fabs(c->h));
        }
        c->hprime = c->h * c->eta;
        if (c->qprime < c->q) c->nscon = 0;
    }
}

static double compute_etaqm1(cvmem* c) {
    c->etaqm1 = 0.0;
    if (c->q > 1) {
        double ddn = wrms(c->n, c->zn[c->q], c->ewt);
        if (c->nq && c->errconQ) ddn = upd_norm(ddn, wrms(c->nq, c->znQ[c->q], c->ewtQ));
        if (c->ns > 0) ddn = fmax(ddn, sens_norm(c, c->znS[c->q], c->ewtS));
        ddn *= c->tq[1];
        c->etaqm1 = 1.0 / (powr(BIAS1 * ddn, 1.0 / c->q) + ADDON);
    }
    return c->etaqm1;
}

static double compute_etaqp1(cvmem* c) {
    const int n = c->n, ne = c->n * c->ns;
    c->etaqp1 = 0.0;
    if (c->q != QMAX) {
        if (c->saved_tq5 == 0.0) return c->etaqp1;
        double cquot = (c->tq[5] / c->saved_tq5) * powi(c->h / c->tau[2], c->L);
        for (int i = 0; i < n; i++) c->tempv[i] = -cquot * c->zn[QMAX][i] + c->acor[i];
        double dup = wrms(n, c->tempv, c->ewt);
        if (c->nq && c->errconQ) {
            for (int e = 0; e < c->nq; e++) c->tempvQ[e] = -cquot * c->znQ[QMAX][e] + c->acorQ[e];
            dup = upd_norm(dup, wrms(c->nq, c->tempvQ, c->ewtQ));
        }
        if (ne) {
            for (int e = 0; e < ne; e++) c->tempvS[e] = -cquot * c->znS[QMAX][e] + c->acorS[e];
            dup = fmax(dup, sens_norm(c, c->tempvS, c->ewtS));
        }
        dup *= c->tq[3];
        c->etaqp1 = 1.0 / (powr(BIAS3 * dup, 1.0 / (c->L + 1)) + ADDON);
    }
    return c->etaqp1;
}

static void choose_eta(cvmem* c) {
    double etam = fmax(c->etaqm1, fmax(c->etaq, c->etaqp1));
    if (etam > ETA_MIN_FX && etam < ETA_MAX_FX) {
        c->eta = 1.0;
        c->qprime = c->q;
        return;
    }
    if (etam == c->etaq) {
        c->eta = c->etaq;
        c->qprime = c->q;
    } else if (etam == c->etaqm1) {
        c->eta = c->etaqm1;
        c->qprime = c->q - 1;
    } else {
        c->eta = c->etaqp1;
        c->qprime = c->q + 1;
        memcpy(c->zn[QMAX], c->acor, sizeof(double) * c->n);
        if (c->nq && c->errconQ) memcpy(c->znQ[QMAX], c->acorQ, sizeof(double) * c->nq);
        if (c->ns) memcpy(c->znS[QMAX], c->acorS, sizeof(double) * c->n * c->ns);
    }
}

static void prepare_next_step(cvmem* c, double dsm) { /* cvodes.c:7747 */
    if (c->etamax == 1.0) {
        c->qwait = c->qwait > 2 ? c->qwait : 2;
        c->qprime = c->q;
        c->hprime = c->h;
        c->eta = 1.0;
        return;
    }
    c->etaq = 1.0 / (powr(BIAS2 * dsm, 1.0 / c->L) + ADDON);
    if (c->qwait != 0) {
        c->eta = c->etaq;
        c->qprime = c->q;
        set_eta(c);
    } else {
        c->qwait = 2;
        compute_etaqm1(c);
        compute_etaqp1(c);
        choose_eta(c);
        set_eta(c);
    }
}

/* ---- BDF stability-limit detection (cvBDFStab / cvSLdet, cvodes.c:8147-8576)
 * After every step at order q >= 3 the scaled norms of the derivatives of
 * orders q-1, q and q+1 are pushed into a five-step history; once the step
 * size and order have been constant for q + 5 steps, the dominant
 * characteristic root of the method applied to the problem is estimated from
 * that history, and a root above 0.98 (the stability boundary) lowers the
 * order by one. */
#define SLD_TINY 1.0e-10
static double sld_min(double a, double b) { return a < b ? a : b; } /* SUNMIN */
static double sld_max(double a, double b) { return a > b ? a : b; } /* SUNMAX */

/* the quartic q_k(r) = c5 + r (c4 + r^2 (c2 + r c1)) of history column k */
static double sld_quartic(const double qc[6][4], int k, double r) {
    return qc[5][k] + r * (qc[4][k] + r * r * (qc[2][k] + r * qc[1][k]));
}

/* Root estimate from ss[i][k] (i = 1 newest .. 5, k = 1..3).  Returns 1..3
 * for a stable root (equal ratios; quartic; quartic with Newton
 * correction), 4..6 for the same cases with the root above the cutoff, and
 * -1..-9 when the data admit no estimate (the reference's kflag values). */
static int sl_detect(const double ss[6][4], int q) {
    const double rrcut = 0.98, vrrtol = 1.0e-4, vrrt2 = 5.0e-4, sqtol = 1.0e-3, rrtol = 1.0e-2;
    double smax[4], ssmax[4], rav[4], vrat[4], qc[6][4], qco[6][4];
    double rr;
    int kflag;
    for (int k = 1; k <= 3; k++) {
        double lo = ss[1][k], hi = 0.0;
        for (int i = 1; i <= 5; i++) {
            lo = sld_min(lo, ss[i][k]);
            hi = sld_max(hi, ss[i][k]);
        }
        if (lo < SLD_TINY * hi) return -1;
        smax[k] = hi;
        ssmax[k] = hi * hi;
        double sum = 0.0, sumsq = 0.0;
        for (int i = 1; i <= 4; i++) {
            const double r = ss[i][k] / ss[i + 1][k];
            sum = sum + r;
            sumsq = sumsq + r * r;
        }
        rav[k] = 0.25 * sum;
        vrat[k] = fabs(0.25 * sumsq - rav[k] * rav[k]);
        qc[5][k] = ss[1][k] * ss[3][k] - ss[2][k] * ss[2][k];
        qc[4][k] = ss[2][k] * ss[3][k] - ss[1][k] * ss[4][k];
        qc[3][k] = 0.0;
        qc[2][k] = ss[2][k] * ss[5][k] - ss[3][k] * ss[4][k];
        qc[1][k] = ss[4][k] * ss[4][k] - ss[3][k] * ss[5][k];
        for (int i = 1; i <= 5; i++) qco[i][k] = qc[i][k];
    }
    const double vmin = sld_min(vrat[1], sld_min(vrat[2], vrat[3]));
    const double vmax = sld_max(vrat[1], sld_max(vrat[2], vrat[3]));
    if (vmin < vrrtol * vrrtol) {
        /* nearly normal case: the three ratio sequences share one root */
        if (vmax > vrrt2 * vrrt2) return -2;
        rr = (rav[1] + rav[2] + rav[3]) / 3.0;
        double dev = 0.0;
        for (int k = 1; k <= 3; k++) dev = sld_max(dev, fabs(rav[k] - rr));
        if (dev > vrrt2) return -3;
        kflag = 1;
    } else {
        /* eliminate between the three quartics for a common root */
        if (fabs(qco[1][1]) < SLD_TINY * ssmax[1]) return -4;
        double f = qco[1][2] / qco[1][1];
        for (int i = 2; i <= 5; i++) qco[i][2] = qco[i][2] - f * qco[i][1];
        qco[1][2] = 0.0;
        f = qco[1][3] / qco[1][1];
        for (int i = 2; i <= 5; i++) qco[i][3] = qco[i][3] - f * qco[i][1];
        qco[1][3] = 0.0;
        if (fabs(qco[2][2]) < SLD_TINY * ssmax[2]) return -4;
        f = qco[2][3] / qco[2][2];
        for (int i = 3; i <= 5; i++) qco[i][3] = qco[i][3] - f * qco[i][2];
        if (fabs(qco[4][3]) < SLD_TINY * ssmax[3]) return -4;
        rr = -qco[5][3] / qco[4][3];
        if (rr < SLD_TINY || rr > 100.0) return -5;
        double qkr[4], worst = 0.0;
        for (int k = 1; k <= 3; k++) qkr[k] = sld_quartic(qc, k, rr);
        for (int k = 1; k <= 3; k++) {
            const double a = fabs(qkr[k]) / ssmax[k];
            if (a > worst) worst = a;
        }
        if (worst < sqtol) {
            kflag = 2;
        } else {
            /* up to three Newton corrections of rr, keeping the candidate
             * whose worst quartic residual is smallest */
            double best = 0.0;
            int kb = 0;
            kflag = 0;
            for (int it = 1; it <= 3; it++) {
                double cand[4], resid[4], qj[4][4];
                for (int k = 1; k <= 3; k++) {
                    const double dq = qc[4][k] + rr * rr * (3.0 * qc[2][k] + rr * 4.0 * qc[1][k]);
                    double d = 0.0;
                    if (fabs(dq) > SLD_TINY * ssmax[k]) d = -qkr[k] / dq;
                    cand[k] = rr + d;
                }
                for (int k = 1; k <= 3; k++) {
                    double w = 0.0;
                    for (int j = 1; j <= 3; j++) {
                        qj[j][k] = sld_quartic(qc, j, cand[k]);
                        const double a = fabs(qj[j][k]) / ssmax[j];
                        if (a > w) w = a;
                    }
                    resid[k] = w;
                }
                best = resid[1] + 1.0;
                for (int k = 1; k <= 3; k++)
                    if (resid[k] < best) {
                        kb = k;
                        best = resid[k];
                    }
                rr = cand[kb];
                if (best < sqtol) {
                    kflag = 3;
                    break;
                }
                for (int j = 1; j <= 3; j++) qkr[j] = qj[j][kb];
            }
            if (best > sqtol) return -6;
        }
    }
    /* given rr: the variances sigma^2_k and the root they imply must agree */
    double sigsq[4];
    for (int k = 1; k <= 3; k++) {
        const double a = ss[1][k], b = ss[2][k] * rr, c = ss[3][k] * rr * rr, d = ss[4][k] * rr * rr * rr;
        const double d1a = a - b, d1b = b - c, d1c = c - d;
        const double d2a = d1a - d1b, d2b = d1b - d1c, d3a = d2a - d2b;
        if (fabs(d1b) < SLD_TINY * smax[k]) return -7;
        const double cest = -d3a / d1b;
        if (cest < SLD_TINY || cest > 4.0) return -7;
        sigsq[k] = ss[3][k] + (d2b / cest) / (rr * rr);
    }
    if (sigsq[2] < SLD_TINY) return -8;
    const double ratp = sigsq[3] / sigsq[2], ratm = sigsq[1] / sigsq[2];
    const double qfac1 = 0.25 * (q * q - 1.0), qfac2 = 2.0 / (q - 1.0);
    const double bb = ratp * ratm - 1.0 - qfac1 * ratp;
    const double den = 1.0 - qfac2 * bb;
    if (fabs(den) < SLD_TINY) return -8;
    if (fabs(1.0 / den - rr) > rrtol) return -9;
    if (rr > rrcut && kflag >= 1 && kflag <= 3) kflag += 3;
    return kflag;
}

/* Optional record of every detector call (history, order, result) for the
 * test fixtures of the engine's detector; single-threaded runs only. */
static double* g_sld_buf = NULL;
static int64_t g_sld_cap = 0, g_sld_n = 0;

void oracle_record_stability_detector(double* buf, int64_t cap) {
    g_sld_buf = buf;
    g_sld_cap = cap;
    g_sld_n = 0;
}

int64_t oracle_stability_detector_records(void) { return g_sld_n; }

static int sl_detect_recorded(const double ss[6][4], int q) {
    const int r = sl_detect(ss, q);
    if (g_sld_buf && g_sld_n < g_sld_cap) {
        double* d = g_sld_buf + g_sld_n * 17;
        for (int i = 1; i <= 5; i++)
            for (int k = 1; k <= 3; k++) d[3 * (i - 1) + (k - 1)] = ss[i][k];
        d[15] = q;
        d[16] = r;
        g_sld_n++;
    }
    return r;
}

/* cvBDFStab: record this step's scaled derivative norms, and lower the
 * next order when a stability limit is detected */
static void bdf_stab(cvmem* c) {
    const int q = c->q;
    if (q >= 3) {
        for (int k = 1; k <= 3; k++)
            for (int i = 5; i >= 2; i--) c->ssdat[i][k] = c->ssdat[i - 1][k];
        int fact = 1;
        for (int i = 1; i <= q - 1; i++) fact *= i;
        const double sq = fact * q * (q + 1) * c->acnrm / sld_max(c->tq[5], SLD_TINY);
        const double sqm1 = fact * q * wrms(c->n, c->zn[q], c->ewt);
        const double sqm2 = fact * wrms(c->n, c->zn[q - 1], c->ewt);
        c->ssdat[1][1] = sqm2 * sqm2;
        c->ssdat[1][2] = sqm1 * sqm1;
        c->ssdat[1][3] = sq * sq;
    }
    if (c->qprime < q) {
        c->nscon = 0; /* an order decrease is already planned */
        return;
    }
    if (q >= 3 && c->nscon >= q + 5 && sl_detect_recorded(c->ssdat, q) > 3) {
        c->qprime = q - 1;
        c->eta = sld_min(c->etaqm1, c->etamax);
        c->eta = c->eta / sld_max(1.0, fabs(c->h) * c->hmax_inv * c->eta);
        c->hprime = c->h * c->eta;
        c->nor++;
    }
}

/* cvStep (cvodes.c:5800-6110) */
static int cv_step(cvmem* c) {
    int ncf = 0, nef = 0, ncfS = 0, nefS = 0, nefQ = 0, nflag, kflag, eflag;
    double dsm = 0.0, dsmS;
    if (c->nst > 0 && c->hprime != c->h) adjust_params(c);
    double saved_t = c->tn;
    nflag = FIRST_CALL;
    for (;;) {
        predict(c);
        cv_set(c);
        nflag = cv_nls(c, nflag);
        kflag = handle_nflag(c, &nflag, saved_t, &ncf, &c->st.ncfn);
        if (kflag == PREDICT_AGAIN) continue;
        if (kflag != DO_ERROR_TEST) return kflag;
        eflag = do_error_test(c, &nflag, saved_t, c->acnrm, &nef, &c->st.netf, &dsm);
        if (eflag == TRY_AGAIN) continue;
        if (eflag != CV_SUCCESS) return eflag;
        if (c->nq) { /* cvQuadNls (cvodes.c:7089) and the quadrature error test (:5909-5937) */
            ncf = nef = 0;
            rhsQ(c, c->tn, c->y, c->acorQ);
            for (int e = 0; e < c->nq; e++) c->acorQ[e] = c->h * c->acorQ[e] - c->znQ[1][e];
            for (int e = 0; e < c->nq; e++) c->acorQ[e] = c->rl1 * c->acorQ[e];
            for (int e = 0; e < c->nq; e++) c->yQ[e] = c->znQ[0][e] + c->acorQ[e];
            if (c->errconQ) {
                double dsmQ;
                c->acnrmQ = wrms(c->nq, c->acorQ, c->ewtQ);
                eflag = do_error_test(c, &nflag, saved_t, c->acnrmQ, &nefQ, &c->st.netf, &dsmQ);
                if (eflag == TRY_AGAIN) continue;
                if (eflag != CV_SUCCESS) return eflag;
                if (dsmQ > dsm) dsm = dsmQ;
            }
        }
        if (c->ns > 0) {
            ncf = nef = 0;
            rhs(c, c->tn, c->y, c->ftemp);
            nflag = stgr_nls(c);
            kflag = handle_nflag(c, &nflag, saved_t, &ncfS, &c->st.ncfnS);
            if (kflag == PREDICT_AGAIN) continue;
            if (kflag != DO_ERROR_TEST) return kflag;
            eflag = do_error_test(c, &nflag, saved_t, c->acnrmS, &nefS, &c->st.netfS, &dsmS);
            if (eflag == TRY_AGAIN) continue;
            if (eflag != CV_SUCCESS) return eflag;
            if (dsmS > dsm) dsm = dsmS;
        }
        break;
    }
    complete_step(c);
    prepare_next_step(c, dsm);
    if (c->sldeton) bdf_stab(c);
    c->etamax = (c->nst <= SMALL_NST) ? ETA_MAX_ES : ETA_MAX_GS;
    return CV_SUCCESS;
}

/* cvHin and helpers (cvodes.c:5436-5798) */
static double upper_bound_h0(cvmem* c, double tdist) {
    const int n = c->n;
    double hub_inv = 0.0;
    for (int i = 0; i < n; i++) {
        double w = 1.0 / c->ewt[i];
        double t = HUB_FACTOR * fabs(c->zn[0][i]) + w;
        double v = fabs(c->zn[1][i]) / t;
        if (v > hub_inv) hub_inv = v;
    }
    for (int e = 0; e < n * c->ns; e++) {
        double w = 1.0 / c->ewtS[e];
        double t = HUB_FACTOR * fabs(c->znS[0][e]) + w;
        double v = fabs(c->znS[1][e]) / t;
        if (v > hub_inv) hub_inv = v;
    }
    if (c->nq && c->errconQ) { /* bound from |yQ|/|yQ'| (cvodes.c:5588-5606) */
        double hubQ_inv = 0.0;
        quad_ewt_set(c, c->znQ[0], c->tempvQ);
        for (int e = 0; e < c->nq; e++) {
            double t = HUB_FACTOR * fabs(c->znQ[0][e]) + 1.0 / c->tempvQ[e];
            double v = fabs(c->znQ[1][e]) / t;
            if (v > hubQ_inv) hubQ_inv = v;
        }
        if (hubQ_inv > hub_inv) hub_inv = hubQ_inv;
    }
    double hub = HUB_FACTOR * tdist;
    if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
    return hub;
}

static double ydd_norm(cvmem* c, double hg) {
    const int n = c->n, ne = c->n * c->ns;
    for (int i = 0; i < n; i++) c->y[i] = hg * c->zn[1][i] + c->zn[0][i];
    rhs(c, c->tn + hg, c->y, c->tempv);
    /* N_VLinearSum(1/hg, tempv, -1/hg, zn1) takes the a == -b branch: (1/hg)*(tempv - zn1) */
    for (int i = 0; i < n; i++) c->tempv[i] = (1.0 / hg) * (c->tempv[i] - c->zn[1][i]);
    double nrm = wrms(n, c->tempv, c->ewt);
    if (c->nq && c->errconQ) {
        rhsQ(c, c->tn + hg, c->y, c->tempvQ);
        for (int e = 0; e < c->nq; e++) c->tempvQ[e] = (1.0 / hg) * (c->tempvQ[e] - c->znQ[1][e]);
        nrm = upd_norm(nrm, wrms(c->nq, c->tempvQ, c->ewtQ));
    }
    if (ne) {
        for (int e = 0; e < ne; e++) c->yS[e] = hg * c->znS[1][e] + c->znS[0][e];
        sens_rhs(c, c->tn + hg, c->y, c->yS, c->tempvS);
        for (int e = 0; e < ne; e++)
            c->tempvS[e] = (1.0 / hg) * (c->tempvS[e] - c->znS[1][e]);
        nrm = fmax(nrm, sens_norm(c, c->tempvS, c->ewtS));
    }
    return nrm;
}

static int cv_hin(cvmem* c, double tout) {
    double tdiff = tout - c->tn;
    if (tdiff == 0.0) return CV_TOO_CLOSE;
    int sign = tdiff > 0.0 ? 1 : -1;
    double tdist = fabs(tdiff);
    double tround = UROUND * fmax(fabs(c->tn), fabs(tout));
    if (tdist < 2.0 * tround) return CV_TOO_CLOSE;
    double hlb = HLB_FACTOR * tround;
    double hub = upper_bound_h0(c, tdist);
    double hg = sqrt(hlb * hub);
    if (hub < hlb) {
        c->h = sign == -1 ? -hg : hg;
        return CV_SUCCESS;
    }
    double hs = hg, hnew = hg, yddnrm = 0.0;
    for (int count1 = 1; count1 <= MAX_ITERS; count1++) {
        int hgOK = 0;
        for (int count2 = 1; count2 <= MAX_ITERS; count2++) {
            double hgs = hg * sign;
            yddnrm = ydd_norm(c, hgs);
            if (isfinite(yddnrm)) { hgOK = 1; break; }
            hg *= 0.2;
        }
        if (!hgOK) { hnew = hs; break; }
        hs = hg;
        hnew = (yddnrm * hub * hub > 2.0) ? sqrt(2.0 / yddnrm) : sqrt(hg * hub);
        if (count1 == MAX_ITERS) break;
        double hrat = hnew / hg;
        if (hrat > 0.5 && hrat < 2.0) break;
        if (count1 > 1 && hrat > 2.0) { hnew = hg; break; }
        hg = hnew;
    }
    double h0 = H_BIAS * hnew;
    if (h0 < hlb) h0 = hlb;
    if (h0 > hub) h0 = hub;
    if (sign == -1) h0 = -h0;
    c->h = h0;
    return CV_SUCCESS;
}

/* CVode in NORMAL mode with tstop = tout (cvodes.c:2890-3640), restricted to
 * the branches AMICI's forward loop reaches.  mxstep is the remaining step
 * budget (solver.cpp:107-119). */
static int get_dky(cvmem* c, double t, double* const* zn, int len, double* dky);

static void gfun(cvmem* c, double t, const double* y, double* g) { c->m->root(g, t, y, c->p, c->k); }

/* cvRcheck1 (cvodes.c:8576-8626): zeros of g at and near the initial point */
static void rcheck1(cvmem* c) {
    for (int i = 0; i < c->nrtfn; i++) c->iroots[i] = 0;
    c->tlo = c->tn;
    c->ttol = (fabs(c->tn) + fabs(c->h)) * UROUND * 100.0;
    gfun(c, c->tlo, c->zn[0], c->glo);
    int zroot = 0;
    for (int i = 0; i < c->nrtfn; i++)
        if (fabs(c->glo[i]) == 0.0) {
            zroot = 1;
            c->gactive[i] = 0;
        }
    if (!zroot) return;
    const double hratio = fmax(c->ttol / fabs(c->h), 0.1);
    const double smallh = hratio * c->h;
    const double tplus = c->tlo + smallh;
    for (int i = 0; i < c->n; i++) c->y[i] = c->zn[0][i] + hratio * c->zn[1][i];
    gfun(c, tplus, c->y, c->ghi);
    for (int i = 0; i < c->nrtfn; i++)
        if (!c->gactive[i] && fabs(c->ghi[i]) != 0.0) {
            c->gactive[i] = 1;
            c->glo[i] = c->ghi[i];
        }
}

/* cvRcheck2 (cvodes.c:8648-8711): exact zeros at the last root found, a
 * close pair of zeros, a new root just after it */
static int rcheck2(cvmem* c) {
    if (c->irfnd == 0) return CV_SUCCESS;
    get_dky(c, c->tlo, c->zn, c->n, c->y);
    gfun(c, c->tlo, c->y, c->glo);
    int zroot = 0;
    for (int i = 0; i < c->nrtfn; i++) c->iroots[i] = 0;
    for (int i = 0; i < c->nrtfn; i++) {
        if (!c->gactive[i]) continue;
        if (fabs(c->glo[i]) == 0.0) {
            zroot = 1;
            c->iroots[i] = 1;
        }
    }
    if (!zroot) return CV_SUCCESS;
    c->ttol = (fabs(c->tn) + fabs(c->h)) * UROUND * 100.0;
    const double smallh = (c->h > 0.0) ? c->ttol : -c->ttol;
    const double tplus = c->tlo + smallh;
    if ((tplus - c->tn) * c->h >= 0.0) {
        const double hratio = smallh / c->h;
        for (int i = 0; i < c->n; i++) c->y[i] = c->y[i] + hratio * c->zn[1][i];
    } else {
        get_dky(c, tplus, c->zn, c->n, c->y);
    }
    gfun(c, tplus, c->y, c->ghi);
    zroot = 0;
    for (int i = 0; i < c->nrtfn; i++) {
        if (!c->gactive[i]) continue;
        if (fabs(c->ghi[i]) == 0.0) {
            if (c->iroots[i] == 1) return CLOSERT;
            zroot = 1;
            c->iroots[i] = 1;
        } else if (c->iroots[i] == 1) {
            c->glo[i] = c->ghi[i];
        }
    }
    return zroot ? RTFOUND : CV_SUCCESS;
}

#define DIFFERENT_SIGN(a, b) (((a) < 0 && (b) > 0) || ((a) > 0 && (b) < 0))

/* cvRootfind (cvodes.c:8859-9060): the Illinois algorithm on (tlo, thi)
 * (no rootdir: every crossing counts) */
static int rootfind(cvmem* c) {
    const int nr = c->nrtfn;
    int imax = 0, zroot = 0, sgnchg = 0;
    double maxfrac = 0.0;
    for (int i = 0; i < nr; i++) {
        if (!c->gactive[i]) continue;
        if (fabs(c->ghi[i]) == 0.0) {
            zroot = 1;
        } else if (DIFFERENT_SIGN(c->glo[i], c->ghi[i])) {
            const double gfrac = fabs(c->ghi[i] / (c->ghi[i] - c->glo[i]));
            if (gfrac > maxfrac) {
                sgnchg = 1;
                maxfrac = gfrac;
                imax = i;
            }
        }
    }
    if (!sgnchg) {
        c->trout = c->thi;
        for (int i = 0; i < nr; i++) c->grout[i] = c->ghi[i];
        if (!zroot) return CV_SUCCESS;
        for (int i = 0; i < nr; i++) {
            c->iroots[i] = 0;
            if (!c->gactive[i]) continue;
            if (fabs(c->ghi[i]) == 0.0) c->iroots[i] = c->glo[i] > 0 ? -1 : 1;
        }
        return RTFOUND;
    }
    double alph = 1.0;
    int side = 0, sideprev = -1;
    for (;;) {
        if (fabs(c->thi - c->tlo) <= c->ttol) break;
        if (sideprev == side) alph = (side == 2) ? alph * 2.0 : alph * 0.5;
        else alph = 1.0;
        double tmid = c->thi - (c->thi - c->tlo) * c->ghi[imax] / (c->ghi[imax] - alph * c->glo[imax]);
        if (fabs(tmid - c->tlo) < 0.5 * c->ttol) {
            const double fracint = fabs(c->thi - c->tlo) / c->ttol;
            const double fracsub = (fracint > 5.0) ? 0.1 : 0.5 / fracint;
            tmid = c->tlo + fracsub * (c->thi - c->tlo);
        }
        if (fabs(c->thi - tmid) < 0.5 * c->ttol) {
            const double fracint = fabs(c->thi - c->tlo) / c->ttol;
            const double fracsub = (fracint > 5.0) ? 0.1 : 0.5 / fracint;
            tmid = c->thi - fracsub * (c->thi - c->tlo);
        }
        get_dky(c, tmid, c->zn, c->n, c->y);
        gfun(c, tmid, c->y, c->grout);
        maxfrac = 0.0;
        zroot = 0;
        sgnchg = 0;
        sideprev = side;
        for (int i = 0; i < nr; i++) {
            if (!c->gactive[i]) continue;
            if (fabs(c->grout[i]) == 0.0) {
                zroot = 1;
            } else if (DIFFERENT_SIGN(c->glo[i], c->grout[i])) {
                const double gfrac = fabs(c->grout[i] / (c->grout[i] - c->glo[i]));
                if (gfrac > maxfrac) {
                    sgnchg = 1;
                    maxfrac = gfrac;
                    imax = i;
                }
            }
        }
        if (sgnchg) {
            c->thi = tmid;
            for (int i = 0; i < nr; i++) c->ghi[i] = c->grout[i];
            side = 1;
            if (fabs(c->thi - c->tlo) <= c->ttol) break;
            continue;
        }
        if (zroot) {
            c->thi = tmid;
            for (int i = 0; i < nr; i++) c->ghi[i] = c->grout[i];
            break;
        }
        c->tlo = tmid;
        for (int i = 0; i < nr; i++) c->glo[i] = c->grout[i];
        side = 2;
        if (fabs(c->thi - c->tlo) <= c->ttol) break;
    }
    c->trout = c->thi;
    for (int i = 0; i < nr; i++) {
        c->grout[i] = c->ghi[i];
        c->iroots[i] = 0;
        if (!c->gactive[i]) continue;
        if (fabs(c->ghi[i]) == 0.0) c->iroots[i] = c->glo[i] > 0 ? -1 : 1;
        if (DIFFERENT_SIGN(c->glo[i], c->ghi[i])) c->iroots[i] = c->glo[i] > 0 ? -1 : 1;
    }
    return RTFOUND;
}

/* cvRcheck3 (cvodes.c:8725-8780): a root between tlo and tn (or tout) */
static int rcheck3(cvmem* c) {
    if (c->taskc == 1 || (c->toutc - c->tn) * c->h >= 0.0) {
        c->thi = c->tn;
        memcpy(c->y, c->zn[0], sizeof(double) * c->n);
    } else {
        c->thi = c->toutc;
        get_dky(c, c->thi, c->zn, c->n, c->y);
    }
    gfun(c, c->thi, c->y, c->ghi);
    c->ttol = (fabs(c->tn) + fabs(c->h)) * UROUND * 100.0;
    const int ier = rootfind(c);
    for (int i = 0; i < c->nrtfn; i++)
        if (!c->gactive[i] && c->grout[i] != 0.0) c->gactive[i] = 1;
    c->tlo = c->trout;
    for (int i = 0; i < c->nrtfn; i++) c->glo[i] = c->grout[i];
    if (ier == CV_SUCCESS) return CV_SUCCESS;
    get_dky(c, c->trout, c->zn, c->n, c->y);
    return RTFOUND;
}

/* CVode's first-call block with the stop time tout (cvInitialSetup, with
 * cvLsInitialize's counter reset, cvodes_ls.c:1567; cvHin; the first step
 * size bounded by hmax and the stop time; zn[1] = h f) */
static int first_call(cvmem* c, double tout) {
    const int n = c->n, ne = c->n * c->ns;
    if (ewt_set(n, c->rtol, c->atol, c->zn[0], c->ewt)) return CV_ILL_INPUT;
    if (ne && sens_ewt_set(c, c->znS[0], c->ewtS)) return CV_ILL_INPUT;
    c->nstlj = 0;
    rhs(c, c->tn, c->zn[0], c->zn[1]);
    if (ne) sens_rhs(c, c->tn, c->zn[0], c->znS[0], c->znS[1]);
    int hflag = cv_hin(c, tout);
    if (hflag != CV_SUCCESS) return CV_ILL_INPUT;
    double rh = fabs(c->h) * c->hmax_inv;
    if (rh > 1.0) c->h /= rh;
    if (fabs(c->h) < c->hmin) c->h *= c->hmin / fabs(c->h);
    if ((c->tn + c->h - c->tstop) * c->h > 0.0) c->h = (c->tstop - c->tn) * (1.0 - 4.0 * UROUND);
    c->hscale = c->h;
    c->h0u = c->h;
    c->hprime = c->h;
    for (int i = 0; i < n; i++) c->zn[1][i] *= c->h;
    for (int e = 0; e < ne; e++) c->znS[1][e] *= c->h;
    return CV_SUCCESS;
}

/* CVode(tout, NORMAL) with the stop time tout; with trigger functions the
 * root checks of cvodes.c:3179-3275,3516-3530: cvRcheck1 on the first call,
 * cvRcheck2 and cvRcheck3 on entry, cvRcheck3 after every step; a root found
 * returns CV_ROOT_RETURN with the state at the root in c->y */
static int cv_solve(cvmem* c, double tout, int64_t mxstep) {
    const int n = c->n, ne = c->n * c->ns;
    c->tstop = tout;
    c->tstopset = 1;
    c->toutc = tout;
    c->taskc = 0;
    if (c->nst == 0) {
        c->tretlast = c->tn;
        int flag = first_call(c, tout);
        if (flag != CV_SUCCESS) return flag;
        if (c->nrtfn) rcheck1(c);
    } else {
        double troundoff = FUZZ_FACTOR * UROUND * (fabs(c->tn) + fabs(c->h));
        if (c->nrtfn) {
            int r = rcheck2(c);
            if (r == CLOSERT) return CV_ILL_INPUT;
            if (r == RTFOUND) {
                c->tretlast = c->tlo;
                return CV_ROOT_RETURN;
            }
            if (fabs(c->tn - c->tretlast) > troundoff) {
                r = rcheck3(c);
                if (r == CV_SUCCESS) {
                    c->irfnd = 0;
                } else if (r == RTFOUND) {
                    c->irfnd = 1;
                    c->tretlast = c->tlo;
                    return CV_ROOT_RETURN;
                }
            }
        }
        if (fabs(c->tn - c->tstop) <= troundoff) {
            memcpy(c->y, c->zn[0], sizeof(double) * n);
            c->tretlast = c->tstop;
            c->tstopset = 0;
            return CV_TSTOP_RETURN;
        }
        if ((c->tn + c->hprime - c->tstop) * c->h > 0.0) {
            c->hprime = (c->tstop - c->tn) * (1.0 - 4.0 * UROUND);
            c->eta = c->hprime / c->h;
        }
    }
    int64_t nstloc = 0;
    for (;;) {
        if (c->nst > 0) {
            if (ewt_set(n, c->rtol, c->atol, c->zn[0], c->ewt)) return CV_ILL_INPUT;
            if (ne && sens_ewt_set(c, c->znS[0], c->ewtS)) return CV_ILL_INPUT;
        }
        if (mxstep > 0 && nstloc >= mxstep) return CV_TOO_MUCH_WORK;
        double nrm = wrms(n, c->zn[0], c->ewt);
        if (ne) nrm = fmax(nrm, sens_norm(c, c->znS[0], c->ewtS));
        if (UROUND * nrm > 1.0) return CV_TOO_MUCH_ACC;
        int kflag = cv_step(c);
        if (kflag != CV_SUCCESS) return kflag;
        nstloc++;
        double troundoff = FUZZ_FACTOR * UROUND * (fabs(c->tn) + fabs(c->h));
        if (fabs(c->tn - c->tstop) <= troundoff) c->tn = c->tstop;
        if (c->nrtfn && rcheck3(c) == RTFOUND) {
            c->irfnd = 1;
            c->tretlast = c->tlo;
            return CV_ROOT_RETURN;
        }
        /* CVodeF (cvodea.c:560-575): store the step for the interpolant */
        if (c->store) c->store(c->store_into, c->zn[0], c->tn, c->qu);
        troundoff = FUZZ_FACTOR * UROUND * (fabs(c->tn) + fabs(c->h));
        if (fabs(c->tn - c->tstop) <= troundoff) {
            memcpy(c->y, c->zn[0], sizeof(double) * n);
            c->tretlast = c->tstop;
            c->tstopset = 0;
            return CV_TSTOP_RETURN;
        }
        if ((c->tn + c->hprime - c->tstop) * c->h > 0.0) {
            c->hprime = (c->tstop - c->tn) * (1.0 - 4.0 * UROUND);
            c->eta = c->hprime / c->h;
        }
    }
}

/* ---- integrator interface used by the AMICI glue (amici_glue.c) --------- */
static void* port_create(const oracle_model* m, const oracle_options* o, const double* p,
                         const double* k, int ns, const int32_t* plist, const double* x0,
                         const double* sx0) {
    const int n = m->nx, np = m->np;
    cvmem* c = (cvmem*)calloc(1, sizeof(cvmem));
    c->m = m;
    c->p = p;
    c->k = k;
    c->n = n;
    c->ns = ns;
    c->plist = plist;
    c->rtol = o->rtol;
    c->atol = o->atol;
    c->rtolS = isnan(o->rtol_fsa) ? o->rtol : o->rtol_fsa;
    c->atolS = isnan(o->atol_fsa) ? o->atol : o->atol_fsa;
    c->maxcor = o->max_nonlin_iters > 0 ? o->max_nonlin_iters : 3;
    c->maxncf = o->max_conv_fails > 0 ? o->max_conv_fails : 10;
    c->lu_f32 = o->lu_f32;
    c->hmin = 0.0;
    c->hmax_inv = (o->max_step_size > 0.0 && isfinite(o->max_step_size)) ? 1.0 / o->max_step_size : 0.0;
    c->sldeton = o->stldet != 0;
    const size_t ne = (size_t)n * (ns > 0 ? ns : 1);
    double* w = (double*)calloc((size_t)(LMAX + 5) * n + (size_t)(LMAX + 5) * ne + 3 * (size_t)n * n +
                                    (size_t)np * n + 8, sizeof(double));
    c->buf = w;
    for (int j = 0; j < LMAX; j++) { c->zn[j] = w; w += n; }
    c->ewt = w; w += n; c->acor = w; w += n; c->tempv = w; w += n; c->ftemp = w; w += n; c->y = w; w += n;
    for (int j = 0; j < LMAX; j++) { c->znS[j] = w; w += ne; }
    c->ewtS = w; w += ne; c->acorS = w; w += ne; c->tempvS = w; w += ne; c->ftempS = w; w += ne; c->yS = w; w += ne;
    c->savedJ = w; w += (size_t)n * n; c->M = w; w += (size_t)n * n; c->Jtmp = w; w += (size_t)n * n;
    c->dfdp = w;
    c->Mf = (float*)malloc(sizeof(float) * (size_t)n * n + 4);
    c->piv = (int*)malloc(sizeof(int) * (n + 1));
    /* CVodeInit defaults (cvodes.c:800-835) */
    c->q = 1; c->L = 2; c->qwait = c->L; c->etamax = ETA_MAX_FS;
    c->tn = 0.0;
    memcpy(c->zn[0], x0, sizeof(double) * n);
    if (ns) memcpy(c->znS[0], sx0, sizeof(double) * n * ns);
    memcpy(c->y, x0, sizeof(double) * n);
    c->sxret = (double*)calloc(ne + 1, sizeof(double));
    /* trigger functions (CVodeRootInit): every function active, no direction */
    c->nrtfn = m->nroot;
    if (c->nrtfn) {
        const int nr = c->nrtfn;
        c->glo = (double*)calloc((size_t)4 * nr, sizeof(double));
        c->ghi = c->glo + nr;
        c->grout = c->ghi + nr;
        c->iroots = (int*)calloc((size_t)2 * nr, sizeof(int));
        c->gactive = c->iroots + nr;
        for (int i = 0; i < nr; i++) c->gactive[i] = 1;
    }
    return c;
}

/* CVode(tout, ONE_STEP) without a stop time (Solver::step, solver.cpp:162-178):
 * the first call sets the integrator up as cv_solve does, every call takes
 * one step and returns the state at tn */
static int port_one_step(void* h, double tout, double* tret) {
    cvmem* c = (cvmem*)h;
    const int n = c->n, ne = c->n * c->ns;
    c->tstopset = 0;
    if (c->nst == 0) {
        if (ewt_set(n, c->rtol, c->atol, c->zn[0], c->ewt)) return CV_ILL_INPUT;
        if (ne && sens_ewt_set(c, c->znS[0], c->ewtS)) return CV_ILL_INPUT;
        rhs(c, c->tn, c->zn[0], c->zn[1]);
        if (ne) sens_rhs(c, c->tn, c->zn[0], c->znS[0], c->znS[1]);
        if (cv_hin(c, tout) != CV_SUCCESS) return CV_ILL_INPUT;
        double rh = fabs(c->h) * c->hmax_inv;
        if (rh > 1.0) c->h /= rh;
        if (fabs(c->h) < c->hmin) c->h *= c->hmin / fabs(c->h);
        c->hscale = c->h;
        c->h0u = c->h;
        c->hprime = c->h;
        for (int i = 0; i < n; i++) c->zn[1][i] *= c->h;
        for (int e = 0; e < ne; e++) c->znS[1][e] *= c->h;
    } else {
        if (ewt_set(n, c->rtol, c->atol, c->zn[0], c->ewt)) return CV_ILL_INPUT;
        if (ne && sens_ewt_set(c, c->znS[0], c->ewtS)) return CV_ILL_INPUT;
    }
    double nrm = wrms(n, c->zn[0], c->ewt);
    if (ne) nrm = fmax(nrm, sens_norm(c, c->znS[0], c->ewtS));
    if (UROUND * nrm > 1.0) return CV_TOO_MUCH_ACC;
    int kflag = cv_step(c);
    *tret = c->tn;
    c->tretlast = c->tn;
    memcpy(c->y, c->zn[0], sizeof(double) * n);
    return kflag;
}

/* CVodeSolver::reInit_post_process (solver_cvodes.cpp:531-583): with the
 * step counter at 0, CVode(tout, ONE_STEP) with the stop time tout sets the
 * integrator up as on its first call and takes one step; the counter then
 * continues.  Any return but CV_SUCCESS (a stop time reached already
 * included) is a CvodeException, AMICI_ERROR (amici.cpp:156-168). */
static int reinit_post_process(cvmem* c, double tout) {
    const int n = c->n, ne = c->n * c->ns;
    const int64_t nst_tmp = c->nst;
    c->nst = 0;
    c->tstop = tout;
    c->tstopset = 1;
    c->toutc = tout;
    c->taskc = 1;
    c->tretlast = c->tn;
    int flag = first_call(c, tout);
    if (flag != CV_SUCCESS) return flag;
    if (c->nrtfn) rcheck1(c);
    double nrm = wrms(n, c->zn[0], c->ewt);
    if (ne) nrm = fmax(nrm, sens_norm(c, c->znS[0], c->ewtS));
    if (UROUND * nrm > 1.0) return CV_TOO_MUCH_ACC;
    int kflag = cv_step(c);
    if (kflag != CV_SUCCESS) return kflag;
    double troundoff = FUZZ_FACTOR * UROUND * (fabs(c->tn) + fabs(c->h));
    if (fabs(c->tn - c->tstop) <= troundoff) c->tn = c->tstop;
    if (c->nrtfn && rcheck3(c) == RTFOUND) {
        c->irfnd = 1;
        return -99; /* CV_ROOT_RETURN after a reinitialisation: AMICI throws */
    }
    if (fabs(c->tn - c->tstop) <= troundoff) {
        c->tstopset = 0;
        return -99; /* CV_TSTOP_RETURN: AMICI throws */
    }
    c->tretlast = c->tn;
    if ((c->tn + c->hprime - c->tstop) * c->h > 0.0) {
        c->hprime = (c->tstop - c->tn) * (1.0 - 4.0 * UROUND);
        c->eta = c->hprime / c->h;
    }
    c->nst = nst_tmp + 1;
    c->force_reinit = 0;
    return 0;
}

static int port_solve(void* h, double tout, int64_t mxstep, double* tret) {
    cvmem* c = (cvmem*)h;
    if (c->force_reinit) {
        /* any failure of this step is a CvodeException: AMICI_ERROR */
        if (reinit_post_process(c, tout)) {
            *tret = c->tn;
            return -99;
        }
    }
    c->called = 1;
    int flag = cv_solve(c, tout, mxstep);
    /* CV_TSTOP_RETURN reports tret = tstop (cvodes.c:3300-3306), a root
     * return the root */
    *tret = (flag == CV_TSTOP_RETURN) ? tout : (flag == CV_ROOT_RETURN ? c->tretlast : c->tn);
    return flag;
}

/* CVodeGetRootInfo: +1 / -1 for a root function that crossed zero upwards /
 * downwards at the root returned, 0 otherwise */
static void port_root_info(void* h, int* iroots) {
    cvmem* c = (cvmem*)h;
    for (int i = 0; i < c->nrtfn; i++) iroots[i] = c->iroots[i];
}

/* CVodeSolver::reinit + reset_state, and sens_reinit (solver_cvodes.cpp:
 * 471-505,586-616): time t, state x (and sensitivities sx) into the first
 * history column, order 1; the next solve takes reInit_post_process's step */
static void port_reinit(void* h, double t, const double* x, const double* sx) {
    cvmem* c = (cvmem*)h;
    c->tn = t;
    if (c->called) c->force_reinit = 1;
    c->q = 1;
    c->L = 2;
    c->qwait = c->L;
    c->qu = 0;
    c->hu = 0.0;
    c->h0u = 0.0;
    memcpy(c->zn[0], x, sizeof(double) * c->n);
    memcpy(c->y, x, sizeof(double) * c->n); /* the state reported at t is the reinitialised one */
    if (c->ns && sx) memcpy(c->znS[0], sx, sizeof(double) * c->n * c->ns);
}

/* the state of the last return (yout: at tout, at the stop time or at the
 * root) and the sensitivities there (CVodeGetSens: CVodeGetSensDky at
 * tretlast, cvodes.c:4018) */
static const double* port_x(void* h) { return ((cvmem*)h)->y; }
static const double* port_sx(void* h) {
    cvmem* c = (cvmem*)h;
    if (!c->ns || c->tretlast == c->tn) return c->znS[0];
    get_dky(c, c->tretlast, c->znS, c->n * c->ns, c->sxret);
    return c->sxret;
}
static int64_t port_nst(void* h) { return ((cvmem*)h)->nst; }
static void port_destroy(void* h) {
    cvmem* c = (cvmem*)h;
    free(c->sxret);
    if (c->nrtfn) { free(c->glo); free(c->iroots); }
    free(c->Mf); free(c->piv); free(c->buf); free(c);
}

const oracle_integrator oracle_integrator_impl = {port_create, port_solve, port_one_step, port_x,
                                                  port_sx, port_nst, port_destroy, port_reinit,
                                                  port_root_info};

/* ======================================================================== */
/* Adjoint sensitivity analysis: forward storage, interpolation, backward    */
/* problem (cvodea.c) and the solver operations AMICI's backward loop uses   */
/* (src/solver_cvodes.cpp:470-640,700-860).                                  */
/* ======================================================================== */
#define CV_BAD_T (-25)

/* CVApolynomialStorePnt (cvodea.c:3236): y = zn[0] and the order of the step */
static void asa_store(asa_mem* a, const double* y, double t, int order) {
    const int n = a->n;
    if (a->np == a->cap) {
        int64_t cap = a->cap ? 2 * a->cap : 1024;
        a->t = (double*)realloc(a->t, sizeof(double) * (size_t)cap);
        a->y = (double*)realloc(a->y, sizeof(double) * (size_t)cap * (size_t)(n > 0 ? n : 1));
        a->order = (int*)realloc(a->order, sizeof(int) * (size_t)cap);
        a->cap = cap;
    }
    a->t[a->np] = t;
    memcpy(a->y + (size_t)a->np * n, y, sizeof(double) * n);
    a->order[a->np] = order;
    a->np++;
    a->newdata = 1; /* CVodeF: ca_IMnewData = SUNTRUE */
}

/* CVAfindIndex (cvodea.c:2548) for a forward run in the positive direction */
static int asa_find_index(asa_mem* a, double t, int64_t* indx) {
    if (a->newdata) {
        a->ilast = a->np - 1;
        a->newdata = 0;
    }
    const int to_left = (t - a->t[a->ilast - 1]) < 0.0;
    const int to_right = (t - a->t[a->ilast]) > 0.0;
    if (to_left) {
        *indx = a->ilast;
        for (;;) {
            if (*indx == 0) break;
            if (t - a->t[*indx - 1] <= 0.0) (*indx)--;
            else break;
        }
        a->ilast = (*indx == 0) ? 1 : *indx;
        if (*indx == 0 && fabs(t - a->t[0]) > FUZZ_FACTOR * UROUND) return CV_BAD_T;
    } else if (to_right) {
        *indx = a->ilast;
        for (;;) {
            if (*indx < a->np - 1 && t - a->t[*indx] > 0.0) (*indx)++;
            else break;
        }
        a->ilast = *indx;
    } else {
        *indx = a->ilast;
    }
    return 0;
}

/* CVApolynomialGetY (cvodea.c:3270): Newton divided differences over the
 * order+1 stored points ending at the base point, evaluated by nested
 * products; vector operations in the order of nvector_serial. */
static void asa_get_y(asa_mem* a, double t, double* y) {
    const int n = a->n;
    int64_t indx;
    if (a->np < 2 || asa_find_index(a, t, &indx) != 0) {
        for (int i = 0; i < n; i++) y[i] = NAN;
        return;
    }
    if (indx == 0) {
        memcpy(y, a->y, sizeof(double) * n);
        return;
    }
    const double dt = fabs(a->t[indx] - a->t[indx - 1]);
    int64_t base = indx;
    const int order = a->order[base];
    if (indx < order) base += order - indx;
    double* Y = a->Y;
    for (int j = 0; j <= order; j++) {
        a->T[j] = a->t[base - j];
        memcpy(Y + (size_t)j * n, a->y + (size_t)(base - j) * n, sizeof(double) * n);
    }
    for (int i = 1; i <= order; i++)
        for (int j = order; j >= i; j--) {
            const double factor = dt / (a->T[j] - a->T[j - i]);
            double* yj = Y + (size_t)j * n;
            const double* yjm = Y + (size_t)(j - 1) * n;
            for (int e = 0; e < n; e++) yj[e] = factor * (yj[e] - yjm[e]);
        }
    double cv[LMAX + 1];
    cv[0] = 1.0;
    for (int i = 0; i < order; i++) cv[i + 1] = cv[i] * (t - a->T[i]) / dt;
    for (int e = 0; e < n; e++) y[e] = cv[0] * Y[e];
    for (int i = 1; i <= order; i++)
        for (int e = 0; e < n; e++) y[e] += cv[i] * Y[(size_t)i * n + e];
}

/* z = sum_j c_j X_j in the order of N_VLinearCombination_Serial */
static void lincomb(int nv, const double* cv, double* const* X, int n, double* z) {
    for (int e = 0; e < n; e++) z[e] = cv[0] * X[0][e];
    for (int i = 1; i < nv; i++)
        for (int e = 0; e < n; e++) z[e] += cv[i] * X[i][e];
}

/* CVodeGetDky / CVodeGetQuadDky with k = 0 (cvodes.c:3742,3864) */
static int get_dky(cvmem* c, double t, double* const* zn, int len, double* dky) {
    double tfuzz = FUZZ_FACTOR * UROUND * (fabs(c->tn) + fabs(c->hu));
    if (c->hu < 0.0) tfuzz = -tfuzz;
    const double tp = c->tn - c->hu - tfuzz, tn1 = c->tn + tfuzz;
    if ((t - tp) * (t - tn1) > 0.0) return CV_BAD_T;
    const double s = (t - c->tn) / c->h;
    double cv[LMAX];
    double* X[LMAX];
    int nv = 0;
    for (int j = c->q; j >= 0; j--) {
        double v = 1.0;
        for (int i = 0; i < j; i++) v *= s;
        cv[nv] = v;
        X[nv] = zn[j];
        nv++;
    }
    lincomb(nv, cv, X, len, dky);
    return CV_SUCCESS;
}

/* CVode(tout, itask) (cvodes.c:2890-3640) for a problem without
 * sensitivities, with quadratures and an optional stop time: the branches
 * AMICI's backward problem reaches (CVodeB in NORMAL mode with the stop
 * time at the check point, and one step in ONE_STEP mode after a reinit). */
static int cv_ode(cvmem* c, double tout, int one_step, int64_t mxstep, double* yout, double* tret) {
    const int n = c->n;
    if (c->nst == 0) {
        c->tretlast = *tret = c->tn;
        /* cvInitialSetup (cvodes.c:5140) incl. cvLsInitialize's counter reset (cvodes_ls.c:1567) */
        if (ewt_set(n, c->rtol, c->atol, c->zn[0], c->ewt)) return CV_ILL_INPUT;
        if (c->nq && c->errconQ && quad_ewt_set(c, c->znQ[0], c->ewtQ)) return CV_ILL_INPUT;
        c->nstlj = 0;
        rhs(c, c->tn, c->zn[0], c->zn[1]);
        if (c->nq) rhsQ(c, c->tn, c->zn[0], c->znQ[1]);
        if (c->tstopset && (c->tstop - c->tn) * (tout - c->tn) <= 0.0) return CV_ILL_INPUT;
        double tout_hin = tout;
        if (c->tstopset && (tout - c->tn) * (tout - c->tstop) > 0.0) tout_hin = c->tstop;
        int hflag = cv_hin(c, tout_hin);
        if (hflag != CV_SUCCESS) return hflag;
        double rh = fabs(c->h) * c->hmax_inv;
        if (rh > 1.0) c->h /= rh;
        if (fabs(c->h) < c->hmin) c->h *= c->hmin / fabs(c->h);
        if (c->tstopset && (c->tn + c->h - c->tstop) * c->h > 0.0)
            c->h = (c->tstop - c->tn) * (1.0 - 4.0 * UROUND);
        c->hscale = c->h;
        c->h0u = c->h;
        c->hprime = c->h;
        for (int i = 0; i < n; i++) c->zn[1][i] *= c->h;
        for (int e = 0; e < c->nq; e++) c->znQ[1][e] *= c->h;
    } else {
        double troundoff = FUZZ_FACTOR * UROUND * (fabs(c->tn) + fabs(c->h));
        if (c->tstopset) {
            if (fabs(c->tn - c->tstop) <= troundoff) {
                if ((tout - c->tstop) * c->h >= 0.0 || fabs(tout - c->tstop) <= troundoff) {
                    memcpy(yout, c->zn[0], sizeof(double) * n);
                    c->tretlast = *tret = c->tstop;
                    c->tstopset = 0;
                    return CV_TSTOP_RETURN;
                }
            } else if ((c->tn + c->hprime - c->tstop) * c->h > 0.0) {
                c->hprime = (c->tstop - c->tn) * (1.0 - 4.0 * UROUND);
                c->eta = c->hprime / c->h;
            }
        }
        if (!one_step && (c->tn - tout) * c->h >= 0.0) {
            c->tretlast = *tret = tout;
            return get_dky(c, tout, c->zn, n, yout) == CV_SUCCESS ? CV_SUCCESS : CV_ILL_INPUT;
        }
        if (one_step && fabs(c->tn - c->tretlast) > troundoff) {
            c->tretlast = *tret = c->tn;
            memcpy(yout, c->zn[0], sizeof(double) * n);
            return CV_SUCCESS;
        }
    }
    int64_t nstloc = 0;
    for (;;) {
        if (c->nst > 0) {
            if (ewt_set(n, c->rtol, c->atol, c->zn[0], c->ewt)) goto fail_ill;
            if (c->nq && c->errconQ && quad_ewt_set(c, c->znQ[0], c->ewtQ)) goto fail_ill;
        }
        if (mxstep > 0 && nstloc >= mxstep) {
            c->tretlast = *tret = c->tn;
            memcpy(yout, c->zn[0], sizeof(double) * n);
            return CV_TOO_MUCH_WORK;
        }
        double nrm = wrms(n, c->zn[0], c->ewt);
        if (c->nq && c->errconQ) nrm = upd_norm(nrm, wrms(c->nq, c->znQ[0], c->ewtQ));
        if (UROUND * nrm > 1.0) {
            c->tretlast = *tret = c->tn;
            memcpy(yout, c->zn[0], sizeof(double) * n);
            return CV_TOO_MUCH_ACC;
        }
        int kflag = cv_step(c);
        if (kflag != CV_SUCCESS) {
            c->tretlast = *tret = c->tn;
            memcpy(yout, c->zn[0], sizeof(double) * n);
            return kflag;
        }
        nstloc++;
        if (c->tstopset) {
            double troundoff = FUZZ_FACTOR * UROUND * (fabs(c->tn) + fabs(c->h));
            if (fabs(c->tn - c->tstop) <= troundoff) c->tn = c->tstop;
        }
        if (c->tstopset) {
            double troundoff = FUZZ_FACTOR * UROUND * (fabs(c->tn) + fabs(c->h));
            if (fabs(c->tn - c->tstop) <= troundoff) {
                if ((tout - c->tstop) * c->h >= 0.0 || fabs(tout - c->tstop) <= troundoff) {
                    memcpy(yout, c->zn[0], sizeof(double) * n);
                    c->tretlast = *tret = c->tstop;
                    c->tstopset = 0;
                    return CV_TSTOP_RETURN;
                }
            } else if ((c->tn + c->hprime - c->tstop) * c->h > 0.0) {
                c->hprime = (c->tstop - c->tn) * (1.0 - 4.0 * UROUND);
                c->eta = c->hprime / c->h;
            }
        }
        if (!one_step && (c->tn - tout) * c->h >= 0.0) {
            c->tretlast = *tret = tout;
            get_dky(c, tout, c->zn, n, yout);
            return CV_SUCCESS;
        }
        if (one_step) {
            c->tretlast = *tret = c->tn;
            memcpy(yout, c->zn[0], sizeof(double) * n);
            return CV_SUCCESS;
        }
    }
fail_ill:
    c->tretlast = *tret = c->tn;
    memcpy(yout, c->zn[0], sizeof(double) * n);
    return CV_ILL_INPUT;
}

typedef struct {
    cvmem* f;   /* forward problem */
    cvmem* b;   /* backward problem (after setup_b) */
    asa_mem a;
    oracle_options o;
    double* yB; /* cvB_mem->cv_y */
    double* ytmp;
    double toutB;
    int force_reinit, called_b;
} adjport;

static void* adj_create(const oracle_model* m, const oracle_options* o, const double* p,
                        const double* k, int nplist, const int32_t* plist, const double* x0) {
    adjport* A = (adjport*)calloc(1, sizeof(adjport));
    const int n = m->nx;
    A->o = *o;
    A->f = (cvmem*)port_create(m, o, p, k, 0, NULL, x0, NULL);
    asa_mem* a = &A->a;
    a->m = m;
    a->p = p;
    a->k = k;
    a->plist = plist;
    a->n = n;
    a->nplist = nplist;
    a->Y = (double*)calloc((size_t)LMAX * n + 1, sizeof(double));
    a->xt = (double*)calloc((size_t)n + 1, sizeof(double));
    a->J = (double*)calloc((size_t)n * n + 1, sizeof(double));
    a->dfdp = (double*)calloc((size_t)m->np * n + 1, sizeof(double));
    A->f->store = asa_store;
    A->f->store_into = a;
    /* CVodeF's first call stores the initial point with order qu = 0 */
    asa_store(a, x0, 0.0, 0);
    A->yB = (double*)calloc((size_t)n + 1, sizeof(double));
    A->ytmp = (double*)calloc((size_t)n + 1, sizeof(double));
    return A;
}

static int adj_solve_f(void* h, double tout, int64_t mxstep, double* tret) {
    return port_solve(((adjport*)h)->f, tout, mxstep, tret);
}
static const double* adj_x(void* h) { return ((adjport*)h)->f->zn[0]; }
static int64_t adj_nst(void* h) { return ((adjport*)h)->f->nst; }

/* Solver::setup_b: CVodeCreateB + CVodeInitB (a fresh CVODES memory at tB0),
 * CVodeQuadInitB, CVodeSStolerancesB, CVodeQuadSStolerancesB and
 * CVodeSetQuadErrConB (solver.cpp:267-298,658-691) */
static int adj_setup_b(void* h, double tB0, const double* xB0, const double* xQB0) {
    adjport* A = (adjport*)h;
    const oracle_options* o = &A->o;
    const int n = A->a.n, nq = A->a.nplist;
    oracle_options ob = *o;
    ob.rtol = isnan(o->rtol_b) ? o->rtol : o->rtol_b;
    ob.atol = isnan(o->atol_b) ? o->atol : o->atol_b;
    ob.max_nonlin_iters = 3; /* CVODES defaults: AMICI sets neither for the backward problem */
    ob.max_conv_fails = 10;
    ob.lu_f32 = 0;
    ob.max_step_size = INFINITY;
    cvmem* b = (cvmem*)port_create(A->a.m, &ob, A->a.p, A->a.k, 0, NULL, xB0, NULL);
    b->tn = tB0;
    b->adj = &A->a;
    b->nq = nq;
    const double rq = isnan(o->rtol_quad) ? o->rtol : o->rtol_quad;
    const double aq = isnan(o->atol_quad) ? o->atol : o->atol_quad;
    b->rtolQ = rq;
    b->atolQ = aq;
    b->errconQ = !isinf(aq) && !isinf(rq);
    double* w = (double*)calloc((size_t)(LMAX + 4) * (nq > 0 ? nq : 1), sizeof(double));
    for (int j = 0; j < LMAX; j++) { b->znQ[j] = w; w += nq; }
    b->ewtQ = w; w += nq; b->acorQ = w; w += nq; b->tempvQ = w; w += nq; b->yQ = w;
    memcpy(b->znQ[0], xQB0, sizeof(double) * nq);
    A->b = b;
    A->toutB = tB0;
    (void)n;
    return 0;
}

/* CVodeSolver::reInit_post_process for the backward problem
 * (solver_cvodes.cpp:512-560): one step from the reinitialised state with a
 * stop time at the next output, run as if it were the first step */
static int adj_reinit_post_process(adjport* A, double tnext, int64_t mxstep) {
    cvmem* b = A->b;
    int64_t nst_tmp = b->nst;
    b->nst = 0;
    b->tstop = tnext;
    b->tstopset = 1;
    double tret;
    int flag = cv_ode(b, tnext, 1, mxstep, A->ytmp, &tret);
    if (flag != CV_SUCCESS) return -99; /* a CvodeException: AMICI_ERROR */
    b->nst = nst_tmp + 1;
    A->toutB = tret;
    A->force_reinit = 0;
    return 0;
}

/* Solver::run_b -> CVodeSolver::solve_b -> CVodeB(tBout, CV_NORMAL) with the
 * single check point at t0 (cvodea.c:1365-1640) */
static int adj_run_b(void* h, double tBout, int64_t mxstepsB) {
    adjport* A = (adjport*)h;
    if (A->force_reinit) {
        int r = adj_reinit_post_process(A, tBout, mxstepsB);
        if (r) return r;
    }
    cvmem* b = A->b;
    b->tstop = A->a.t[0];
    b->tstopset = 1;
    double tret;
    int flag = cv_ode(b, tBout, 0, mxstepsB, A->yB, &tret);
    A->toutB = tret;
    A->called_b = 1;
    return flag < 0 ? flag : 0;
}

/* write_solution_b: CVodeGetB (cv_y at cv_tout) and CVodeGetQuadB (cvodea.c:1640-1720) */
static void adj_get_b(void* h, double* xB, double* xQB) {
    adjport* A = (adjport*)h;
    cvmem* b = A->b;
    memcpy(xB, A->yB, sizeof(double) * A->a.n);
    if (b->nst == 0) memcpy(xQB, b->znQ[0], sizeof(double) * b->nq);
    else get_dky(b, b->tretlast, b->znQ, b->nq, xQB);
}

/* CVodeSolver::reinit_b + reset_state + reinit_quad_b (solver_cvodes.cpp:471-505,618-648) */
static void adj_reinit_b(void* h, double t, const double* xB, const double* xQB) {
    adjport* A = (adjport*)h;
    cvmem* b = A->b;
    if (A->called_b) A->force_reinit = 1;
    b->tn = t;
    b->q = 1;
    b->L = 2;
    b->qwait = b->L;
    b->qu = 0;
    b->hu = 0.0;
    memcpy(b->zn[0], xB, sizeof(double) * A->a.n);
    memcpy(b->znQ[0], xQB, sizeof(double) * b->nq);
}

static int64_t adj_nst_b(void* h) {
    adjport* A = (adjport*)h;
    return A->b ? A->b->nst : 0;
}

static void adj_destroy(void* h) {
    adjport* A = (adjport*)h;
    port_destroy(A->f);
    if (A->b) {
        free(A->b->znQ[0]);
        port_destroy(A->b);
    }
    free(A->a.t); free(A->a.y); free(A->a.order); free(A->a.Y); free(A->a.xt); free(A->a.J);
    free(A->a.dfdp); free(A->yB); free(A->ytmp); free(A);
}

const oracle_adjoint_ops oracle_adjoint_impl = {adj_create, adj_solve_f, adj_x, adj_nst,
                                                adj_setup_b, adj_run_b, adj_get_b, adj_reinit_b,
                                                adj_nst_b, adj_destroy};
