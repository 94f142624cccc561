/*
 * AMICI simulation glue of the CPU oracle — TEST INFRASTRUCTURE ONLY.
 *
 * Restates amici::run_simulation for an ODE model without events: parameter
 * unscaling, x0/sx0 (src/model.cpp:251-280,1907-1990), the output loop with a
 * stop time at every output (src/forwardproblem.cpp:53-151), outputs
 * x, y, sigmay (ExpData overrides, src/model.cpp:2143-2184), the Gaussian
 * negative log-likelihood Jy = 0.5*log(2*pi*sigma^2) + 0.5*((y-m)/sigma)^2
 * (models/model_robertson_py/Jy.cpp:15-26; llh -= Jy, src/model.cpp:1194-1210),
 * forward-sensitivity outputs sx, sy and sllh (src/rdata.cpp:406-432,
 * src/model.cpp:1212-1240), the parameter-scale chain rule
 * (src/rdata.cpp:749-968) and invalidation after a failure
 * (src/rdata.cpp:684-747).  The integrator behind it is chosen at link time
 * (oracle_integrator.h).
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_integrator.h"

#ifdef _OPENMP
#include <omp.h>
#endif

static double unscale(double v, int32_t scale) {
    switch (scale) {
    case 1: return exp(v);
    case 2: return pow(10.0, v);
    default: return v;
    }
}

/* d p_unscaled / d p_scaled (src/rdata.cpp:749-968) */
static double scale_factor(double punscaled, int32_t scale) {
    switch (scale) {
    case 1: return punscaled;
    case 2: return punscaled * log(10.0);
    default: return 1.0;
    }
}

/* is_next_t_too_close (src/forwardproblem.cpp:26-38) */
static int t_too_close(double cur, double next) {
    double tdiff = next - cur;
    if (tdiff == 0.0) return 1;
    double tround = DBL_EPSILON * fmax(fabs(cur), fabs(next));
    return fabs(tdiff) < 2.0 * tround;
}

int oracle_simulate(const oracle_model* m, const oracle_options* o, const double* p_scaled,
                    const int32_t* pscale, const double* k, int nt, const double* ts,
                    const double* my, const double* sigma_data, int nplist, const int32_t* plist,
                    double* x, double* y, double* sigmay, double* llh, double* sx, double* sy,
                    double* sllh, int32_t* numsteps, oracle_stats* stats) {
    const oracle_integrator* I = &oracle_integrator_impl;
    const int n = m->nx, ny = m->ny, np = m->np;
    const int ns = (o->sensi == 1) ? nplist : 0;
    const double t0 = 0.0;
    double* p = (double*)malloc(sizeof(double) * (np > 0 ? np : 1));
    for (int j = 0; j < np; j++) p[j] = unscale(p_scaled[j], pscale ? pscale[j] : 0);
    double* x0 = (double*)calloc((size_t)n + 1, sizeof(double));
    double* sx0 = (double*)calloc((size_t)n * (ns > 0 ? ns : 1) + 1, sizeof(double));
    m->x0(x0, p, k);
    if (ns) {
        double* dx0 = (double*)calloc((size_t)np * n + 1, sizeof(double));
        m->dx0dp(dx0, p, k);
        for (int is = 0; is < ns; is++)
            memcpy(sx0 + (size_t)is * n, dx0 + (size_t)plist[is] * n, sizeof(double) * n);
        free(dx0);
    }
    void* h = I->create(m, o, p, k, ns, plist, x0, sx0);
    double* sig = (double*)malloc(sizeof(double) * (ny > 0 ? ny : 1));
    m->sigmay(sig, p, k);
    double* dydx = (double*)calloc((size_t)n * ny + 1, sizeof(double));
    double* dydp = (double*)calloc((size_t)np * ny + 1, sizeof(double));
    const int have_data = (my != NULL);
    *llh = have_data ? 0.0 : NAN;
    for (int is = 0; is < nplist; is++) sllh[is] = have_data ? 0.0 : NAN;
    int status = 0, it;
    double tcur = t0;
    const double* xt = x0;
    const double* sxt = sx0;
    for (it = 0; it < nt; it++) {
        double tout = ts[it];
        if (tout > t0) {
            while (tcur < tout) {
                if (t_too_close(tcur, tout)) break;
                int64_t remaining = o->maxsteps - I->nst(h);
                if (remaining <= 0) { status = -99; break; } /* AmiException -> AMICI_ERROR */
                int flag = I->solve(h, tout, remaining, &tcur);
                if (flag < 0) { status = flag; break; } /* CVODES flag == AMICI_* code */
                xt = I->x(h);
                sxt = I->sx(h);
            }
            if (status != 0) break;
        }
        memcpy(x + (size_t)it * n, xt, sizeof(double) * n);
        m->y(y + (size_t)it * ny, tout, xt, p, k);
        double* sgy = sigmay + (size_t)it * ny;
        for (int iy = 0; iy < ny; iy++) {
            double s = sig[iy];
            if (sigma_data && !isnan(sigma_data[(size_t)it * ny + iy])) s = sigma_data[(size_t)it * ny + iy];
            sgy[iy] = s;
        }
        if (have_data) {
            for (int iy = 0; iy < ny; iy++) {
                double mv = my[(size_t)it * ny + iy];
                if (isnan(mv)) continue;
                double s = sgy[iy], r = (y[(size_t)it * ny + iy] - mv) / s;
                *llh -= 0.5 * log(2.0 * M_PI * s * s) + 0.5 * r * r;
            }
        }
        if (ns) {
            m->dydx(dydx, tout, xt, p, k);
            m->dydp(dydp, tout, xt, p, k);
            for (int is = 0; is < ns; is++) {
                const double* s = sxt + (size_t)is * n;
                double f = scale_factor(p[plist[is]], pscale ? pscale[plist[is]] : 0);
                double* sxo = sx + ((size_t)it * nplist + is) * n;
                for (int i = 0; i < n; i++) sxo[i] = s[i] * f;
                double* syo = sy + ((size_t)it * nplist + is) * ny;
                for (int iy = 0; iy < ny; iy++) {
                    double v = dydp[(size_t)plist[is] * ny + iy];
                    for (int j = 0; j < n; j++) v += dydx[(size_t)j * ny + iy] * s[j];
                    syo[iy] = v * f;
                    double mv = have_data ? my[(size_t)it * ny + iy] : NAN;
                    if (!isnan(mv)) {
                        double sg = sgy[iy], yv = y[(size_t)it * ny + iy];
                        sllh[is] -= (yv - mv) / (sg * sg) * v * f;
                    }
                }
            }
        }
        numsteps[it] = (int32_t)I->nst(h);
    }
    if (status != 0) {
        for (int jt = it; jt < nt; jt++) {
            for (int i = 0; i < n; i++) x[(size_t)jt * n + i] = NAN;
            for (int iy = 0; iy < ny; iy++) y[(size_t)jt * ny + iy] = NAN;
            for (int iy = 0; iy < ny; iy++) sigmay[(size_t)jt * ny + iy] = NAN;
            if (ns) {
                for (size_t e = 0; e < (size_t)nplist * n; e++) sx[(size_t)jt * nplist * n + e] = NAN;
                for (size_t e = 0; e < (size_t)nplist * ny; e++) sy[(size_t)jt * nplist * ny + e] = NAN;
            }
            numsteps[jt] = (int32_t)I->nst(h);
        }
        *llh = NAN;
        for (int is = 0; is < nplist; is++) sllh[is] = NAN;
    }
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->nst = I->nst(h);
    }
    I->destroy(h);
    free(dydx); free(dydp); free(sig); free(x0); free(sx0); free(p);
    return status;
}

int oracle_run_simulations(const oracle_model* m, const oracle_options* o, int n,
                           const double* p, const int32_t* pscale, const double* k, int nt,
                           const double* ts, const double* my, const double* sigma_data,
                           int nplist, const int32_t* plist, double* x, double* y,
                           double* sigmay, double* llh, double* sx, double* sy, double* sllh,
                           int32_t* numsteps, int32_t* status, int nthreads) {
    const int nx = m->nx, ny = m->ny, np = m->np, nk = m->nk;
    int nfail = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : nfail)
#endif
    for (int i = 0; i < n; i++) {
        int s = oracle_simulate(
            m, o, p + (size_t)i * np, pscale, k + (size_t)i * nk, nt, ts + (size_t)i * nt,
            my ? my + (size_t)i * nt * ny : NULL, sigma_data ? sigma_data + (size_t)i * nt * ny : NULL,
            nplist, plist, x + (size_t)i * nt * nx, y + (size_t)i * nt * ny,
            sigmay + (size_t)i * nt * ny, llh + i, sx ? sx + (size_t)i * nt * nplist * nx : NULL,
            sy ? sy + (size_t)i * nt * nplist * ny : NULL, sllh + (size_t)i * nplist,
            numsteps + (size_t)i * nt, NULL);
        status[i] = s;
        if (s < 0) nfail++;
    }
    (void)nthreads;
    return nfail;
}

/* ======================================================================== */
/* Adjoint sensitivities: amici::run_simulation with SensitivityMethod::    */
/* adjoint for an ODE model without events or equilibration.                */
/*   forward  ForwardProblem::run with CVodeF storage (forwardproblem.cpp), */
/*            outputs and llh as above, the partial objective sensitivity   */
/*            sllh -= dJy/dp (rdata.cpp:387-395, model.cpp:1241-1251),     */
/*            dJy/dx per output (forwardproblem.cpp:675-701);              */
/*   backward EventHandlingBwdSimulator::run (backwardproblem.cpp:267-332): */
/*            xB jumps by dJy/dx at every output, the solver reinitialised  */
/*            after each jump, quadratures carried through;                */
/*   gradient ReturnData::process_backward_problem + handle_sx0_forward     */
/*            (rdata.cpp:514-629): sllh -= xB(t0).sx0 + xQB, then the       */
/*            parameter-scale chain rule (rdata.cpp:749-968).               */
/* ======================================================================== */
#include "oracle_adjoint.h"

int oracle_simulate_asa(const oracle_model* m, const oracle_options* o, const double* p_scaled,
                        const int32_t* pscale, const double* k, int nt, const double* ts,
                        const double* my, const double* sigma_data, int nplist,
                        const int32_t* plist, double* x, double* y, double* sigmay, double* llh,
                        double* sllh, int32_t* numsteps, int64_t* nst_b) {
    const oracle_adjoint_ops* A = &oracle_adjoint_impl;
    const int n = m->nx, ny = m->ny, np = m->np;
    const double t0 = 0.0;
    double* p = (double*)malloc(sizeof(double) * (np > 0 ? np : 1));
    for (int j = 0; j < np; j++) p[j] = unscale(p_scaled[j], pscale ? pscale[j] : 0);
    double* x0 = (double*)calloc((size_t)n + 1, sizeof(double));
    m->x0(x0, p, k);
    void* h = A->create(m, o, p, k, nplist, plist, x0);
    double* sig = (double*)malloc(sizeof(double) * (ny > 0 ? ny : 1));
    m->sigmay(sig, p, k);
    double* dydx = (double*)calloc((size_t)n * ny + 1, sizeof(double));
    double* dydp = (double*)calloc((size_t)np * ny + 1, sizeof(double));
    double* dJydx = (double*)calloc((size_t)nt * n + 1, sizeof(double));
    const int have_data = (my != NULL);
    *llh = have_data ? 0.0 : NAN;
    for (int is = 0; is < nplist; is++) sllh[is] = have_data ? 0.0 : NAN;
    int status = 0, it;
    double tcur = t0;
    const double* xt = x0;
    for (it = 0; it < nt; it++) {
        double tout = ts[it];
        if (tout > t0) {
            while (tcur < tout) {
                if (t_too_close(tcur, tout)) break;
                int64_t remaining = o->maxsteps - A->nst(h);
                if (remaining <= 0) { status = -99; break; }
                int flag = A->solve_f(h, tout, remaining, &tcur);
                if (flag < 0) { status = flag; break; }
                xt = A->x(h);
            }
            if (status != 0) break;
        }
        memcpy(x + (size_t)it * n, xt, sizeof(double) * n);
        m->y(y + (size_t)it * ny, tout, xt, p, k);
        double* sgy = sigmay + (size_t)it * ny;
        for (int iy = 0; iy < ny; iy++) {
            double s = sig[iy];
            if (sigma_data && !isnan(sigma_data[(size_t)it * ny + iy])) s = sigma_data[(size_t)it * ny + iy];
            sgy[iy] = s;
        }
        if (have_data) {
            m->dydx(dydx, tout, xt, p, k);
            m->dydp(dydp, tout, xt, p, k);
            for (int iy = 0; iy < ny; iy++) {
                double mv = my[(size_t)it * ny + iy];
                if (isnan(mv)) continue;
                double s = sgy[iy], yv = y[(size_t)it * ny + iy], r = (yv - mv) / s;
                *llh -= 0.5 * log(2.0 * M_PI * s * s) + 0.5 * r * r;
                double dJdy = (yv - mv) / (s * s); /* Gaussian dJy/dy */
                for (int i = 0; i < n; i++) dJydx[(size_t)it * n + i] += dJdy * dydx[(size_t)i * ny + iy];
                for (int is = 0; is < nplist; is++) sllh[is] -= dJdy * dydp[(size_t)plist[is] * ny + iy];
            }
        }
        numsteps[it] = (int32_t)A->nst(h);
    }
    int64_t nstb = 0;
    if (status == 0 && have_data && nplist > 0 && nt > 0) {
        double* xB = (double*)calloc((size_t)n + 1, sizeof(double));
        double* xQB = (double*)calloc((size_t)nplist + 1, sizeof(double));
        const int64_t maxsteps_b = o->maxsteps_b > 0 ? o->maxsteps_b : 100 * o->maxsteps;
        double t = ts[nt - 1] > t0 ? ts[nt - 1] : t0; /* the forward problem's final time */
        int jt = nt - 1;
        int bstat = 0;
        if (ts[jt] == t) {
            for (int i = 0; i < n; i++) xB[i] += dJydx[(size_t)jt * n + i];
            A->setup_b(h, t, xB, xQB);
            jt--;
        } else {
            A->setup_b(h, t, xB, xQB);
        }
        while (jt >= 0 && !bstat) {
            double tnext = ts[jt];
            if (tnext < t) {
                int64_t rem = maxsteps_b - A->nst_b(h);
                if (rem <= 0) { bstat = -99; break; }
                int flag = A->run_b(h, tnext, rem);
                if (flag < 0) { bstat = flag; break; }
                A->get_b(h, xB, xQB);
                t = tnext;
            }
            for (int i = 0; i < n; i++) xB[i] += dJydx[(size_t)jt * n + i];
            jt--;
            A->reinit_b(h, t, xB, xQB);
        }
        if (!bstat && t > t0) {
            int64_t rem = maxsteps_b - A->nst_b(h);
            int flag = rem <= 0 ? -99 : A->run_b(h, t0, rem);
            if (flag < 0) bstat = flag;
            else A->get_b(h, xB, xQB);
        }
        nstb = A->nst_b(h);
        if (bstat) {
            status = bstat;
            for (int is = 0; is < nplist; is++) sllh[is] = NAN;
        } else {
            double* dx0 = (double*)calloc((size_t)np * n + 1, sizeof(double));
            m->dx0dp(dx0, p, k);
            for (int is = 0; is < nplist; is++) {
                double s0 = 0.0;
                for (int i = 0; i < n; i++) s0 += xB[i] * dx0[(size_t)plist[is] * n + i];
                sllh[is] -= s0 + xQB[is];
                sllh[is] *= scale_factor(p[plist[is]], pscale ? pscale[plist[is]] : 0);
            }
            free(dx0);
        }
        free(xB);
        free(xQB);
    }
    if (status != 0) {
        for (int jt = it; jt < nt; jt++) {
            for (int i = 0; i < n; i++) x[(size_t)jt * n + i] = NAN;
            for (int iy = 0; iy < ny; iy++) y[(size_t)jt * ny + iy] = NAN;
            for (int iy = 0; iy < ny; iy++) sigmay[(size_t)jt * ny + iy] = NAN;
            numsteps[jt] = (int32_t)A->nst(h);
        }
        *llh = NAN;
        for (int is = 0; is < nplist; is++) sllh[is] = NAN;
    }
    if (nst_b) *nst_b = nstb;
    A->destroy(h);
    free(dJydx); free(dydx); free(dydp); free(sig); free(x0); free(p);
    return status;
}

int oracle_run_simulations_asa(const oracle_model* m, const oracle_options* o, int n,
                               const double* p, const int32_t* pscale, const double* k, int nt,
                               const double* ts, const double* my, const double* sigma_data,
                               int nplist, const int32_t* plist, double* x, double* y,
                               double* sigmay, double* llh, double* sllh, int32_t* numsteps,
                               int32_t* status, int64_t* nst_b, int nthreads) {
    const int nx = m->nx, ny = m->ny, np = m->np, nk = m->nk;
    int nfail = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : nfail)
#endif
    for (int i = 0; i < n; i++) {
        int s = oracle_simulate_asa(
            m, o, p + (size_t)i * np, pscale, k + (size_t)i * nk, nt, ts + (size_t)i * nt,
            my ? my + (size_t)i * nt * ny : NULL, sigma_data ? sigma_data + (size_t)i * nt * ny : NULL,
            nplist, plist, x + (size_t)i * nt * nx, y + (size_t)i * nt * ny,
            sigmay + (size_t)i * nt * ny, llh + i, sllh + (size_t)i * nplist,
            numsteps + (size_t)i * nt, nst_b ? nst_b + i : NULL);
        status[i] = s;
        if (s < 0) nfail++;
    }
    (void)nthreads;
    return nfail;
}
