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

/* Negative log-likelihood of one measurement m of the simulated y with
 * scale sigma, and its derivatives w.r.t. y and sigma, for the noise
 * distributions of python/sdist/amici/importers/utils.py:110-130 (the
 * generated Jy, dJydy, dJydsigma; e.g. models/model_robertson_py/Jy.cpp):
 *   normal          0.5 log(2 pi s^2) + 0.5 ((y - m) / s)^2
 *   log-normal      0.5 log(2 pi s^2 m^2) + 0.5 ((ln y - ln m) / s)^2
 *   log10-normal    0.5 log(2 pi s^2 m^2 ln(10)^2) + 0.5 ((lg y - lg m) / s)^2
 *   laplace         log(2 s) + |y - m| / s
 *   log-laplace     log(2 s m) + |ln y - ln m| / s
 *   log10-laplace   log(2 s m ln 10) + |lg y - lg m| / s */
static double noise_jy(int kind, double y, double m, double s, double* djdy, double* djds) {
    const double ln10 = log(10.0);
    double r, e;
    switch (kind) {
    case 1:
        r = (log(y) - log(m)) / s;
        *djdy = r / (s * y);
        *djds = 1.0 / s - r * r / s;
        return 0.5 * log(2.0 * M_PI * s * s * m * m) + 0.5 * r * r;
    case 2:
        r = (log10(y) - log10(m)) / s;
        *djdy = r / (s * y * ln10);
        *djds = 1.0 / s - r * r / s;
        return 0.5 * log(2.0 * M_PI * s * s * m * m * ln10 * ln10) + 0.5 * r * r;
    case 3:
        e = y - m;
        *djdy = (e > 0.0 ? 1.0 : (e < 0.0 ? -1.0 : 0.0)) / s;
        *djds = 1.0 / s - fabs(e) / (s * s);
        return log(2.0 * s) + fabs(e) / s;
    case 4:
        e = log(y) - log(m);
        *djdy = (e > 0.0 ? 1.0 : (e < 0.0 ? -1.0 : 0.0)) / (s * y);
        *djds = 1.0 / s - fabs(e) / (s * s);
        return log(2.0 * s * m) + fabs(e) / s;
    case 5:
        e = log10(y) - log10(m);
        *djdy = (e > 0.0 ? 1.0 : (e < 0.0 ? -1.0 : 0.0)) / (s * y * ln10);
        *djds = 1.0 / s - fabs(e) / (s * s);
        return log(2.0 * s * m * ln10) + fabs(e) / s;
    default:
        r = (y - m) / s;
        *djdy = (y - m) / (s * s);
        *djds = 1.0 / s - r * r / s;
        return 0.5 * log(2.0 * M_PI * s * s) + 0.5 * r * r;
    }
}

/* the noise scale of output it, observable iy comes from ExpData (then it
 * is a constant: Model::fdsigmaydp sets its parameter derivative to zero) */
static int sigma_from_data(const double* sigma_data, int it, int ny, int iy) {
    return sigma_data && !isnan(sigma_data[(size_t)it * ny + iy]);
}

/* is_next_t_too_close (src/forwardproblem.cpp:26-38) */
static int t_too_close(double cur, double next) {
    double tdiff = next - cur;
    if (tdiff == 0.0) return 1;
    double tround = DBL_EPSILON * fmax(fabs(cur), fabs(next));
    return fabs(tdiff) < 2.0 * tround;
}

/* One instance's rows of a batch's pre-equilibration and override arrays. */
typedef struct {
    const double *k_preeq, *x0, *sx0;
    double *x_ss, *sx_ss, *preeq_t, *preeq_wrms, *posteq_t, *posteq_wrms;
    int32_t *preeq_status, *preeq_numsteps, *posteq_status, *posteq_numsteps;
} inst_ext;

static inst_ext instance_ext(const oracle_batch_ext* e, int i, int nx, int nk, int nplist) {
    inst_ext r;
    memset(&r, 0, sizeof(r));
    if (!e) return r;
    if (e->k_preeq) r.k_preeq = e->k_preeq + (size_t)i * nk;
    if (e->x0) r.x0 = e->x0 + (size_t)i * nx;
    if (e->sx0) r.sx0 = e->sx0 + (size_t)i * nplist * nx;
    if (e->x_ss) r.x_ss = e->x_ss + (size_t)i * nx;
    if (e->sx_ss) r.sx_ss = e->sx_ss + (size_t)i * nplist * nx;
    if (e->preeq_t) r.preeq_t = e->preeq_t + i;
    if (e->preeq_wrms) r.preeq_wrms = e->preeq_wrms + i;
    if (e->preeq_status) r.preeq_status = e->preeq_status + i;
    if (e->preeq_numsteps) r.preeq_numsteps = e->preeq_numsteps + i;
    if (e->posteq_t) r.posteq_t = e->posteq_t + i;
    if (e->posteq_wrms) r.posteq_wrms = e->posteq_wrms + i;
    if (e->posteq_status) r.posteq_status = e->posteq_status + i;
    if (e->posteq_numsteps) r.posteq_numsteps = e->posteq_numsteps + i;
    return r;
}

/* ---- pre-equilibration: simulation to steady state ----------------------
 * SteadyStateProblem with the reference's default settings (steady-state
 * computation mode integrationOnly, model.h:2296; Newton steps 0,
 * solver.h:2043): from x0 (and sx0) at the pre-equilibration's fixed
 * parameters, one CVODES step at a time towards tout = max(t, 1) * 10
 * (EventHandlingSimulator::run_steady_state, forwardproblem.cpp:153-230)
 * until the WRMS norm of xdot, with weights 1/(rtol_ss |x| + atol_ss), is
 * below 1 (checked before every step, steadystateproblem.cpp:29-52,
 * forwardproblem.cpp:1040-1092) and, with forward sensitivities, so is the
 * norm of every sensitivity's right-hand side J sx_i + df/dp_i with weights
 * from |sx_i| (get_wrms_fsa, forwardproblem.cpp:989-1017).  The steady-state
 * tolerances are 100 x the solver's (ss_tol_factor, solver.h:2081,2090).  A
 * fresh solver with the same settings runs it (forwardproblem.cpp:944-975).
 * Returns the simulation stage's SteadyStateStatus: 1 success, -2 step budget
 * exhausted, -5 time overflow, -1 any other integration failure. */
#define SS_TOL_FACTOR 100.0

/* getWrmsNorm (steadystateproblem.cpp:29-52) */
static double ss_wrms(int n, const double* v, const double* xref, double atol, double rtol) {
    double sum = 0.0;
    for (int i = 0; i < n; i++) {
        const double w = 1.0 / (rtol * fabs(xref[i]) + atol);
        const double t = v[i] * w;
        sum += t * t;
    }
    return sqrt(sum / n);
}

/* The simulation to steady state on the integrator h, from the state xc (and
 * sensitivities sxc) at time *t: the steady-state check before every step,
 * one step at a time.  On return xc / sxc point at the last state, *t is its
 * time, *nsteps the steps taken and *wrms_ss the last norm. */
static int ss_simulate(const oracle_integrator* I, void* h, const oracle_model* m, const oracle_options* o,
                       const double* p, const double* kp, int ns, const int32_t* plist, const double** xcp,
                       const double** sxcp, double* tp, int32_t* nsteps, double* wrms_ss) {
    const int n = m->nx, np = m->np;
    const double atol = o->atol * SS_TOL_FACTOR, rtol = o->rtol * SS_TOL_FACTOR;
    double* xdot = (double*)calloc((size_t)n + 1, sizeof(double));
    double* sxdot = (double*)calloc((size_t)n + 1, sizeof(double));
    double* J = ns ? (double*)calloc((size_t)n * n + 1, sizeof(double)) : NULL;
    double* dfdp = ns ? (double*)calloc((size_t)np * n + 1, sizeof(double)) : NULL;
    const double* xc = *xcp;
    const double* sxc = *sxcp;
    double t = *tp, w = INFINITY;
    int steps = 0, st = 1;
    for (;;) {
        m->xdot(xdot, t, xc, p, kp);
        w = ss_wrms(n, xdot, xc, atol, rtol);
        int converged = w < 1.0;
        if (converged && ns) {
            m->jac(J, t, xc, p, kp);
            m->dxdotdp(dfdp, t, xc, p, kp);
            for (int is = 0; is < ns && converged; is++) {
                const double* s = sxc + (size_t)is * n;
                for (int i = 0; i < n; i++) {
                    double v = 0.0;
                    for (int j = 0; j < n; j++) v += J[(size_t)j * n + i] * s[j];
                    sxdot[i] = v + dfdp[(size_t)plist[is] * n + i];
                }
                converged = ss_wrms(n, sxdot, s, atol, rtol) < 1.0;
            }
        }
        if (converged) break;
        if (steps >= o->maxsteps) {
            st = -2;
            break;
        }
        steps++;
        const double tout = (t > 1.0 ? t : 1.0) * 10.0;
        if (!isfinite(tout)) {
            st = -5;
            break;
        }
        const int flag = I->one_step(h, tout, &t);
        if (flag < 0) {
            st = flag == -1 ? -2 : -1; /* AMICI_TOO_MUCH_WORK: failed_convergence */
            break;
        }
        xc = I->x(h);
        sxc = I->sx(h);
    }
    *xcp = xc;
    *sxcp = sxc;
    *nsteps = steps;
    *tp = t;
    *wrms_ss = w;
    free(xdot); free(sxdot); free(J); free(dfdp);
    return st;
}

static int preequilibrate(const oracle_model* m, const oracle_options* o, const double* p, const double* kp,
                          int ns, const int32_t* plist, double* x, double* sx, int32_t* nsteps,
                          double* t_ss, double* wrms_ss) {
    const oracle_integrator* I = &oracle_integrator_impl;
    const int n = m->nx;
    void* h = I->create(m, o, p, kp, ns, plist, x, sx);
    const double* xc = x;
    const double* sxc = sx;
    double t = 0.0;
    const int st = ss_simulate(I, h, m, o, p, kp, ns, plist, &xc, &sxc, &t, nsteps, wrms_ss);
    if (xc != x) memcpy(x, xc, sizeof(double) * n);
    if (ns && sxc != sx) memcpy(sx, sxc, sizeof(double) * n * ns);
    *t_ss = t;
    I->destroy(h);
    return st;
}

/* Initial state and its sensitivities (w.r.t. the unscaled parameters of
 * plist) of one instance, pre-equilibrated if the instance has
 * pre-equilibration parameters: ExpData x0 / sx0 override the model's x0 and
 * dx0/dp (ConditionContext, edata.cpp:472-490; sx0 given w.r.t. the scaled
 * parameters, Model::set_initial_state_sensitivities, model.cpp:986-1021).
 * Returns 0, or AMICI_ERROR (-99) when no steady state was found. */
static int initial_state(const oracle_model* m, const oracle_options* o, const double* p, const int32_t* pscale,
                         const double* k, int ns, const int32_t* plist, const inst_ext* e, double* x0,
                         double* sx0) {
    const int n = m->nx, np = m->np;
    /* events are handled in the main simulation only: a pre-equilibration of
     * a model with events is not restated */
    if (e && e->k_preeq && m->ne) return -99;
    const double* k0 = (e && e->k_preeq) ? e->k_preeq : k;
    if (e && e->x0) memcpy(x0, e->x0, sizeof(double) * n);
    else m->x0(x0, p, k0);
    if (ns) {
        if (e && e->sx0) {
            for (int is = 0; is < ns; is++) {
                const double f = scale_factor(p[plist[is]], pscale ? pscale[plist[is]] : 0);
                for (int i = 0; i < n; i++) sx0[(size_t)is * n + i] = e->sx0[(size_t)is * n + i] / f;
            }
        } else {
            double* dx0 = (double*)calloc((size_t)np * n + 1, sizeof(double));
            m->dx0dp(dx0, p, k0);
            for (int is = 0; is < ns; is++)
                memcpy(sx0 + (size_t)is * n, dx0 + (size_t)plist[is] * n, sizeof(double) * n);
            free(dx0);
        }
    }
    if (!(e && e->k_preeq)) return 0;
    int32_t steps = 0;
    double t_ss = NAN, w = NAN;
    const int st = preequilibrate(m, o, p, e->k_preeq, ns, plist, x0, sx0, &steps, &t_ss, &w);
    if (e->preeq_status) *e->preeq_status = st;
    if (e->preeq_numsteps) *e->preeq_numsteps = steps;
    if (e->preeq_t) *e->preeq_t = t_ss;
    if (e->preeq_wrms) *e->preeq_wrms = w;
    if (e->x_ss) memcpy(e->x_ss, x0, sizeof(double) * n);
    if (e->sx_ss)
        for (int is = 0; is < ns; is++) {
            const double f = scale_factor(p[plist[is]], pscale ? pscale[plist[is]] : 0);
            for (int i = 0; i < n; i++) e->sx_ss[(size_t)is * n + i] = sx0[(size_t)is * n + i] * f;
        }
    return st == 1 ? 0 : -99;
}

/* ---- events ----------------------------------------------------------------
 * EventHandlingSimulator::run (forwardproblem.cpp:53-151).  Events with
 * explicit trigger times: the times within (t0, last output], ascending
 * (Model::get_trigger_timepoints, the keys of explicit_roots_,
 * model.cpp:444-470), are stop times next to the outputs; at one of them the
 * events whose time it is fire with roots_found = copysign(1, -root value at
 * the previous event), the root value of an explicit trigger being
 * direction * (t - te).
 * Events with trigger functions: the solver's root finding returns at a
 * zero crossing, with roots_found from CVodeGetRootInfo. */
#define EV_QUEUE 64  /* queued events (primary and secondary) per time, times ne */
#define EV_PENDING 4 /* events waiting in the queue, times ne */
typedef struct {
    int ne, ns, nroot, ntimes, next;
    double *te, *rootvals, *rval_tmp, *times, *dtedp, *g, *dgdx, *dgdp;
    int *found, *queue, *root_of;
    double tlastroot;
    double *xold, *xdot_old, *xdot, *dx, *ddx, *ddp, *stau, *sx, *x;
    /* the Heaviside indicators of the right-hand side (k[nk + j]); NULL
     * without any */
    double* h;
    int nh;
    const int* h_event;
} evsched;

/* Model::update_heaviside (model.cpp:1588-1592): h_j += roots_found of
 * its event */
static void update_heaviside(evsched* e) {
    for (int j = 0; j < e->nh; j++) e->h[j] += (double)e->found[e->h_event[j]];
}

static int cmp_double(const void* a, const void* b) {
    const double x = *(const double*)a, y = *(const double*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* Model::froot for every event: direction * (t - te) for an explicit trigger, the trigger
 * function otherwise */
static void froot_all(evsched* e, const oracle_model* m, const double* p, const double* k, double t,
                      const double* x, double* rv) {
    if (e->nroot) m->root(e->g, t, x, p, k);
    for (int ie = 0; ie < e->ne; ie++)
        rv[ie] = e->root_of[ie] >= 0 ? e->g[e->root_of[ie]] : m->event_dir[ie] * (t - e->te[ie]);
}

static void events_begin(evsched* e, const oracle_model* m, const double* p, const double* k, double t0,
                         double tlast, int ns, const double* x0) {
    memset(e, 0, sizeof(*e));
    e->ne = m->ne;
    e->ns = ns;
    e->nroot = m->nroot;
    e->tlastroot = t0;
    if (!e->ne) return;
    const int ne = e->ne, n = m->nx, np = m->np, nr = m->nroot;
    e->te = (double*)malloc(sizeof(double) * ne * 4);
    e->rootvals = e->te + ne;
    e->rval_tmp = e->rootvals + ne;
    e->times = e->rval_tmp + ne;
    e->found = (int*)calloc((size_t)(2 + EV_QUEUE) * ne + 1, sizeof(int));
    e->root_of = e->found + ne;
    e->queue = e->root_of + ne;
    e->dtedp = (double*)calloc((size_t)np * ne + 1, sizeof(double));
    e->g = (double*)calloc((size_t)nr + n + np + 1, sizeof(double));
    e->dgdx = e->g + nr;
    e->dgdp = e->dgdx + n;
    e->xold = (double*)calloc((size_t)n * 5 + (size_t)n * n + (size_t)np * n + (size_t)ns + (size_t)n * ns + 8,
                              sizeof(double));
    e->xdot_old = e->xold + n;
    e->xdot = e->xdot_old + n;
    e->dx = e->xdot + n;
    e->x = e->dx + n;
    e->ddx = e->x + n;
    e->ddp = e->ddx + (size_t)n * n;
    e->stau = e->ddp + (size_t)np * n;
    e->sx = e->stau + ns;
    for (int ie = 0; ie < ne; ie++) e->root_of[ie] = -1;
    for (int ir = 0; ir < nr; ir++) e->root_of[m->root_event[ir]] = ir;
    m->event_times(e->te, p, k);
    m->devent_times_dp(e->dtedp, p, k);
    int nt = 0;
    for (int ie = 0; ie < ne; ie++)
        if (e->root_of[ie] < 0 && e->te[ie] > t0 && e->te[ie] <= tlast) e->times[nt++] = e->te[ie];
    qsort(e->times, nt, sizeof(double), cmp_double);
    int u = 0;
    for (int i = 0; i < nt; i++)
        if (u == 0 || e->times[i] != e->times[u - 1]) e->times[u++] = e->times[i];
    e->ntimes = u;
    (void)x0;
}

static void events_end(evsched* e) {
    if (!e->ne) return;
    free(e->te); free(e->found); free(e->dtedp); free(e->g); free(e->xold);
}

/* get_event_time_sensitivity (model.cpp:1464-1479; de_model.py "stau"):
 * stau = sroot / drootdt_total, sroot = dg/dx sx + dg/dp, drootdt_total =
 * dg/dt + dg/dx xdot; for an explicit trigger t - te, stau = -dte/dp */
static void event_time_sensitivity(evsched* e, const oracle_model* m, const double* p, const double* k, int ie,
                                   double t, int n, int ns, const int32_t* plist) {
    const int ir = e->root_of[ie];
    if (ir < 0) {
        for (int is = 0; is < ns; is++) e->stau[is] = -e->dtedp[(size_t)plist[is] * e->ne + ie];
        return;
    }
    m->drootdx(e->dgdx, ir, t, e->x, p, k);
    m->drootdp(e->dgdp, ir, t, e->x, p, k);
    double dt = m->drootdt(ir, t, e->x, p, k);
    for (int j = 0; j < n; j++) dt += e->dgdx[j] * e->xdot_old[j];
    for (int is = 0; is < ns; is++) {
        double sr = e->dgdp[plist[is]];
        const double* s = e->sx + (size_t)is * n;
        for (int j = 0; j < n; j++) sr += e->dgdx[j] * s[j];
        e->stau[is] = dt != 0.0 ? sr / dt : 0.0;
    }
}

/* store_pre_event_info (forwardproblem.cpp:404-426, 573-604): root values
 * now, state and xdot before the events and, for a primary event with
 * forward sensitivities, the event-time sensitivity of the last firing event
 * ("just use the last ie") */
static void store_pre_event(evsched* e, const oracle_model* m, const double* p, const double* k, double t,
                            int n, int ns, const int32_t* plist, int seflag, int initial) {
    froot_all(e, m, p, k, t, e->x, e->rootvals);
    memcpy(e->rval_tmp, e->rootvals, sizeof(double) * e->ne);
    memcpy(e->xold, e->x, sizeof(double) * n);
    m->xdot(e->xdot_old, t, e->x, p, k);
    if (!ns) return;
    if (!seflag && !initial) {
        for (int is = 0; is < ns; is++) e->stau[is] = 0.0;
        for (int ie = 0; ie < e->ne; ie++)
            if (e->found[ie] == 1) event_time_sensitivity(e, m, p, k, ie, t, n, ns, plist);
    }
    if (initial)
        for (int is = 0; is < ns; is++) e->stau[is] = 0.0;
}

/* detect_secondary_events (forwardproblem.cpp:605-660): the root values
 * after the boluses; an event that did not fire and whose Heaviside value
 * changed fires when its root value rose (roots_found 1, queued) and is
 * marked -1 when it fell; the events that fired are cleared */
static int detect_secondary(evsched* e, const oracle_model* m, const double* p, const double* k, double t,
                            int* nq) {
    froot_all(e, m, p, k, t, e->x, e->rootvals);
    int second = 0;
    for (int ie = 0; ie < e->ne; ie++) {
        if (e->found[ie] == 0) {
            const double a = e->rval_tmp[ie], b = e->rootvals[ie];
            if ((a < 0.0 && b >= 0.0) || (a >= 0.0 && b < 0.0)) { /* heaviside_differs, misc.h:280 */
                if (a < b) {
                    e->found[ie] = 1;
                    e->queue[(*nq)++] = ie;
                } else {
                    e->found[ie] = -1;
                }
                second++;
            } else {
                e->found[ie] = 0;
            }
        } else {
            e->found[ie] = 0;
        }
    }
    return second;
}

/* handle_events (forwardproblem.cpp:388-516) with roots_found in e->found,
 * the state and sensitivities in e->x, e->sx: the events with roots_found 1
 * in index order (the queue of events without priorities keeps that order,
 * event.h:163-212) add their boluses (add_state_event_update,
 * model.cpp:1481-1503) and, with sensitivities, the bolus of the
 * sensitivities, deltasx = (xdot - xdot_old) stau + ddeltax/dp
 * + ddeltax/dx (sx - xdot_old stau) (de_model.py "deltasx";
 * model.cpp:1505-1534); after each, secondary events.  Returns -99 for an
 * event at the time of the last one ("stuck in an event"). */
static int handle_events(evsched* e, const oracle_model* m, const double* p, const double* k, double t, int n,
                         int ns, const int32_t* plist, int initial) {
    if (!initial && t == e->tlastroot) return -99;
    e->tlastroot = t;
    store_pre_event(e, m, p, k, t, n, ns, plist, 0, initial);
    if (!initial) update_heaviside(e);
    int nq = 0, head = 0;
    for (int ie = 0; ie < e->ne; ie++)
        if (e->found[ie] == 1) e->queue[nq++] = ie;
    while (head < nq) {
        const int ie = e->queue[head++];
        m->deltax(e->dx, ie, t, e->x, p, k);
        for (int i = 0; i < n; i++) e->x[i] += e->dx[i];
        if (ns) {
            m->xdot(e->xdot, t, e->x, p, k);
            m->ddeltaxdx(e->ddx, ie);
            m->ddeltaxdp(e->ddp, ie, p, k);
            for (int is = 0; is < ns; is++) {
                double* s = e->sx + (size_t)is * n;
                const double st = e->stau[is];
                double* d = e->dx; /* deltasx of this column */
                for (int i = 0; i < n; i++)
                    d[i] = (e->xdot[i] - e->xdot_old[i]) * st + e->ddp[(size_t)plist[is] * n + i];
                for (int j = 0; j < n; j++) {
                    const double v = s[j] - e->xdot_old[j] * st;
                    const double* col = e->ddx + (size_t)j * n;
                    for (int i = 0; i < n; i++) d[i] += col[i] * v;
                }
                for (int i = 0; i < n; i++) s[i] += d[i];
            }
        }
        /* the queue is full (AMICI's is unbounded): at most EV_QUEUE * ne
         * events at one time, at most EV_PENDING * ne of them waiting */
        if (nq + e->ne > EV_QUEUE * e->ne || nq - head + e->ne > EV_PENDING * e->ne) break;
        if (detect_secondary(e, m, p, k, t, &nq)) {
            store_pre_event(e, m, p, k, t, n, ns, plist, 1, initial);
            update_heaviside(e);
        }
    }
    return 0;
}

/* handle_initial_events (forwardproblem.cpp:518-525) after
 * Model::initialize_events (model.cpp:407-440): at t0 an event whose root
 * value is not negative while its trigger's initial value is false fires;
 * its event-time sensitivity is zero; the solver has not run, so the
 * boluses change the initial state */
static void initial_events(evsched* e, const oracle_model* m, const double* p, const double* k, double t0,
                           int n, int ns, const int32_t* plist, double* x0, double* sx0) {
    const int ne = e->ne;
    if (!ne) return;
    froot_all(e, m, p, k, t0, x0, e->rootvals);
    int any = 0;
    for (int ie = 0; ie < ne; ie++) {
        e->found[ie] = (!(e->rootvals[ie] < 0.0) && !m->event_initial_value[ie]) ? 1 : 0;
        any |= e->found[ie];
    }
    if (any) {
        memcpy(e->x, x0, sizeof(double) * n);
        if (ns) memcpy(e->sx, sx0, sizeof(double) * n * ns);
        handle_events(e, m, p, k, t0, n, ns, plist, 1);
        memcpy(x0, e->x, sizeof(double) * n);
        if (ns) memcpy(sx0, e->sx, sizeof(double) * n * ns);
    }
    /* the root values at t0 (forwardproblem.cpp:66-67) */
    froot_all(e, m, p, k, t0, x0, e->rootvals);
    for (int ie = 0; ie < ne; ie++) e->found[ie] = 0;
}

/* after a solve that stopped at a trigger time or returned a root: the
 * events' roots_found, handle_events, the solver reinitialised at t */
static int events_at(evsched* e, const oracle_model* m, const double* p, const double* k, double t, int flag,
                     double tev, int n, int ns, const int32_t* plist, const oracle_integrator* I, void* h) {
    const int ne = e->ne;
    if (flag == 2 && e->nroot) { /* CV_ROOT_RETURN: CVodeGetRootInfo */
        int ir_found[64];
        int* rf = e->nroot <= 64 ? ir_found : (int*)malloc(sizeof(int) * e->nroot);
        I->root_info(h, rf);
        for (int ie = 0; ie < ne; ie++) e->found[ie] = e->root_of[ie] >= 0 ? rf[e->root_of[ie]] : 0;
        if (rf != ir_found) free(rf);
    } else {
        for (int ie = 0; ie < ne; ie++) e->found[ie] = 0;
    }
    if (t == tev) {
        for (int ie = 0; ie < ne; ie++)
            if (e->root_of[ie] < 0 && e->te[ie] == t)
                e->found[ie] = (-e->rootvals[ie] >= 0.0 && !signbit(-e->rootvals[ie])) ? 1 : -1;
        e->next++;
    }
    memcpy(e->x, I->x(h), sizeof(double) * n);
    if (ns) memcpy(e->sx, I->sx(h), sizeof(double) * n * ns);
    if (handle_events(e, m, p, k, t, n, ns, plist, 0)) return -99;
    I->reinit(h, t, e->x, ns ? e->sx : NULL);
    return 0;
}

/* Outputs of an instance whose pre-equilibration failed: the main simulation
 * never ran (AMICI_ERROR, every output invalid, no steps). */
static void invalidate_all(int nt, int n, int ny, int nplist, int ns, double* x, double* y, double* sigmay,
                           double* llh, double* sx, double* sy, double* sllh, int32_t* numsteps) {
    for (size_t e = 0; e < (size_t)nt * n; e++) x[e] = NAN;
    for (size_t e = 0; e < (size_t)nt * ny; e++) y[e] = sigmay[e] = NAN;
    if (ns && sx)
        for (size_t e = 0; e < (size_t)nt * nplist * n; e++) sx[e] = NAN;
    if (ns && sy)
        for (size_t e = 0; e < (size_t)nt * nplist * ny; e++) sy[e] = NAN;
    for (int it = 0; it < nt; it++) numsteps[it] = 0;
    *llh = NAN;
    for (int is = 0; is < nplist; is++) sllh[is] = NAN;
}

static int simulate_one(const oracle_model* m, const oracle_options* o, const double* p_scaled,
                        const int32_t* pscale, const double* k, int nt, const double* ts,
                        const double* my, const double* sigma_data, int nplist, const int32_t* plist,
                        double* x, double* y, double* sigmay, double* llh, double* sx, double* sy,
                        double* sllh, int32_t* numsteps, oracle_stats* stats, const inst_ext* e) {
    const oracle_integrator* I = &oracle_integrator_impl;
    const int n = m->nx, ny = m->ny, np = m->np;
    const int ns = (o->sensi == 1) ? nplist : 0;
    const double t0 = 0.0;
    double* p = (double*)malloc(sizeof(double) * (np > 0 ? np : 1));
    for (int j = 0; j < np; j++) p[j] = unscale(p_scaled[j], pscale ? pscale[j] : 0);
    double* x0 = (double*)calloc((size_t)n + 1, sizeof(double));
    double* sx0 = (double*)calloc((size_t)n * (ns > 0 ? ns : 1) + 1, sizeof(double));
    if (initial_state(m, o, p, pscale, k, ns, plist, e, x0, sx0)) {
        invalidate_all(nt, n, ny, nplist, ns, x, y, sigmay, llh, sx, sy, sllh, numsteps);
        if (stats) memset(stats, 0, sizeof(*stats));
        free(x0); free(sx0); free(p);
        return -99;
    }
    /* the fixed parameters followed by the Heaviside indicators, which the
     * event handling updates in place (the integrator reads them through
     * this pointer) */
    double* kx = (double*)calloc((size_t)m->nk + m->nh + 1, sizeof(double));
    if (m->nk) memcpy(kx, k, sizeof(double) * m->nk);
    k = kx;
    evsched ev;
    events_begin(&ev, m, p, k, t0, nt > 0 ? ts[nt - 1] : t0, ns, x0);
    ev.h = kx + m->nk;
    ev.nh = m->nh;
    ev.h_event = m->h_event;
    if (m->nh) {
        /* Model::initialize_events (model.cpp:407-440): h_j = 1 where the
         * trigger is not negative at t0 */
        froot_all(&ev, m, p, k, t0, x0, ev.rootvals);
        for (int j = 0; j < m->nh; j++) ev.h[j] = ev.rootvals[m->h_event[j]] < 0.0 ? 0.0 : 1.0;
    }
    /* handle_initial_events (forwardproblem.cpp:518-525): events whose
     * trigger is already true at t0 and was false before fire at t0; the
     * solver has not run, so their boluses change the initial state */
    initial_events(&ev, m, p, k, t0, n, ns, plist, x0, sx0);
    void* h = I->create(m, o, p, k, ns, plist, x0, sx0);
    double* sig = (double*)malloc(sizeof(double) * (ny > 0 ? ny : 1));
    m->sigmay(sig, p, k);
    double* dydx = (double*)calloc((size_t)n * ny + 1, sizeof(double));
    double* dydp = (double*)calloc((size_t)np * ny + 1, sizeof(double));
    double* dsig = (double*)calloc((size_t)np * ny + 1, sizeof(double));
    m->dsigmaydp(dsig, p, k);
    const int have_data = (my != NULL);
    *llh = have_data ? 0.0 : NAN;
    for (int is = 0; is < nplist; is++) sllh[is] = have_data ? 0.0 : NAN;
    int status = 0, it, pe_status = 0;
    double tcur = t0;
    const double* xt = x0;
    const double* sxt = sx0;
    for (it = 0; it < nt; it++) {
        double tout = ts[it];
        if (isinf(tout)) {
            /* handle_postequilibration (forwardproblem.cpp:376-387): the
             * outputs at t = inf come from the steady state that the main
             * solver, continued from the last output in ONE_STEP mode,
             * reaches (SteadyStateProblem::run with is_preeq false: no new
             * solver, forwardproblem.cpp:862-900,1009-1105); outputs at
             * t = inf carry no step count (Solver::store_diagnosis runs at
             * the finite outputs only) */
            if (!pe_status) {
                double tpe = tcur, pw = NAN;
                int32_t psteps = 0;
                pe_status = ss_simulate(I, h, m, o, p, k, ns, plist, &xt, &sxt, &tpe, &psteps, &pw);
                if (e && e->posteq_status) *e->posteq_status = pe_status;
                if (e && e->posteq_numsteps) *e->posteq_numsteps = psteps;
                if (e && e->posteq_t) *e->posteq_t = pe_status == 1 ? tpe : NAN;
                if (e && e->posteq_wrms) *e->posteq_wrms = pw;
            }
        } else if (tout > t0) {
            while (tcur < tout) {
                if (t_too_close(tcur, tout)) break;
                /* the next stop is the output or the next trigger time */
                const double tev = ev.next < ev.ntimes ? ev.times[ev.next] : INFINITY;
                const double tstop = tout < tev ? tout : tev;
                int64_t remaining = o->maxsteps - I->nst(h);
                if (remaining <= 0) { status = -99; break; } /* AmiException -> AMICI_ERROR */
                int flag = I->solve(h, tstop, remaining, &tcur);
                if (flag < 0) { status = flag; break; } /* CVODES flag == AMICI_* code */
                xt = I->x(h);
                sxt = I->sx(h);
                if (flag == 2 || tcur == tev) { /* CV_ROOT_RETURN or a trigger time */
                    if (events_at(&ev, m, p, k, tcur, flag, tev, n, ns, plist, I, h)) {
                        status = -99;
                        break;
                    }
                    xt = I->x(h);
                    sxt = I->sx(h);
                }
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
                double djdy, djds;
                *llh -= noise_jy(m->noise[iy], y[(size_t)it * ny + iy], mv, sgy[iy], &djdy, &djds);
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
                        double djdy, djds;
                        noise_jy(m->noise[iy], y[(size_t)it * ny + iy], mv, sgy[iy], &djdy, &djds);
                        sllh[is] -= djdy * v * f;
                        /* a noise scale from the data does not depend on the parameters */
                        if (!sigma_from_data(sigma_data, it, ny, iy))
                            sllh[is] -= djds * dsig[(size_t)plist[is] * ny + iy] * f;
                    }
                }
            }
        }
        numsteps[it] = isinf(tout) ? 0 : (int32_t)I->nst(h);
    }
    /* a failed post-equilibration is an AmiException (AMICI_ERROR) that
     * leaves every output in place (rdata.cpp:288-313,336-347) */
    if (status == 0 && pe_status != 0 && pe_status != 1) status = -99;
    else if (status != 0) {
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
    events_end(&ev);
    free(dydx); free(dydp); free(dsig); free(sig); free(x0); free(sx0); free(p); free(kx);
    return status;
}

int oracle_simulate(const oracle_model* m, const oracle_options* o, const double* p_scaled,
                    const int32_t* pscale, const double* k, int nt, const double* ts,
                    const double* my, const double* sigma_data, int nplist, const int32_t* plist,
                    double* x, double* y, double* sigmay, double* llh, double* sx, double* sy,
                    double* sllh, int32_t* numsteps, oracle_stats* stats) {
    return simulate_one(m, o, p_scaled, pscale, k, nt, ts, my, sigma_data, nplist, plist, x, y, sigmay, llh,
                        sx, sy, sllh, numsteps, stats, NULL);
}

int oracle_run_simulations_ext(const oracle_model* m, const oracle_options* o, int n,
                               const double* p, const int32_t* pscale, const double* k, int nt,
                               const double* ts, const double* my, const double* sigma_data,
                               int nplist, const int32_t* plist, double* x, double* y,
                               double* sigmay, double* llh, double* sx, double* sy, double* sllh,
                               int32_t* numsteps, int32_t* status, const oracle_batch_ext* ext,
                               int nthreads) {
    const int nx = m->nx, ny = m->ny, np = m->np, nk = m->nk;
    int nfail = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : nfail)
#endif
    for (int i = 0; i < n; i++) {
        const inst_ext e = instance_ext(ext, i, nx, nk, nplist);
        int s = simulate_one(
            m, o, p + (size_t)i * np, pscale, k + (size_t)i * nk, nt, ts + (size_t)i * nt,
            my ? my + (size_t)i * nt * ny : NULL, sigma_data ? sigma_data + (size_t)i * nt * ny : NULL,
            nplist, plist, x + (size_t)i * nt * nx, y + (size_t)i * nt * ny,
            sigmay + (size_t)i * nt * ny, llh + i, sx ? sx + (size_t)i * nt * nplist * nx : NULL,
            sy ? sy + (size_t)i * nt * nplist * ny : NULL, sllh + (size_t)i * nplist,
            numsteps + (size_t)i * nt, NULL, &e);
        status[i] = s;
        if (s < 0) nfail++;
    }
    (void)nthreads;
    return nfail;
}

int oracle_run_simulations(const oracle_model* m, const oracle_options* o, int n,
                           const double* p, const int32_t* pscale, const double* k, int nt,
                           const double* ts, const double* my, const double* sigma_data,
                           int nplist, const int32_t* plist, double* x, double* y,
                           double* sigmay, double* llh, double* sx, double* sy, double* sllh,
                           int32_t* numsteps, int32_t* status, int nthreads) {
    return oracle_run_simulations_ext(m, o, n, p, pscale, k, nt, ts, my, sigma_data, nplist, plist, x, y,
                                      sigmay, llh, sx, sy, sllh, numsteps, status, NULL, nthreads);
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

static int simulate_asa_one(const oracle_model* m, const oracle_options* o, const double* p_scaled,
                            const int32_t* pscale, const double* k, int nt, const double* ts,
                            const double* my, const double* sigma_data, int nplist,
                            const int32_t* plist, double* x, double* y, double* sigmay, double* llh,
                            double* sllh, int32_t* numsteps, int64_t* nst_b, const inst_ext* e) {
    const oracle_adjoint_ops* A = &oracle_adjoint_impl;
    const int n = m->nx, ny = m->ny, np = m->np;
    const double t0 = 0.0;
    double* p = (double*)malloc(sizeof(double) * (np > 0 ? np : 1));
    for (int j = 0; j < np; j++) p[j] = unscale(p_scaled[j], pscale ? pscale[j] : 0);
    double* x0 = (double*)calloc((size_t)n + 1, sizeof(double));
    /* sx0 enters the gradient (handle_sx0_forward); a pre-equilibration runs
     * with forward sensitivities (the default sensi_meth_preeq, solver.h:2034) */
    double* sx0 = (double*)calloc((size_t)n * (nplist > 0 ? nplist : 1) + 1, sizeof(double));
    oracle_options of = *o;
    of.sensi = 1;
    /* the adjoint of a model with events is not restated */
    if (m->ne || initial_state(m, &of, p, pscale, k, nplist, plist, e, x0, sx0)) {
        invalidate_all(nt, n, ny, nplist, 0, x, y, sigmay, llh, NULL, NULL, sllh, numsteps);
        if (nst_b) *nst_b = 0;
        free(x0); free(sx0); free(p);
        return -99;
    }
    void* h = A->create(m, o, p, k, nplist, plist, x0);
    double* sig = (double*)malloc(sizeof(double) * (ny > 0 ? ny : 1));
    m->sigmay(sig, p, k);
    double* dydx = (double*)calloc((size_t)n * ny + 1, sizeof(double));
    double* dydp = (double*)calloc((size_t)np * ny + 1, sizeof(double));
    double* dsig = (double*)calloc((size_t)np * ny + 1, sizeof(double));
    m->dsigmaydp(dsig, p, k);
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
                double dJdy, dJds;
                *llh -= noise_jy(m->noise[iy], y[(size_t)it * ny + iy], mv, sgy[iy], &dJdy, &dJds);
                for (int i = 0; i < n; i++) dJydx[(size_t)it * n + i] += dJdy * dydx[(size_t)i * ny + iy];
                for (int is = 0; is < nplist; is++) sllh[is] -= dJdy * dydp[(size_t)plist[is] * ny + iy];
                if (!sigma_from_data(sigma_data, it, ny, iy))
                    for (int is = 0; is < nplist; is++) sllh[is] -= dJds * dsig[(size_t)plist[is] * ny + iy];
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
            for (int is = 0; is < nplist; is++) {
                double s0 = 0.0;
                for (int i = 0; i < n; i++) s0 += xB[i] * sx0[(size_t)is * n + i];
                sllh[is] -= s0 + xQB[is];
                sllh[is] *= scale_factor(p[plist[is]], pscale ? pscale[plist[is]] : 0);
            }
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
    free(dJydx); free(dydx); free(dydp); free(dsig); free(sig); free(x0); free(sx0); free(p);
    return status;
}

int oracle_simulate_asa(const oracle_model* m, const oracle_options* o, const double* p_scaled,
                        const int32_t* pscale, const double* k, int nt, const double* ts,
                        const double* my, const double* sigma_data, int nplist,
                        const int32_t* plist, double* x, double* y, double* sigmay, double* llh,
                        double* sllh, int32_t* numsteps, int64_t* nst_b) {
    return simulate_asa_one(m, o, p_scaled, pscale, k, nt, ts, my, sigma_data, nplist, plist, x, y, sigmay,
                            llh, sllh, numsteps, nst_b, NULL);
}

int oracle_run_simulations_asa_ext(const oracle_model* m, const oracle_options* o, int n,
                                   const double* p, const int32_t* pscale, const double* k, int nt,
                                   const double* ts, const double* my, const double* sigma_data,
                                   int nplist, const int32_t* plist, double* x, double* y,
                                   double* sigmay, double* llh, double* sllh, int32_t* numsteps,
                                   int32_t* status, int64_t* nst_b, const oracle_batch_ext* ext,
                                   int nthreads) {
    const int nx = m->nx, ny = m->ny, np = m->np, nk = m->nk;
    int nfail = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(+ : nfail)
#endif
    for (int i = 0; i < n; i++) {
        const inst_ext e = instance_ext(ext, i, nx, nk, nplist);
        int s = simulate_asa_one(
            m, o, p + (size_t)i * np, pscale, k + (size_t)i * nk, nt, ts + (size_t)i * nt,
            my ? my + (size_t)i * nt * ny : NULL, sigma_data ? sigma_data + (size_t)i * nt * ny : NULL,
            nplist, plist, x + (size_t)i * nt * nx, y + (size_t)i * nt * ny,
            sigmay + (size_t)i * nt * ny, llh + i, sllh + (size_t)i * nplist,
            numsteps + (size_t)i * nt, nst_b ? nst_b + i : NULL, &e);
        status[i] = s;
        if (s < 0) nfail++;
    }
    (void)nthreads;
    return nfail;
}

int oracle_run_simulations_asa(const oracle_model* m, const oracle_options* o, int n,
                               const double* p, const int32_t* pscale, const double* k, int nt,
                               const double* ts, const double* my, const double* sigma_data,
                               int nplist, const int32_t* plist, double* x, double* y,
                               double* sigmay, double* llh, double* sllh, int32_t* numsteps,
                               int32_t* status, int64_t* nst_b, int nthreads) {
    return oracle_run_simulations_asa_ext(m, o, n, p, pscale, k, nt, ts, my, sigma_data, nplist, plist, x, y,
                                          sigmay, llh, sllh, numsteps, status, nst_b, NULL, nthreads);
}
