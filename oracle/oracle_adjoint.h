/*
 * Adjoint sensitivity analysis (ASA) in the CPU oracle — TEST INFRASTRUCTURE
 * ONLY.
 *
 * The operations AMICI's backward problem asks of its solver
 * (src/backwardproblem.cpp:267-332, src/solver.cpp:180-191,267-298,
 * src/solver_cvodes.cpp:470-640,700-860), implemented twice: by the restated
 * integrator (bdf_oracle.c) and by the reference's own CVODES
 * (ref_cvodes_driver.c).  The AMICI glue above them (amici_glue.c) restates
 * the backward loop and the gradient assembly once.
 *
 * The backward right-hand sides are those of an ODE model in AMICI
 * (src/model_ode.cpp:305-374): xBdot = -J(x(t))^T xB, the backward Jacobian
 * -J^T, and the quadrature qBdot_ip = -(dxdot/dp_{plist[ip]})^T xB.
 */
#ifndef AMICI_GB300_ORACLE_ADJOINT_H
#define AMICI_GB300_ORACLE_ADJOINT_H

#include <stddef.h>
#include <stdint.h>

#include "bdf_oracle.h"

typedef struct oracle_adjoint_ops {
    /* forward memory with adjoint storage (CVodeAdjInit(maxsteps + 1,
     * CV_POLYNOMIAL), solver_cvodes.cpp:726-739); p unscaled */
    void* (*create)(const oracle_model* m, const oracle_options* o, const double* p,
                    const double* k, int nplist, const int32_t* plist, const double* x0);
    /* forward to tout with stop time tout (CVodeF, cvodea.c:395) */
    int (*solve_f)(void* h, double tout, int64_t mxstep, double* tret);
    const double* (*x)(void* h);
    int64_t (*nst)(void* h);
    /* Solver::setup_b: CVodeCreateB/InitB/QuadInitB, tolerances, quadrature
     * error control (solver.cpp:267-298,658-691) */
    int (*setup_b)(void* h, double tB0, const double* xB0, const double* xQB0);
    /* Solver::run_b (solver.cpp:180-191) with its step budget
     * (apply_max_num_steps_B, solver.cpp:121-139) */
    int (*run_b)(void* h, double tBout, int64_t mxstepsB);
    /* write_solution_b: CVodeGetB, CVodeGetQuadB */
    void (*get_b)(void* h, double* xB, double* xQB);
    /* CVodeSolver::reinit_b / reinit_quad_b (solver_cvodes.cpp:618-648) */
    void (*reinit_b)(void* h, double t, const double* xB, const double* xQB);
    int64_t (*nst_b)(void* h);
    void (*destroy)(void* h);
} oracle_adjoint_ops;

extern const oracle_adjoint_ops oracle_adjoint_impl;

/* ---- backward right-hand sides of an ODE model (model_ode.cpp:305-374) --- */
/* J is column-major: J[j*n + i] = d xdot_i / d x_j */
static inline void oracle_fxBdot(const oracle_model* m, const double* p, const double* k, double* J,
                                 double t, const double* x, const double* xB, double* xBdot) {
    const int n = m->nx;
    m->jac(J, t, x, p, k);
    for (int j = 0; j < n; j++) {
        const double* col = J + (size_t)j * n;
        double s = 0.0;
        for (int i = 0; i < n; i++) s += col[i] * xB[i];
        xBdot[j] = -s;
    }
}

/* JB = -J^T, column-major */
static inline void oracle_fJB(const oracle_model* m, const double* p, const double* k, double* J,
                              double t, const double* x, double* JB) {
    const int n = m->nx;
    m->jac(J, t, x, p, k);
    for (int c = 0; c < n; c++)
        for (int r = 0; r < n; r++) JB[(size_t)c * n + r] = -J[(size_t)r * n + c];
}

/* qBdot[ip] = -sum_i dxdot_i/dp_{plist[ip]} * xB_i */
static inline void oracle_fqBdot(const oracle_model* m, const double* p, const double* k, double* dfdp,
                                 int nplist, const int32_t* plist, double t, const double* x,
                                 const double* xB, double* qBdot) {
    const int n = m->nx;
    m->dxdotdp(dfdp, t, x, p, k);
    for (int ip = 0; ip < nplist; ip++) {
        const double* col = dfdp + (size_t)plist[ip] * n;
        double s = 0.0;
        for (int i = 0; i < n; i++) s += col[i] * xB[i];
        qBdot[ip] = -s;
    }
}

#ifdef __cplusplus
extern "C" {
#endif

/* One instance with adjoint sensitivities: outputs as oracle_simulate plus
 * sllh[nplist] from the backward problem; nst_b (may be NULL) receives the
 * number of backward steps. */
int oracle_simulate_asa(const oracle_model* m, const oracle_options* o, const double* p,
                        const int32_t* pscale, const double* k, int nt, const double* ts,
                        const double* my, const double* sigma_data, int nplist,
                        const int32_t* plist, double* x, double* y, double* sigmay, double* llh,
                        double* sllh, int32_t* numsteps, int64_t* nst_b);

int oracle_run_simulations_asa(const oracle_model* m, const oracle_options* o, int n,
                               const double* p, const int32_t* pscale, const double* k, int nt,
                               const double* ts, const double* my, const double* sigma_data,
                               int nplist, const int32_t* plist, double* x, double* y,
                               double* sigmay, double* llh, double* sllh, int32_t* numsteps,
                               int32_t* status, int64_t* nst_b, int nthreads);

/* oracle_run_simulations_asa with pre-equilibration (run with forward
 * sensitivities, the reference's default pre-equilibration sensitivity
 * method) and initial-state overrides; ext may be NULL. */
int oracle_run_simulations_asa_ext(const oracle_model* m, const oracle_options* o, int n,
                                   const double* p, const int32_t* pscale, const double* k, int nt,
                                   const double* ts, const double* my, const double* sigma_data,
                                   int nplist, const int32_t* plist, double* x, double* y,
                                   double* sigmay, double* llh, double* sllh, int32_t* numsteps,
                                   int32_t* status, int64_t* nst_b, const oracle_batch_ext* ext,
                                   int nthreads);

#ifdef __cplusplus
}
#endif
#endif
