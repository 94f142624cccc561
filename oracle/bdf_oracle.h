/*
 * CPU oracle for the batched stiff-ODE path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement of what AMICI's simulation path computes for an ODE
 * model: amici::run_simulation (src/amici.cpp:65-218) driving CVODES' BDF
 * integrator (ThirdParty/sundials/src/cvodes/cvodes.c) with a stop time at
 * every output (src/solver.cpp:141-160), dense LU (sundials_dense.c:82-175),
 * staggered forward sensitivities (cvodes.c:7167-7218, cvodes_nls_stg.c) and
 * the Gaussian log-likelihood of ReturnData (src/rdata.cpp:368-432,
 * src/model.cpp:1194-1240).  Only tests, the smoke check and the CPU baseline
 * of the benchmark use this library; the product path never does.
 */
#ifndef AMICI_GB300_BDF_ORACLE_H
#define AMICI_GB300_BDF_ORACLE_H

#include <stdint.h>

#include "oracle_model.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_options {
    double rtol, atol;         /* Solver::set_relative/absolute_tolerance */
    double rtol_fsa, atol_fsa; /* NaN = inherit (solver.h:2063-2072) */
    int64_t maxsteps;          /* cumulative over outputs (solver.cpp:107-119) */
    int32_t sensi;             /* 0 none, 1 forward sensitivities (staggered) */
    int32_t max_nonlin_iters;  /* solver.h:2108, default 3 */
    int32_t max_conv_fails;    /* solver.h:2112, default 10 */
    int32_t lu_f32;            /* 1: iteration matrix factorised in float */
    double max_step_size;      /* <=0 or inf: unlimited */
    int32_t stldet;            /* stability-limit detection (Solver::set_stability_limit_flag, default on) */
    /* adjoint problem (solver.cpp:658-691, solver.h:2063-2078) */
    double rtol_b, atol_b;       /* NaN = inherit rtol/atol */
    double rtol_quad, atol_quad; /* NaN = inherit rtol/atol; inf disables error control */
    int64_t maxsteps_b;          /* 0: 100 * maxsteps (solver.cpp:125) */
} oracle_options;

/* Pre-equilibration and initial-state overrides of a batch (ExpData
 * fixed_parameters_pre_equilibration, x0, sx0; include/amici/edata.h and
 * simulation_parameters.h:174,183) and the steady-state results (ReturnData
 * x_ss, sx_ss, preeq_status, preeq_numsteps, preeq_t, preeq_wrms).  Arrays
 * are [n, ...]; every pointer may be NULL.  sx0 and sx_ss are w.r.t. the
 * scaled parameters of plist, [n, nplist, nx].  preeq_status is the status
 * of the simulation stage (SteadyStateStatus: 1 success, -1 failed, -2 too
 * much work, -5 simulation too long; 0 not run).  posteq_status,
 * posteq_numsteps, posteq_t, posteq_wrms: the same for the
 * post-equilibration (outputs at t = inf; ReturnData posteq_*). */
typedef struct oracle_batch_ext {
    const double* k_preeq;
    const double* x0;
    const double* sx0;
    double* x_ss;
    double* sx_ss;
    int32_t* preeq_status;
    int32_t* preeq_numsteps;
    double* preeq_t;
    double* preeq_wrms;
    int32_t* posteq_status;
    int32_t* posteq_numsteps;
    double* posteq_t;
    double* posteq_wrms;
} oracle_batch_ext;

/* Per-instance counters (ReturnData diagnostics, rdata.h:267-301). */
typedef struct oracle_stats {
    int64_t nst, nfe, nni, nsetups, nje, netf, ncfn, netfS, ncfnS;
} oracle_stats;

/* One instance.  p is SCALED by pscale (0 lin, 1 ln, 2 log10).
 * Outputs (row-major): x[nt*nx], y[nt*ny], sigmay[nt*ny], sx[nt*nplist*nx],
 * sy[nt*nplist*ny], sllh[nplist], numsteps[nt].  my/sigma_data may be NULL. */
int oracle_simulate(const oracle_model* m, const oracle_options* o,
                    const double* p, const int32_t* pscale, const double* k,
                    int nt, const double* ts, const double* my,
                    const double* sigma_data, int nplist, const int32_t* plist,
                    double* x, double* y, double* sigmay, double* llh,
                    double* sx, double* sy, double* sllh, int32_t* numsteps,
                    oracle_stats* stats);

/* Batch over n instances with arrays laid out [n, ...]; nthreads <= 0 means
 * all host threads (OpenMP).  Returns the number of instances with status<0. */
int oracle_run_simulations(const oracle_model* m, const oracle_options* o, int n,
                           const double* p, const int32_t* pscale,
                           const double* k, int nt, const double* ts,
                           const double* my, const double* sigma_data,
                           int nplist, const int32_t* plist, double* x,
                           double* y, double* sigmay, double* llh, double* sx,
                           double* sy, double* sllh, int32_t* numsteps,
                           int32_t* status, int nthreads);

/* oracle_run_simulations with pre-equilibration and initial-state
 * overrides (ext may be NULL). */
int oracle_run_simulations_ext(const oracle_model* m, const oracle_options* o, int n,
                               const double* p, const int32_t* pscale,
                               const double* k, int nt, const double* ts,
                               const double* my, const double* sigma_data,
                               int nplist, const int32_t* plist, double* x,
                               double* y, double* sigmay, double* llh, double* sx,
                               double* sy, double* sllh, int32_t* numsteps,
                               int32_t* status, const oracle_batch_ext* ext, int nthreads);

const oracle_model* oracle_get_model(void);

#ifdef __cplusplus
}
#endif
#endif
