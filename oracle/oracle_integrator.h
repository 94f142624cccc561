/*
 * Integrator interface between the AMICI glue (amici_glue.c) and an ODE
 * integrator — TEST INFRASTRUCTURE ONLY.  Two implementations exist: the
 * restated BDF integrator (bdf_oracle.c) and the reference's own CVODES,
 * compiled from the reference sources (ref_cvodes_driver.c, built by
 * Makefile.ref).  Mirrors the Solver calls AMICI makes per output
 * (src/solver.cpp:141-160: set_stop_time(tout), remaining-step budget,
 * CVode(tout, NORMAL)).
 */
#ifndef AMICI_GB300_ORACLE_INTEGRATOR_H
#define AMICI_GB300_ORACLE_INTEGRATOR_H

#include <stdint.h>

#include "bdf_oracle.h"

typedef struct oracle_integrator {
    /* x0[nx], sx0[ns*nx] (w.r.t. unscaled parameters); p unscaled */
    void* (*create)(const oracle_model* m, const oracle_options* o, const double* p,
                    const double* k, int ns, const int32_t* plist, const double* x0,
                    const double* sx0);
    /* integrate to tout with stop time tout; returns a CVODES flag (<0 fails) */
    int (*solve)(void* h, double tout, int64_t mxstep, double* tret);
    /* one step towards tout without a stop time (CVode ONE_STEP, as
     * Solver::step runs it for the simulation to steady state) */
    int (*one_step)(void* h, double tout, double* tret);
    const double* (*x)(void* h);
    const double* (*sx)(void* h);
    int64_t (*nst)(void* h);
    void (*destroy)(void* h);
    /* CVodeSolver::reinit + reset_state and sens_reinit after an event
     * (solver_cvodes.cpp:471-505,586-616): the state (and sensitivities, may
     * be NULL) at t, order 1; the next solve starts with reInit_post_process */
    void (*reinit)(void* h, double t, const double* x, const double* sx);
    /* CVodeGetRootInfo after a CV_ROOT_RETURN (2): per trigger function +1 /
     * -1 for a zero crossing upwards / downwards, 0 otherwise */
    void (*root_info)(void* h, int* iroots);
} oracle_integrator;

extern const oracle_integrator oracle_integrator_impl;

#endif
