/*
 * Model ABI of the CPU oracle (test infrastructure only).
 *
 * The same function set as AMICI's generated model files for an ODE model
 * (python/sdist/amici/exporters/sundials/cxx_functions.py:102-410, overridden
 * in models/model_robertson_py/model_robertson_py.h:200-540): initial states,
 * right-hand side, Jacobian, parameter derivative of the right-hand side,
 * observables and noise scales.  All parameters passed in are UNSCALED.
 * Dense matrices are column-major: J[j*nx + i] = d xdot_i / d x_j.
 */
#ifndef AMICI_GB300_ORACLE_MODEL_H
#define AMICI_GB300_ORACLE_MODEL_H

typedef struct oracle_model {
    const char* name;
    int nx, np, nk, ny;
    void (*x0)(double* x0, const double* p, const double* k);
    /* sx0[j*nx + i] = d x0_i / d p_j, all np parameters */
    void (*dx0dp)(double* sx0, const double* p, const double* k);
    void (*xdot)(double* xdot, double t, const double* x, const double* p, const double* k);
    void (*jac)(double* J, double t, const double* x, const double* p, const double* k);
    /* dfdp[j*nx + i] = d xdot_i / d p_j */
    void (*dxdotdp)(double* dfdp, double t, const double* x, const double* p, const double* k);
    void (*y)(double* y, double t, const double* x, const double* p, const double* k);
    /* dydx[j*ny + i] = d y_i / d x_j */
    void (*dydx)(double* dydx, double t, const double* x, const double* p, const double* k);
    /* dydp[j*ny + i] = d y_i / d p_j */
    void (*dydp)(double* dydp, double t, const double* x, const double* p, const double* k);
    void (*sigmay)(double* sigmay, const double* p, const double* k);
    /* dsigmay[j*ny + i] = d sigmay_i / d p_j */
    void (*dsigmaydp)(double* dsigmay, const double* p, const double* k);
    /* noise distribution per observable (importers/utils.py:110-130): 0
     * normal, 1 log-normal, 2 log10-normal, 3 laplace, 4 log-laplace, 5
     * log10-laplace */
    const int* noise;
    /* events whose triggers are explicit in time (Model::reinit_explicit_roots,
     * model.cpp:444-470): event ie fires at t = te_ie(p, k), then the states
     * jump by deltax (fdeltax, model.cpp:1481-1503), affine in x */
    int ne;
    void (*event_times)(double* te, const double* p, const double* k);
    /* d[j*ne + ie] = d te_ie / d p_j */
    void (*devent_times_dp)(double* d, const double* p, const double* k);
    void (*deltax)(double* dx, int ie, double t, const double* x, const double* p, const double* k);
    /* d[j*nx + i] = d deltax_i / d x_j (constant) */
    void (*ddeltaxdx)(double* d, int ie);
    /* d[j*nx + i] = d deltax_i / d p_j */
    void (*ddeltaxdp)(double* d, int ie, const double* p, const double* k);
    /* the trigger's value before t0 (1 true: no event at t0) */
    const int* event_initial_value;
    /* events with a trigger function g(t, x, p, k) (CVODES root finding);
     * root function ir belongs to event root_event[ir]; the other events
     * have explicit trigger times */
    int nroot;
    const int* root_event;
    void (*root)(double* g, double t, const double* x, const double* p, const double* k);
    /* d g_ir / d x (nx), d g_ir / d p (np), d g_ir / d t */
    void (*drootdx)(double* d, int ir, double t, const double* x, const double* p, const double* k);
    void (*drootdp)(double* d, int ir, double t, const double* x, const double* p, const double* k);
    double (*drootdt)(int ir, double t, const double* x, const double* p, const double* k);
    /* Heaviside indicators of the right-hand side (Model::update_heaviside,
     * model.cpp:1588-1592): indicator j is k[nk + j], the Heaviside of the
     * trigger function of event h_event[j] */
    int nh;
    const int* h_event;
    /* explicit trigger times: the trigger is event_dir[ie] * (t - te) */
    const int* event_dir;
} oracle_model;

#endif
