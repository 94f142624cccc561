/*
 * amici_gb300 — C ABI of the GB300-native batched stiff-ODE simulation engine.
 *
 * Every compiled model is one shared library (libamici_gb300_<model>.so, as
 * every AMICI model is its own compiled module) exporting the functions
 * below.  Plain C types only; buffers are caller-owned.  No exception or
 * C++ type crosses this boundary: every failure is a return code (per call)
 * or a per-instance status (AMICI_* codes, include/amici/defines.h:66-104 of
 * the reference).
 *
 * Reference interfaces replaced:
 *   amici::run_simulations(Solver const&, std::vector<ExpData*> const&,
 *       Model const&, bool failfast, int num_threads)
 *       -- include/amici/amici.h:29-40, src/amici.cpp:220-264
 *   amici::run_simulation(Solver&, ExpData const*, Model&, bool rethrow)
 *       -- include/amici/amici.h:21-27, src/amici.cpp:65-218
 *   ReturnData fields x, y, sigmay, llh, sx, sy, sllh, numsteps, status
 *       -- include/amici/rdata.h:129-498 (shapes: python/sdist/amici/sim/
 *          sundials/_numpy.py:414-440)
 *   Solver options -- include/amici/solver.h (setters, defaults :1869-2112)
 */
#ifndef AMICI_GB300_H
#define AMICI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AMICI_GB300_ABI_VERSION 3

/* call-level return codes */
#define AMICI_GB300_OK 0
#define AMICI_GB300_ERR_ARG (-1)     /* invalid argument (NULL pointer, size) */
#define AMICI_GB300_ERR_CUDA (-2)    /* CUDA runtime error */
#define AMICI_GB300_ERR_UNSUPPORTED (-3)

/* per-instance status codes (subset of AMICI's defines.h) */
#define AMICI_GB300_SUCCESS 0
#define AMICI_GB300_TOO_MUCH_WORK (-1)
#define AMICI_GB300_TOO_MUCH_ACC (-2)
#define AMICI_GB300_ERR_FAILURE (-3)
#define AMICI_GB300_CONV_FAILURE (-4)
#define AMICI_GB300_ILL_INPUT (-22)
#define AMICI_GB300_ERROR (-99)
#define AMICI_GB300_NOT_RUN (-1001)

/* sensitivity method (amici::SensitivityMethod, defines.h) */
#define AMICI_GB300_SENSI_NONE 0
#define AMICI_GB300_SENSI_FORWARD 1
#define AMICI_GB300_SENSI_ADJOINT 2

/* parameter scale (amici::ParameterScaling) */
#define AMICI_GB300_PSCALE_LIN 0
#define AMICI_GB300_PSCALE_LN 1
#define AMICI_GB300_PSCALE_LOG10 2

/* Model dimensions (amici::ModelDimensions, include/amici/model_dimensions.h). */
typedef struct amici_gb300_model_dims {
    int32_t nx;   /* states */
    int32_t np;   /* free parameters */
    int32_t nk;   /* fixed parameters */
    int32_t ny;   /* observables */
    int32_t nw;   /* fluxes (AMICI "expressions") */
    int32_t nnz_jac; /* structural nonzeros of dxdot/dx */
} amici_gb300_model_dims;

/* Solver options (amici::Solver setters; NaN = inherit, as in the reference). */
typedef struct amici_gb300_solver_options {
    double rtol, atol;           /* set_relative_tolerance / set_absolute_tolerance */
    double rtol_fsa, atol_fsa;   /* set_relative/absolute_tolerance_fsa */
    double rtol_b, atol_b;       /* backward problem */
    double rtol_quad, atol_quad; /* quadratures */
    int64_t maxsteps;            /* set_max_steps (cumulative over outputs) */
    double max_step_size;        /* set_max_step_size; <=0 or inf: none */
    int32_t sensi_order;         /* 0 none, 1 first */
    int32_t sensi_meth;          /* AMICI_GB300_SENSI_* */
    int32_t max_nonlin_iters;    /* set_max_nonlin_iters (default 3) */
    int32_t max_conv_fails;      /* set_max_conv_fails (default 10) */
    int32_t lu_precision;        /* 32: factorise M = I - gamma*J in FP32; 64: FP64 */
    int32_t lanes_per_instance;  /* 0: autotuned; else 1,2,4,8,16,32 */
    int32_t checkpoint_steps;    /* adjoint: forward checkpoint spacing (0: default) */
    int32_t control_precision;   /* 32: step-size/order heuristics in FP32; 64: FP64 */
    int32_t launch_mode;         /* 0: one persistent batched launch; 1: one launch per instance */
    int32_t instances_per_sm;    /* 0: automatic; else at most this many resident instances per SM,
                                    the rest of the SM's on-chip memory left to the L1 cache */
    int32_t stldet;              /* set_stability_limit_flag: BDF stability-limit detection in the
                                    forward and backward problems (default 1, solver.h:2037) */
    int32_t reserved;            /* 0 */
} amici_gb300_solver_options;

/* One batch of instances (the ExpData list) and its results (ReturnData).
 * Arrays are row-major with the instance index outermost; shapes:
 *   p[N,np] (scaled), pscale[np], k[N,nk], ts[N,nt], my[N,nt,ny] (NaN =
 *   missing; NULL = no data -> llh NaN), sigma_y[N,nt,ny] (NaN = model
 *   value; NULL = model values), plist[nplist];
 *   x[N,nt,nx], y[N,nt,ny], sigmay[N,nt,ny], llh[N], sx[N,nt,nplist,nx],
 *   sy[N,nt,nplist,ny], sllh[N,nplist], numsteps[N,nt], status[N].
 * Output pointers may be NULL when not wanted (x, y, sigmay, sx, sy, diag).
 * diag[N,8] (int32) receives per-instance solver counters (ReturnData
 * diagnostics, rdata.h:267-301): steps, RHS evaluations, Newton iterations,
 * linear-solver setups, error-test failures, convergence failures, Jacobian
 * evaluations, backward steps (adjoint sensitivities; else 0).
 * With sensi_meth AMICI_GB300_SENSI_ADJOINT, sllh comes from the backward
 * problem with quadratures (AMICI's BackwardProblem) and sx, sy are not
 * written; my is required (sllh is NaN without data).
 *
 * Initial states and pre-equilibration (ExpData x0, sx0 and
 * fixed_parameters_pre_equilibration, include/amici/edata.h,
 * simulation_parameters.h:145-247; ReturnData x_ss, sx_ss, preeq_*,
 * rdata.h): x0[N,nx] replaces the model's initial states, sx0[N,nplist,nx]
 * (w.r.t. the scaled parameters of plist) its initial state sensitivities.
 * With k_preeq[N,nk] every instance is first brought to steady state at
 * those fixed parameters (the reference's default: simulation only, one
 * step at a time until the WRMS norm of xdot, and with sensitivities of
 * every sensitivity right-hand side, is below 1 at 100 x the tolerances;
 * with adjoint sensitivities the pre-equilibration runs with forward
 * sensitivities, as the reference's default sensi_meth_preeq), and the main
 * simulation starts from that steady state at k.  x_ss[N,nx], sx_ss[N,
 * nplist,nx] (scaled parameters), preeq_status[N] (1 steady state found, -2
 * step budget exhausted or too much work, -5 time overflow, -1 other
 * failure), preeq_numsteps[N], preeq_t[N] and preeq_wrms[N] receive its
 * results when not NULL.  An instance without a steady state is not
 * simulated: status AMICI_GB300_ERROR, outputs NaN, no steps.  Models compiled
 * without the pre-equilibration kernels refuse k_preeq
 * (AMICI_GB300_ERR_UNSUPPORTED), as does launch_mode 1.
 *
 * Post-equilibration (ExpData output times inf; ForwardProblem::
 * handle_postequilibration, forwardproblem.cpp:376-387; ReturnData posteq_*):
 * with posteq = 1 the output times may end with inf; after the last finite
 * output the solver continues, one step at a time, to steady state (the same
 * criterion as the pre-equilibration), and the outputs at inf are taken
 * there (numsteps 0 at those outputs).  posteq_status[N], posteq_numsteps[N],
 * posteq_t[N] and posteq_wrms[N] receive its results when not NULL; a failed
 * post-equilibration gives status AMICI_GB300_ERROR with every output kept,
 * as the reference does.  The host entry sets posteq itself when ts holds
 * inf.  Refused (AMICI_GB300_ERR_UNSUPPORTED): adjoint sensitivities, models
 * with events, models compiled without the post-equilibration kernels,
 * launch_mode 1. */
typedef struct amici_gb300_batch {
    int32_t n_instances;
    int32_t nt;
    int32_t nplist;
    int32_t posteq;
    const double* p;
    const int32_t* pscale;
    const double* k;
    const double* ts;
    const double* my;
    const double* sigma_y;
    const int32_t* plist;
    double* x;
    double* y;
    double* sigmay;
    double* llh;
    double* sx;
    double* sy;
    double* sllh;
    int32_t* numsteps;
    int32_t* status;
    int32_t* diag;
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
} amici_gb300_batch;

/* ABI version of the library (must equal AMICI_GB300_ABI_VERSION). */
int32_t amici_gb300_abi_version(void);

/* Model name and dimensions (amici::Model::get_name / dimensions). */
const char* amici_gb300_model_name(void);
int32_t amici_gb300_model_dims_get(amici_gb300_model_dims* out);

/* Default solver options (the reference Solver's defaults, solver.h:1869-2112). */
void amici_gb300_default_options(amici_gb300_solver_options* out);

/* Batched simulation with DEVICE buffers on the caller's CUDA stream
 * (cudaStream_t passed as void*; NULL = default stream).  Replaces
 * amici::run_simulations for an ODE model (with events, trigger functions and
 * Heaviside switches in forward simulation and forward sensitivities; the
 * adjoint of a model with events is refused); asynchronous.  Temporary device
 * memory is allocated with stream-ordered cudaMallocAsync: the work-queue
 * counters, with pre-equilibration its steady states, and with forward or
 * adjoint sensitivities a per-group scratch of groups x stride doubles (the
 * sensitivity history or the check points and backward work arrays). */
int32_t amici_gb300_run_simulations_device(const amici_gb300_solver_options* opts,
                                           const amici_gb300_batch* batch, void* stream);

/* Same with HOST buffers: copies inputs host->device, runs, copies results
 * device->host and synchronises the stream before returning.  Device buffers
 * are cached in the library and reused across calls. */
int32_t amici_gb300_run_simulations_host(const amici_gb300_solver_options* opts,
                                         const amici_gb300_batch* batch, void* stream);

/* Allocation-free variant of amici_gb300_run_simulations_device (no
 * counterpart in the reference, which has no device path).  For callers that
 * cannot let a library enter the CUDA allocator: applications that reserve all
 * device memory up front in their own pool, and latency-critical callers for
 * which a stream-ordered allocation that has to grow its pool is an unbounded
 * stall.  Forward simulation only: it takes the same options, device buffers
 * and stream, but a request with sensitivities (sensi_order > 0, forward or
 * adjoint) fails with AMICI_GB300_ERR_UNSUPPORTED, because the sensitivity
 * kernels need per-call scratch proportional to the batch.  It allocates
 * nothing: its only scratch (the persistent kernel's work-queue counters) is
 * a fixed device array of AMICI_GB300_NOALLOC_MAX_COUNTERS unsigned ints in
 * the library, held by every GPU that loads it until exit.  One counter is
 * used per call, one per instance in per-instance launch mode (launch_mode
 * 1), which is therefore limited to AMICI_GB300_NOALLOC_MAX_COUNTERS
 * instances; larger requests fail with AMICI_GB300_ERR_UNSUPPORTED.  The
 * first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current and keeps it for the life
 * of the process; make that first call before any stream capture, and do not
 * call this entry point again after a cudaDeviceReset of that device (the
 * kept address belongs to the destroyed context).  All calls share the array
 * and zero the counters they use on the given stream, so calls that overlap
 * on the GPU (other streams, other host threads) race: serialise them. */
#define AMICI_GB300_NOALLOC_MAX_COUNTERS 4096
int32_t amici_gb300_run_simulations_device_noalloc(const amici_gb300_solver_options* opts,
                                                   const amici_gb300_batch* batch, void* stream);

/* Message for the last failing call on this thread ("" if none). */
const char* amici_gb300_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
