// GB300 (sm_103a) batched BDF engine: forward simulation of many model
// instances in one persistent kernel.
//
// Execution model.  A *group* of G consecutive lanes of a warp (G in
// {1,2,4,8,16,32}) integrates one instance; a warp holds 32/G instances.
// On GB300 an FP64 warp instruction occupies the FP64 pipe for the same time
// whatever its active mask (measured: one active lane costs as much as 32),
// and FP64 runs at 1/64 of the FP32 rate.  The kernel is built around that:
//   * element i of a state-sized vector lives in register slot i / G of lane
//     i % G; all loops over the BDF order q are specialised at compile time,
//     so the Nordsieck history never leaves registers;
//   * only the quantities that set the solution accuracy are FP64: states,
//     Newton residuals and corrections, the weighted RMS norms, the Nordsieck
//     history, t, h and the BDF coefficients l (hence gamma);
//   * the iteration matrix M = I - gamma*J is factorised in FP32 (shared
//     memory, partial pivoting) and the triangular solves run in FP32 with
//     warp shuffles; modified Newton on FP64 residuals tolerates the
//     approximate M;
//   * the step-size/order heuristics (eta, error constants, convergence-rate
//     estimates) run in the control type R (FP32 by default, using the SFU
//     for powers), so their cost is not paid at the FP64 rate;
//   * several instances per warp amortise the remaining group-uniform scalar
//     work; groups pull instance indices from a global work queue, so
//     instances with very different step counts keep every group busy.
//
// Algorithm.  The integrator restates CVODES' variable-order BDF method as
// AMICI drives it (the reference's ThirdParty/sundials/src/cvodes/cvodes.c,
// cvodes_nls.c, cvodes_ls.c; src/solver.cpp:141-160): Nordsieck predictor
// (cvPredict, cvodes.c:6507), BDF coefficients (cvSetBDF/cvSetTqBDF
// :6788-6892), modified Newton with the linear-solver setup heuristics (cvNls
// :6894, cvNlsConvTest cvodes_nls.c:303, cvLsSetup cvodes_ls.c:1611, msbp=20,
// dgmax=0.3, msbj=51, dgmax_jbad=0.2), local error test (cvDoErrorTest
// :7461), history update and order/step selection (cvCompleteStep :7634,
// cvPrepareNextStep :7747, cvChooseEta :7935), initial step (cvHin :5436)
// and a stop time at every output (cvodes.c:3270-3330).  With R = double and
// an FP64 LU the arithmetic follows CVODES operation for operation (up to
// fused multiply-adds and the order of the norm reductions).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace agb {

constexpr int QMAX = 5;
constexpr int LMAX = QMAX + 1;
// cvodes_impl.h:55-135,178-204; cvodes.c:280-305; cvodes_ls_impl.h:40-41
constexpr double ETA_MIN_FX = 0.0, ETA_MAX_FX = 1.5, ETA_MAX_FS = 10000.0;
constexpr double ETA_MAX_ES = 10.0, ETA_MAX_GS = 10.0, ETA_MIN = 0.1;
constexpr double ETA_MAX_EF = 0.2, ETA_MIN_EF = 0.1, ETA_CF = 0.25;
constexpr int SMALL_NST = 10, SMALL_NEF = 2, LONG_WAIT = 10, MXNEF = 7, MXNEF1 = 3;
constexpr double ADDON = 0.000001, BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0;
constexpr double CRDOWN = 0.3, RDIV = 2.0, FUZZ_FACTOR = 100.0, HLB_FACTOR = 100.0;
constexpr double HUB_FACTOR = 0.1, H_BIAS = 0.5, CORTES = 0.1, DGMAX_LSETUP = 0.3;
constexpr double DGMAX_JBAD = 0.2;
constexpr int MAX_ITERS = 4, MSBP = 20, MSBJ = 51;
constexpr double UROUND = 2.220446049250313e-16;
constexpr double SLD_TINY = 1.0e-10;  // TINY of cvodes.c:204

// internal flags (cvodes_impl.h:178-185)
constexpr int CV_SUCCESS = 0, CV_TSTOP_RETURN = 1, CV_ROOT_RETURN = 2, CV_TOO_MUCH_WORK = -1, CV_TOO_MUCH_ACC = -2,
              CV_ERR_FAILURE = -3, CV_CONV_FAILURE = -4, CV_ILL_INPUT = -22;
constexpr int DO_ERROR_TEST = 2, PREDICT_AGAIN = 3, TRY_AGAIN = 5, FIRST_CALL = 6,
              PREV_CONV_FAIL = 7, PREV_ERR_FAIL = 9, NLS_CONV_RECVR = 901, NLS_CONTINUE = 902;
constexpr int CV_NO_FAILURES = 0, CV_FAIL_BAD_J = 1, CV_FAIL_OTHER = 2;

struct Opts {
    double rtol, atol, rtolS, atolS;
    int64_t maxsteps;
    int maxcor, maxncf;
    double hmax_inv;
    // adjoint problem: backward state and quadrature tolerances
    // (Solver::apply_tolerances_asa / apply_quad_tolerances_asa, solver.cpp:658-691)
    double rtolB, atolB, rtolQ, atolQ;
    int errconQ;
    int64_t maxstepsB;
    int ipsm;  // launch: cap on resident instances per SM (0: automatic)
    // BDF stability-limit detection (CVodeSetStabLimDet; on by default in the
    // reference Solver, include/amici/solver.h:2037), forward and backward
    int stldet;
};

// Device-side view of one batch (all device pointers; see amici_gb300.h).
struct Batch {
    int n, nt, nplist;
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
    int32_t* diag;        // [n, 8] solver counters, or NULL
    unsigned int* queue;  // work-queue counter (scratch, zeroed before launch)
    // forward sensitivities: per-group scratch for the sensitivity columns
    // (Nordsieck history, weights, corrections, residuals), sens_stride doubles per group
    double* sens_scratch;
    long long sens_stride;
    int nsp;              // nplist rounded up to a multiple of the group size
    // adjoint sensitivities: per-group scratch holding the forward steps for
    // the interpolant (times, states, orders), dJy/dx per output and the
    // quadrature history; adj_stride doubles per group, adj_cap points
    double* adj_scratch;
    long long adj_stride;
    long long adj_cap;
    int ck_k;             // adjoint check-point spacing in steps (0: every step stored)
    long long ck_cap;     // check points per group
    // initial states [n, NX] and their sensitivities [n, nplist, NX] w.r.t.
    // the scaled parameters of plist (ExpData x0 / sx0, or the steady state of
    // a pre-equilibration); NULL: the model's x0(p, k) and dx0/dp
    const double* x0;
    const double* sx0;
    // [n] status of this batch's pre-equilibration (1: steady state found);
    // an instance without one is not simulated (status AMICI_ERROR, outputs
    // invalid, no steps); NULL: no pre-equilibration
    const int32_t* preeq_in;
    // a pre-equilibration launch: simulation to steady state at the fixed
    // parameters k, writing the steady state [n, NX], its sensitivities [n,
    // nplist, NX] (scaled parameters), the simulation stage's status (1
    // success, -2 step budget, -5 time overflow, -1 other failure), steps,
    // time and residual norm
    int preeq;
    double* x_ss;
    double* sx_ss;
    int32_t* preeq_status;
    int32_t* preeq_numsteps;
    double* preeq_t;
    double* preeq_wrms;
    // post-equilibration (outputs at t = inf; kernels compiled with POSTEQ):
    // status of the simulation stage, its steps, time and norm per instance
    int32_t* posteq_status;
    int32_t* posteq_numsteps;
    double* posteq_t;
    double* posteq_wrms;
};

// Negative log-likelihood of one measurement m of the simulated y with scale
// s, and its derivatives w.r.t. y and s, for the reference's noise
// distributions (python/sdist/amici/importers/utils.py:110-130; the generated
// Jy, dJydy, dJydsigma): 0 normal, 1 log-normal, 2 log10-normal, 3 laplace,
// 4 log-laplace, 5 log10-laplace.
__device__ __forceinline__ double noise_jy(int kind, double y, double m, double s, double& djdy, double& djds) {
    constexpr double ln10 = 2.302585092994046, two_pi = 6.283185307179586;
    auto sgn = [](double e) { return e > 0.0 ? 1.0 : (e < 0.0 ? -1.0 : 0.0); };
    double r, e;
    switch (kind) {
    case 1:
        r = (log(y) - log(m)) / s;
        djdy = r / (s * y);
        djds = 1.0 / s - r * r / s;
        return 0.5 * log(two_pi * s * s * m * m) + 0.5 * r * r;
    case 2:
        r = (log10(y) - log10(m)) / s;
        djdy = r / (s * y * ln10);
        djds = 1.0 / s - r * r / s;
        return 0.5 * log(two_pi * s * s * m * m * ln10 * ln10) + 0.5 * r * r;
    case 3:
        e = y - m;
        djdy = sgn(e) / s;
        djds = 1.0 / s - fabs(e) / (s * s);
        return log(2.0 * s) + fabs(e) / s;
    case 4:
        e = log(y) - log(m);
        djdy = sgn(e) / (s * y);
        djds = 1.0 / s - fabs(e) / (s * s);
        return log(2.0 * s * m) + fabs(e) / s;
    case 5:
        e = log10(y) - log10(m);
        djdy = sgn(e) / (s * y * ln10);
        djds = 1.0 / s - fabs(e) / (s * s);
        return log(2.0 * s * m * ln10) + fabs(e) / s;
    default:
        r = (y - m) / s;
        djdy = (y - m) / (s * s);
        djds = 1.0 / s - r * r / s;
        return 0.5 * log(two_pi * s * s) + 0.5 * r * r;
    }
}

// d p / d (scaled p) of the parameter scale: p (ln), p ln 10 (log10), 1 (lin)
__device__ __forceinline__ double scale_factor(const int32_t* pscale, const double* pu, int j) {
    const int scl = pscale ? pscale[j] : 0;
    return scl == 1 ? pu[j] : (scl == 2 ? pu[j] * 2.302585092994046 : 1.0);
}

// Per-group adjoint scratch layout (doubles): step times [cap], step orders
// [cap], states [cap][NX], dJy/dx [nt][NX], quadrature vectors [QV_N][nqp].
struct AdjLayout {
    long long cap, nt, nx, nqp;
    __host__ __device__ long long t_off() const { return 0; }
    __host__ __device__ long long q_off() const { return cap; }
    __host__ __device__ long long y_off() const { return 2 * cap; }
    __host__ __device__ long long dj_off() const { return 2 * cap + cap * nx; }
    __host__ __device__ long long qv_off() const { return dj_off() + nt * nx; }
    __host__ __device__ long long stride(int nqv) const { return qv_off() + (long long)nqv * nqp; }
};

// A group of G lanes inside one warp.
template <int G>
struct Group {
    unsigned mask;
    int lane;
    __device__ __forceinline__ Group() {
        int wl = threadIdx.x & 31;
        lane = wl % G;
        mask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (wl - lane));
    }
    __device__ __forceinline__ void sync() const {
        if (G > 1) __syncwarp(mask);
    }
    template <class T>
    __device__ __forceinline__ T sum(T v) const {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, G);
        return v;
    }
    template <class T>
    __device__ __forceinline__ T max(T v) const {  // propagates NaN
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            T w = __shfl_xor_sync(mask, v, o, G);
            v = (w > v || w != w) ? w : v;
        }
        return v;
    }
    template <class T>
    __device__ __forceinline__ T bcast(T v, int src) const {
        if (G == 1) return v;
        return __shfl_sync(mask, v, src, G);
    }
};

// control-type helpers: SUNRpowerR / SUNRpowerI (sundials_math.c:25-51)
__device__ __forceinline__ float powr(float base, float e) { return base <= 0.0f ? 0.0f : __powf(base, e); }
__device__ __forceinline__ double powr(double base, double e) { return base <= 0.0 ? 0.0 : pow(base, e); }
template <class R>
__device__ __forceinline__ R powi(R base, int e) {
    R prod = R(1);
    for (int i = 1; i <= e; i++) prod *= base;
    return prod;
}

// division in the control type: the SFU reciprocal for FP32 heuristics
__device__ __forceinline__ float rdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return a / b; }

// 1/j, j = 1..6 (ONE/j in cvSetBDF/cvIncreaseBDF)
__device__ __forceinline__ double inv_int(int j) {
    return j == 1 ? 1.0 : j == 2 ? 0.5 : j == 3 ? 1.0 / 3.0 : j == 4 ? 0.25 : j == 5 ? 0.2 : 1.0 / 6.0;
}

// BDF stability-limit detection (cvSLdet, cvodes.c:8221-8576).  ss holds
// the scaled derivative norms of the last five steps, ss[3 * (i - 1) + k - 1]
// for step i = 1 (newest) .. 5 and k = 1, 2, 3 (derivative orders q-1, q,
// q+1).  Estimates the dominant characteristic root rr of the method on the
// problem: equal norm ratios (the nearly normal case) or the common root of
// three quartics, refined by up to three Newton corrections, then checked
// against the variances it implies.  Returns 1..3 for a stable root, 4..6
// for a root above the cutoff 0.98 (the step size sits on the stability
// boundary of order q), negative when the data admit no estimate.  FP64: the
// quartic coefficients are products of squared norms.  Group-uniform (every
// lane computes the same value); not inlined, as it runs once per step only
// after q + 5 steps of constant step size and order.
static __device__ __noinline__ int sl_detect(const double* ss, int q) {
    constexpr double rrcut = 0.98, vrrtol = 1.0e-4, vrrt2 = 5.0e-4, sqtol = 1.0e-3, rrtol = 1.0e-2;
    auto S = [ss](int i, int k) { return ss[3 * (i - 1) + (k - 1)]; };
    auto mn = [](double a, double b) { return a < b ? a : b; };
    auto mx = [](double a, double b) { return a > b ? a : b; };
    double smax[3], ssmax[3], rav[3], vrat[3];
    double c1[3], c2[3], c4[3], c5[3];  // quartic q_k(r) = c5 + r (c4 + r^2 (c2 + r c1))
    for (int k = 1; k <= 3; k++) {
        double lo = S(1, k), hi = 0.0;
        for (int i = 1; i <= 5; i++) {
            lo = mn(lo, S(i, k));
            hi = mx(hi, S(i, k));
        }
        if (lo < SLD_TINY * hi) return -1;
        smax[k - 1] = hi;
        ssmax[k - 1] = hi * hi;
        double sum = 0.0, sumsq = 0.0;
        for (int i = 1; i <= 4; i++) {
            const double r = S(i, k) / S(i + 1, k);
            sum += r;
            sumsq += r * r;
        }
        rav[k - 1] = 0.25 * sum;
        vrat[k - 1] = fabs(0.25 * sumsq - rav[k - 1] * rav[k - 1]);
        c5[k - 1] = S(1, k) * S(3, k) - S(2, k) * S(2, k);
        c4[k - 1] = S(2, k) * S(3, k) - S(1, k) * S(4, k);
        c2[k - 1] = S(2, k) * S(5, k) - S(3, k) * S(4, k);
        c1[k - 1] = S(4, k) * S(4, k) - S(3, k) * S(5, k);
    }
    auto quartic = [&](int k, double r) { return c5[k] + r * (c4[k] + r * r * (c2[k] + r * c1[k])); };
    double rr;
    int kflag;
    const double vmin = mn(vrat[0], mn(vrat[1], vrat[2])), vmax = mx(vrat[0], mx(vrat[1], vrat[2]));
    if (vmin < vrrtol * vrrtol) {
        if (vmax > vrrt2 * vrrt2) return -2;
        rr = (rav[0] + rav[1] + rav[2]) / 3.0;
        double dev = 0.0;
        for (int k = 0; k < 3; k++) dev = mx(dev, fabs(rav[k] - rr));
        if (dev > vrrt2) return -3;
        kflag = 1;
    } else {
        // Gaussian elimination of c1, then c2, between the three quartics
        // (rows: coefficients c1, c2, c4, c5 of quartics 1, 2, 3)
        double e1[3] = {c1[0], c1[1], c1[2]}, e2[3] = {c2[0], c2[1], c2[2]};
        double e4[3] = {c4[0], c4[1], c4[2]}, e5[3] = {c5[0], c5[1], c5[2]};
        if (fabs(e1[0]) < SLD_TINY * ssmax[0]) return -4;
        for (int k = 1; k < 3; k++) {
            const double f = e1[k] / e1[0];
            e2[k] -= f * e2[0];
            e4[k] -= f * e4[0];
            e5[k] -= f * e5[0];
        }
        if (fabs(e2[1]) < SLD_TINY * ssmax[1]) return -4;
        const double f = e2[2] / e2[1];
        e4[2] -= f * e4[1];
        e5[2] -= f * e5[1];
        if (fabs(e4[2]) < SLD_TINY * ssmax[2]) return -4;
        rr = -e5[2] / e4[2];
        if (rr < SLD_TINY || rr > 100.0) return -5;
        double qkr[3], worst = 0.0;
        for (int k = 0; k < 3; k++) {
            qkr[k] = quartic(k, rr);
            worst = mx(worst, fabs(qkr[k]) / ssmax[k]);
        }
        if (worst < sqtol) {
            kflag = 2;
        } else {
            double best = 0.0;
            int kb = -1;
            kflag = 0;
            for (int it = 0; it < 3; it++) {
                double cand[3], resid[3], qj[3][3];
                for (int k = 0; k < 3; k++) {
                    const double dq = c4[k] + rr * rr * (3.0 * c2[k] + rr * 4.0 * c1[k]);
                    cand[k] = rr + ((fabs(dq) > SLD_TINY * ssmax[k]) ? -qkr[k] / dq : 0.0);
                }
                for (int k = 0; k < 3; k++) {
                    double w = 0.0;
                    for (int j = 0; j < 3; j++) {
                        qj[j][k] = quartic(j, cand[k]);
                        w = mx(w, fabs(qj[j][k]) / ssmax[j]);
                    }
                    resid[k] = w;
                }
                best = resid[0] + 1.0;
                for (int k = 0; k < 3; k++)
                    if (resid[k] < best) {
                        kb = k;
                        best = resid[k];
                    }
                if (kb < 0) return -6;
                rr = cand[kb];
                if (best < sqtol) {
                    kflag = 3;
                    break;
                }
                for (int j = 0; j < 3; j++) qkr[j] = qj[j][kb];
            }
            if (best > sqtol) return -6;
        }
    }
    double sigsq[3];
    for (int k = 1; k <= 3; k++) {
        const double a = S(1, k), b = S(2, k) * rr, c = S(3, k) * rr * rr, d = S(4, k) * rr * rr * rr;
        const double d1a = a - b, d1b = b - c, d1c = c - d;
        const double d2a = d1a - d1b, d2b = d1b - d1c, d3a = d2a - d2b;
        if (fabs(d1b) < SLD_TINY * smax[k - 1]) return -7;
        const double cest = -d3a / d1b;
        if (cest < SLD_TINY || cest > 4.0) return -7;
        sigsq[k - 1] = S(3, k) + (d2b / cest) / (rr * rr);
    }
    if (sigsq[1] < SLD_TINY) return -8;
    const double ratp = sigsq[2] / sigsq[1], ratm = sigsq[0] / sigsq[1];
    const double bb = ratp * ratm - 1.0 - 0.25 * (q * q - 1.0) * ratp;
    const double den = 1.0 - (2.0 / (q - 1.0)) * bb;
    if (fabs(den) < SLD_TINY) return -8;
    if (fabs(1.0 / den - rr) > rrtol) return -9;
    if (rr > rrcut && kflag >= 1) kflag += 3;
    return kflag;
}

// The same estimate computed by a group of G >= 4 lanes: lane k < 3 takes
// history column k (its extremes, ratios and quartic coefficients; in the
// Newton corrections candidate k and its residuals; then sigma^2_k) and the
// lanes exchange the per-column results by shuffles.  On GB300 an FP64 warp
// instruction costs the same whatever its active lanes, so this takes about
// a third of the FP64 instructions of the one-lane form; the divisions by
// the columns' squared extremes become multiplications by their reciprocals.
template <int G>
__device__ __noinline__ int sl_detect_group(const double* ss, int q, unsigned mask, int lane) {
    constexpr double rrcut = 0.98, vrrtol = 1.0e-4, vrrt2 = 5.0e-4, sqtol = 1.0e-3, rrtol = 1.0e-2;
    auto get = [&](double v, int src) { return __shfl_sync(mask, v, src, G); };
    auto mn = [](double a, double b) { return a < b ? a : b; };
    auto mx = [](double a, double b) { return a > b ? a : b; };
    const int k = lane < 3 ? lane : 0;  // this lane's column (lanes >= 3 repeat column 0)
    double sk[6];
#pragma unroll
    for (int i = 1; i <= 5; i++) sk[i] = ss[3 * (i - 1) + k];
    double lo = sk[1], hi = 0.0;
#pragma unroll
    for (int i = 1; i <= 5; i++) {
        lo = mn(lo, sk[i]);
        hi = mx(hi, sk[i]);
    }
    if (__any_sync(mask, lo < SLD_TINY * hi)) return -1;
    const double ssmax_k = hi * hi, inv_ssmax_k = 1.0 / ssmax_k;
    double sum = 0.0, sumsq = 0.0;
#pragma unroll
    for (int i = 1; i <= 4; i++) {
        const double r = sk[i] / sk[i + 1];
        sum += r;
        sumsq += r * r;
    }
    const double rav_k = 0.25 * sum, vrat_k = fabs(0.25 * sumsq - rav_k * rav_k);
    const double c5_k = sk[1] * sk[3] - sk[2] * sk[2], c4_k = sk[2] * sk[3] - sk[1] * sk[4];
    const double c2_k = sk[2] * sk[5] - sk[3] * sk[4], c1_k = sk[4] * sk[4] - sk[3] * sk[5];
    auto quartic = [](double c1, double c2, double c4, double c5, double r) {
        return c5 + r * (c4 + r * r * (c2 + r * c1));
    };
    const double v0 = get(vrat_k, 0), v1 = get(vrat_k, 1), v2 = get(vrat_k, 2);
    const double vmin = mn(v0, mn(v1, v2)), vmax = mx(v0, mx(v1, v2));
    double rr;
    int kflag;
    if (vmin < vrrtol * vrrtol) {
        if (vmax > vrrt2 * vrrt2) return -2;
        const double a0 = get(rav_k, 0), a1 = get(rav_k, 1), a2 = get(rav_k, 2);
        rr = (a0 + a1 + a2) / 3.0;
        if (mx(fabs(a0 - rr), mx(fabs(a1 - rr), fabs(a2 - rr))) > vrrt2) return -3;
        kflag = 1;
    } else {
        // every column's quartic on every lane, then elimination of c1 and c2
        double c1[3], c2[3], c4[3], c5[3], ssm[3], issm[3];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            c1[j] = get(c1_k, j);
            c2[j] = get(c2_k, j);
            c4[j] = get(c4_k, j);
            c5[j] = get(c5_k, j);
            ssm[j] = get(ssmax_k, j);
            issm[j] = get(inv_ssmax_k, j);
        }
        double e1[3], e2[3], e4[3], e5[3];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            e1[j] = c1[j];
            e2[j] = c2[j];
            e4[j] = c4[j];
            e5[j] = c5[j];
        }
        if (fabs(e1[0]) < SLD_TINY * ssm[0]) return -4;
        const double inv_e10 = 1.0 / e1[0];
#pragma unroll
        for (int j = 1; j < 3; j++) {
            const double f = e1[j] * inv_e10;
            e2[j] -= f * e2[0];
            e4[j] -= f * e4[0];
            e5[j] -= f * e5[0];
        }
        if (fabs(e2[1]) < SLD_TINY * ssm[1]) return -4;
        const double f = e2[2] / e2[1];
        e4[2] -= f * e4[1];
        e5[2] -= f * e5[1];
        if (fabs(e4[2]) < SLD_TINY * ssm[2]) return -4;
        rr = -e5[2] / e4[2];
        if (rr < SLD_TINY || rr > 100.0) return -5;
        // quartic residual of column k at rr, relative to the column's scale
        double qk = quartic(c1_k, c2_k, c4_k, c5_k, rr);
        double worst = fabs(qk) * inv_ssmax_k;
        worst = mx(get(worst, 0), mx(get(worst, 1), get(worst, 2)));
        if (worst < sqtol) {
            kflag = 2;
        } else {
            // Newton corrections: lane k refines rr on quartic k and measures
            // the candidate against all three quartics
            double best = 0.0;
            kflag = 0;
            int kb = -1;
            for (int it = 0; it < 3; it++) {
                const double dq = c4_k + rr * rr * (3.0 * c2_k + rr * 4.0 * c1_k);
                const double cand = rr + ((fabs(dq) > SLD_TINY * ssmax_k) ? -qk / dq : 0.0);
                double qj[3], w = 0.0;
#pragma unroll
                for (int j = 0; j < 3; j++) {
                    qj[j] = quartic(c1[j], c2[j], c4[j], c5[j], cand);
                    w = mx(w, fabs(qj[j]) * issm[j]);
                }
                const double r0 = get(w, 0), r1 = get(w, 1), r2 = get(w, 2);
                best = r0 + 1.0;
                if (r0 < best) { kb = 0; best = r0; }
                if (r1 < best) { kb = 1; best = r1; }
                if (r2 < best) { kb = 2; best = r2; }
                if (kb < 0) return -6;
                rr = get(cand, kb);
                if (best < sqtol) {
                    kflag = 3;
                    break;
                }
                // the chosen candidate's residual on quartic k becomes this lane's
                const double q0 = get(qj[0], kb), q1 = get(qj[1], kb), q2 = get(qj[2], kb);
                qk = k == 0 ? q0 : (k == 1 ? q1 : q2);
            }
            if (best > sqtol) return -6;
        }
    }
    // given rr: sigma^2 of column k, and the root it implies
    const double a = sk[1], b = sk[2] * rr, c = sk[3] * rr * rr, d = sk[4] * rr * rr * rr;
    const double d1a = a - b, d1b = b - c, d1c = c - d;
    const double d2a = d1a - d1b, d2b = d1b - d1c, d3a = d2a - d2b;
    int bad = fabs(d1b) < SLD_TINY * hi;
    const double cest = -d3a / d1b;
    bad |= cest < SLD_TINY || cest > 4.0;
    if (__any_sync(mask, bad && lane < 3)) return -7;
    const double sig_k = sk[3] + (d2b / cest) / (rr * rr);
    const double sg0 = get(sig_k, 0), sg1 = get(sig_k, 1), sg2 = get(sig_k, 2);
    if (sg1 < SLD_TINY) return -8;
    const double inv_sg1 = 1.0 / sg1;
    const double ratp = sg2 * inv_sg1, ratm = sg0 * inv_sg1;
    const double bb = ratp * ratm - 1.0 - 0.25 * (q * q - 1.0) * ratp;
    const double den = 1.0 - (2.0 / (q - 1.0)) * bb;
    if (fabs(den) < SLD_TINY) return -8;
    if (fabs(1.0 / den - rr) > rrtol) return -9;
    if (rr > rrcut && kflag >= 1) kflag += 3;
    return kflag;
}

// Mixed-precision form for the FP32 control type, computed by a group of
// G >= 16 lanes.  The parts that cancel stay in FP64: the ratio statistics
// (their variance is compared with 1e-8) and the quartic coefficients
// ss_a ss_b - ss_c ss_d; lane e < 15 takes history entry (i, k) =
// (e / 3 + 1, e % 3), lane e < 12 also the ratio ss[i][k] / ss[i+1][k] and
// quartic coefficient e (c5, c4, c2, c1 of column e % 3).  Each column is
// first scaled by the power of two 2^-e_k that brings its largest entry into
// [0.5, 1) (an exact exponent shift), so everything after the FP64 part fits
// FP32's range; the rest runs in FP32 with the column scales put back where
// the reference compares across columns or with absolute thresholds.  In
// the Newton corrections lane 3j + k (of the first nine) evaluates quartic j
// at candidate k, and lane k (of the first three) computes sigma^2_k.  On
// histories recorded from the restatement (tens of thousands of calls) this
// form returns the same result in all but a few in 10^4 calls and the same
// order decision in every one; on GB300 it takes a small fraction of the
// FP64 form's FP64 instructions.
__device__ __forceinline__ float sel3(int k, float a, float b, float c) { return k == 0 ? a : (k == 1 ? b : c); }

template <int G>
__device__ __noinline__ int sl_detect_mixed(const double* ss, int q, unsigned mask, int lane) {
    static_assert(G >= 16, "the mixed form takes one history entry per lane");
    constexpr float rrcut = 0.98f, vrrt2 = 5.0e-4f, sqtol = 1.0e-3f, rrtol = 1.0e-2f;
    constexpr float tiny = float(SLD_TINY);
    // every lane: extremes and scale exponent of every column (bit patterns of
    // nonnegative doubles order like the numbers)
    long long lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        lo[k] = hi[k] = __double_as_longlong(ss[k]);
#pragma unroll
        for (int i = 1; i < 5; i++) {
            const long long b = __double_as_longlong(ss[3 * i + k]);
            lo[k] = b < lo[k] ? b : lo[k];
            hi[k] = b > hi[k] ? b : hi[k];
        }
    }
    int ex[3], bad = 0;
    float hn[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double h = __longlong_as_double(hi[k]);
        bad |= !(h > 0.0) || __longlong_as_double(lo[k]) < SLD_TINY * h || !isfinite(h);
        ex[k] = int((hi[k] >> 52) & 0x7FF) - 1022;
        hn[k] = float(__longlong_as_double(hi[k] - ((long long)ex[k] << 52)));
    }
    if (bad) return -1;
    // FP64 part: lane e takes entry (i, k) scaled, ratio and quartic coefficient e
    const int e = lane < 15 ? lane : 0, ke = e % 3, ie = e / 3;  // ie = 0..4 (history rows 1..5)
    const long long shift = (long long)(ke == 0 ? ex[0] : (ke == 1 ? ex[1] : ex[2])) << 52;
    auto scaled = [&](int row) {  // ss[row+1][ke] * 2^-e_ke, exact
        return __longlong_as_double(__double_as_longlong(ss[3 * row + ke]) - shift);
    };
    const float s_e = float(scaled(ie));
    double r = 0.0, cf = 0.0;
    if (e < 12) {
        r = ss[e] / ss[e + 3];
        const double s1 = scaled(0), s2 = scaled(1), s3 = scaled(2), s4 = scaled(3), s5 = scaled(4);
        // ie = 0: c5 = s1 s3 - s2^2, 1: c4 = s2 s3 - s1 s4, 2: c2 = s2 s5 - s3 s4, 3: c1 = s4^2 - s3 s5
        const double pa = ie == 0 ? s1 : (ie == 3 ? s4 : s2);
        const double pb = ie == 2 ? s5 : (ie == 3 ? s4 : s3);
        const double na = ie == 0 ? s2 : (ie == 1 ? s1 : s3);
        const double nb = ie == 0 ? s2 : (ie == 3 ? s5 : s4);
        cf = fma(pa, pb, -(na * nb));
    }
    // ratio sums of column k on lane k: (r1 + r3) + (r2 + r4)
    double sum = r, sumsq = r * r;
    sum += __shfl_down_sync(mask, sum, 6, G);
    sumsq += __shfl_down_sync(mask, sumsq, 6, G);
    sum += __shfl_down_sync(mask, sum, 3, G);
    sumsq += __shfl_down_sync(mask, sumsq, 3, G);
    const double rav = 0.25 * sum;
    const float rav_f = float(rav), vrat_f = float(fabs(fma(0.25, sumsq, -(rav * rav))));
    const float cf_f = float(cf);
    // FP32 part.  Every lane: the three columns' coefficients (index 0 = c1,
    // 1 = c2, 2 = c4, 3 = c5; c5 of column k on lane k, c4 on 3 + k, c2 on
    // 6 + k, c1 on 9 + k) and statistics
    float C[3][4], ravs[3], vrats[3], sm[3], ism[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        C[k][0] = __shfl_sync(mask, cf_f, 9 + k, G);
        C[k][1] = __shfl_sync(mask, cf_f, 6 + k, G);
        C[k][2] = __shfl_sync(mask, cf_f, 3 + k, G);
        C[k][3] = __shfl_sync(mask, cf_f, k, G);
        ravs[k] = __shfl_sync(mask, rav_f, k, G);
        vrats[k] = __shfl_sync(mask, vrat_f, k, G);
        sm[k] = hn[k] * hn[k];
        ism[k] = __frcp_rn(sm[k]);
    }
    auto quartic = [](float c1, float c2, float c4, float c5, float x) { return c5 + x * (c4 + x * x * (c2 + x * c1)); };
    const float vmin = fminf(vrats[0], fminf(vrats[1], vrats[2]));
    const float vmax = fmaxf(vrats[0], fmaxf(vrats[1], vrats[2]));
    // this lane's column / candidate k and quartic j (lanes >= 9 repeat)
    const int l9 = lane % 9, k = l9 % 3, j = l9 / 3;
    float rr;
    int kflag;
    if (vmin < 1.0e-8f) {  // vrrtol^2
        if (vmax > vrrt2 * vrrt2) return -2;
        rr = (ravs[0] + ravs[1] + ravs[2]) * (1.0f / 3.0f);
        const float dev = fmaxf(fabsf(ravs[0] - rr), fmaxf(fabsf(ravs[1] - rr), fabsf(ravs[2] - rr)));
        if (dev > vrrt2) return -3;
        kflag = 1;
    } else {
        // eliminate c1 and c2 between the three quartics (uniform)
        float o[3][4];
#pragma unroll
        for (int kk = 0; kk < 3; kk++)
#pragma unroll
            for (int m = 0; m < 4; m++) o[kk][m] = C[kk][m];
        if (fabsf(o[0][0]) < tiny * sm[0]) return -4;
#pragma unroll
        for (int kk = 1; kk < 3; kk++) {
            const float f = __fdividef(o[kk][0], o[0][0]);
#pragma unroll
            for (int m = 1; m < 4; m++) o[kk][m] -= f * o[0][m];
        }
        if (fabsf(o[1][1]) < tiny * sm[1]) return -4;
        const float f = __fdividef(o[2][1], o[1][1]);
        o[2][2] -= f * o[1][2];
        o[2][3] -= f * o[1][3];
        if (fabsf(o[2][2]) < tiny * sm[2]) return -4;
        float rc = -__fdividef(o[2][3], o[2][2]);
        if (rc < tiny || rc > 100.0f) return -5;
        // this lane's rows: quartic k (its candidate's) and quartic j
        const float k1 = sel3(k, C[0][0], C[1][0], C[2][0]), k2 = sel3(k, C[0][1], C[1][1], C[2][1]);
        const float k4 = sel3(k, C[0][2], C[1][2], C[2][2]), k5 = sel3(k, C[0][3], C[1][3], C[2][3]);
        const float j1 = sel3(j, C[0][0], C[1][0], C[2][0]), j2 = sel3(j, C[0][1], C[1][1], C[2][1]);
        const float j4 = sel3(j, C[0][2], C[1][2], C[2][2]), j5 = sel3(j, C[0][3], C[1][3], C[2][3]);
        const float smk = sel3(k, sm[0], sm[1], sm[2]), ismj = sel3(j, ism[0], ism[1], ism[2]);
        const float ismk = sel3(k, ism[0], ism[1], ism[2]);
        float qk = quartic(k1, k2, k4, k5, rc);  // residual of quartic k at rr
        const float wk = fabsf(qk) * ismk;
        const float worst = fmaxf(__shfl_sync(mask, wk, 0, G), fmaxf(__shfl_sync(mask, wk, 1, G),
                                                                      __shfl_sync(mask, wk, 2, G)));
        if (worst < sqtol) {
            kflag = 2;
        } else {
            float best = 0.0f;
            kflag = 0;
            int kb = 0;
            #pragma unroll 1
            for (int it = 0; it < 3; it++) {
                // candidate k: one Newton correction of rr on quartic k
                const float dq = k4 + rc * rc * (3.0f * k2 + rc * 4.0f * k1);
                const float cand = rc + ((fabsf(dq) > tiny * smk) ? -__fdividef(qk, dq) : 0.0f);
                // quartic j at candidate k, relative to column j's scale
                const float qjk = quartic(j1, j2, j4, j5, cand);
                const float a = fabsf(qjk) * ismj;
                // residual of candidate k: the largest over the quartics j
                const float res = fmaxf(__shfl_sync(mask, a, k, G),
                                        fmaxf(__shfl_sync(mask, a, 3 + k, G), __shfl_sync(mask, a, 6 + k, G)));
                const float r0 = __shfl_sync(mask, res, 0, G), r1 = __shfl_sync(mask, res, 1, G),
                            r2 = __shfl_sync(mask, res, 2, G);
                best = r0 + 1.0f;
                if (r0 < best) { kb = 0; best = r0; }
                if (r1 < best) { kb = 1; best = r1; }
                if (r2 < best) { kb = 2; best = r2; }
                rc = __shfl_sync(mask, cand, kb, G);
                if (best < sqtol) {
                    kflag = 3;
                    break;
                }
                // the chosen candidate's residual on quartic k becomes this lane's
                qk = __shfl_sync(mask, qjk, 3 * k + kb, G);
            }
            if (best > sqtol) return -6;
        }
        rr = rc;
    }
    // given rr: sigma^2 of column k on lane k, and the root they imply
    const float s0 = __shfl_sync(mask, s_e, k, G), s1 = __shfl_sync(mask, s_e, 3 + k, G);
    const float s2 = __shfl_sync(mask, s_e, 6 + k, G), s3 = __shfl_sync(mask, s_e, 9 + k, G);
    const float hk = sel3(k, hn[0], hn[1], hn[2]);
    const float ta = s0, tb = s1 * rr, tc = s2 * rr * rr, td = s3 * rr * rr * rr;
    const float d1a = ta - tb, d1b = tb - tc, d1c = tc - td;
    const float d2a = d1a - d1b, d2b = d1b - d1c, d3a = d2a - d2b;
    int badk = fabsf(d1b) < tiny * hk;
    const float cest = -__fdividef(d3a, d1b);
    badk |= cest < tiny || cest > 4.0f;
    if (__any_sync(mask, badk)) return -7;
    const float sgk = s2 + __fdividef(__fdividef(d2b, cest), rr * rr);
    const float sg0 = __shfl_sync(mask, sgk, 0, G), sg1 = __shfl_sync(mask, sgk, 1, G),
                sg2 = __shfl_sync(mask, sgk, 2, G);
    if (sg1 < ldexpf(tiny, -ex[1])) return -8;
    const float ratp = ldexpf(__fdividef(sg2, sg1), ex[2] - ex[1]), ratm = ldexpf(__fdividef(sg0, sg1), ex[0] - ex[1]);
    const float bb = ratp * ratm - 1.0f - 0.25f * float(q * q - 1) * ratp;
    const float den = 1.0f - __fdividef(2.0f, float(q - 1)) * bb;
    if (fabsf(den) < tiny) return -8;
    if (fabsf(__frcp_rn(den) - rr) > rrtol) return -9;
    if (rr > rrcut && kflag >= 1) kflag += 3;
    return kflag;
}

// Shared-memory layout of one instance.
template <class M, class LUT, bool SENS = false>
struct InstanceLayout {
    static constexpr int N = M::NX;
    static constexpr int NW = M::NW;
    // y, w, coefficients c, p (unscaled), k; with sensitivities also dw/dy_a,
    // dw/dy_b, dw/dc (for monomials: the monomial) and the coefficient
    // derivatives dc/dp
    static constexpr int n_base = N + NW + M::NC + M::NP + M::NK + M::NH + (SENS ? 2 * NW + M::NC + M::ND : 0);
    // the stability-limit detector's five-step history of scaled derivative
    // norms (5 x 3 doubles, padded)
    static constexpr int ssd_off = n_base;
    // with sensitivities and events: xdot before and after an event's bolus
    static constexpr int ev_off = n_base + 16;
    static constexpr int n_double = ev_off + ((SENS && M::NE > 0) ? 2 * N : 0);
    // saved J (on its pattern for the sparse-LU models, else dense), M (LU:
    // dense N x N, or the compressed rows of the factor pattern), 1/pivots,
    // rhs; with sensitivities also M^-1 (register path)
    static constexpr int n_jsv = M::SPARSE_LU ? M::NNZ_J : N * N;
    static constexpr int n_lut = n_jsv + M::LU_STORE + 2 * N + (SENS ? N * N : 0);
    static constexpr size_t bytes_double = sizeof(double) * n_double;
    static constexpr size_t bytes_lut = ((sizeof(LUT) * (size_t)n_lut + 7) / 8) * 8;
    static constexpr size_t bytes_int = sizeof(int16_t) * N;  // composed row permutation
    static constexpr size_t bytes = ((bytes_double + bytes_lut + bytes_int + 15) / 16) * 16;
};

// Per-group adjoint scratch with check points (doubles): check points
// [ck_cap][ck_stride], one segment's Hermite data: times [k+2], states
// [k+2][NX], derivatives [k+2][NX]; dJy/dx [nt][NX]; quadrature vectors
// [QV_N][nqp]; the backward problem's saved state [ck_stride + 8 + NX].
struct AdjCkLayout {
    long long k, cap, nt, nx, nqp, ck_stride;
    __host__ __device__ long long ck_off() const { return 0; }
    __host__ __device__ long long st_off() const { return cap * ck_stride; }
    __host__ __device__ long long sy_off() const { return st_off() + (k + 2); }
    __host__ __device__ long long syd_off() const { return sy_off() + (k + 2) * nx; }
    __host__ __device__ long long dj_off() const { return syd_off() + (k + 2) * nx; }
    __host__ __device__ long long qv_off() const { return dj_off() + nt * nx; }
    __host__ __device__ long long bs_off(int nqv) const { return qv_off() + (long long)nqv * nqp; }
    __host__ __device__ long long stride(int nqv) const { return bs_off(nqv) + ck_stride + 8 + nx; }
};
// scalars of a saved integrator state (check point, backward resume), then
// the Nordsieck history
constexpr int CK_NSCAL = 80;
template <class M>
__host__ __device__ constexpr long long ck_stride_of() { return CK_NSCAL + (long long)(QMAX + 1) * M::NX; }

// Shared memory the backward (adjoint) problem adds after an instance's
// forward layout: interpolated forward state, flux partials dw/dx_a, dw/dx_b,
// dw/dc (for monomials: the monomial), the adjoint flux projections
// u = S^T xB, the divided differences of the interpolant and their abscissae.
template <class M>
struct BwdLayout {
    static constexpr int N = M::NX;
    static constexpr int NW = M::NW;
    static constexpr int n_double = N + 3 * NW + M::NC + (QMAX + 1) * N + (QMAX + 1) + M::ND;
    static constexpr size_t bytes = ((sizeof(double) * n_double + 15) / 16) * 16;
};

// Dense LU with partial pivoting of the column-major N x N matrix Mm in shared
// memory (SUNDlsMat_denseGETRF, sundials_dense.c:82), by the G lanes of one
// group: dinv[k] = 1/U(k,k), the composed row permutation in perm, bf used as
// pivot scratch.  Not inlined into the integrator: the factorisation then has
// the full register budget to itself (the caller's live state is saved around
// the call) and its chunked trailing update does not spill.  Returns 1 for a
// singular matrix.
template <class LUT, int N, int G>
__device__ __noinline__ int dense_getrf(LUT* Mm, LUT* dinv, LUT* bf, int16_t* perm, unsigned mask, int lane) {
    if (G > 1) __syncwarp(mask);
    for (int k = 0; k < N; k++) {
        LUT* colk = Mm + k * N;
        LUT best = LUT(-1);
        int bi = N;
        for (int i = k + lane; i < N; i += G) {
            const LUT v = fabs(colk[i]);
            if (v > best) {
                best = v;
                bi = i;
            }
        }
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1) {
            const LUT ob = __shfl_xor_sync(mask, best, off, G);
            const int oi = __shfl_xor_sync(mask, bi, off, G);
            if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        if (bi >= N) return 1;  // no finite pivot
        const int lp = bi;
        if (colk[lp] == LUT(0)) return 1;
        if (lane == 0) bf[k] = LUT(lp);  // pivot row (bf doubles as scratch here)
        if (lp != k)
            for (int j = lane; j < N; j += G) {
                const LUT t = Mm[j * N + lp];
                Mm[j * N + lp] = Mm[j * N + k];
                Mm[j * N + k] = t;
            }
        if (G > 1) __syncwarp(mask);
        const LUT mult = LUT(1) / colk[k];
        if (lane == 0) dinv[k] = mult;
        // rank-1 update of the trailing columns, one row of the lane at a
        // time; the column loop is unrolled by 4 with its loads issued ahead
        // of the stores, so shared-memory latency is paid once per 4 columns
        for (int i = k + 1 + lane; i < N; i += G) {
            const LUT lik = colk[i] * mult;
            colk[i] = lik;
            int j = k + 1;
            for (; j + 3 < N; j += 4) {
                const LUT u0 = Mm[j * N + k], u1 = Mm[(j + 1) * N + k], u2 = Mm[(j + 2) * N + k],
                          u3 = Mm[(j + 3) * N + k];
                LUT a0 = Mm[j * N + i], a1 = Mm[(j + 1) * N + i], a2 = Mm[(j + 2) * N + i],
                    a3 = Mm[(j + 3) * N + i];
                a0 -= u0 * lik;
                a1 -= u1 * lik;
                a2 -= u2 * lik;
                a3 -= u3 * lik;
                Mm[j * N + i] = a0;
                Mm[(j + 1) * N + i] = a1;
                Mm[(j + 2) * N + i] = a2;
                Mm[(j + 3) * N + i] = a3;
            }
            for (; j < N; j++) Mm[j * N + i] -= Mm[j * N + k] * lik;
        }
        if (G > 1) __syncwarp(mask);
    }
    if (lane == 0) {
        for (int i = 0; i < N; i++) perm[i] = (int16_t)i;
        for (int k = 0; k < N; k++) {
            const int pk = (int)bf[k];
            const int16_t t = perm[k];
            perm[k] = perm[pk];
            perm[pk] = t;
        }
    }
    if (G > 1) __syncwarp(mask);
    return 0;
}

// LU without row exchanges in the model's static order (the codegen's
// minimum-degree ordering of the pattern of I - gamma*J with its fill): for
// pivot k only the rows of column k of L and the columns of row k of U that
// are structurally nonzero take part, each lane updating whole rows.  Mm holds
// the already permuted matrix (dense storage, zeros outside the pattern stay
// zero), dinv[k] = 1/U(k,k).  TR: the matrix has the transposed pattern (the
// backward problem's I + gamma*J^T); its column k of L has the pattern of row
// k of U of the forward plan and its row k of U that of column k of L, so the
// two index lists trade places.  Returns 1 for a zero or non-finite pivot.
template <class M, class LUT, int N, int G, bool TR>
__device__ __noinline__ int sparse_getrf(LUT* Mm, LUT* dinv, unsigned mask, int lane) {
    if (G > 1) __syncwarp(mask);
    for (int k = 0; k < N; k++) {
        const LUT piv = Mm[k * N + k];
        if (!(fabs(piv) > LUT(0)) || !isfinite(piv)) return 1;
        const LUT mult = LUT(1) / piv;
        if (lane == 0) dinv[k] = mult;
        const int c0 = TR ? M::lu_rbegin(k) : M::lu_cbegin(k), c1 = TR ? M::lu_rend(k) : M::lu_cend(k);
        const int r1 = TR ? M::lu_cend(k) : M::lu_rend(k);
        for (int e = (TR ? M::lu_cbegin(k) : M::lu_rbegin(k)) + lane; e < r1; e += G) {
            const int i = TR ? M::lu_col(e) : M::lu_row(e);
            auto ucol = [](int c) { return TR ? M::lu_row(c) : M::lu_col(c); };
            const LUT lik = Mm[k * N + i] * mult;
            Mm[k * N + i] = lik;
            int c = c0;
            for (; c + 3 < c1; c += 4) {
                const int j0 = ucol(c), j1 = ucol(c + 1), j2 = ucol(c + 2), j3 = ucol(c + 3);
                const LUT u0 = Mm[j0 * N + k], u1 = Mm[j1 * N + k], u2 = Mm[j2 * N + k], u3 = Mm[j3 * N + k];
                LUT a0 = Mm[j0 * N + i], a1 = Mm[j1 * N + i], a2 = Mm[j2 * N + i], a3 = Mm[j3 * N + i];
                a0 -= u0 * lik;
                a1 -= u1 * lik;
                a2 -= u2 * lik;
                a3 -= u3 * lik;
                Mm[j0 * N + i] = a0;
                Mm[j1 * N + i] = a1;
                Mm[j2 * N + i] = a2;
                Mm[j3 * N + i] = a3;
            }
            for (; c < c1; c++) {
                const int j = ucol(c);
                Mm[j * N + i] -= Mm[j * N + k] * lik;
            }
        }
        if (G > 1) __syncwarp(mask);
    }
    return 0;
}

// The same elimination on the factors in compressed rows (models whose dense
// N x N storage would crowd the shared memory out): row i of val holds its
// pattern entries with columns ascending (L part, diagonal, U part).  For
// pivot k the U row is scattered into the dense row urow (zero elsewhere),
// and every L row i of the pivot sweeps its entries after (i, k) up to the
// last column of that U row: val(i, j) -= l(i, k) * urow(j).  The stretch
// holds every target (the pattern is closed under the elimination) plus a
// few entries whose urow value is zero; the loads are independent, so the
// sweep pipelines like a dense row update.  TR: the transposed plan (the
// backward problem's I + gamma*J^T).  Returns 1 for a zero or non-finite
// pivot.
template <class M, class LUT, int N, int G, bool TR>
__device__ __noinline__ int packed_getrf(LUT* val, LUT* dinv, LUT* urow, unsigned mask, int lane) {
    for (int j = lane; j < N; j += G) urow[j] = LUT(0);
    if (G > 1) __syncwarp(mask);
    for (int k = 0; k < N; k++) {
        const int dk = M::template pk_diag<TR>(k), q1 = M::template pk_rptr<TR>(k + 1);
        const LUT piv = val[dk];
        if (!(fabs(piv) > LUT(0)) || !isfinite(piv)) return 1;
        const LUT mult = LUT(1) / piv;
        if (lane == 0) dinv[k] = mult;
        for (int q = dk + 1 + lane; q < q1; q += G) urow[M::template pk_col<TR>(q)] = val[q];
        if (G > 1) __syncwarp(mask);
        const int e1 = TR ? M::lu_cend(k) : M::lu_rend(k);
        for (int e = (TR ? M::lu_cbegin(k) : M::lu_rbegin(k)) + lane; e < e1; e += G) {
            const int p = M::template pk_lpos<TR>(e), pend = p + 1 + M::template pk_span<TR>(e);
            const LUT lik = val[p] * mult;
            val[p] = lik;
            int pp = p + 1;
            for (; pp + 3 < pend; pp += 4) {
                const int c0 = M::template pk_col<TR>(pp), c1 = M::template pk_col<TR>(pp + 1),
                          c2 = M::template pk_col<TR>(pp + 2), c3 = M::template pk_col<TR>(pp + 3);
                LUT a0 = val[pp], a1 = val[pp + 1], a2 = val[pp + 2], a3 = val[pp + 3];
                a0 -= urow[c0] * lik;
                a1 -= urow[c1] * lik;
                a2 -= urow[c2] * lik;
                a3 -= urow[c3] * lik;
                val[pp] = a0;
                val[pp + 1] = a1;
                val[pp + 2] = a2;
                val[pp + 3] = a3;
            }
            for (; pp < pend; pp++) val[pp] -= urow[M::template pk_col<TR>(pp)] * lik;
        }
        if (G > 1) __syncwarp(mask);
        for (int q = dk + 1 + lane; q < q1; q += G) urow[M::template pk_col<TR>(q)] = LUT(0);
        if (G > 1) __syncwarp(mask);
    }
    return 0;
}

#define AGB_DISPATCH_Q(qv, F) \
    switch (qv) {             \
    case 1: F<1>(); break;    \
    case 2: F<2>(); break;    \
    case 3: F<3>(); break;    \
    case 4: F<4>(); break;    \
    default: F<5>(); break;   \
    }

template <class M, int G, class LUT, class R, bool SENS = false, bool BWD = false>
struct Integrator {
    static constexpr int N = M::NX;
    static constexpr int NW = M::NW;
    static constexpr int S = (N + G - 1) / G;  // register slots per lane
    static constexpr int FM = (NW + G - 1) / G;  // fluxes per lane
    static constexpr int RM = M::RMAX;           // longest stoichiometry row
    // model tables cached in registers for the whole kernel when small enough
    static constexpr bool TREG = (S * RM <= 16);
    // flux reactants and coefficients in registers for up to 8 fluxes per
    // lane; above that the rate law reads the shared coefficients and the
    // (L1-resident) reactant table, which frees the registers the n = 100+
    // kernels would otherwise spill
    static constexpr bool FREG = (FM <= 8) && !M::GENERAL;
    static constexpr int FMR = FREG ? FM : 1;
    // one row of M per lane: Gauss-Jordan inverse in registers, shuffle mat-vec solves
    static constexpr bool REG = (S == 1);
    static constexpr int NPS = (M::NP + G - 1) / G;  // sensitivity columns per lane (at most)
    using LY = InstanceLayout<M, LUT, SENS>;
    static_assert(!(SENS && M::PACKED_LU), "forward sensitivities need the dense factor storage");

    Group<G> g;
    // shared memory of this instance
    double *ys, *ws, *cs, *pu, *ku;
    LUT *Jsv, *Mm, *dinv, *bf;
    int16_t* perm;
    const Opts* o;
    // register-resident vectors (element s*G + lane)
    double zn[LMAX][S], acor[S], tmp[S], ftmp[S];
    // error weights in the control type: they only scale norms compared with
    // thresholds near 1, and on GB300 every FP64 warp instruction (a
    // conversion included) takes the FP64 pipe's full issue cost
    R ewt[S];
    // FP64 scalars: time, step size, step ratio, gamma = h/l1
    double tn, h, hprime, hscale, tstop, gamma;
    // BDF coefficients in the control type: an error eps in l (rl1 and gamma
    // share it) moves the corrector's fixed point by eps*|correction|, i.e.
    // eps*O(local error); ld is the FP64 copy used by the history update
    R rl1, gammap, gamrat;
    R tau[LMAX + 1], l[LMAX];
    double ld[LMAX];
    // step ratio: FP64, because a stop time is reached by h = hscale * (hprime / h)
    double eta;
    // control scalars (heuristics)
    R etamax, crate, delp, acnrm, saved_tq5, etaqm1, etaq, etaqp1;
    R tq[6];
    int q, qprime, qwait, L, convfail, jcur, jcur_nls, tstopset;
    int nst, nstlp, nstlj;
    // steps since the last change of step size or order (cv_nscon); the
    // stability-limit detector runs once it reaches q + 5
    int nscon;
    int nfe, nni, nsetups, netf, ncfn, nje;  // diagnostics (CVodeGetNum*)
    // a restart from saved state (check point, backward resume): the first
    // step refreshes the Jacobian and the iteration matrix (their shared
    // memory is not part of the saved state), as CVODES' cv_forceSetup does
    // at its check points
    int force_setup;
    // a reinitialisation after an event (CVodeSolver::reinit, solver_cvodes.cpp:
    // 586-616): the next solve first takes reInit_post_process's step;
    // called = solver_was_called_F_
    int force_reinit, called;
    // root finding (CVodeRootInit, cvodes.c:2674): the trigger functions'
    // values and the search state of cvRcheck1-3 / cvRootfind, the same on
    // every lane; rt_taskc 1 = ONE_STEP; yret: the state returned at a root
    static constexpr int NRR = M::NR > 0 ? M::NR : 1;
    double rt_glo[NRR], rt_ghi[NRR], rt_grout[NRR];
    int rt_iroots[NRR], rt_gactive[NRR];
    double rt_tlo, rt_thi, rt_trout, rt_ttol, rt_toutc, tlastroot;
    int rt_irfnd, rt_taskc;
    double yret[S];
    // forward check points (adjoint with checkpoint_steps k > 0): the state
    // before step nst = 0, k, 2k, ... goes to ck_buf + (nst / k) * CK_STRIDE
    double* ck_buf;
    int ck_k, ck_next, ck_n;
    int it_cur;         // output index the current stop time belongs to
    double tcur_cur;    // time reported at the last output
    // per-lane model tables: packed flux reactants (a+1 | (b+1)<<16) and their
    // per-instance coefficients; packed stoichiometry entries (flux | coef<<16)
    int fab[FMR];
    double fcr[FMR];
    int srow[TREG ? S : 1][TREG ? RM : 1];
    double scoef[TREG ? S : 1][TREG ? RM : 1];
    int slen[S];
    // register path: saved Jacobian row and the row of M^-1 held by this lane
    LUT jrow[REG ? N : 1], irow[REG ? N : 1];
    int inv_src;
    // the pivot lane of every Gauss-Jordan step, 5 bits per step
    static constexpr int NPK = REG ? (N + 5) / 6 : 1;
    unsigned pivlanes[NPK];
    __device__ __forceinline__ int pivot_lane(int j) const { return int((pivlanes[j / 6] >> (5 * (j % 6))) & 31u); }
    // staggered forward sensitivities
    double *fda, *fdb, *fmo, *dcs;  // shared: dw_r/dy_a, dw_r/dy_b, dw/dc, dc/dp
    LUT* Minv;                      // shared: M^-1 (register path)
    double* sb;                     // this group's sensitivity scratch
    const int32_t* plist;
    int ns, nsp;
    R crateS, acnrmS;
    int jcur_stg;
    double incA1;                   // coefficient of the last order increase
    // forward run with adjoint storage: every accepted step's time, state and
    // order go to the group's scratch (CVodeF + CVApolynomialStorePnt,
    // cvodea.c:395,3236); NULL when not storing
    double *st_t, *st_q, *st_y, *st_dj;
    long long st_n, st_cap;
    // backward (adjoint) problem: shared interpolant and flux work, the
    // forward steps to interpolate, quadratures in the group's scratch
    double *xs, *fwa, *fwb, *fmo_b, *us, *Yd, *Td;
    const double *pt_t, *pt_q, *pt_y;
    long long npts, ilast;
    int newdata, dd_base, dd_order;
    double t_interp, hu, tretlast;
    double* qb;                     // quadrature vectors [QV_N][nqp]
    const double* pt_yd;            // Hermite interpolant: derivatives at the stored points (NULL: polynomial)
    const int* tb;                  // model tables in shared memory (M::TB_* offsets)
    int nq, nqp, qu;
    static constexpr int QV_EWT = LMAX, QV_ACOR = LMAX + 1, QV_TMP = LMAX + 2, QV_Y = LMAX + 3, QV_N = LMAX + 4;

    __device__ __forceinline__ Integrator(unsigned char* base) {
        double* d = reinterpret_cast<double*>(base);
        ys = d;
        ws = ys + N;
        cs = ws + NW;
        pu = cs + M::NC;
        ku = pu + M::NP;
        LUT* lb = reinterpret_cast<LUT*>(base + LY::bytes_double);
        Jsv = lb;
        Mm = lb + LY::n_jsv;
        dinv = Mm + M::LU_STORE;
        bf = dinv + N;
        perm = reinterpret_cast<int16_t*>(base + LY::bytes_double + LY::bytes_lut);
        fda = ku + M::NK + M::NH;
        fdb = fda + NW;
        fmo = fdb + NW;
        dcs = fmo + M::NC;
        Minv = bf + N;
        sb = nullptr;
        plist = nullptr;
        ns = nsp = 0;
        st_t = st_q = st_y = st_dj = nullptr;
        st_n = st_cap = 0;
        force_setup = 0;
        force_reinit = called = 0;
        rt_irfnd = rt_taskc = 0;
        rt_tlo = rt_thi = rt_trout = rt_ttol = rt_toutc = tretlast = tlastroot = 0.0;
#pragma unroll
        for (int i = 0; i < NRR; i++) {
            rt_glo[i] = rt_ghi[i] = rt_grout[i] = 0.0;
            rt_iroots[i] = 0;
            rt_gactive[i] = 1;
        }
        ck_buf = nullptr;
        ck_k = ck_next = ck_n = 0;
        it_cur = 0;
        tcur_cur = 0.0;
        qb = nullptr;
        pt_yd = nullptr;
        nq = nqp = 0;
        if constexpr (BWD) {
            double* e = reinterpret_cast<double*>(base + LY::bytes);
            xs = e;
            fwa = xs + N;
            fwb = fwa + NW;
            fmo_b = fwb + NW;
            us = fmo_b + M::NC;
            Yd = us + NW;
            Td = Yd + (QMAX + 1) * N;
            dcs = Td + (QMAX + 1);
        }
    }

    __device__ __forceinline__ int idx(int s) const { return s * G + g.lane; }
    // the stability-limit detector's history in this instance's shared memory
    __device__ __forceinline__ double* ssd() const { return ys + LY::ssd_off; }
    __device__ void clear_stab() {
        nscon = 0;
        for (int j = g.lane; j < 15; j += G) ssd()[j] = 0.0;
        g.sync();
    }
    __device__ __forceinline__ bool own(int s) const { return (N % G == 0) || (s * G + g.lane < N); }

    // ---------------- model evaluation ------------------------------------
    __device__ void load_tables() {
        if constexpr (FREG) {
#pragma unroll
            for (int m = 0; m < FM; m++) {
                const int r = m * G + g.lane;
                fab[m] = r < NW ? M::flux_ab(r) : 0;
                fcr[m] = 0.0;
            }
        }
#pragma unroll
        for (int s = 0; s < S; s++) {
            slen[s] = own(s) ? M::row_end(idx(s)) - M::row_begin(idx(s)) : 0;
            if constexpr (TREG) {
#pragma unroll
                for (int e = 0; e < RM; e++) {
                    const int pk = e < slen[s] ? M::row_packed(M::row_begin(idx(s)) + e) : 0;
                    srow[s][e] = pk & 0xFFFF;
                    scoef[s][e] = double(pk >> 16);
                }
            }
        }
    }

    __device__ __forceinline__ static double stoich_term(int pk, const double* w) {
        const double t = w[pk & 0xFFFF];
        const int c = pk >> 16;
        return c == 1 ? t : c == -1 ? -t : c == 2 ? t + t : c == -2 ? -(t + t) : double(c) * t;
    }

    // f = S * w(y) for y in ys (complete in shared memory; callers sync first);
    // for the backward problem f = -J(x(t))^T y at the interpolated x(t)
    __device__ __forceinline__ void rhs(double (&f)[S]) {
        nfe++;
        if constexpr (BWD) {
            rhs_bwd(f);
            return;
        }
        if constexpr (FREG) {
#pragma unroll
            for (int m = 0; m < FM; m++) {
                const int r = m * G + g.lane;
                if (r < NW) {
                    const int a = (fab[m] & 0xFFFF) - 1, b = (fab[m] >> 16) - 1;
                    double v = fcr[m];
                    if (a >= 0) v *= ys[a];
                    if (b >= 0) v *= ys[b];
                    ws[r] = v;
                }
            }
        } else if constexpr (M::GENERAL) {
            for (int r = g.lane; r < NW; r += G) ws[r] = M::flux_value(r, ys, cs);
        } else {
            for (int r = g.lane; r < NW; r += G) {
                const int ab = M::flux_ab(r);
                const int a = (ab & 0xFFFF) - 1, b = (ab >> 16) - 1;
                double v = cs[r];
                if (a >= 0) v *= ys[a];
                if (b >= 0) v *= ys[b];
                ws[r] = v;
            }
        }
        g.sync();
#pragma unroll
        for (int s = 0; s < S; s++) {
            double s0 = 0.0, s1 = 0.0;  // two partial sums halve the dependency chain
            if constexpr (TREG) {
#pragma unroll
                for (int e = 0; e < RM; e++) {
                    // padded entries have coefficient 0 and point at flux 0
                    if (e & 1) s1 = fma(scoef[s][e], ws[srow[s][e]], s1);
                    else s0 = fma(scoef[s][e], ws[srow[s][e]], s0);
                }
            } else if (own(s)) {
                const int e0 = M::row_begin(idx(s)), e1 = M::row_end(idx(s));
                for (int e = e0; e < e1; e++) {
                    const double t = stoich_term(M::row_packed(e), ws);
                    if ((e - e0) & 1) s1 += t;
                    else s0 += t;
                }
            }
            f[s] = s0 + s1;
        }
    }

    __device__ __forceinline__ void rhs_at(double t, double (&f)[S]) {
        if constexpr (BWD) interp_at(t);
        rhs(f);
    }

    // ---------------- backward (adjoint) right-hand sides -----------------
    // u = S^T y (one flux per lane), then xBdot_j = -sum over the fluxes r
    // with reactant j of dw_r/dx_j * u_r (model_ode.cpp:355-362 with the
    // sparse Jacobian written as S * dw/dx)
    __device__ void flux_projection() {
        for (int r = g.lane; r < NW; r += G) {
            double u = 0.0;
            const int e1 = tb[M::TB_SC_PTR + r + 1];
            for (int e = tb[M::TB_SC_PTR + r]; e < e1; e++) {
                const int pk = tb[M::TB_SC_PK + e];
                u = fma(double(pk >> 16), ys[pk & 0xFFFF], u);
            }
            us[r] = u;
        }
        g.sync();
    }
    __device__ void rhs_bwd(double (&f)[S]) {
        flux_projection();
#pragma unroll
        for (int s = 0; s < S; s++) {
            double acc = 0.0;
            if (own(s)) {
                const int i = idx(s);
                const int e1 = tb[M::TB_RI_PTR + i + 1];
                for (int e = tb[M::TB_RI_PTR + i]; e < e1; e++) {
                    const int pk = tb[M::TB_RI_PK + e], r = pk >> 1;
                    acc = fma((pk & 1) ? fwb[r] : fwa[r], us[r], acc);
                }
            }
            f[s] = -acc;
        }
        g.sync();
    }
    // quadrature right-hand side qBdot_c = -(dxdot/dp_{plist[c]})^T y into QV(dst)
    // (model_ode.cpp:364-374), y in ys
    __device__ void rhsQ_at(double t, int dst) {
        interp_at(t);
        flux_projection();
        for (int c = g.lane; c < nq; c += G) {
            const int pj = plist[c];
            double acc = 0.0;
            const int d1 = tb[M::TB_DP_PTR + pj + 1];
            for (int d = tb[M::TB_DP_PTR + pj]; d < d1; d++) {
                const int ci = tb[M::TB_DP_R + d];
                acc = fma(dcs[d] * fmo_b[ci], us[M::coef_flux(ci)], acc);
            }
            QV(dst, c) = -acc;
        }
        g.sync();
    }
    __device__ __forceinline__ double& QV(int v, int c) const { return qb[(size_t)v * nqp + c]; }

    // Forward state at t from the stored steps (CVAfindIndex + CVApolynomialGetY,
    // cvodea.c:2548,3270): divided differences over the order+1 points ending at
    // the base point, cached per (base, order); then dw/dx and the monomials at x(t)
    __device__ void interp_at(double t) {
        if (t == t_interp) return;
        long long indx;
        int bad = 0;
        if (newdata) {
            ilast = npts - 1;
            newdata = 0;
        }
        const bool to_left = (t - pt_t[ilast - 1]) < 0.0;
        const bool to_right = (t - pt_t[ilast]) > 0.0;
        if (to_left) {
            indx = ilast;
            for (;;) {
                if (indx == 0) break;
                if (t - pt_t[indx - 1] <= 0.0) indx--;
                else break;
            }
            ilast = (indx == 0) ? 1 : indx;
            if (indx == 0 && fabs(t - pt_t[0]) > FUZZ_FACTOR * UROUND) bad = 1;
        } else if (to_right) {
            indx = ilast;
            for (;;) {
                if (indx < npts - 1 && t - pt_t[indx] > 0.0) indx++;
                else break;
            }
            ilast = indx;
        } else {
            indx = ilast;
        }
        if (indx == 0 || bad) {
#pragma unroll
            for (int s = 0; s < S; s++)
                if (own(s)) xs[idx(s)] = bad ? NAN : pt_y[idx(s)];
        } else if (pt_yd) {
            // cubic Hermite between the stored points indx-1 and indx (CVAhermiteGetY,
            // cvodea.c:2906): y = y0 + f1 yd0 + f2 Y0 + f3 Y1 with Y0 = y1 - y0 - d yd0
            // and Y1 = d (yd1 + yd0) - 2 (y1 - y0), cached per interval
            const double t0i = pt_t[indx - 1], t1i = pt_t[indx], delta = t1i - t0i;
            // per interval, shared: Y0, Y1 and the left point's y0, yd0
            const double* y0 = Yd + 2 * N;
            const double* yd0 = Yd + 3 * N;
            if (indx != dd_base) {
                const double* gy0 = pt_y + (size_t)(indx - 1) * N;
                const double* gyd0 = pt_yd + (size_t)(indx - 1) * N;
                const double* y1 = pt_y + (size_t)indx * N;
                const double* yd1 = pt_yd + (size_t)indx * N;
#pragma unroll
                for (int s = 0; s < S; s++) {
                    if (!own(s)) continue;
                    const int i = idx(s);
                    const double a0 = gy0[i], ad0 = gyd0[i], a1 = y1[i], ad1 = yd1[i];
                    double y1v = -2.0 * a1;
                    y1v += 2.0 * a0;
                    y1v += delta * ad1;
                    y1v += delta * ad0;
                    double y0v = 1.0 * a1;
                    y0v += -1.0 * a0;
                    y0v += -delta * ad0;
                    Yd[i] = y0v;
                    Yd[N + i] = y1v;
                    Yd[2 * N + i] = a0;
                    Yd[3 * N + i] = ad0;
                }
                dd_base = (int)indx;
            }
            const double f1 = t - t0i;
            double f2 = f1 / delta;
            f2 = f2 * f2;
            const double f3 = f2 * (t - t1i) / delta;
#pragma unroll
            for (int s = 0; s < S; s++) {
                if (!own(s)) continue;
                const int i = idx(s);
                double v = y0[i];
                v += f1 * yd0[i];
                v += f2 * Yd[i];
                v += f3 * Yd[N + i];
                xs[i] = v;
            }
        } else {
            const double dt = fabs(pt_t[indx] - pt_t[indx - 1]);
            long long base = indx;
            const int order = int(pt_q[base]);
            if (indx < order) base += order - indx;
            if (base != dd_base || order != dd_order) {
#pragma unroll
                for (int s = 0; s < S; s++) {
                    if (!own(s)) continue;
                    const int i = idx(s);
                    for (int j = 0; j <= order; j++) Yd[j * N + i] = pt_y[(size_t)(base - j) * N + i];
                    for (int k = 1; k <= order; k++)
                        for (int j = order; j >= k; j--) {
                            const double factor = dt / (pt_t[base - j] - pt_t[base - j + k]);
                            Yd[j * N + i] = factor * (Yd[j * N + i] - Yd[(j - 1) * N + i]);
                        }
                }
                dd_base = (int)base;
                dd_order = order;
            }
            double cv = 1.0;
            double c[QMAX + 1];
            c[0] = 1.0;
#pragma unroll
            for (int k = 0; k < QMAX; k++) {
                if (k < order) cv = cv * (t - pt_t[base - k]) / dt;
                c[k + 1] = cv;
            }
#pragma unroll
            for (int s = 0; s < S; s++) {
                if (!own(s)) continue;
                const int i = idx(s);
                double v = c[0] * Yd[i];
#pragma unroll
                for (int k = 1; k <= QMAX; k++)
                    if (k <= order) v += c[k] * Yd[k * N + i];
                xs[i] = v;
            }
        }
        g.sync();
        if constexpr (M::GENERAL) {
            for (int r = g.lane; r < NW; r += G) M::flux_partials(r, xs, cs, fwa[r], fwb[r]);
            for (int ci = g.lane; ci < M::NC; ci += G) fmo_b[ci] = M::flux_dwdc(ci, xs, cs);
        } else {
            for (int r = g.lane; r < NW; r += G) {
                const int ab = tb[M::TB_W_AB + r], a = (ab & 0xFFFF) - 1, b = (ab >> 16) - 1;
                const double cr = cs[r];
                double da = 0.0, db = 0.0, mo = 1.0;
                if (a >= 0 && b >= 0) {
                    if (a == b) {
                        da = 2.0 * cr * xs[a];
                        mo = xs[a] * xs[a];
                    } else {
                        da = cr * xs[b];
                        db = cr * xs[a];
                        mo = xs[a] * xs[b];
                    }
                } else if (a >= 0) {
                    da = cr;
                    mo = xs[a];
                }
                fwa[r] = da;
                fwb[r] = db;
                fmo_b[r] = mo;
            }
        }
        g.sync();
        t_interp = t;
    }

    // quadrature WRMS norm over the lanes' entries of QV(v) with weights QV(QV_EWT)
    __device__ R quad_wrms(int v) {
        double s2 = 0.0;
        for (int c = g.lane; c < nq; c += G) {
            const double t = QV(v, c) * QV(QV_EWT, c);
            s2 += t * t;
        }
        const R sr = g.sum(R(s2));
        return sqrt(sr * R(1.0 / nq));
    }
    __device__ __forceinline__ static R upd_norm(R old_nrm, R nrm) { return (old_nrm > nrm) ? old_nrm : nrm; }
    __device__ int quad_ewt_set() {  // cvQuadEwtSetSS (cvodes.c:9177)
        int bad = 0;
        for (int c = g.lane; c < nq; c += G) {
            const double t = o->rtolQ * fabs(QV(0, c)) + o->atolQ;
            bad |= (o->atolQ == 0.0) && !(t > 0.0);
            QV(QV_EWT, c) = double(rdiv(R(1), R(t)));  // weights only scale norms compared with 1
        }
        return g.max(bad);
    }
    template <int Q, int SIGN>
    __device__ void quad_pascal_q() {
        for (int c = g.lane; c < nq; c += G) {
            double z[Q + 1];
#pragma unroll
            for (int j = 0; j <= Q; j++) z[j] = QV(j, c);
#pragma unroll
            for (int j = 0; j < Q; j++) {
                double a0 = z[j], a1 = 0.0;
#pragma unroll
                for (int m = j + 1; m <= Q; m++) {
                    const double cf = ((SIGN < 0) && ((m - j) & 1)) ? -binom(m, j) : binom(m, j);
                    if ((m - j) & 1) a1 = fma(cf, z[m], a1);
                    else a0 = fma(cf, z[m], a0);
                }
                QV(j, c) = a0 + a1;
            }
        }
    }
    template <int Q> __device__ void quad_predict_q() { quad_pascal_q<Q, 1>(); }
    template <int Q> __device__ void quad_restore_q() { quad_pascal_q<Q, -1>(); }
    template <int Q>
    __device__ void quad_rescale_q() {
        for (int c = g.lane; c < nq; c += G) {
            double f = eta;
#pragma unroll
            for (int j = 1; j <= Q; j++) {
                QV(j, c) *= f;
                f *= eta;
            }
        }
    }
    template <int Q>
    __device__ void quad_complete_q() {
        for (int c = g.lane; c < nq; c += G) {
            const double a = QV(QV_ACOR, c);
#pragma unroll
            for (int j = 0; j <= Q; j++) QV(j, c) += ld[j] * a;
        }
    }
    template <int Q>
    __device__ void quad_increase_q() {
        if constexpr (Q < QMAX) {
            for (int c = g.lane; c < nq; c += G) {
                const double zl = incA1 * QV(QMAX, c);
                QV(Q + 1, c) = zl;
#pragma unroll
                for (int j = 2; j <= Q; j++) QV(j, c) += double(l[j]) * zl;
            }
        }
    }
    template <int Q>
    __device__ void quad_decrease_q() {
        if constexpr (Q > 2) {
            for (int c = g.lane; c < nq; c += G) {
                const double zq = QV(Q, c);
#pragma unroll
                for (int j = 2; j < Q; j++) QV(j, c) += -double(l[j]) * zq;
            }
        }
    }
    __device__ void quad_copy(int vdst, int vsrc) {
        for (int c = g.lane; c < nq; c += G) QV(vdst, c) = QV(vsrc, c);
    }

    __device__ __forceinline__ void store_y(const double (&v)[S]) {
#pragma unroll
        for (int s = 0; s < S; s++)
            if (own(s)) ys[idx(s)] = v[s];
        g.sync();
    }

    // weighted RMS norm (N_VWrmsNorm) in the control type: one conversion per
    // element, the weighting, squares and sums in R (relative error ~1e-7 in
    // FP32, in a quantity only compared against thresholds near 1)
    __device__ __forceinline__ R wrms(const double (&v)[S]) {
        R s2 = R(0);
#pragma unroll
        for (int s = 0; s < S; s++) {
            const R t = R(v[s]) * ewt[s];
            s2 += t * t;
        }
        const R sr = g.sum(s2);
        return sqrt(sr * R(1.0 / N));
    }

    // error weights (cvEwtSetSS): 1/(rtol*|y| + atol); a nonpositive weight is an error
    __device__ __forceinline__ int ewt_set() {
        int bad = 0;
#pragma unroll
        for (int s = 0; s < S; s++) {
            if (own(s)) {
                const R t = R(BWD ? o->rtolB : o->rtol) * fabs(R(zn[0][s])) + R(BWD ? o->atolB : o->atol);
                bad |= !(t > R(0));
                ewt[s] = rdiv(R(1), t);
            } else {
                ewt[s] = R(0);
            }
        }
        return g.max(bad);
    }

    // ---------------- linear algebra: M = I - gamma*J, LU, solve -----------
    __device__ void jac_eval() {
        if constexpr (M::SPARSE_LU && !REG) {
            // J on its pattern at the forward state (the backward problem's -J^T is
            // formed when the iteration matrix is assembled)
#pragma unroll
            for (int s = 0; s < S; s++)
                if (own(s)) M::template jac_row_sparse<LUT>(idx(s), cs, BWD ? xs : ys, Jsv);
            g.sync();
            return;
        }
        if constexpr (BWD) {
            // J at the interpolated forward state (in Mm as scratch), then J_B = -J^T
            // (Model_ODE::fJB, model_ode.cpp:305-322)
#pragma unroll
            for (int s = 0; s < S; s++) {
                if (!own(s)) continue;
                const int i = idx(s);
                for (int j = 0; j < N; j++) Mm[j * N + i] = LUT(0);
                M::template jac_row<LUT>(i, cs, xs, Mm);
            }
            g.sync();
#pragma unroll
            for (int s = 0; s < S; s++) {
                if (!own(s)) continue;
                const int c = idx(s);
                for (int r = 0; r < N; r++) Jsv[c * N + r] = -Mm[r * N + c];
            }
            g.sync();
            return;
        }
#pragma unroll
        for (int s = 0; s < S; s++) {
            if (!own(s)) continue;
            const int i = idx(s);
            for (int j = 0; j < N; j++) Jsv[j * N + i] = LUT(0);
            M::template jac_row<LUT>(i, cs, ys, Jsv);
        }
    }

    // cvLsSetup (cvodes_ls.c:1611) + GETRF; returns 0, or 1 for a singular M
    __device__ int lsetup() {
        nsetups++;
        const R dgamma = fabs(R(gamma) / gammap - R(1));
        const int jbad = force_setup || (nst == 0) || (nst >= nstlj + MSBJ) ||
                         ((convfail == CV_FAIL_BAD_J) && (dgamma < DGMAX_JBAD)) || (convfail == CV_FAIL_OTHER);
        if (!jbad) {
            jcur = 0;
        } else {
            jac_eval();  // J at the predicted y in ys
            nje++;
            jcur = 1;
            nstlj = nst;
            if constexpr (REG) {
#pragma unroll
                for (int j = 0; j < N; j++) jrow[j] = g.lane < N ? Jsv[j * N + g.lane] : LUT(0);
            }
        }
        force_setup = 0;
        if constexpr (REG) {
            const int ret = gauss_jordan();
            gamrat = R(1);
            gammap = R(gamma);
            crate = R(1);
            crateS = R(1);
            nstlp = nst;
            return ret;
        }
        const LUT mg = LUT(-gamma);
        int ret;
        if constexpr (M::PACKED_LU) {
            // the same matrix into the compressed rows of its factor pattern
            g.sync();
            for (int q = g.lane; q < M::LU_STORE; q += G) Mm[q] = LUT(0);
            for (int i = g.lane; i < N; i += G) perm[i] = (int16_t)M::lu_order(i);
            g.sync();
            const LUT sg = BWD ? LUT(gamma) : mg;
            for (int p = g.lane; p < M::NNZ_J; p += G) Mm[M::template pk_jpos<BWD>(p)] = sg * Jsv[p];
            g.sync();
            for (int i = g.lane; i < N; i += G) Mm[M::template pk_diag<BWD>(i)] += LUT(1);
            ret = packed_getrf<M, LUT, N, G, BWD>(Mm, dinv, bf, g.mask, g.lane);
            g.sync();
        } else if constexpr (M::SPARSE_LU) {
            // M = I - gamma*J in the static order, Mm(i, j) = M(order[i], order[j]):
            // zeros, the pattern entries scattered from the compact J (for the
            // backward problem M = I + gamma*J^T), then the unit diagonal
            g.sync();
#pragma unroll
            for (int s = 0; s < S; s++) {
                if (!own(s)) continue;
                const int i = idx(s);
                for (int j = 0; j < N; j++) Mm[j * N + i] = LUT(0);
                perm[i] = (int16_t)M::lu_order(i);
            }
            g.sync();
            for (int p = g.lane; p < M::NNZ_J; p += G) {
                const int rc = M::j_rc(p), r = M::lu_iorder(rc & 0xFFFF), c = M::lu_iorder(rc >> 16);
                if constexpr (BWD) Mm[r * N + c] = LUT(gamma) * Jsv[p];
                else Mm[c * N + r] = mg * Jsv[p];
            }
            g.sync();
#pragma unroll
            for (int s = 0; s < S; s++)
                if (own(s)) Mm[idx(s) * N + idx(s)] += LUT(1);
            ret = sparse_getrf<M, LUT, N, G, BWD>(Mm, dinv, g.mask, g.lane);
            g.sync();
        } else {
#pragma unroll
            for (int s = 0; s < S; s++) {
                if (!own(s)) continue;
                const int i = idx(s);
                for (int j = 0; j < N; j++) Mm[j * N + i] = mg * Jsv[j * N + i] + (i == j ? LUT(1) : LUT(0));
            }
            ret = getrf();
        }
        gamrat = R(1);
        gammap = R(gamma);
        crate = R(1);
        crateS = R(1);
        nstlp = nst;
        return ret;
    }

    // Register path (one row of M per lane): M^-1 by in-place Gauss-Jordan
    // elimination with partial pivoting, rows never move.  Step k pivots on
    // the unused row lp with the largest |a_lp,k| (ties: lowest row), chosen
    // with one warp reduction on (|a| bits, row); the pivot row is scaled,
    // column k is eliminated from every other row and takes the multipliers.
    // Afterwards lane P[k] holds row k of M^-1 with its entry for column P[j]
    // in slot j (P: the pivot lanes, kept in pivlanes).  Returns 1 if singular.
    __device__ int gauss_jordan() {
        const int lane = g.lane;
        const bool live = lane < N;
        const LUT mg = LUT(-gamma);
#pragma unroll
        for (int j = 0; j < N; j++) irow[j] = live ? mg * jrow[j] + (lane == j ? LUT(1) : LUT(0)) : LUT(0);
#pragma unroll
        for (int w = 0; w < NPK; w++) pivlanes[w] = 0u;
        bool used = !live;
        inv_src = 0;
        int my_step = -1;
        // the pivot loop stays rolled (its body selects column k of the
        // register row by predicates): unrolled, the N steps are most of the
        // kernel's code, and fetching that code on every setup costs more
        // than the predicated work
#pragma unroll 1
        for (int k = 0; k < N; k++) {
            // a_k by a tree of selects on the bits of k (dependent depth log2 N)
            LUT t[N];
#pragma unroll
            for (int j = 0; j < N; j++) t[j] = irow[j];
#pragma unroll
            for (int lv = 0; (1 << lv) < N; lv++) {
                const int w = 1 << lv;
                const bool hi = (k & w) != 0;
#pragma unroll
                for (int j = 0; j + w < N; j += 2 * w) t[j] = hi ? t[j + w] : t[j];
            }
            const LUT ak = t[0];
            const float v = fabsf(float(ak));
            unsigned key = 0u;
            if (!used) key = (v != v) ? 0xFFFFFFFFu : (v > 0.0f ? ((__float_as_uint(v) & ~31u) | (31u - lane)) : 0u);
            const unsigned kmax = __reduce_max_sync(g.mask, key);
            if (kmax == 0u) return 1;
            const int lp = 31 - int(kmax & 31u);
            const LUT piv = g.bcast(ak, lp);
            if (!(fabs(piv) > LUT(0)) || !isfinite(piv)) return 1;
            const LUT rp = LUT(1) / piv;
            const bool me = (lane == lp);
            const LUT gk = me ? LUT(0) : ak * rp;
#pragma unroll
            for (int j = 0; j < N; j++) {
                const LUT pj = g.bcast(irow[j], lp);
                const LUT u = me ? pj * rp : irow[j] - gk * pj;
                irow[j] = (j == k) ? (me ? rp : -gk) : u;
            }
            used = used || me;
            if (lane == k) inv_src = lp;
            if (me) my_step = k;
        }
        // P[j] = inv_src of lane j, packed (compile-time slots: no local memory)
#pragma unroll
        for (int j = 0; j < N; j++) pivlanes[j / 6] |= unsigned(g.bcast(inv_src, j)) << (5 * (j % 6));
        if constexpr (SENS) {
            if (my_step >= 0)
#pragma unroll
                for (int j = 0; j < N; j++) Minv[my_step * N + pivot_lane(j)] = irow[j];
            g.sync();
        }
        return 0;
    }

    __device__ int getrf() { return dense_getrf<LUT, N, G>(Mm, dinv, bf, perm, g.mask, g.lane); }

    // b <- M^{-1} b (cvLsSolve + GETRS), scaled by 2/(1+gamrat) (cvodes_ls.c:1851)
    // triangular sweeps over compressed rows: each slot walks its row's L
    // entries forward and its U entries backward with one pointer, matching
    // the entry's column against the pivot being broadcast
    __device__ __forceinline__ void packed_sweeps(LUT (&x)[S]) {
        int ptr[S], nxt[S], dg[S];
#pragma unroll
        for (int s = 0; s < S; s++) {
            const int i = s * G + g.lane;
            if (i < N) {
                ptr[s] = M::template pk_rptr<BWD>(i);
                dg[s] = M::template pk_diag<BWD>(i);
                nxt[s] = ptr[s] < dg[s] ? M::template pk_col<BWD>(ptr[s]) : N;
            } else {
                ptr[s] = dg[s] = 0;
                nxt[s] = N;
            }
        }
#pragma unroll
        for (int sk = 0; sk < S; sk++) {
            for (int kk = 0; kk < G; kk++) {
                const int k = sk * G + kk;
                if (k >= N - 1) break;
                const LUT xk = g.bcast(x[sk], kk);
#pragma unroll
                for (int s = sk; s < S; s++) {
                    if (nxt[s] == k) {
                        x[s] -= Mm[ptr[s]] * xk;
                        ptr[s]++;
                        nxt[s] = ptr[s] < dg[s] ? M::template pk_col<BWD>(ptr[s]) : N;
                    }
                }
            }
        }
#pragma unroll
        for (int s = 0; s < S; s++) {
            const int i = s * G + g.lane;
            ptr[s] = i < N ? M::template pk_rptr<BWD>(i + 1) - 1 : 0;
            nxt[s] = ptr[s] > dg[s] ? M::template pk_col<BWD>(ptr[s]) : -1;
        }
#pragma unroll
        for (int sk = S - 1; sk >= 0; sk--) {
            for (int kk = G - 1; kk >= 0; kk--) {
                const int k = sk * G + kk;
                if (k >= N) continue;
                const LUT xk = g.bcast(x[sk], kk) * dinv[k];
                if (g.lane == kk) x[sk] = xk;
#pragma unroll
                for (int s = 0; s <= sk; s++) {
                    if (nxt[s] == k) {
                        x[s] -= Mm[ptr[s]] * xk;
                        ptr[s]--;
                        nxt[s] = ptr[s] > dg[s] ? M::template pk_col<BWD>(ptr[s]) : -1;
                    }
                }
            }
        }
    }
    __device__ void lsolve(double (&b)[S]) {
        if constexpr (REG) {
            const LUT bme = g.lane < N ? LUT(b[0]) : LUT(0);
            LUT acc[4] = {LUT(0), LUT(0), LUT(0), LUT(0)};
#pragma unroll
            for (int j = 0; j < N; j++) acc[j & 3] += irow[j] * g.bcast(bme, pivot_lane(j));
            const LUT xk = (acc[0] + acc[1]) + (acc[2] + acc[3]);
            const LUT x = g.bcast(xk, inv_src);
            const double sc = (gamrat != R(1)) ? double(R(2) / (R(1) + gamrat)) : 1.0;
            b[0] = g.lane < N ? double(x) * sc : 0.0;
            return;
        }
#pragma unroll
        for (int s = 0; s < S; s++)
            if (own(s)) bf[idx(s)] = LUT(b[s]);
        g.sync();
        LUT x[S];
#pragma unroll
        for (int s = 0; s < S; s++) x[s] = own(s) ? bf[perm[idx(s)]] : LUT(0);
        g.sync();
        // sweeps over the LU factors with the solution in registers (element i
        // in slot i / G of lane i % G) and x_k broadcast by shuffle: no shared
        // round trip or barrier on the dependent chain
        if constexpr (M::PACKED_LU) {
            packed_sweeps(x);
        } else {
#pragma unroll
        for (int sk = 0; sk < S; sk++) {
            for (int kk = 0; kk < G; kk++) {
                const int k = sk * G + kk;
                if (k >= N - 1) break;
                const LUT xk = g.bcast(x[sk], kk);
                const LUT* Lk = Mm + k * N;
#pragma unroll
                for (int s = sk; s < S; s++) {
                    const int i = s * G + g.lane;
                    if (i > k && i < N) x[s] -= Lk[i] * xk;
                }
            }
        }
#pragma unroll
        for (int sk = S - 1; sk >= 0; sk--) {
            for (int kk = G - 1; kk >= 0; kk--) {
                const int k = sk * G + kk;
                if (k >= N) continue;
                const LUT xk = g.bcast(x[sk], kk) * dinv[k];
                if (g.lane == kk) x[sk] = xk;
                const LUT* Uk = Mm + k * N;
#pragma unroll
                for (int s = 0; s <= sk; s++) {
                    const int i = s * G + g.lane;
                    if (i < k) x[s] -= Uk[i] * xk;
                }
            }
        }
        }
        if constexpr (M::SPARSE_LU) {  // the solution back from the static order
#pragma unroll
            for (int s = 0; s < S; s++)
                if (own(s)) bf[perm[idx(s)]] = x[s];
            g.sync();
#pragma unroll
            for (int s = 0; s < S; s++) x[s] = own(s) ? bf[idx(s)] : LUT(0);
            g.sync();
        }
        const double sc = (gamrat != R(1)) ? double(R(2) / (R(1) + gamrat)) : 1.0;
#pragma unroll
        for (int s = 0; s < S; s++) b[s] = double(x[s]) * sc;
    }

    // ---------------- Nordsieck history (cvodes.c:6112-6506) --------------
    // cvPredict: zn <- zn * Pascal matrix.  Written as zn'_j = sum_{m>=j} C(m,j) zn_m
    // so every new entry is a short independent sum instead of one long chain
    // of dependent additions (same operation count, depth ~3 instead of ~15).
    __host__ __device__ static constexpr double binom(int m, int j) {
        double c = 1.0;
        for (int i = 0; i < j; i++) c = c * (m - i) / (i + 1);
        return c;
    }
    template <int Q, int SIGN>
    __device__ __forceinline__ void pascal_q() {
#pragma unroll
        for (int s = 0; s < S; s++) {
            double z[Q + 1];
#pragma unroll
            for (int j = 0; j <= Q; j++) z[j] = zn[j][s];
#pragma unroll
            for (int j = 0; j < Q; j++) {
                double a0 = z[j], a1 = 0.0;
#pragma unroll
                for (int m = j + 1; m <= Q; m++) {
                    const double c = ((SIGN < 0) && ((m - j) & 1)) ? -binom(m, j) : binom(m, j);
                    if ((m - j) & 1) a1 = fma(c, z[m], a1);
                    else a0 = fma(c, z[m], a0);
                }
                zn[j][s] = a0 + a1;
            }
        }
    }
    template <int Q>
    __device__ __forceinline__ void predict_q() { pascal_q<Q, 1>(); }
    // cvRestore: the inverse Pascal matrix has entries (-1)^(m-j) C(m,j)
    template <int Q>
    __device__ __forceinline__ void restore_q() { pascal_q<Q, -1>(); }
    template <int Q>
    __device__ __forceinline__ void rescale_q() {
        const double e = eta;
        double f = e;
#pragma unroll
        for (int j = 1; j <= Q; j++) {
#pragma unroll
            for (int s = 0; s < S; s++) zn[j][s] *= f;
            f *= e;
        }
    }
    template <int Q>
    __device__ __forceinline__ void complete_q() {
#pragma unroll
        for (int j = 0; j <= Q; j++)
#pragma unroll
            for (int s = 0; s < S; s++) zn[j][s] += ld[j] * acor[s];
    }
    template <int Q>
    __device__ __forceinline__ void znq_to_tmp() {
#pragma unroll
        for (int s = 0; s < S; s++) tmp[s] = zn[Q][s];
    }
    // cvIncreaseBDF (cvodes.c:6256): zn[q+1] from the saved correction zn[QMAX]
    template <int Q>
    __device__ __forceinline__ void increase_q() {
        if constexpr (Q < QMAX) {
            const R hsc = R(hscale);
            R alpha0 = R(-1), alpha1 = R(1), prod = R(1), xiold = R(1), hsum = hsc;
#pragma unroll
            for (int i = 0; i <= QMAX; i++) l[i] = R(0);
            l[2] = R(1);
#pragma unroll
            for (int j = 1; j < Q; j++) {
                hsum += tau[j + 1];
                const R xi = rdiv(hsum, hsc);
                prod *= xi;
                alpha0 -= R(inv_int(j + 1));
                alpha1 += rdiv(R(1), xi);
#pragma unroll
                for (int i = j + 2; i >= 2; i--) l[i] = l[i] * xiold + l[i - 1];
                xiold = xi;
            }
            const double A1 = double(rdiv(-alpha0 - alpha1, prod));
            incA1 = A1;
            double lj[LMAX];
#pragma unroll
            for (int j = 2; j <= Q; j++) lj[j] = double(l[j]);
#pragma unroll
            for (int s = 0; s < S; s++) {
                const double zl = A1 * zn[QMAX][s];
                zn[Q + 1][s] = zl;
#pragma unroll
                for (int j = 2; j <= Q; j++) zn[j][s] += lj[j] * zl;
            }
        }
    }
    // cvDecreaseBDF (cvodes.c:6363)
    template <int Q>
    __device__ __forceinline__ void decrease_q() {
        if constexpr (Q > 2) {
            const R hsc = R(hscale);
            R hsum = R(0);
#pragma unroll
            for (int i = 0; i <= QMAX; i++) l[i] = R(0);
            l[2] = R(1);
#pragma unroll
            for (int j = 1; j <= Q - 2; j++) {
                hsum += tau[j];
                const R xi = rdiv(hsum, hsc);
#pragma unroll
                for (int i = j + 2; i >= 2; i--) l[i] = l[i] * xi + l[i - 1];
            }
            double lj[LMAX];
#pragma unroll
            for (int j = 2; j < Q; j++) lj[j] = -double(l[j]);
#pragma unroll
            for (int s = 0; s < S; s++)
#pragma unroll
                for (int j = 2; j < Q; j++) zn[j][s] += lj[j] * zn[Q][s];
        }
    }
    // cvSetBDF + cvSetTqBDF (cvodes.c:6788-6892)
    template <int Q>
    __device__ __forceinline__ void set_bdf_q() {
        const R hr = R(h);
        R alpha0 = R(-1), alpha0_hat = R(-1), xi_inv = R(1), xistar_inv = R(1), hsum = hr;
        l[0] = l[1] = R(1);
#pragma unroll
        for (int i = 2; i <= QMAX; i++) l[i] = R(0);
        if constexpr (Q > 1) {
#pragma unroll
            for (int j = 2; j < Q; j++) {
                hsum += tau[j - 1];
                xi_inv = rdiv(hr, hsum);
                alpha0 -= R(inv_int(j));
#pragma unroll
                for (int i = j; i >= 1; i--) l[i] += l[i - 1] * xi_inv;
            }
            alpha0 -= R(inv_int(Q));
            xistar_inv = -l[1] - alpha0;
            hsum += tau[Q - 1];
            xi_inv = rdiv(hr, hsum);
            alpha0_hat = -l[1] - xi_inv;
#pragma unroll
            for (int i = Q; i >= 1; i--) l[i] += l[i - 1] * xistar_inv;
        }
        const R A1 = R(1) - alpha0_hat + alpha0;
        const R A2 = R(1) + R(Q) * A1;
        tq[2] = fabs(rdiv(A1, alpha0 * A2));
        tq[5] = fabs(rdiv(A2 * xistar_inv, l[Q] * xi_inv));
        if (qwait == 1) {
            if constexpr (Q > 1) {
                const R C = rdiv(xistar_inv, l[Q]);
                const R A3 = alpha0 + R(inv_int(Q));
                const R A4 = alpha0_hat + xi_inv;
                const R Cpinv = rdiv(R(1) - A4 + A3, A3);
                tq[1] = fabs(C * Cpinv);
            } else {
                tq[1] = R(1);
            }
            hsum += tau[Q];
            const R xi2 = rdiv(hr, hsum);
            const R A5 = alpha0 - R(inv_int(Q + 1));
            const R A6 = alpha0_hat - xi2;
            const R Cppinv = rdiv(R(1) - A6 + A5, A2);
            tq[3] = fabs(rdiv(Cppinv, xi2 * R(Q + 2) * A5));
        }
        tq[4] = rdiv(R(CORTES), tq[2]);
#pragma unroll
        for (int j = 0; j <= Q; j++) ld[j] = double(l[j]);
    }

    __device__ void predict() {
        tn += h;
        if (tstopset && (tn - tstop) * h > 0.0) tn = tstop;
        AGB_DISPATCH_Q(q, predict_q)
        if constexpr (SENS) AGB_DISPATCH_Q(q, sens_predict_q)
        if constexpr (BWD) AGB_DISPATCH_Q(q, quad_predict_q)
    }
    __device__ void restore(double saved_t) {
        tn = saved_t;
        AGB_DISPATCH_Q(q, restore_q)
        if constexpr (SENS) AGB_DISPATCH_Q(q, sens_restore_q)
        if constexpr (BWD) AGB_DISPATCH_Q(q, quad_restore_q)
    }
    __device__ void rescale() {
        AGB_DISPATCH_Q(q, rescale_q)
        if constexpr (SENS) AGB_DISPATCH_Q(q, sens_rescale_q)
        if constexpr (BWD) AGB_DISPATCH_Q(q, quad_rescale_q)
        h = hscale * eta;
        hscale = h;
        nscon = 0;
    }
    __device__ void adjust_order(int dq) {
        if (q == 2 && dq != 1) return;  // cvAdjustOrder (cvodes.c:6134)
        if (dq == 1) {
            AGB_DISPATCH_Q(q, increase_q)
            if constexpr (SENS) AGB_DISPATCH_Q(q, sens_increase_q)
            if constexpr (BWD) AGB_DISPATCH_Q(q, quad_increase_q)
        } else if (dq == -1) {
            AGB_DISPATCH_Q(q, decrease_q)
            if constexpr (SENS) AGB_DISPATCH_Q(q, sens_decrease_q)
            if constexpr (BWD) AGB_DISPATCH_Q(q, quad_decrease_q)
        }
    }
    __device__ void adjust_params() {
        if (qprime != q) {
            adjust_order(qprime - q);
            q = qprime;
            L = q + 1;
            qwait = L;
        }
        rescale();
    }
    __device__ void cv_set() {
        AGB_DISPATCH_Q(q, set_bdf_q)
        rl1 = rdiv(R(1), l[1]);
        gamma = h * double(rl1);
        if (nst == 0) gammap = R(gamma);
        gamrat = (nst > 0) ? rdiv(R(gamma), gammap) : R(1);
    }


    // ---------------- staggered forward sensitivities ----------------------
    // Column c of the sensitivities (parameter plist[c]) belongs to lane
    // c % G; vector v (Nordsieck 0..QMAX, weights, correction, residual,
    // RHS) of column c lives at sb[(v*N + i)*nsp + c], so the lanes of a group
    // touch consecutive addresses.  cvStgrNls, cvodes.c:7167-7218;
    // cvodes_nls_stg.c; sensitivity RHS Model_ODE::fsxdot, model_ode.cpp:419-450.
    static constexpr int V_EWT = LMAX, V_ACOR = LMAX + 1, V_TMP = LMAX + 2, V_F = LMAX + 3;
    __device__ __forceinline__ double& SV(int v, int i, int c) const {
        return sb[((size_t)v * N + i) * nsp + c];
    }

    // dw/dy and dw/dc at the state in ys (complete); coefficient derivatives
    // are per instance
    __device__ void sens_prepare() {
        if constexpr (M::GENERAL) {
            for (int r = g.lane; r < NW; r += G) M::flux_partials(r, ys, cs, fda[r], fdb[r]);
            for (int ci = g.lane; ci < M::NC; ci += G) fmo[ci] = M::flux_dwdc(ci, ys, cs);
            g.sync();
            return;
        }
        for (int r = g.lane; r < NW; r += G) {
            const int ab = M::flux_ab(r), a = (ab & 0xFFFF) - 1, b = (ab >> 16) - 1;
            const double c = cs[r];
            double da = 0.0, db = 0.0, mo = 1.0;
            if (a >= 0 && b >= 0) {
                if (a == b) {
                    da = 2.0 * c * ys[a];
                    mo = ys[a] * ys[a];
                } else {
                    da = c * ys[b];
                    db = c * ys[a];
                    mo = ys[a] * ys[b];
                }
            } else if (a >= 0) {
                da = c;
                mo = ys[a];
            }
            fda[r] = da;
            fdb[r] = db;
            fmo[r] = mo;
        }
        g.sync();
    }

    // vout(:, c) = J * vin(:, c) + dxdot/dp_{plist[c]}
    __device__ void sens_rhs_col(int c, int vin, int vout) {
        auto v = [&](int j) { return SV(vin, j, c); };
        for (int i = 0; i < N; i++) {
            double acc = 0.0;
            for (int e = M::row_begin(i); e < M::row_end(i); e++) {
                const int pk = M::row_packed(e), r = pk & 0xFFFF;
                const int ab = M::flux_ab(r), a = (ab & 0xFFFF) - 1, b = (ab >> 16) - 1;
                double wsv = a >= 0 ? fda[r] * v(a) : 0.0;
                if (b >= 0 && b != a) wsv = fma(fdb[r], v(b), wsv);
                acc = fma(double(pk >> 16), wsv, acc);
            }
            SV(vout, i, c) = acc;
        }
        const int pj = plist[c];
        for (int d = M::dp_begin(pj); d < M::dp_end(pj); d++) {
            const int ci = M::dp_coef(d), r = M::coef_flux(ci);
            const double v = dcs[d] * fmo[ci];
            for (int e = M::col_begin(r); e < M::col_end(r); e++) {
                const int pk = M::col_packed(e);
                SV(vout, pk & 0xFFFF, c) += double(pk >> 16) * v;
            }
        }
    }
    __device__ void sens_rhs(int vin, int vout) {
        for (int c = g.lane; c < ns; c += G) sens_rhs_col(c, vin, vout);
    }

    // max over columns of the WRMS norms (cvSensNorm), FP64 sums per column
    __device__ R sens_norm(int v) {
        R mx = R(0);
        for (int c = g.lane; c < ns; c += G) {
            double s2 = 0.0;
            for (int i = 0; i < N; i++) {
                const double t = SV(v, i, c) * SV(V_EWT, i, c);
                s2 += t * t;
            }
            const R nrm = sqrt(R(s2) * R(1.0 / N));
            mx = (nrm > mx || nrm != nrm) ? nrm : mx;
        }
        return g.max(mx);
    }

    __device__ int sens_ewt_set() {  // cvSensEwtSetSS
        int bad = 0;
        for (int c = g.lane; c < ns; c += G)
            for (int i = 0; i < N; i++) {
                const double t = o->rtolS * fabs(SV(0, i, c)) + o->atolS;
                bad |= !(t > 0.0);
                SV(V_EWT, i, c) = double(rdiv(R(1), R(t)));
            }
        return g.max(bad);
    }
    // the weights as sens_ewt_set, and with them sens_norm(0) in the same pass
    __device__ int sens_ewt_set_norm0(R& nrm0) {
        int bad = 0;
        R mx = R(0);
        for (int c = g.lane; c < ns; c += G) {
            double s2 = 0.0;
            for (int i = 0; i < N; i++) {
                const double z = SV(0, i, c);
                const double t = o->rtolS * fabs(z) + o->atolS;
                bad |= !(t > 0.0);
                const double w = double(rdiv(R(1), R(t)));
                SV(V_EWT, i, c) = w;
                const double u = z * w;
                s2 += u * u;
            }
            const R nrm = sqrt(R(s2) * R(1.0 / N));
            mx = (nrm > mx || nrm != nrm) ? nrm : mx;
        }
        nrm0 = g.max(mx);
        return g.max(bad);
    }

    // column solve with the state's iteration matrix, scaled by 2/(1+gamrat),
    // added to the correction V_ACOR; returns the largest WRMS norm of the
    // solutions over the columns (cvSensNorm of the Newton update), so the
    // update itself is never stored
    __device__ R sens_lsolve_update(int v) {
        R mx = R(0);
        const double sc = (gamrat != R(1)) ? double(R(2) / (R(1) + gamrat)) : 1.0;
        for (int c = g.lane; c < ns; c += G) {
            LUT x[N];
            if constexpr (REG) {
                LUT bl[N];
                for (int i = 0; i < N; i++) bl[i] = LUT(SV(v, i, c));
                for (int i = 0; i < N; i++) {
                    LUT acc = LUT(0);
                    for (int j = 0; j < N; j++) acc += Minv[i * N + j] * bl[j];
                    x[i] = acc;
                }
            } else if constexpr (M::SPARSE_LU) {
                // only the structurally nonzero factor entries of the static order:
                // L by columns, U by rows (x_k -= U(k, j) x_j over row k, then / U(k, k))
                for (int i = 0; i < N; i++) x[i] = LUT(SV(v, perm[i], c));
                for (int k = 0; k < N - 1; k++) {
                    const LUT xk = x[k];
                    for (int e = M::lu_rbegin(k); e < M::lu_rend(k); e++) {
                        const int i = M::lu_row(e);
                        x[i] -= Mm[k * N + i] * xk;
                    }
                }
                for (int k = N - 1; k >= 0; k--) {
                    LUT xk = x[k];
                    for (int e = M::lu_cbegin(k); e < M::lu_cend(k); e++) {
                        const int j = M::lu_col(e);
                        xk -= Mm[j * N + k] * x[j];
                    }
                    x[k] = xk * dinv[k];
                }
            } else {
                for (int i = 0; i < N; i++) x[i] = LUT(SV(v, perm[i], c));
                for (int k = 0; k < N - 1; k++) {
                    const LUT xk = x[k];
                    for (int i = k + 1; i < N; i++) x[i] -= Mm[k * N + i] * xk;
                }
                for (int k = N - 1; k >= 0; k--) {
                    x[k] *= dinv[k];
                    const LUT xk = x[k];
                    for (int i = 0; i < k; i++) x[i] -= Mm[k * N + i] * xk;
                }
            }
            double s2 = 0.0;
            for (int i = 0; i < N; i++) {
                const int oi = (M::SPARSE_LU && !REG) ? perm[i] : i;
                const double d = double(x[i]) * sc;
                SV(V_ACOR, oi, c) += d;
                const double t = d * SV(V_EWT, oi, c);
                s2 += t * t;
            }
            const R nrm = sqrt(R(s2) * R(1.0 / N));
            mx = (nrm > mx || nrm != nrm) ? nrm : mx;
        }
        return g.max(mx);
    }

    template <int Q, int SIGN>
    __device__ __forceinline__ void sens_pascal_q() {
        for (int c = g.lane; c < ns; c += G)
            for (int i = 0; i < N; i++) {
                double z[Q + 1];
#pragma unroll
                for (int j = 0; j <= Q; j++) z[j] = SV(j, i, c);
#pragma unroll
                for (int j = 0; j < Q; j++) {
                    double a0 = z[j], a1 = 0.0;
#pragma unroll
                    for (int m = j + 1; m <= Q; m++) {
                        const double cf = ((SIGN < 0) && ((m - j) & 1)) ? -binom(m, j) : binom(m, j);
                        if ((m - j) & 1) a1 = fma(cf, z[m], a1);
                        else a0 = fma(cf, z[m], a0);
                    }
                    SV(j, i, c) = a0 + a1;
                }
            }
    }
    template <int Q> __device__ void sens_predict_q() { sens_pascal_q<Q, 1>(); }
    template <int Q> __device__ void sens_restore_q() { sens_pascal_q<Q, -1>(); }
    template <int Q>
    __device__ void sens_rescale_q() {
        for (int c = g.lane; c < ns; c += G)
            for (int i = 0; i < N; i++) {
                double f = eta;
#pragma unroll
                for (int j = 1; j <= Q; j++) {
                    SV(j, i, c) *= f;
                    f *= eta;
                }
            }
    }
    template <int Q>
    __device__ void sens_complete_q() {
        for (int c = g.lane; c < ns; c += G)
            for (int i = 0; i < N; i++) {
                const double a = SV(V_ACOR, i, c);
#pragma unroll
                for (int j = 0; j <= Q; j++) SV(j, i, c) += ld[j] * a;
            }
    }
    template <int Q>
    __device__ void sens_increase_q() {
        if constexpr (Q < QMAX) {
            for (int c = g.lane; c < ns; c += G)
                for (int i = 0; i < N; i++) {
                    const double zl = incA1 * SV(QMAX, i, c);
                    SV(Q + 1, i, c) = zl;
#pragma unroll
                    for (int j = 2; j <= Q; j++) SV(j, i, c) += double(l[j]) * zl;
                }
        }
    }
    template <int Q>
    __device__ void sens_decrease_q() {
        if constexpr (Q > 2) {
            for (int c = g.lane; c < ns; c += G)
                for (int i = 0; i < N; i++) {
                    const double zq = SV(Q, i, c);
#pragma unroll
                    for (int j = 2; j < Q; j++) SV(j, i, c) += -double(l[j]) * zq;
                }
        }
    }
    __device__ void sens_copy(int vdst, int vsrc) {
        for (int c = g.lane; c < ns; c += G)
            for (int i = 0; i < N; i++) SV(vdst, i, c) = SV(vsrc, i, c);
    }

    // the Newton right-hand side -resS, resS = rl1*znS1 + ycorS - gamma*fS(znS0 +
    // ycorS), into V_TMP (ycorS = V_ACOR), one column at a time; the iterate
    // znS0 + ycorS is stored in V_F once (reading it formed from two vectors
    // at every Jacobian entry measured 15% slower)
    __device__ void stg_residual() {
        const double rl1d = double(rl1);
        for (int c = g.lane; c < ns; c += G) {
            for (int i = 0; i < N; i++) SV(V_F, i, c) = SV(0, i, c) + SV(V_ACOR, i, c);
            sens_rhs_col(c, V_F, V_TMP);
            for (int i = 0; i < N; i++)
                SV(V_TMP, i, c) = -((rl1d * SV(1, i, c) + SV(V_ACOR, i, c)) + (-gamma) * SV(V_TMP, i, c));
        }
    }

    // Del: the norm of the Newton update
    __device__ int stg_convtest(int m, R Del) {  // cvNlsConvTestSensStg (cvodes_nls_stg.c:332)
        if (m > 0) crateS = fmax(R(CRDOWN) * crateS, rdiv(Del, delp));
        const R dcon = rdiv(Del * fmin(R(1), crateS), tq[4]);
        if (dcon <= R(1)) {
            acnrmS = (m == 0) ? Del : sens_norm(V_ACOR);
            return CV_SUCCESS;
        }
        if (m >= 1 && Del > R(RDIV) * delp) return NLS_CONV_RECVR;
        delp = Del;
        return NLS_CONTINUE;
    }

    __device__ int stgr_nls() {
        for (int c = g.lane; c < ns; c += G)
            for (int i = 0; i < N; i++) SV(V_ACOR, i, c) = 0.0;
        int callSetup = 0, jbad = 0, retval;
        for (;;) {
            int curiter = 0;
            stg_residual();
            if (callSetup) {
                if (jbad) convfail = CV_FAIL_BAD_J;
                retval = lsetup();
                crateS = R(1);
                jcur_stg = jcur;
                if (retval != 0) return NLS_CONV_RECVR;
            }
            for (;;) {
                const R Del = sens_lsolve_update(V_TMP);
                retval = stg_convtest(curiter, Del);
                curiter++;
                if (retval == CV_SUCCESS) {
                    jcur = 0;
                    jcur_stg = 0;
                    return CV_SUCCESS;
                }
                if (retval != NLS_CONTINUE) break;
                if (curiter >= o->maxcor) {
                    retval = NLS_CONV_RECVR;
                    break;
                }
                stg_residual();
            }
            if (retval == NLS_CONV_RECVR && !jcur_stg) {
                callSetup = 1;
                jbad = 1;
                for (int c = g.lane; c < ns; c += G)
                    for (int i = 0; i < N; i++) SV(V_ACOR, i, c) = 0.0;
                continue;
            }
            break;
        }
        return retval;
    }

    // ---------------- Newton iteration (cvNls + SUNNonlinSolSolve_Newton) -
    // tmp = rl1*zn1 + acor - gamma*f(zn0 + acor)  (cvNlsResidual)
    __device__ void nls_residual() {
        double yv[S];
#pragma unroll
        for (int s = 0; s < S; s++) yv[s] = zn[0][s] + acor[s];
        store_y(yv);
        rhs_at(tn, ftmp);
        const double rl1d = double(rl1);
#pragma unroll
        for (int s = 0; s < S; s++) tmp[s] = (rl1d * zn[1][s] + acor[s]) + (-gamma) * ftmp[s];
    }

    __device__ int nls_convtest(int m) {  // cvNlsConvTest (cvodes_nls.c:303)
        const R del = wrms(tmp);
        if (m > 0) crate = fmax(R(CRDOWN) * crate, rdiv(del, delp));
        const R dcon = rdiv(del * fmin(R(1), crate), tq[4]);
        if (dcon <= R(1)) {
            acnrm = (m == 0) ? del : wrms(acor);
            return CV_SUCCESS;
        }
        if (m >= 1 && del > R(RDIV) * delp) return NLS_CONV_RECVR;
        delp = del;
        return NLS_CONTINUE;
    }

    __device__ int cv_nls(int nflag) {
        convfail = ((nflag == FIRST_CALL) || (nflag == PREV_ERR_FAIL)) ? CV_NO_FAILURES : CV_FAIL_OTHER;
        int callSetup = force_setup || (nflag == PREV_CONV_FAIL) || (nflag == PREV_ERR_FAIL) || (nst == 0) ||
                        (nst >= nstlp + MSBP) || (fabs(gamrat - R(1)) > R(DGMAX_LSETUP));
#pragma unroll
        for (int s = 0; s < S; s++) acor[s] = 0.0;
        int jbad = 0, retval;
        for (;;) {
            int curiter = 0;
            nls_residual();
            if (callSetup) {
                if (jbad) convfail = CV_FAIL_BAD_J;
                retval = lsetup();
                jcur_nls = jcur;
                if (retval != 0) return NLS_CONV_RECVR;
            }
            for (;;) {
                nni++;
#pragma unroll
                for (int s = 0; s < S; s++) tmp[s] = -tmp[s];
                lsolve(tmp);
#pragma unroll
                for (int s = 0; s < S; s++) acor[s] += tmp[s];
                retval = nls_convtest(curiter);
                curiter++;
                if (retval == CV_SUCCESS) {
                    jcur = 0;
                    jcur_nls = 0;
                    return CV_SUCCESS;
                }
                if (retval != NLS_CONTINUE) break;
                if (curiter >= o->maxcor) {
                    retval = NLS_CONV_RECVR;
                    break;
                }
                nls_residual();
            }
            if (retval == NLS_CONV_RECVR && !jcur_nls) {
                callSetup = 1;
                jbad = 1;
#pragma unroll
                for (int s = 0; s < S; s++) acor[s] = 0.0;
                continue;
            }
            break;
        }
        return retval;
    }

    // ---------------- step control ----------------------------------------
    __device__ int handle_nflag(int* nflag, double saved_t, int* ncf) {  // cvodes.c:7309
        if (*nflag == CV_SUCCESS) return DO_ERROR_TEST;
        ncfn++;
        restore(saved_t);
        (*ncf)++;
        etamax = R(1);
        if (*ncf == o->maxncf) return CV_CONV_FAILURE;
        eta = ETA_CF;
        *nflag = PREV_CONV_FAIL;
        rescale();
        return PREDICT_AGAIN;
    }

    __device__ int do_error_test(int* nflag, double saved_t, int* nef, R* dsmp, R acor_nrm) {  // cvodes.c:7461
        const R dsm = acor_nrm * tq[2];
        *dsmp = dsm;
        if (dsm <= R(1)) return CV_SUCCESS;
        (*nef)++;
        netf++;
        *nflag = PREV_ERR_FAIL;
        restore(saved_t);
        if (*nef == MXNEF) return CV_ERR_FAILURE;
        etamax = R(1);
        if (*nef <= MXNEF1) {
            eta = double(rdiv(R(1), powr(R(BIAS2) * dsm, rdiv(R(1), R(L))) + R(ADDON)));
            eta = fmax(ETA_MIN_EF, eta);
            if (*nef >= SMALL_NEF) eta = fmin(eta, ETA_MAX_EF);
            rescale();
            return TRY_AGAIN;
        }
        if (q > 1) {
            eta = ETA_MIN_EF;
            adjust_order(-1);
            L = q;
            q--;
            qwait = L;
            rescale();
            return TRY_AGAIN;
        }
        eta = ETA_MIN_EF;
        h *= eta;
        hscale = h;
        qwait = LONG_WAIT;
        nscon = 0;
        store_y(zn[0]);
        rhs_at(tn, tmp);
#pragma unroll
        for (int s = 0; s < S; s++) zn[1][s] = h * tmp[s];
        if constexpr (BWD) {  // cvodes.c:7559-7568
            rhsQ_at(tn, 1);
            for (int c = g.lane; c < nq; c += G) QV(1, c) *= h;
        }
        if constexpr (SENS) {
            sens_prepare();
            sens_rhs(0, 1);
            for (int c = g.lane; c < ns; c += G)
                for (int i = 0; i < N; i++) SV(1, i, c) *= h;
        }
        return TRY_AGAIN;
    }

    __device__ void complete_step() {  // cvCompleteStep (cvodes.c:7634)
        nst++;
        nscon++;
#pragma unroll
        for (int i = QMAX; i >= 2; i--)
            if (i <= q) tau[i] = tau[i - 1];
        if (q == 1 && nst > 1) tau[2] = tau[1];
        tau[1] = R(h);
        if constexpr (BWD) {
            hu = h;
            qu = q;
        }
        AGB_DISPATCH_Q(q, complete_q)
        if constexpr (SENS) AGB_DISPATCH_Q(q, sens_complete_q)
        if constexpr (BWD) AGB_DISPATCH_Q(q, quad_complete_q)
        qwait--;
        if (qwait == 1 && q != QMAX) {
#pragma unroll
            for (int s = 0; s < S; s++) zn[QMAX][s] = acor[s];
            if constexpr (SENS) sens_copy(QMAX, V_ACOR);
            if constexpr (BWD) quad_copy(QMAX, QV_ACOR);
            saved_tq5 = tq[5];
        }
    }

    __device__ void set_eta() {  // cvSetEta (cvodes.c:7798)
        if (eta > ETA_MIN_FX && eta < ETA_MAX_FX) {
            eta = 1.0;
            hprime = h;
        } else {
            if (eta >= ETA_MAX_FX) {
                eta = fmin(eta, double(etamax));
                if (!BWD && o->hmax_inv > 0.0) eta /= fmax(1.0, fabs(h) * o->hmax_inv * eta);
            } else {
                eta = fmax(eta, ETA_MIN);
            }
            hprime = h * eta;
            if (qprime < q) nscon = 0;
        }
    }

    __device__ void prepare_next_step(R dsm) {  // cvPrepareNextStep (cvodes.c:7747)
        if (etamax == R(1)) {
            qwait = qwait > 2 ? qwait : 2;
            qprime = q;
            hprime = h;
            eta = 1.0;
            return;
        }
        etaq = rdiv(R(1), powr(R(BIAS2) * dsm, rdiv(R(1), R(L))) + R(ADDON));
        if (qwait != 0) {
            eta = double(etaq);
            qprime = q;
            set_eta();
            return;
        }
        qwait = 2;
        etaqm1 = R(0);  // cvComputeEtaqm1 (cvodes.c:7836)
        if (q > 1) {
            AGB_DISPATCH_Q(q, znq_to_tmp)
            R ddn = wrms(tmp);
            if constexpr (SENS) ddn = fmax(ddn, sens_norm(q));
            if constexpr (BWD)
                if (o->errconQ) ddn = upd_norm(ddn, quad_wrms(q));
            ddn *= tq[1];
            etaqm1 = rdiv(R(1), powr(R(BIAS1) * ddn, rdiv(R(1), R(q))) + R(ADDON));
        }
        etaqp1 = R(0);  // cvComputeEtaqp1 (cvodes.c:7877)
        if (q != QMAX && saved_tq5 != R(0)) {
            const R cquot = rdiv(tq[5], saved_tq5) * powi(rdiv(R(h), tau[2]), L);
            const double cq = double(cquot);
#pragma unroll
            for (int s = 0; s < S; s++) tmp[s] = -cq * zn[QMAX][s] + acor[s];
            R dup = wrms(tmp);
            if constexpr (BWD) {
                if (o->errconQ) {
                    for (int c = g.lane; c < nq; c += G) QV(QV_TMP, c) = -cq * QV(QMAX, c) + QV(QV_ACOR, c);
                    dup = upd_norm(dup, quad_wrms(QV_TMP));
                }
            }
            if constexpr (SENS) {
                for (int c = g.lane; c < ns; c += G)
                    for (int i = 0; i < N; i++) SV(V_TMP, i, c) = -cq * SV(QMAX, i, c) + SV(V_ACOR, i, c);
                dup = fmax(dup, sens_norm(V_TMP));
            }
            dup *= tq[3];
            etaqp1 = rdiv(R(1), powr(R(BIAS3) * dup, rdiv(R(1), R(L + 1))) + R(ADDON));
        }
        const R etam = fmax(etaqm1, fmax(etaq, etaqp1));  // cvChooseEta (cvodes.c:7935)
        if (etam > R(ETA_MIN_FX) && etam < R(ETA_MAX_FX)) {
            eta = 1.0;
            qprime = q;
        } else if (etam == etaq) {
            eta = double(etaq);
            qprime = q;
        } else if (etam == etaqm1) {
            eta = double(etaqm1);
            qprime = q - 1;
        } else {
            eta = double(etaqp1);
            qprime = q + 1;
#pragma unroll
            for (int s = 0; s < S; s++) zn[QMAX][s] = acor[s];
            if constexpr (SENS) sens_copy(QMAX, V_ACOR);
            if constexpr (BWD)
                if (o->errconQ) quad_copy(QMAX, QV_ACOR);
        }
        set_eta();
    }

    // cvBDFStab (cvodes.c:8158-8219): at order q >= 3 push the scaled norms of
    // the derivatives of orders q-1, q and q+1 into the five-step history;
    // after q + 5 steps at constant step size and order, a detected stability
    // limit lowers the next order by one with the step ratio of order q-1
    __device__ void bdf_stab() {
        double* ss = ssd();
        if (q >= 3) {
            // zn[q] and zn[q-1] by selects (one norm loop each, no per-order copies)
            double zq[S], zqm1[S];
#pragma unroll
            for (int s = 0; s < S; s++) {
                zq[s] = q == 3 ? zn[3][s] : (q == 4 ? zn[4][s] : zn[5][s]);
                zqm1[s] = q == 3 ? zn[2][s] : (q == 4 ? zn[3][s] : zn[4][s]);
            }
            const R nrm_q = wrms(zq), nrm_qm1 = wrms(zqm1);
            int fact = 1;
            for (int i = 2; i < q; i++) fact *= i;
            // the scaled norms in the control type (their inputs are), squared in FP64
            const R t5 = tq[5] > R(SLD_TINY) ? tq[5] : R(SLD_TINY);
            const R sq = rdiv(R(fact * q * (q + 1)) * acnrm, t5);
            const R sqm1 = R(fact * q) * nrm_q, sqm2 = R(fact) * nrm_qm1;
            // the history is read only by the detector below, after a group barrier
            if constexpr (G >= 12) {  // entry j moves to j + 3, one entry per lane
                const double v = g.lane < 12 ? ss[g.lane] : 0.0;
                g.sync();
                if (g.lane < 12) ss[g.lane + 3] = v;
                if (g.lane < 3) {
                    const double a = double(g.lane == 0 ? sqm2 : (g.lane == 1 ? sqm1 : sq));
                    ss[g.lane] = a * a;
                }
            } else if (g.lane == 0) {
                for (int j = 14; j >= 3; j--) ss[j] = ss[j - 3];
                const double a = double(sqm2), b = double(sqm1), c = double(sq);
                ss[0] = a * a;
                ss[1] = b * b;
                ss[2] = c * c;
            }
        }
        if (qprime < q) {  // an order decrease is already planned
            nscon = 0;
            return;
        }
        if (q >= 3 && nscon >= q + 5) {
            g.sync();
            int ldflag;
            if constexpr (G >= 16 && sizeof(R) == sizeof(float)) ldflag = sl_detect_mixed<G>(ss, q, g.mask, g.lane);
            else if constexpr (G >= 4) ldflag = sl_detect_group<G>(ss, q, g.mask, g.lane);
            else ldflag = sl_detect(ss, q);
            if (ldflag > 3) {
                qprime = q - 1;
                const double em = double(etaqm1), ex = double(etamax);
                eta = em < ex ? em : ex;
                const double d = fabs(h) * (BWD ? 0.0 : o->hmax_inv) * eta;
                eta = eta / (d > 1.0 ? d : 1.0);
                hprime = h * eta;
            }
        }
    }

    __device__ int cv_step() {  // cvStep (cvodes.c:5800)
        int ncf = 0, nef = 0, ncfS = 0, nefS = 0, nefQ = 0, nflag, kflag, eflag;
        R dsm = R(0);
        if (nst > 0 && hprime != h) adjust_params();
        const double saved_t = tn;
        nflag = FIRST_CALL;
        for (;;) {
            predict();
            cv_set();
            nflag = cv_nls(nflag);
            kflag = handle_nflag(&nflag, saved_t, &ncf);
            if (kflag == PREDICT_AGAIN) continue;
            if (kflag != DO_ERROR_TEST) return kflag;
            eflag = do_error_test(&nflag, saved_t, &nef, &dsm, acnrm);
            if (eflag == TRY_AGAIN) continue;
            if (eflag != CV_SUCCESS) return eflag;
            if constexpr (BWD) {  // cvQuadNls (cvodes.c:7089) and the quadrature error test (:5909-5937)
                ncf = nef = 0;
                double yv[S];
#pragma unroll
                for (int s = 0; s < S; s++) yv[s] = zn[0][s] + acor[s];
                store_y(yv);
                rhsQ_at(tn, QV_ACOR);
                const double rl1d = double(rl1);
                for (int c = g.lane; c < nq; c += G) QV(QV_ACOR, c) = rl1d * (h * QV(QV_ACOR, c) - QV(1, c));
                if (o->errconQ) {
                    R dsmQ = R(0);
                    eflag = do_error_test(&nflag, saved_t, &nefQ, &dsmQ, quad_wrms(QV_ACOR));
                    if (eflag == TRY_AGAIN) continue;
                    if (eflag != CV_SUCCESS) return eflag;
                    if (dsmQ > dsm) dsm = dsmQ;
                }
            }
            if constexpr (SENS) {  // staggered sensitivities (cvodes.c:5938-5990)
                ncf = nef = 0;
                double yv[S];
#pragma unroll
                for (int s = 0; s < S; s++) yv[s] = zn[0][s] + acor[s];
                store_y(yv);
                sens_prepare();
                nflag = stgr_nls();
                kflag = handle_nflag(&nflag, saved_t, &ncfS);
                if (kflag == PREDICT_AGAIN) continue;
                if (kflag != DO_ERROR_TEST) return kflag;
                R dsmS = R(0);
                eflag = do_error_test(&nflag, saved_t, &nefS, &dsmS, acnrmS);
                if (eflag == TRY_AGAIN) continue;
                if (eflag != CV_SUCCESS) return eflag;
                if (dsmS > dsm) dsm = dsmS;
            }
            break;
        }
        complete_step();
        prepare_next_step(dsm);
        if (o->stldet) bdf_stab();
        etamax = (nst <= SMALL_NST) ? R(ETA_MAX_ES) : R(ETA_MAX_GS);
        return CV_SUCCESS;
    }

    // ---------------- initial step (cvHin, cvodes.c:5436-5798), FP64 ------
    __device__ double ydd_norm(double hg) {
        double yv[S];
#pragma unroll
        for (int s = 0; s < S; s++) yv[s] = hg * zn[1][s] + zn[0][s];
        store_y(yv);
        rhs_at(tn + hg, tmp);
#pragma unroll
        for (int s = 0; s < S; s++) tmp[s] = (1.0 / hg) * (tmp[s] - zn[1][s]);
        double s2 = 0.0;
#pragma unroll
        for (int s = 0; s < S; s++) {
            const double t = tmp[s] * double(ewt[s]);
            s2 += t * t;
        }
        double nrm = sqrt(g.sum(s2) / N);
        if constexpr (BWD) {
            if (o->errconQ) {
                rhsQ_at(tn + hg, QV_TMP);
                double q2 = 0.0;
                for (int c = g.lane; c < nq; c += G) {
                    const double t = (1.0 / hg) * (QV(QV_TMP, c) - QV(1, c)) * QV(QV_EWT, c);
                    q2 += t * t;
                }
                const double qn = sqrt(g.sum(q2) / nq);
                nrm = (nrm > qn) ? nrm : qn;
            }
        }
        if constexpr (SENS) {
            sens_prepare();
            for (int c = g.lane; c < ns; c += G)
                for (int i = 0; i < N; i++) SV(V_ACOR, i, c) = hg * SV(1, i, c) + SV(0, i, c);
            sens_rhs(V_ACOR, V_F);
            double mx = 0.0;
            for (int c = g.lane; c < ns; c += G) {
                double s2c = 0.0;
                for (int i = 0; i < N; i++) {
                    const double t = (1.0 / hg) * (SV(V_F, i, c) - SV(1, i, c)) * SV(V_EWT, i, c);
                    s2c += t * t;
                }
                const double nc = sqrt(s2c / N);
                mx = (nc > mx || nc != nc) ? nc : mx;
            }
            mx = g.max(mx);
            nrm = (mx > nrm || mx != mx) ? mx : nrm;
            for (int c = g.lane; c < ns; c += G)
                for (int i = 0; i < N; i++) SV(V_ACOR, i, c) = 0.0;
        }
        return nrm;
    }

    __device__ int cv_hin(double tout) {
        const double tdiff = tout - tn;
        if (tdiff == 0.0) return CV_ILL_INPUT;
        const int sign = tdiff > 0.0 ? 1 : -1;
        const double tdist = fabs(tdiff);
        const double tround = UROUND * fmax(fabs(tn), fabs(tout));
        if (tdist < 2.0 * tround) return CV_ILL_INPUT;
        const double hlb = HLB_FACTOR * tround;
        double hub_inv = 0.0;  // cvUpperBoundH0
#pragma unroll
        for (int s = 0; s < S; s++) {
            if (!own(s)) continue;
            const double t = HUB_FACTOR * fabs(zn[0][s]) + double(rdiv(R(1), ewt[s]));
            hub_inv = fmax(hub_inv, fabs(zn[1][s]) / t);
        }
        if constexpr (SENS) {
            for (int c = g.lane; c < ns; c += G)
                for (int i = 0; i < N; i++) {
                    const double t = HUB_FACTOR * fabs(SV(0, i, c)) + 1.0 / SV(V_EWT, i, c);
                    hub_inv = fmax(hub_inv, fabs(SV(1, i, c)) / t);
                }
        }
        if constexpr (BWD) {  // bound from |yQ|/|yQ'| (cvodes.c:5588-5603)
            if (o->errconQ)
                for (int c = g.lane; c < nq; c += G) {
                    const double t = HUB_FACTOR * fabs(QV(0, c)) + 1.0 / QV(QV_EWT, c);
                    hub_inv = fmax(hub_inv, fabs(QV(1, c)) / t);
                }
        }
        hub_inv = g.max(hub_inv);
        double hub = HUB_FACTOR * tdist;
        if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
        double hg = sqrt(hlb * hub);
        if (hub < hlb) {
            h = sign == -1 ? -hg : hg;
            return CV_SUCCESS;
        }
        double hs = hg, hnew = hg, yddnrm = 0.0;
        for (int count1 = 1; count1 <= MAX_ITERS; count1++) {
            int hgOK = 0;
            for (int count2 = 1; count2 <= MAX_ITERS; count2++) {
                yddnrm = ydd_norm(hg * sign);
                if (isfinite(yddnrm)) {
                    hgOK = 1;
                    break;
                }
                hg *= 0.2;
            }
            if (!hgOK) {
                hnew = hs;
                break;
            }
            hs = hg;
            hnew = (yddnrm * hub * hub > 2.0) ? sqrt(2.0 / yddnrm) : sqrt(hg * hub);
            if (count1 == MAX_ITERS) break;
            const double hrat = hnew / hg;
            if (hrat > 0.5 && hrat < 2.0) break;
            if (count1 > 1 && hrat > 2.0) {
                hnew = hg;
                break;
            }
            hg = hnew;
        }
        double h0 = H_BIAS * hnew;
        if (h0 < hlb) h0 = hlb;
        if (h0 > hub) h0 = hub;
        if (sign == -1) h0 = -h0;
        h = h0;
        return CV_SUCCESS;
    }

    // ---------------- root finding (cvodes.c:8576-9060) --------------------
    // the trigger functions at (t, y) on every lane
    __device__ void gfun(double t, const double (&y)[S], double (&gv)[NRR]) {
        g.sync();
        store_y(y);
        g.sync();
#pragma unroll
        for (int ir = 0; ir < M::NR; ir++) gv[ir] = M::root(ir, t, ys, pu, ku);
    }
    // CVodeGetDky, k = 0: the Nordsieck polynomial at t (terms of order q down to 0)
    __device__ void dky(double t, double (&y)[S]) const {
        const double sv = (t - tn) / h;
#pragma unroll
        for (int s = 0; s < S; s++) {
            double z = 0.0;
            bool first = true;
#pragma unroll
            for (int j = QMAX; j >= 0; j--) {
                if (j > q) continue;
                double v = 1.0;
#pragma unroll
                for (int i = 0; i < j; i++) v *= sv;
                z = first ? v * zn[j][s] : z + v * zn[j][s];
                first = false;
            }
            y[s] = z;
        }
    }
    // the same for the sensitivities, into vector vout
    __device__ void sens_dky(double t, int vout) {
        if constexpr (SENS) {
            const double sv = (t - tn) / h;
            for (int c = g.lane; c < ns; c += G)
                for (int i = 0; i < N; i++) {
                    double z = 0.0;
                    for (int j = q; j >= 0; j--) {
                        double v = 1.0;
                        for (int m = 0; m < j; m++) v *= sv;
                        z = (j == q) ? v * SV(j, i, c) : z + v * SV(j, i, c);
                    }
                    SV(vout, i, c) = z;
                }
        }
    }
    // cvRcheck1: zeros of g at and near the initial point
    __device__ void rcheck1() {
#pragma unroll
        for (int i = 0; i < M::NR; i++) rt_iroots[i] = 0;
        rt_tlo = tn;
        rt_ttol = (fabs(tn) + fabs(h)) * UROUND * 100.0;
        gfun(rt_tlo, zn[0], rt_glo);
        bool zroot = false;
#pragma unroll
        for (int i = 0; i < M::NR; i++)
            if (fabs(rt_glo[i]) == 0.0) {
                zroot = true;
                rt_gactive[i] = 0;
            }
        if (!zroot) return;
        const double hratio = fmax(rt_ttol / fabs(h), 0.1);
        const double tplus = rt_tlo + hratio * h;
        double yv[S];
#pragma unroll
        for (int s = 0; s < S; s++) yv[s] = zn[0][s] + hratio * zn[1][s];
        gfun(tplus, yv, rt_ghi);
#pragma unroll
        for (int i = 0; i < M::NR; i++)
            if (!rt_gactive[i] && fabs(rt_ghi[i]) != 0.0) {
                rt_gactive[i] = 1;
                rt_glo[i] = rt_ghi[i];
            }
    }
    // cvRcheck2: exact zeros at the last root, a close pair, a root just after
    __device__ int rcheck2() {
        if (rt_irfnd == 0) return CV_SUCCESS;
        double yv[S];
        dky(rt_tlo, yv);
        gfun(rt_tlo, yv, rt_glo);
        bool zroot = false;
#pragma unroll
        for (int i = 0; i < M::NR; i++) rt_iroots[i] = 0;
#pragma unroll
        for (int i = 0; i < M::NR; i++)
            if (rt_gactive[i] && fabs(rt_glo[i]) == 0.0) {
                zroot = true;
                rt_iroots[i] = 1;
            }
        if (!zroot) return CV_SUCCESS;
        rt_ttol = (fabs(tn) + fabs(h)) * UROUND * 100.0;
        const double smallh = (h > 0.0) ? rt_ttol : -rt_ttol;
        const double tplus = rt_tlo + smallh;
        if ((tplus - tn) * h >= 0.0) {
            const double hratio = smallh / h;
#pragma unroll
            for (int s = 0; s < S; s++) yv[s] = yv[s] + hratio * zn[1][s];
        } else {
            dky(tplus, yv);
        }
        gfun(tplus, yv, rt_ghi);
        zroot = false;
#pragma unroll
        for (int i = 0; i < M::NR; i++) {
            if (!rt_gactive[i]) continue;
            if (fabs(rt_ghi[i]) == 0.0) {
                if (rt_iroots[i] == 1) return 3;  // CLOSERT
                zroot = true;
                rt_iroots[i] = 1;
            } else if (rt_iroots[i] == 1) {
                rt_glo[i] = rt_ghi[i];
            }
        }
#pragma unroll
        for (int s = 0; s < S; s++) yret[s] = yv[s];
        return zroot ? 1 : CV_SUCCESS;  // RTFOUND
    }
    // cvRootfind: the Illinois algorithm on (tlo, thi); every crossing counts
    __device__ int rootfind() {
        auto diff = [](double a, double b) { return (a < 0.0 && b > 0.0) || (a > 0.0 && b < 0.0); };
        int imax = 0;
        bool zroot = false, sgnchg = false;
        double maxfrac = 0.0;
#pragma unroll
        for (int i = 0; i < M::NR; i++) {
            if (!rt_gactive[i]) continue;
            if (fabs(rt_ghi[i]) == 0.0) {
                zroot = true;
            } else if (diff(rt_glo[i], rt_ghi[i])) {
                const double gfrac = fabs(rt_ghi[i] / (rt_ghi[i] - rt_glo[i]));
                if (gfrac > maxfrac) {
                    sgnchg = true;
                    maxfrac = gfrac;
                    imax = i;
                }
            }
        }
        if (!sgnchg) {
            rt_trout = rt_thi;
#pragma unroll
            for (int i = 0; i < M::NR; i++) rt_grout[i] = rt_ghi[i];
            if (!zroot) return CV_SUCCESS;
#pragma unroll
            for (int i = 0; i < M::NR; i++) {
                rt_iroots[i] = 0;
                if (rt_gactive[i] && fabs(rt_ghi[i]) == 0.0) rt_iroots[i] = rt_glo[i] > 0 ? -1 : 1;
            }
            return 1;
        }
        double alph = 1.0;
        int side = 0, sideprev = -1;
        for (int iter = 0; iter < 10000; iter++) {  // the interval shrinks every pass; a bound all the same
            if (fabs(rt_thi - rt_tlo) <= rt_ttol) break;
            if (sideprev == side) alph = (side == 2) ? alph * 2.0 : alph * 0.5;
            else alph = 1.0;
            double ghim = 0.0, glom = 0.0;
#pragma unroll
            for (int i = 0; i < M::NR; i++)
                if (i == imax) {
                    ghim = rt_ghi[i];
                    glom = rt_glo[i];
                }
            double tmid = rt_thi - (rt_thi - rt_tlo) * ghim / (ghim - alph * glom);
            if (fabs(tmid - rt_tlo) < 0.5 * rt_ttol) {
                const double fracint = fabs(rt_thi - rt_tlo) / rt_ttol;
                const double fracsub = (fracint > 5.0) ? 0.1 : 0.5 / fracint;
                tmid = rt_tlo + fracsub * (rt_thi - rt_tlo);
            }
            if (fabs(rt_thi - tmid) < 0.5 * rt_ttol) {
                const double fracint = fabs(rt_thi - rt_tlo) / rt_ttol;
                const double fracsub = (fracint > 5.0) ? 0.1 : 0.5 / fracint;
                tmid = rt_thi - fracsub * (rt_thi - rt_tlo);
            }
            double yv[S];
            dky(tmid, yv);
            gfun(tmid, yv, rt_grout);
            maxfrac = 0.0;
            zroot = sgnchg = false;
            sideprev = side;
#pragma unroll
            for (int i = 0; i < M::NR; i++) {
                if (!rt_gactive[i]) continue;
                if (fabs(rt_grout[i]) == 0.0) {
                    zroot = true;
                } else if (diff(rt_glo[i], rt_grout[i])) {
                    const double gfrac = fabs(rt_grout[i] / (rt_grout[i] - rt_glo[i]));
                    if (gfrac > maxfrac) {
                        sgnchg = true;
                        maxfrac = gfrac;
                        imax = i;
                    }
                }
            }
            if (sgnchg) {
                rt_thi = tmid;
#pragma unroll
                for (int i = 0; i < M::NR; i++) rt_ghi[i] = rt_grout[i];
                side = 1;
                if (fabs(rt_thi - rt_tlo) <= rt_ttol) break;
                continue;
            }
            if (zroot) {
                rt_thi = tmid;
#pragma unroll
                for (int i = 0; i < M::NR; i++) rt_ghi[i] = rt_grout[i];
                break;
            }
            rt_tlo = tmid;
#pragma unroll
            for (int i = 0; i < M::NR; i++) rt_glo[i] = rt_grout[i];
            side = 2;
            if (fabs(rt_thi - rt_tlo) <= rt_ttol) break;
        }
        rt_trout = rt_thi;
#pragma unroll
        for (int i = 0; i < M::NR; i++) {
            rt_grout[i] = rt_ghi[i];
            rt_iroots[i] = 0;
            if (!rt_gactive[i]) continue;
            if (fabs(rt_ghi[i]) == 0.0) rt_iroots[i] = rt_glo[i] > 0 ? -1 : 1;
            if (diff(rt_glo[i], rt_ghi[i])) rt_iroots[i] = rt_glo[i] > 0 ? -1 : 1;
        }
        return 1;
    }
    // cvRcheck3: a root between tlo and tn (or tout); the state at it in yret
    __device__ int rcheck3() {
        double yv[S];
        if (rt_taskc == 1 || (rt_toutc - tn) * h >= 0.0) {
            rt_thi = tn;
#pragma unroll
            for (int s = 0; s < S; s++) yv[s] = zn[0][s];
        } else {
            rt_thi = rt_toutc;
            dky(rt_thi, yv);
        }
        gfun(rt_thi, yv, rt_ghi);
        rt_ttol = (fabs(tn) + fabs(h)) * UROUND * 100.0;
        const int ier = rootfind();
#pragma unroll
        for (int i = 0; i < M::NR; i++)
            if (!rt_gactive[i] && rt_grout[i] != 0.0) rt_gactive[i] = 1;
        rt_tlo = rt_trout;
#pragma unroll
        for (int i = 0; i < M::NR; i++) rt_glo[i] = rt_grout[i];
        if (ier == CV_SUCCESS) return CV_SUCCESS;
        dky(rt_trout, yret);
        return 1;
    }

    // CVode's first-call block with the stop time tout (cvInitialSetup, with
    // cvLsInitialize's counter reset, cvodes_ls.c:1567; cvHin; the first step
    // bounded by hmax and the stop time; zn[1] = h f)
    __device__ int first_call(double tout) {
        if (ewt_set()) return CV_ILL_INPUT;
        if constexpr (SENS)
            if (sens_ewt_set()) return CV_ILL_INPUT;
        nstlj = 0;
        store_y(zn[0]);
        rhs_at(tn, zn[1]);
        if constexpr (SENS) {
            sens_prepare();
            sens_rhs(0, 1);
        }
        if (cv_hin(tout) != CV_SUCCESS) return CV_ILL_INPUT;
        const double rh = fabs(h) * o->hmax_inv;
        if (rh > 1.0) h /= rh;
        if ((tn + h - tstop) * h > 0.0) h = (tstop - tn) * (1.0 - 4.0 * UROUND);
        hscale = h;
        hprime = h;
#pragma unroll
        for (int s = 0; s < S; s++) zn[1][s] *= h;
        if constexpr (SENS)
            for (int c = g.lane; c < ns; c += G)
                for (int i = 0; i < N; i++) SV(1, i, c) *= h;
        return CV_SUCCESS;
    }

    // CVode(tout, NORMAL) with tstop = tout, as AMICI calls it (cvodes.c:2890).
    // After an event the call starts with CVodeSolver::reInit_post_process
    // (solver_cvodes.cpp:531-583): with the step counter at 0, one step in
    // ONE_STEP mode with the stop time tout, the integrator set up as on its
    // first call; the counter then continues, and any failure of that step (a
    // stop time reached included) is a CvodeException, AMICI_ERROR.  The
    // post-process step runs through the same loop as the others, so the step
    // code is emitted once.
    __device__ int cv_solve(double tout, int64_t mxstep) {
        bool post = force_reinit != 0;
        int nst_tmp = 0;
        if (post) {
            nst_tmp = nst;
            nst = 0;
        } else {
            called = 1;
        }
        tstop = tout;
        tstopset = 1;
        rt_toutc = tout;
        rt_taskc = post ? 1 : 0;
        if (nst == 0) {
            tretlast = tn;
            const int f = first_call(tout);
            if (f != CV_SUCCESS) return post ? -99 : f;
            if constexpr (M::NR > 0) rcheck1();
        } else {
            const double troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
            if constexpr (M::NR > 0) {  // the root checks on entry (cvodes.c:3216-3275)
                int r = rcheck2();
                if (r == 3) return CV_ILL_INPUT;
                if (r == 1) {
                    tretlast = rt_tlo;
                    return CV_ROOT_RETURN;
                }
                if (fabs(tn - tretlast) > troundoff) {
                    r = rcheck3();
                    if (r == CV_SUCCESS) {
                        rt_irfnd = 0;
                    } else if (r == 1) {
                        rt_irfnd = 1;
                        tretlast = rt_tlo;
                        return CV_ROOT_RETURN;
                    }
                }
            }
            if (fabs(tn - tstop) <= troundoff) {
                tretlast = tstop;
                return CV_TSTOP_RETURN;
            }
            if ((tn + hprime - tstop) * h > 0.0) {
                hprime = (tstop - tn) * (1.0 - 4.0 * UROUND);
                eta = hprime / h;
            }
        }
        int64_t nstloc = 0;
        for (;;) {
            if (ck_buf && !post && nst == ck_next) {  // check point before step nst + 1 (cvodea.c:395-600)
                save_state(ck_buf + (size_t)(nst / ck_k) * CK_STRIDE);
                ck_n = nst / ck_k + 1;
                ck_next += ck_k;
                force_setup = 1;
            }
            if (nst > 0 && ewt_set()) return CV_ILL_INPUT;
            R nrmS = R(0);
            if constexpr (SENS) {
                if (nst > 0) {
                    if (sens_ewt_set_norm0(nrmS)) return CV_ILL_INPUT;
                } else {
                    nrmS = sens_norm(0);
                }
            }
            if (mxstep > 0 && nstloc >= mxstep) return CV_TOO_MUCH_WORK;
            R nrm0 = wrms(zn[0]);
            if constexpr (SENS) nrm0 = fmax(nrm0, nrmS);
            if (nrm0 > R(1.0 / UROUND)) return post ? -99 : CV_TOO_MUCH_ACC;  // UROUND * nrm0 > 1
            const int kflag = cv_step();
            if (kflag != CV_SUCCESS) return post ? -99 : kflag;
            nstloc++;
            double troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
            if (fabs(tn - tstop) <= troundoff) tn = tstop;
            if constexpr (M::NR > 0) {  // a root in the step just taken (cvodes.c:3516-3530)
                if (rcheck3() == 1) {
                    rt_irfnd = 1;
                    tretlast = rt_tlo;
                    return post ? -99 : CV_ROOT_RETURN;
                }
            }
            if (st_t && !post && !store_point(tn, q)) return CV_TOO_MUCH_WORK;
            troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
            if (fabs(tn - tstop) <= troundoff) {
                tstopset = 0;
                tretlast = tstop;
                return post ? -99 : CV_TSTOP_RETURN;
            }
            if ((tn + hprime - tstop) * h > 0.0) {
                hprime = (tstop - tn) * (1.0 - 4.0 * UROUND);
                eta = hprime / h;
            }
            if (post) {  // end of reInit_post_process; CVode(tout, NORMAL) continues
                nst = nst_tmp + 1;
                force_reinit = 0;
                post = false;
                called = 1;
                nstloc = 0;
                tretlast = tn;
                rt_taskc = 0;
                if constexpr (M::NR > 0) {  // the NORMAL call's root checks on entry
                    int r = rcheck2();
                    if (r == 3) return CV_ILL_INPUT;
                    if (r == 1) {
                        tretlast = rt_tlo;
                        return CV_ROOT_RETURN;
                    }
                }
            }
        }
    }

    // CVode(tout, ONE_STEP) without a stop time, as Solver::step runs it for the
    // simulation to steady state (solver.cpp:162-178): the first call sets the
    // integrator up as cv_solve does; every call takes one step
    __device__ int cv_one_step(double tout) {
        tstopset = 0;
        if (nst == 0) {
            if (ewt_set()) return CV_ILL_INPUT;
            if constexpr (SENS)
                if (sens_ewt_set()) return CV_ILL_INPUT;
            store_y(zn[0]);
            rhs_at(tn, zn[1]);
            if constexpr (SENS) {
                sens_prepare();
                sens_rhs(0, 1);
            }
            if (cv_hin(tout) != CV_SUCCESS) return CV_ILL_INPUT;
            const double rh = fabs(h) * o->hmax_inv;
            if (rh > 1.0) h /= rh;
            hscale = h;
            hprime = h;
#pragma unroll
            for (int s = 0; s < S; s++) zn[1][s] *= h;
            if constexpr (SENS)
                for (int c = g.lane; c < ns; c += G)
                    for (int i = 0; i < N; i++) SV(1, i, c) *= h;
        } else {
            if (ewt_set()) return CV_ILL_INPUT;
            if constexpr (SENS)
                if (sens_ewt_set()) return CV_ILL_INPUT;
        }
        R nrm0 = wrms(zn[0]);
        if constexpr (SENS) nrm0 = fmax(nrm0, sens_norm(0));
        if (nrm0 > R(1.0 / UROUND)) return CV_TOO_MUCH_ACC;  // UROUND * nrm0 > 1
        return cv_step();
    }

    // ---------------- pre-equilibration: simulation to steady state ---------
    // SteadyStateProblem with the reference's default settings (computation
    // mode integrationOnly, model.h:2296; no Newton steps, solver.h:2043):
    // from the initial state at the fixed parameters of the pre-equilibration
    // (b.k of this launch), one step at a time towards tout = max(t, 1) * 10
    // (EventHandlingSimulator::run_steady_state, forwardproblem.cpp:153-230)
    // until, checked before every step, the WRMS norm of xdot with weights
    // 1/(rtol_ss |x| + atol_ss) is below 1 and, with sensitivities, so is that
    // of every sensitivity's right-hand side J sx_c + df/dp_c with weights from
    // |sx_c| (steadystateproblem.cpp:29-52; forwardproblem.cpp:989-1092); the
    // steady-state tolerances are 100 x the solver's (solver.h:2081,2090).
    // Writes the steady state, its sensitivities w.r.t. the scaled parameters,
    // the status (1 success, -2 step budget exhausted or too much work, -5
    // time overflow, -1 any other failure), the steps, the time and the norm.
    __device__ void run_preeq(const Batch& b, int inst) {
        begin_instance(b, inst);
        int steps = 0;
        double w = INFINITY;
        const int st = ss_simulate(steps, w);
        if (g.lane == 0) {
            b.preeq_status[inst] = st;
            b.preeq_numsteps[inst] = steps;
            b.preeq_t[inst] = tn;
            b.preeq_wrms[inst] = w;
        }
#pragma unroll
        for (int s = 0; s < S; s++)
            if (own(s)) b.x_ss[(size_t)inst * N + idx(s)] = zn[0][s];
        if constexpr (SENS) {
            if (b.sx_ss)
                for (int c = g.lane; c < ns; c += G) {
                    const double fac = scale_factor(b.pscale, pu, plist[c]);
                    for (int i = 0; i < N; i++) b.sx_ss[((size_t)inst * ns + c) * N + i] = SV(0, i, c) * fac;
                }
        }
        g.sync();
    }

    // the simulation to steady state from the current state at tn (the
    // pre-equilibration's fresh solver, or the main solver continued for the
    // post-equilibration): returns the SteadyStateStatus of the stage, the
    // steps taken and the last norm
    __device__ int ss_simulate(int& steps, double& w) {
        const double atol_ss = o->atol * 100.0, rtol_ss = o->rtol * 100.0;
        int st = 1;
        steps = 0;
        w = INFINITY;
        for (;;) {
            store_y(zn[0]);
            rhs(ftmp);
            double s2 = 0.0;
#pragma unroll
            for (int s = 0; s < S; s++) {
                if (!own(s)) continue;
                const double t = ftmp[s] * (1.0 / (rtol_ss * fabs(zn[0][s]) + atol_ss));
                s2 += t * t;
            }
            w = sqrt(g.sum(s2) / N);
            bool converged = w < 1.0;
            if constexpr (SENS) {
                if (converged) {
                    sens_prepare();
                    sens_rhs(0, V_TMP);
                    double mx = 0.0;
                    for (int c = g.lane; c < ns; c += G) {
                        double s2c = 0.0;
                        for (int i = 0; i < N; i++) {
                            const double t = SV(V_TMP, i, c) * (1.0 / (rtol_ss * fabs(SV(0, i, c)) + atol_ss));
                            s2c += t * t;
                        }
                        const double wc = sqrt(s2c / N);
                        mx = (wc > mx || wc != wc) ? wc : mx;
                    }
                    converged = g.max(mx) < 1.0;
                }
            }
            if (converged) break;
            if (steps >= o->maxsteps) {
                st = -2;
                break;
            }
            steps++;
            const double tout = (tn > 1.0 ? tn : 1.0) * 10.0;
            if (!isfinite(tout)) {
                st = -5;
                break;
            }
            const int flag = cv_one_step(tout);
            if (flag < 0) {
                st = flag == CV_TOO_MUCH_WORK ? -2 : -1;
                break;
            }
        }
        return st;
    }

    // ---------------- integrator state (check points, backward resume) -----
    // Everything the next step reads besides the shared-memory Jacobian and
    // iteration matrix (refreshed after a restart): the Nordsieck history
    // (lane-strided after CK_NSCAL scalars) and the step/order/setup state.
    static constexpr long long CK_STRIDE = ck_stride_of<M>();
    __device__ void save_state(double* buf) {
#pragma unroll
        for (int s = 0; s < S; s++)
            if (own(s))
#pragma unroll
                for (int j = 0; j < LMAX; j++) buf[CK_NSCAL + (size_t)j * N + idx(s)] = zn[j][s];
        if (g.lane == 0) {
            double* d = buf;
            int c = 0;
            d[c++] = tn; d[c++] = h; d[c++] = hprime; d[c++] = hscale; d[c++] = tstop; d[c++] = eta;
            d[c++] = double(etamax); d[c++] = double(crate); d[c++] = double(gammap); d[c++] = double(gamrat);
            d[c++] = double(saved_tq5); d[c++] = double(acnrm); d[c++] = double(delp);
#pragma unroll
            for (int j = 0; j <= LMAX; j++) d[c++] = double(tau[j]);
#pragma unroll
            for (int j = 0; j < 6; j++) d[c++] = double(tq[j]);
            d[c++] = q; d[c++] = qprime; d[c++] = qwait; d[c++] = L; d[c++] = jcur; d[c++] = jcur_nls;
            d[c++] = tstopset; d[c++] = nst; d[c++] = nstlp; d[c++] = nstlj;
            d[c++] = nfe; d[c++] = nni; d[c++] = nsetups; d[c++] = netf; d[c++] = ncfn; d[c++] = nje;
            d[c++] = it_cur; d[c++] = tcur_cur; d[c++] = incA1;
            d[c++] = nscon; d[c++] = double(etaqm1);
            const double* ss = ssd();
#pragma unroll
            for (int j = 0; j < 15; j++) d[c++] = ss[j];
            if constexpr (BWD) {
                d[c++] = hu; d[c++] = qu; d[c++] = tretlast;
            }
        }
        g.sync();
    }
    __device__ void load_state(const double* buf) {
        g.sync();
#pragma unroll
        for (int s = 0; s < S; s++)
#pragma unroll
            for (int j = 0; j < LMAX; j++) zn[j][s] = own(s) ? buf[CK_NSCAL + (size_t)j * N + idx(s)] : 0.0;
        const double* d = buf;
        int c = 0;
        tn = d[c++]; h = d[c++]; hprime = d[c++]; hscale = d[c++]; tstop = d[c++]; eta = d[c++];
        etamax = R(d[c++]); crate = R(d[c++]); gammap = R(d[c++]); gamrat = R(d[c++]);
        saved_tq5 = R(d[c++]); acnrm = R(d[c++]); delp = R(d[c++]);
#pragma unroll
        for (int j = 0; j <= LMAX; j++) tau[j] = R(d[c++]);
#pragma unroll
        for (int j = 0; j < 6; j++) tq[j] = R(d[c++]);
        q = int(d[c++]); qprime = int(d[c++]); qwait = int(d[c++]); L = int(d[c++]); jcur = int(d[c++]);
        jcur_nls = int(d[c++]); tstopset = int(d[c++]); nst = int(d[c++]); nstlp = int(d[c++]); nstlj = int(d[c++]);
        nfe = int(d[c++]); nni = int(d[c++]); nsetups = int(d[c++]); netf = int(d[c++]); ncfn = int(d[c++]);
        nje = int(d[c++]); it_cur = int(d[c++]); tcur_cur = d[c++]; incA1 = d[c++];
        nscon = int(d[c++]); etaqm1 = R(d[c++]);
        for (int j = g.lane; j < 15; j += G) ssd()[j] = d[c + j];
        c += 15;
        if constexpr (BWD) {
            hu = d[c++]; qu = int(d[c++]); tretlast = d[c++];
        }
        force_setup = 1;
        g.sync();
    }

    // ---------------- adjoint storage of the forward run --------------------
    // CVodeF stores the time, zn[0] and the order of every accepted step
    // (cvodea.c:560-575, CVApolynomialStorePnt :3236); false if full
    __device__ bool store_point(double t, int order) {
        if (st_n >= st_cap) return false;
        if (g.lane == 0) {
            st_t[st_n] = t;
            st_q[st_n] = double(order);
        }
        double* yo = st_y + (size_t)st_n * N;
#pragma unroll
        for (int s = 0; s < S; s++)
            if (own(s)) yo[idx(s)] = zn[0][s];
        st_n++;
        return true;
    }

    // ---------------- backward problem: CVode(tout, itask) -----------------
    // CVodeGetDky / CVodeGetQuadDky with k = 0 (cvodes.c:3742,3864): sum of
    // s^j zn[j] from j = q down to 0
    __device__ void get_dky(double t, double (&out)[S]) {
        const double sg = (t - tn) / h;
        double cj[LMAX];
#pragma unroll
        for (int j = 0; j <= QMAX; j++) {
            double v = 1.0;
#pragma unroll
            for (int i = 0; i < j; i++) v *= sg;
            cj[j] = v;
        }
#pragma unroll
        for (int s = 0; s < S; s++) {
            double z = 0.0;
            bool first = true;
#pragma unroll
            for (int j = QMAX; j >= 0; j--)
                if (j <= q) {
                    z = first ? cj[j] * zn[j][s] : z + cj[j] * zn[j][s];
                    first = false;
                }
            out[s] = z;
        }
    }
    __device__ void get_quad_dky(double t, int dst) {
        const double sg = (t - tn) / h;
        for (int c = g.lane; c < nq; c += G) {
            double z = 0.0;
            for (int j = q; j >= 0; j--) {
                double v = 1.0;
                for (int i = 0; i < j; i++) v *= sg;
                z = (j == q) ? v * QV(j, c) : z + v * QV(j, c);
            }
            QV(dst, c) = z;
        }
    }

    // CVode (cvodes.c:2890-3640) without sensitivities, with quadratures and a
    // stop time: NORMAL mode to tout (CVodeB with the stop time at the check
    // point) or ONE_STEP (the step after a reinitialisation).  yout gets
    // y(tout) (NORMAL, interpolated) or zn[0] (ONE_STEP, stop time, failure).
    __device__ int bwd_ode(double tout, bool one_step, int64_t mxstep, double (&yout)[S]) {
        if (nst == 0) {
            tretlast = tn;
            // cvInitialSetup, incl. cvLsInitialize's counter reset (cvodes_ls.c:1567,1980)
            if (ewt_set()) return CV_ILL_INPUT;
            if (o->errconQ && quad_ewt_set()) return CV_ILL_INPUT;
            nstlj = 0;
            store_y(zn[0]);
            rhs_at(tn, zn[1]);
            rhsQ_at(tn, 1);
            if (tstopset && (tstop - tn) * (tout - tn) <= 0.0) return CV_ILL_INPUT;
            double tout_hin = tout;
            if (tstopset && (tout - tn) * (tout - tstop) > 0.0) tout_hin = tstop;
            if (cv_hin(tout_hin) != CV_SUCCESS) return CV_ILL_INPUT;
            if (tstopset && (tn + h - tstop) * h > 0.0) h = (tstop - tn) * (1.0 - 4.0 * UROUND);
            hscale = h;
            hprime = h;
#pragma unroll
            for (int s = 0; s < S; s++) zn[1][s] *= h;
            for (int c = g.lane; c < nq; c += G) QV(1, c) *= h;
        } else {
            const double troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
            if (tstopset) {
                if (fabs(tn - tstop) <= troundoff) {
                    if ((tout - tstop) * h >= 0.0 || fabs(tout - tstop) <= troundoff) {
#pragma unroll
                        for (int s = 0; s < S; s++) yout[s] = zn[0][s];
                        tretlast = tstop;
                        tstopset = 0;
                        return CV_TSTOP_RETURN;
                    }
                } else if ((tn + hprime - tstop) * h > 0.0) {
                    hprime = (tstop - tn) * (1.0 - 4.0 * UROUND);
                    eta = hprime / h;
                }
            }
            if (!one_step && (tn - tout) * h >= 0.0) {
                tretlast = tout;
                get_dky(tout, yout);
                return CV_SUCCESS;
            }
            if (one_step && fabs(tn - tretlast) > troundoff) {
                tretlast = tn;
#pragma unroll
                for (int s = 0; s < S; s++) yout[s] = zn[0][s];
                return CV_SUCCESS;
            }
        }
        int64_t nstloc = 0;
        int flag = CV_SUCCESS;
        for (;;) {
            if (nst > 0) {
                if (ewt_set() || (o->errconQ && quad_ewt_set())) {
                    flag = CV_ILL_INPUT;
                    break;
                }
            }
            if (mxstep > 0 && nstloc >= mxstep) {
                flag = CV_TOO_MUCH_WORK;
                break;
            }
            R nrm0 = wrms(zn[0]);
            if (o->errconQ) nrm0 = upd_norm(nrm0, quad_wrms(0));
            if (nrm0 > R(1.0 / UROUND)) {  // UROUND * nrm0 > 1
                flag = CV_TOO_MUCH_ACC;
                break;
            }
            const int kflag = cv_step();
            if (kflag != CV_SUCCESS) {
                flag = kflag;
                break;
            }
            nstloc++;
            if (tstopset) {
                const double troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
                if (fabs(tn - tstop) <= troundoff) tn = tstop;
            }
            if (tstopset) {
                const double troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
                if (fabs(tn - tstop) <= troundoff) {
                    if ((tout - tstop) * h >= 0.0 || fabs(tout - tstop) <= troundoff) {
#pragma unroll
                        for (int s = 0; s < S; s++) yout[s] = zn[0][s];
                        tretlast = tstop;
                        tstopset = 0;
                        return CV_TSTOP_RETURN;
                    }
                } else if ((tn + hprime - tstop) * h > 0.0) {
                    hprime = (tstop - tn) * (1.0 - 4.0 * UROUND);
                    eta = hprime / h;
                }
            }
            if (!one_step && (tn - tout) * h >= 0.0) {
                tretlast = tout;
                get_dky(tout, yout);
                return CV_SUCCESS;
            }
            if (one_step) {
                tretlast = tn;
#pragma unroll
                for (int s = 0; s < S; s++) yout[s] = zn[0][s];
                return CV_SUCCESS;
            }
        }
        tretlast = tn;
#pragma unroll
        for (int s = 0; s < S; s++) yout[s] = zn[0][s];
        return flag;
    }

    // CVodeInit / CVodeReInit state of a fresh integrator at t0 with y0 (cvodes.c:800-835)
    __device__ void init_state(double t0) {
        q = 1;
        L = 2;
        qwait = L;
        qprime = 1;
        etamax = R(ETA_MAX_FS);
        tn = t0;
        h = hprime = hscale = tstop = 0.0;
        eta = 1.0;
#pragma unroll
        for (int j = 0; j <= LMAX; j++) tau[j] = R(0);
#pragma unroll
        for (int j = 0; j < LMAX; j++) l[j] = R(0), ld[j] = 0.0;
#pragma unroll
        for (int j = 0; j < 6; j++) tq[j] = R(0);
        gamma = 0.0;
        rl1 = gammap = gamrat = R(0);
        crate = delp = acnrm = saved_tq5 = etaqm1 = etaq = etaqp1 = R(0);
        convfail = jcur = jcur_nls = tstopset = 0;
        nst = nstlp = nstlj = 0;
        nfe = nni = nsetups = netf = ncfn = nje = 0;
        incA1 = 0.0;
        clear_stab();
        if constexpr (BWD) {
            hu = 0.0;
            qu = 0;
            tretlast = t0;
        }
    }

    // ---------------- forward replay of one check-point segment -------------
    // From a restored check point, the steps up to nst == nst_end again, with
    // the stop-time logic of run_instance/cv_solve (after a step reaches the
    // stop time, the next output that needs integration becomes the stop
    // time), storing (t, y, y') of the segment's first point and of every
    // step as CVAhermiteStorePnt does (y' = zn[1]/h, cvodea.c:2839).  The
    // check point restores the same state and refreshes the iteration matrix
    // at the same step as the original run, so the replay retraces it.
    // Returns the number of stored points, or a negative CVODES flag.
    __device__ long long replay_segment(const Batch& b, int inst, int nst_end, double* qt, double* qy, double* qyd) {
        const double t0 = 0.0;
        const int nt = b.nt;
        const double* tsi = b.ts + (size_t)inst * nt;
        long long np = 0;
        auto store = [&]() {
            if (g.lane == 0) qt[np] = tn;
            const double hi = 1.0 / h;
#pragma unroll
            for (int s = 0; s < S; s++)
                if (own(s)) {
                    qy[(size_t)np * N + idx(s)] = zn[0][s];
                    qyd[(size_t)np * N + idx(s)] = hi * zn[1][s];
                }
            np++;
        };
        store();
        int it = it_cur;
        double tcur = tcur_cur;
        while (nst < nst_end) {
            if (ewt_set()) return CV_ILL_INPUT;
            const int kflag = cv_step();
            if (kflag != CV_SUCCESS) return kflag;
            double troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
            if (fabs(tn - tstop) <= troundoff) tn = tstop;
            store();
            troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
            if (fabs(tn - tstop) <= troundoff) {
                tstopset = 0;
                tcur = tstop;
                for (;;) {  // the next output that needs integration (run_instance's loop)
                    it++;
                    if (it >= nt) break;
                    const double tout = tsi[it];
                    if (!(tout > t0) || !(tcur < tout)) continue;
                    const double tdiff = tout - tcur;
                    if (tdiff == 0.0 || fabs(tdiff) < 2.0 * UROUND * fmax(fabs(tcur), fabs(tout))) continue;
                    tstop = tout;  // cv_solve(tout) entry
                    tstopset = 1;
                    const double tr = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
                    if (fabs(tn - tstop) <= tr) {
                        tcur = tout;
                        continue;
                    }
                    if ((tn + hprime - tstop) * h > 0.0) {
                        hprime = (tstop - tn) * (1.0 - 4.0 * UROUND);
                        eta = hprime / h;
                    }
                    break;
                }
                if (it >= nt) break;
            } else if ((tn + hprime - tstop) * h > 0.0) {
                hprime = (tstop - tn) * (1.0 - 4.0 * UROUND);
                eta = hprime / h;
            }
        }
        return np;
    }

    // reload the per-lane flux coefficients of a forward integrator that
    // restarts from a check point (the shared-memory p, k and c are intact)
    __device__ void reload_coeffs() {
        if constexpr (FREG) {
#pragma unroll
            for (int m = 0; m < FM; m++) {
                const int r = m * G + g.lane;
                fcr[m] = r < NW ? M::flux_coeff(r, pu, ku) : 0.0;
            }
        }
    }

    // ---------------- backward problem over check-point segments -----------
    // The loop of run_backward as a resumable machine: resume_backward runs
    // the backward problem within the current segment [seg_t0, ...] and
    // returns 1 when it needs the segment before (CVodeB moving to the
    // previous check point, cvodea.c:1500-1620), 0 when done.  Its loop state
    // (output index, time, flags, the adjoint value xB) is kept in ctl and
    // yB between calls, the integrator state by save_state.
    static constexpr int BC_JT = 0, BC_T = 1, BC_CALLED = 2, BC_FORCE = 3, BC_INRUN = 4, BC_POST = 5,
                         BC_TNEXT = 6, BC_STATUS = 7, BC_N = 8;
    __device__ void begin_backward(const Batch& b, int inst, const double* dj, double* ctl, double* yBs) {
        const int nt = b.nt;
        const double* tsi = b.ts + (size_t)inst * nt;
        double t = tsi[nt - 1] > 0.0 ? tsi[nt - 1] : 0.0;
        int jt = nt - 1;
        const bool jump0 = jt >= 0 && tsi[jt] == t;
        init_state(t);
#pragma unroll
        for (int s = 0; s < S; s++) {
            double v = 0.0;
            if (jump0 && own(s)) v += dj[(size_t)jt * N + idx(s)];
            zn[0][s] = v;
            if (own(s)) yBs[idx(s)] = v;
#pragma unroll
            for (int j = 1; j < LMAX; j++) zn[j][s] = 0.0;
        }
        if (jump0) jt--;
        for (int c = g.lane; c < nq; c += G)
            for (int v = 0; v < QV_N; v++) QV(v, c) = 0.0;
        if (g.lane == 0) {
            ctl[BC_JT] = jt;
            ctl[BC_T] = t;
            ctl[BC_CALLED] = 0;
            ctl[BC_FORCE] = 0;
            ctl[BC_INRUN] = 0;
            ctl[BC_POST] = 0;
            ctl[BC_TNEXT] = 0.0;
            ctl[BC_STATUS] = 0;
        }
        g.sync();
    }

    __device__ int resume_backward(const Batch& b, int inst, const double* dj, double* ctl, double* yBs,
                                   double seg_t0, bool has_prev) {
        const int nt = b.nt;
        const double* tsi = b.ts + (size_t)inst * nt;
        for (int d = g.lane; d < M::ND; d += G) dcs[d] = M::dcoeff(d, pu, ku);
        g.sync();
        int jt = int(ctl[BC_JT]);
        double t = ctl[BC_T];
        bool called = ctl[BC_CALLED] != 0.0, force_reinit = ctl[BC_FORCE] != 0.0;
        bool in_run = ctl[BC_INRUN] != 0.0, post = ctl[BC_POST] != 0.0;
        double tnext = ctl[BC_TNEXT];
        int status = int(ctl[BC_STATUS]);
        double yB[S];
#pragma unroll
        for (int s = 0; s < S; s++) yB[s] = own(s) ? yBs[idx(s)] : 0.0;
        int need_prev = 0;
        const int64_t maxstepsB = o->maxstepsB;
        for (;;) {
            if (!in_run) {
                const bool at_data = jt >= 0;
                if (!at_data && !(t > 0.0)) break;
                tnext = at_data ? tsi[jt] : 0.0;
                if (tnext < t) {
                    if (maxstepsB - nst <= 0) {
                        status = -99;
                        break;
                    }
                    in_run = true;
                    post = force_reinit;
                } else {
                    // output at the current time: jump and reinitialise
#pragma unroll
                    for (int s = 0; s < S; s++)
                        if (own(s)) yB[s] += dj[(size_t)jt * N + idx(s)];
                    jt--;
                    if (called) force_reinit = true;
                    tn = t;
                    q = 1;
                    L = 2;
                    qwait = L;
                    qu = 0;
                    hu = 0.0;
#pragma unroll
                    for (int s = 0; s < S; s++) zn[0][s] = yB[s];
                    quad_copy(0, QV_Y);
                    g.sync();
                    continue;
                }
            }
            // a run towards tnext inside the current segment
            const double tr = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
            if (has_prev && tn - seg_t0 <= tr) {
                need_prev = 1;
                break;
            }
            const int64_t rem = maxstepsB - nst;
            if (rem <= 0) {
                status = -99;
                break;
            }
            // one call site for the solver (keeps the integrator in registers):
            // after a reinit, reInit_post_process's single step with the stop
            // time at the next output (kept inside the segment); else CVodeB's
            // NORMAL-mode call with the stop time at the segment's check point
            const bool is_post = post;
            const int nst_tmp = nst;
            if (is_post) nst = 0;
            tstop = is_post ? fmax(tnext, seg_t0) : seg_t0;
            tstopset = 1;
            const int f = bwd_ode(is_post ? tstop : tnext, is_post, rem, yB);
            if (is_post) {
                if (f != CV_SUCCESS) {
                    status = -99;  // a CvodeException of reInit_post_process: AMICI_ERROR
                    break;
                }
                nst = nst_tmp + 1;
                post = false;
                force_reinit = false;
                continue;
            }
            called = true;
            if (f < 0) {
                status = f;
                break;
            }
            if (f == CV_TSTOP_RETURN && fabs(tnext - seg_t0) > FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h))) {
                continue;  // reached the segment start before tnext: the previous segment next
            }
            // passed tnext: CVodeGetB / CVodeGetQuadB
            if (nst == 0) quad_copy(QV_Y, 0);
            else get_quad_dky(tretlast, QV_Y);
            t = tnext;
            in_run = false;
            if (jt < 0) break;  // reached t0
#pragma unroll
            for (int s = 0; s < S; s++)
                if (own(s)) yB[s] += dj[(size_t)jt * N + idx(s)];
            jt--;
            if (called) force_reinit = true;
            tn = t;
            q = 1;
            L = 2;
            qwait = L;
            qu = 0;
            hu = 0.0;
#pragma unroll
            for (int s = 0; s < S; s++) zn[0][s] = yB[s];
            quad_copy(0, QV_Y);
            g.sync();
        }
        g.sync();
#pragma unroll
        for (int s = 0; s < S; s++)
            if (own(s)) yBs[idx(s)] = yB[s];
        if (g.lane == 0) {
            ctl[BC_JT] = jt;
            ctl[BC_T] = t;
            ctl[BC_CALLED] = called;
            ctl[BC_FORCE] = force_reinit;
            ctl[BC_INRUN] = in_run;
            ctl[BC_POST] = post;
            ctl[BC_TNEXT] = tnext;
            ctl[BC_STATUS] = status;
        }
        g.sync();
        return need_prev;
    }

    // sllh = -(xB(t0) . sx0 + xQB) with the chain rule, from the stored xB
    __device__ void write_gradient(const Batch& b, int inst, const double* yBs, int status) {
        if (!b.sllh) return;
        for (int i = g.lane; i < N; i += G) ys[i] = yBs[i];
        g.sync();
        for (int c = g.lane; c < nq; c += G) {
            const int pj = plist[c];
            const double fac = scale_factor(b.pscale, pu, pj);
            b.sllh[(size_t)inst * nq + c] =
                status ? NAN : (direct_terms(b, inst, c) - (sx0_dot(b, inst, c, ys) + QV(QV_Y, c))) * fac;
        }
        g.sync();
    }

    // the objective's direct parameter dependence accumulated by the forward run
    __device__ double direct_terms(const Batch& b, int inst, int c) const {
        if constexpr (M::HAS_DYDP || M::HAS_DSIGMA) return b.sllh[(size_t)inst * nq + c];
        return 0.0;
    }

    // x . sx0 of column c (parameter plist[c]), sx0 w.r.t. the unscaled
    // parameter: dx0/dp, or the given initial sensitivities (ExpData sx0 or a
    // pre-equilibration's steady state, w.r.t. the scaled parameter)
    __device__ double sx0_dot(const Batch& b, int inst, int c, const double* x) const {
        const int pj = plist[c];
        double s0 = 0.0;
        if (b.sx0) {
            const double* s = b.sx0 + ((size_t)inst * nq + c) * N;
            const double rf = 1.0 / scale_factor(b.pscale, pu, pj);
            for (int i = 0; i < N; i++) s0 = fma(x[i], s[i] * rf, s0);
        } else {
            for (int i = 0; i < N; i++) s0 = fma(x[i], M::dx0dp(i, pj, pu, ku), s0);
        }
        return s0;
    }

    // ---------------- backward problem of one instance ---------------------
    // EventHandlingBwdSimulator::run (backwardproblem.cpp:267-332) for an ODE
    // without events: xB jumps by dJy/dx at every output, after each jump the
    // solver is reinitialised the way CVodeSolver::reinit_b/reset_state and
    // reInit_post_process do it (solver_cvodes.cpp:470-560,618-648); then the
    // gradient (rdata.cpp:514-629,749-968).  npts forward steps are stored in
    // the group's scratch; returns the status (0 or a CVODES flag).
    __device__ int run_backward(const Batch& b, int inst, double* scr, long long npts_fwd, int* nst_b_out) {
        const int nt = b.nt;
        const AdjLayout lay{b.adj_cap, nt, N, nqp};
        pt_t = scr + lay.t_off();
        pt_q = scr + lay.q_off();
        pt_y = scr + lay.y_off();
        const double* dj = scr + lay.dj_off();
        qb = scr + lay.qv_off();
        npts = npts_fwd;
        newdata = 1;
        dd_base = -1;
        dd_order = -1;
        t_interp = NAN;
        const double* tsi = b.ts + (size_t)inst * nt;
        for (int d = g.lane; d < M::ND; d += G) dcs[d] = M::dcoeff(d, pu, ku);
        g.sync();
        const int64_t maxstepsB = o->maxstepsB;
        double yB[S];
        // Solver::setup_b at the final time with xB = 0 and xQB = 0
        double t = tsi[nt - 1] > 0.0 ? tsi[nt - 1] : 0.0;
        int jt = nt - 1;
#pragma unroll
        for (int s = 0; s < S; s++) {
            yB[s] = 0.0;
            if (jt >= 0 && tsi[jt] == t && own(s)) yB[s] += dj[(size_t)jt * N + idx(s)];
        }
        if (jt >= 0 && tsi[jt] == t) jt--;
        init_state(t);
#pragma unroll
        for (int s = 0; s < S; s++) {
            zn[0][s] = yB[s];
#pragma unroll
            for (int j = 1; j < LMAX; j++) zn[j][s] = 0.0;
            acor[s] = tmp[s] = ftmp[s] = 0.0;
            ewt[s] = R(0);
        }
        for (int c = g.lane; c < nq; c += G)
            for (int v = 0; v < QV_N; v++) QV(v, c) = 0.0;
        g.sync();
        bool called = false, force_reinit = false;
        int status = 0;
        // targets: every output below the final time (with its jump), then t0;
        // one call site for the solver keeps the inlined step code single
        for (;;) {
            const bool at_data = jt >= 0;
            if (!at_data && !(t > 0.0)) break;
            const double tnext = at_data ? tsi[jt] : 0.0;
            if (tnext < t) {
                // Solver::run_b: the step budget, then (after a reinit) one step as
                // if it were the first (reInit_post_process), then CVodeB in
                // NORMAL mode with the stop time at the single check point t0
                const int64_t rem = maxstepsB - nst;
                if (rem <= 0) {
                    status = -99;
                    break;
                }
                int nst_tmp = nst;
                for (int pass = force_reinit ? 0 : 1; pass < 2; pass++) {
                    const bool post = (pass == 0);
                    if (post) {
                        nst_tmp = nst;
                        nst = 0;
                    }
                    tstop = post ? tnext : 0.0;
                    tstopset = 1;
                    const int f = bwd_ode(tnext, post, rem, yB);
                    if (post) {
                        if (f != CV_SUCCESS) {
                            status = -99;  // a CvodeException of reInit_post_process: AMICI_ERROR
                            break;
                        }
                        nst = nst_tmp + 1;
                        force_reinit = false;
                    } else {
                        called = true;
                        if (f < 0) status = f;
                    }
                }
                if (status) break;
                // write_solution_b: CVodeGetB (yB) and CVodeGetQuadB into QV(QV_Y)
                if (nst == 0) quad_copy(QV_Y, 0);
                else get_quad_dky(tretlast, QV_Y);
                t = tnext;
            }
            if (!at_data) break;
#pragma unroll
            for (int s = 0; s < S; s++)
                if (own(s)) yB[s] += dj[(size_t)jt * N + idx(s)];
            jt--;
            // reinit_b + reset_state + reinit_quad_b
            if (called) force_reinit = true;
            tn = t;
            q = 1;
            L = 2;
            qwait = L;
            qu = 0;
            hu = 0.0;
#pragma unroll
            for (int s = 0; s < S; s++) zn[0][s] = yB[s];
            quad_copy(0, QV_Y);
            g.sync();
        }
        g.sync();
        if (nst_b_out) *nst_b_out = nst;
        // sllh = -(xB(t0) . sx0 + xQB) with the chain rule to the parameter scale
        if (b.sllh) {
            store_y(yB);
            for (int c = g.lane; c < nq; c += G) {
                const double fac = scale_factor(b.pscale, pu, plist[c]);
                b.sllh[(size_t)inst * nq + c] =
                    status ? NAN : (direct_terms(b, inst, c) - (sx0_dot(b, inst, c, ys) + QV(QV_Y, c))) * fac;
            }
        }
        g.sync();
        return status;
    }

    // Model::froot of event ie at (t, ys): its trigger function, or
    // direction * (t - te) for an explicit trigger time
    __device__ double root_value(int ie, double t) const {
        if constexpr (M::NE > 0) {
            const int ir = M::event_root(ie);
            if (ir >= 0) return M::root(ir, t, ys, pu, ku);
            return double(M::event_direction(ie)) * (t - M::event_time(ie, pu, ku));
        }
        return 0.0;
    }

    // the per-instance flux coefficients from p and k (with the Heaviside
    // indicators); with sens also their parameter derivatives
    __device__ void refresh_coefficients(bool sens) {
        for (int ci = g.lane; ci < M::NC; ci += G) cs[ci] = M::flux_coeff(ci, pu, ku);
        if constexpr (FREG) {
#pragma unroll
            for (int m = 0; m < FM; m++) {
                const int r = m * G + g.lane;
                fcr[m] = r < NW ? M::flux_coeff(r, pu, ku) : 0.0;
            }
        }
        if constexpr (SENS)
            if (sens)
                for (int d = g.lane; d < M::ND; d += G) dcs[d] = M::dcoeff(d, pu, ku);
        g.sync();
    }
    // Model::update_heaviside (model.cpp:1588-1592): h_j += roots_found of its
    // event, then the coefficients that contain it
    __device__ void update_heaviside(const int* found) {
        if constexpr (M::NH > 0) {
            g.sync();
            if (g.lane == 0)
                for (int j = 0; j < M::NH; j++) ku[M::NK + j] += double(found[M::heaviside_event(j)]);
            g.sync();
            refresh_coefficients(true);
        }
    }

    // ---------------- one instance: parameters, initial state, integrator ----
    // ParameterScaling, coefficients, x0 (or the given initial state) and,
    // with sensitivities, sx0 (dx0/dp or the given one, w.r.t. the unscaled
    // parameters), then the CVodeInit defaults (cvodes.c:800-835)
    __device__ void begin_instance(const Batch& b, int inst) {
        const double* pin = b.p + (size_t)inst * M::NP;
        for (int j = g.lane; j < M::NP; j += G) {  // ParameterScaling
            const double v = pin[j];
            const int sc = b.pscale ? b.pscale[j] : 0;
            pu[j] = sc == 1 ? exp(v) : (sc == 2 ? exp10(v) : v);
        }
        for (int j = g.lane; j < M::NK; j += G) ku[j] = b.k[(size_t)inst * M::NK + j];
        for (int j = g.lane; j < M::NH; j += G) ku[M::NK + j] = 0.0;
        g.sync();
        refresh_coefficients(false);
#pragma unroll
        for (int s = 0; s < S; s++) {
            zn[0][s] = own(s) ? (b.x0 ? b.x0[(size_t)inst * N + idx(s)] : M::x0(idx(s), pu, ku)) : 0.0;
#pragma unroll
            for (int j = 1; j < LMAX; j++) zn[j][s] = 0.0;
            acor[s] = tmp[s] = ftmp[s] = 0.0;
            ewt[s] = R(0);
        }
        if constexpr (M::NH > 0) {
            // Model::initialize_events (model.cpp:407-440): indicator h_j is 1
            // where the trigger of its event is not negative at t0
            store_y(zn[0]);
            g.sync();
            if (g.lane == 0)
                for (int j = 0; j < M::NH; j++) ku[M::NK + j] = root_value(M::heaviside_event(j), 0.0) < 0.0 ? 0.0 : 1.0;
            g.sync();
            refresh_coefficients(false);
        }
        if constexpr (SENS) {
            ns = b.nplist;
            plist = b.plist;
            for (int d = g.lane; d < M::ND; d += G) dcs[d] = M::dcoeff(d, pu, ku);
            for (int c = g.lane; c < ns; c += G) {
                const double rf = b.sx0 ? 1.0 / scale_factor(b.pscale, pu, plist[c]) : 0.0;
                for (int i = 0; i < N; i++) {
                    SV(0, i, c) = b.sx0 ? b.sx0[((size_t)inst * ns + c) * N + i] * rf : M::dx0dp(i, plist[c], pu, ku);
                    for (int v = 1; v <= V_F; v++) SV(v, i, c) = 0.0;
                }
            }
            crateS = acnrmS = R(0);
            jcur_stg = 0;
            incA1 = 0.0;
        }
        g.sync();
        if (st_t) {  // CVodeF's first call stores the initial point with order 0
            st_n = 0;
            store_point(0.0, 0);
        }
        // CVodeInit defaults (cvodes.c:800-835)
        q = 1;
        L = 2;
        qwait = L;
        qprime = 1;
        etamax = R(ETA_MAX_FS);
        tn = 0.0;
        h = hprime = hscale = tstop = 0.0;
        eta = 1.0;
#pragma unroll
        for (int j = 0; j <= LMAX; j++) tau[j] = R(0);
#pragma unroll
        for (int j = 0; j < LMAX; j++) l[j] = R(0), ld[j] = 0.0;
#pragma unroll
        for (int j = 0; j < 6; j++) tq[j] = R(0);
        gamma = 0.0;
        rl1 = gammap = gamrat = R(0);
        crate = delp = acnrm = saved_tq5 = etaqm1 = etaq = etaqp1 = R(0);
        convfail = jcur = jcur_nls = tstopset = 0;
        nst = nstlp = nstlj = 0;
        nfe = nni = nsetups = netf = ncfn = nje = 0;
        clear_stab();
    }

    // ---------------- one instance through AMICI's output loop -------------
    // ---------------- events ----------------------------------------------
    // EventHandlingSimulator::run (forwardproblem.cpp:53-151): the trigger
    // times te(p, k) of the events with explicit trigger times within
    // (t0, last output] are stop times beside the outputs
    // (Model::get_trigger_timepoints, model.cpp:444-470); the next one after
    // the last handled.  Events with trigger functions: the solver's root
    // finding returns at a zero crossing (CV_ROOT_RETURN).
    __device__ double next_event_time(double after, double tlast) const {
        double best = INFINITY;
        for (int ie = 0; ie < M::NE; ie++) {
            if (M::event_root(ie) >= 0) continue;
            const double te = M::event_time(ie, pu, ku);
            if (te > after && te <= tlast && te < best) best = te;
        }
        return best;
    }

    // bounds of the event queue at one time (AMICI's is unbounded; the oracle
    // stops at the same bounds): EV_QUEUE * NE events, EV_PENDING * NE waiting
    static constexpr int NEE = M::NE > 0 ? M::NE : 1;
    static constexpr int EV_QUEUE = 64, EV_PENDING = 4;

    // get_event_time_sensitivity (model.cpp:1464-1479; de_model.py "stau"):
    // for a trigger function stau = sroot / drootdt_total with sroot = dg/dx sx
    // + dg/dp and drootdt_total = dg/dt + dg/dx xdot; for an explicit trigger
    // t - te, stau = -dte/dp.  ys holds x, fo xdot, SV(0) the sensitivities.
    __device__ void event_time_sensitivity(int ie, double t, const double* fo, double (&stau)[SENS ? NPS : 1]) {
        if constexpr (SENS) {
            const int ir = M::event_root(ie);
            int m = 0;
            if (ir < 0) {
                for (int c = g.lane; c < ns; c += G, m++) stau[m] = -M::devent_time_dp(ie, plist[c], pu, ku);
                return;
            }
            const double dt = M::root_dt(ir, t, ys, pu, ku) + M::root_dx_dot(ir, t, ys, pu, ku, fo, 1);
            for (int c = g.lane; c < ns; c += G, m++) {
                const double sr = M::root_dp(ir, plist[c], t, ys, pu, ku) + M::root_dx_dot(ir, t, ys, pu, ku, &SV(0, 0, c), nsp);
                stau[m] = dt != 0.0 ? sr / dt : 0.0;
            }
        }
    }

    // handle_events (forwardproblem.cpp:388-516) at time t with roots_found
    // in found (1: the event fires); the state in zn[0], the sensitivities in
    // SV(0).  store_pre_event_info (forwardproblem.cpp:404-426, 573-604): the
    // trigger functions' values, xdot before the events and, with
    // sensitivities, the event-time sensitivity of the last firing event.
    // Then the queue of firing events in index order (the queue of events
    // without priorities keeps it, event.h:163-212): each adds its bolus
    // (model.cpp:1481-1503) and, with sensitivities, the sensitivities' bolus
    // deltasx = (xdot - xdot_old) stau + ddeltax/dp + ddeltax/dx
    // (sx - xdot_old stau) (model.cpp:1505-1534); after each,
    // detect_secondary_events (forwardproblem.cpp:605-660): an event that did
    // not fire and whose Heaviside value changed fires when its trigger rose
    // (queued; the pre-event values are taken again) and is marked -1 when it
    // fell; the events that fired are cleared.  An event at the time of the
    // last one is "stuck in an event" (AmiException, AMICI_ERROR -99).  Then
    // the solver is reinitialised at t as CVodeSolver::reinit and reset_state
    // do (solver_cvodes.cpp:471-505,586-616): order 1, the next solve starts
    // with reInit_post_process's step.
    // initial: the events at t0 (Model::initialize_events, model.cpp:407-440),
    // event-time sensitivity zero, the solver not yet started.
    __device__ int handle_events(double t, int (&found)[NEE], bool initial) {
        if (!initial && t == tlastroot) return -99;
        tlastroot = t;
        store_y(zn[0]);
        g.sync();
        double rtmp[NRR];
#pragma unroll
        for (int ir = 0; ir < M::NR; ir++) rtmp[ir] = M::root(ir, t, ys, pu, ku);
        double* fo = nullptr;
        double* fn = nullptr;
        double stau[SENS ? NPS : 1];
        if constexpr (SENS && M::NE > 0) {
            fo = ys + LY::ev_off;
            fn = fo + N;
            double f[S];
            rhs(f);
#pragma unroll
            for (int s = 0; s < S; s++)
                if (own(s)) fo[idx(s)] = f[s];
            g.sync();
            for (int m = 0; m < NPS; m++) stau[m] = 0.0;
            if (!initial)
                for (int ie = 0; ie < M::NE; ie++)
                    if (found[ie] == 1) event_time_sensitivity(ie, t, fo, stau);
        }
        if (!initial) update_heaviside(found);
        int queue[EV_PENDING * NEE];
        int nq = 0, head = 0;
        for (int ie = 0; ie < M::NE; ie++)
            if (found[ie] == 1) queue[nq++ % (EV_PENDING * NEE)] = ie;
        while (head < nq) {
            const int ie = queue[head++ % (EV_PENDING * NEE)];
            double xn[S];
#pragma unroll
            for (int s = 0; s < S; s++) xn[s] = own(s) ? zn[0][s] + M::deltax(ie, idx(s), ys, pu, ku) : 0.0;
            g.sync();  // every lane has read the state before the bolus
#pragma unroll
            for (int s = 0; s < S; s++) zn[0][s] = xn[s];
            store_y(zn[0]);
            g.sync();
            if constexpr (SENS && M::NE > 0) {
                double f[S];
                rhs(f);
#pragma unroll
                for (int s = 0; s < S; s++)
                    if (own(s)) fn[idx(s)] = f[s];
                g.sync();
                int m = 0;
                for (int c = g.lane; c < ns; c += G, m++) {
                    const int pj = plist[c];
                    const double st = stau[m];
                    for (int i = 0; i < N; i++) {
                        double d = fma(fn[i] - fo[i], st, M::ddeltaxdp(ie, i, pj, ys, pu, ku));
                        d += M::ddeltaxdx_times(ie, i, &SV(0, 0, c), nsp) - st * M::ddeltaxdx_times(ie, i, fo, 1);
                        SV(V_TMP, i, c) = d;
                    }
                    for (int i = 0; i < N; i++) SV(0, i, c) += SV(V_TMP, i, c);
                }
                g.sync();
            }
            if (nq + M::NE > EV_QUEUE * M::NE || nq - head + M::NE > EV_PENDING * M::NE) break;
            // detect_secondary_events (an explicit trigger t - te does not
            // change with a bolus, so it gives no secondary event)
            int second = 0;
            for (int je = 0; je < M::NE; je++) {
                const int ir = M::event_root(je);
                if (found[je] == 0 && ir >= 0) {
                    double a = 0.0, bv = 0.0;
#pragma unroll
                    for (int jr = 0; jr < M::NR; jr++)
                        if (jr == ir) a = rtmp[jr];
                    bv = M::root(ir, t, ys, pu, ku);
                    if ((a < 0.0 && bv >= 0.0) || (a >= 0.0 && bv < 0.0)) {  // heaviside_differs, misc.h:280
                        if (a < bv) {
                            found[je] = 1;
                            queue[nq++ % (EV_PENDING * NEE)] = je;
                        } else {
                            found[je] = -1;
                        }
                        second++;
                    } else {
                        found[je] = 0;
                    }
                } else {
                    found[je] = 0;
                }
            }
            if (second) {  // store_pre_event_info again, without a new event-time sensitivity
#pragma unroll
                for (int ir = 0; ir < M::NR; ir++) rtmp[ir] = M::root(ir, t, ys, pu, ku);
                if constexpr (SENS && M::NE > 0) {  // xdot_old: xdot after the last bolus
                    double* sw = fo;
                    fo = fn;
                    fn = sw;
                }
                update_heaviside(found);
            }
        }
        tn = t;
        if (called) force_reinit = 1;
        q = 1;
        L = 2;
        qwait = L;
        qu = 0;
        hu = 0.0;
        return 0;
    }

    // POSTEQ: outputs at t = inf come from the post-equilibration
    // (ForwardProblem::handle_postequilibration, forwardproblem.cpp:376-387):
    // the main solver continues from the last finite output in ONE_STEP mode
    // to steady state (SteadyStateProblem::run with is_preeq false keeps the
    // solver, forwardproblem.cpp:862-900,1009-1105); those outputs carry no
    // step count (Solver::store_diagnosis runs at the finite outputs only),
    // and a failed post-equilibration is AMICI_ERROR with every output kept
    // (rdata.cpp:288-313,336-347)
    template <bool POSTEQ = false>
    __device__ int run_instance(const Batch& b, int inst) {
        const int ny = M::NY;
        const int nt = b.nt;
        begin_instance(b, inst);
        if constexpr (M::HAS_DYDP || M::HAS_DSIGMA) {
            // the adjoint gradient's direct objective terms accumulate in sllh
            if (st_dj && b.sllh)
                for (int c = g.lane; c < b.nplist; c += G) b.sllh[(size_t)inst * b.nplist + c] = 0.0;
        }

        const double t0 = 0.0;
        const double* tsi = b.ts + (size_t)inst * nt;
        const double* myi = b.my ? b.my + (size_t)inst * nt * ny : nullptr;
        const double* sgi = b.sigma_y ? b.sigma_y + (size_t)inst * nt * ny : nullptr;
        double llh_part = 0.0;
        double sllh_part[SENS ? NPS : 1];
        for (int m = 0; m < (SENS ? NPS : 1); m++) sllh_part[m] = 0.0;
        int status = 0, it;
        double tcur = t0;
        double t_ev = t0;  // the last explicit trigger time handled
        const double tlast = nt > 0 ? tsi[nt - 1] : t0;
        (void)t_ev;
        (void)tlast;
        // an instance whose pre-equilibration failed is not simulated
        const bool no_steady_state = b.preeq_in && b.preeq_in[inst] != 1;
        int found[NEE];
        tlastroot = t0;
        // handle_initial_events (forwardproblem.cpp:518-525): an event fires at
        // t0 whose root value there is not negative while its trigger's
        // initial value is false
        if constexpr (M::NE > 0) {
            if (!no_steady_state) {
                store_y(zn[0]);
                g.sync();
                bool any = false;
                for (int ie = 0; ie < M::NE; ie++) {
                    const double rv = root_value(ie, t0);
                    found[ie] = (!(rv < 0.0) && !M::event_initial_value(ie)) ? 1 : 0;
                    any |= found[ie] != 0;
                }
                g.sync();
                if (any) handle_events(t0, found, true);
            }
        }
        int pe_status = 0;
        for (it = no_steady_state ? nt : 0; it < nt; it++) {
            const double tout = tsi[it];
            if (POSTEQ && isinf(tout)) {
                if constexpr (POSTEQ) {
                    if (pe_status == 0) {
                        int steps = 0;
                        double w = INFINITY;
                        pe_status = ss_simulate(steps, w);
                        if (g.lane == 0) {
                            if (b.posteq_status) b.posteq_status[inst] = pe_status;
                            if (b.posteq_numsteps) b.posteq_numsteps[inst] = steps;
                            if (b.posteq_t) b.posteq_t[inst] = pe_status == 1 ? tn : NAN;
                            if (b.posteq_wrms) b.posteq_wrms[inst] = w;
                        }
                    }
                }
            } else if (tout > t0) {
                while (tcur < tout) {
                    const double tdiff = tout - tcur;  // is_next_t_too_close (forwardproblem.cpp:26)
                    if (tdiff == 0.0 || fabs(tdiff) < 2.0 * UROUND * fmax(fabs(tcur), fabs(tout))) break;
                    // the next stop: the output or the next trigger time
                    double tev = INFINITY;
                    if constexpr (M::NE > 0) tev = next_event_time(t_ev, tlast);
                    const double tnext = tout < tev ? tout : tev;
                    const int64_t remaining = o->maxsteps - nst;
                    if (remaining <= 0) {
                        status = -99;
                        break;
                    }
                    it_cur = it;
                    tcur_cur = tcur;
                    const int flag = cv_solve(tnext, remaining);
                    if (flag < 0) {
                        status = flag;
                        break;
                    }
                    // CV_TSTOP_RETURN reports tret = tstop (cvodes.c:3300-3306), a
                    // root return the root
                    tcur = (flag == CV_TSTOP_RETURN) ? tnext : (flag == CV_ROOT_RETURN ? tretlast : tn);
                    if constexpr (M::NE > 0) {
                        if (flag == CV_ROOT_RETURN || tcur == tev) {
                            // roots_found: CVodeGetRootInfo for the trigger functions; for
                            // an explicit trigger time reached, copysign(1, -root value at
                            // the last event), the root value direction * (t_prev - te)
                            // having the sign of -direction
                            for (int ie = 0; ie < M::NE; ie++) {
                                const int ir = M::event_root(ie);
                                int fv = 0;
                                if (ir >= 0 && flag == CV_ROOT_RETURN) {
#pragma unroll
                                    for (int jr = 0; jr < M::NR; jr++)
                                        if (jr == ir) fv = rt_iroots[jr];
                                } else if (ir < 0 && tcur == tev && M::event_time(ie, pu, ku) == tcur) {
                                    fv = M::event_direction(ie);  // the sign of -(root value before)
                                }
                                found[ie] = fv;
                            }
                            if (flag == CV_ROOT_RETURN) {
                                // the state the root return gives (yout) and the
                                // sensitivities at the root (CVodeGetSensDky at
                                // tretlast, cvodes.c:4018)
#pragma unroll
                                for (int s = 0; s < S; s++) zn[0][s] = yret[s];
                                if (tretlast != tn) {
                                    g.sync();
                                    sens_dky(tretlast, 0);
                                    g.sync();
                                }
                            }
                            if (tcur == tev) t_ev = tcur;
                            if (handle_events(tcur, found, false) != 0) {
                                status = -99;
                                break;
                            }
                        }
                    }
                }
                if (status != 0) break;
            }
            // outputs at this time point (ReturnData::get_data_output)
            store_y(zn[0]);
            if (b.x) {
                double* xo = b.x + ((size_t)inst * nt + it) * N;
#pragma unroll
                for (int s = 0; s < S; s++)
                    if (own(s)) xo[idx(s)] = zn[0][s];
            }
            for (int iy = g.lane; iy < ny; iy += G) {
                const double yv = M::observable(iy, ys, pu, ku);
                double sg = M::sigma(iy, pu, ku);
                if (sgi && !isnan(sgi[(size_t)it * ny + iy])) sg = sgi[(size_t)it * ny + iy];
                const size_t oi = ((size_t)inst * nt + it) * ny + iy;
                if (b.y) b.y[oi] = yv;
                if (b.sigmay) b.sigmay[oi] = sg;
                if (myi) {
                    const double mv = myi[(size_t)it * ny + iy];
                    if (!isnan(mv)) {
                        double djdy, djds;
                        llh_part -= noise_jy(M::noise(iy), yv, mv, sg, djdy, djds);
                    }
                }
            }
            if (st_dj) {
                // dJy/dx at this output for the adjoint jumps (forwardproblem.cpp:675-701:
                // dJy/dy times dy/dx), and the objective's direct parameter
                // dependence dJy/dy dy/dp + dJy/dsigma dsigma/dp, which the
                // gradient takes as it is (rdata.cpp:387-395, model.cpp:1241-1251)
                double rr[M::NY > 0 ? M::NY : 1], rs[M::NY > 0 ? M::NY : 1];
#pragma unroll
                for (int iy = 0; iy < ny; iy++) {
                    rr[iy] = rs[iy] = 0.0;
                    if (myi) {
                        const double mv = myi[(size_t)it * ny + iy];
                        if (!isnan(mv)) {
                            double sg = M::sigma(iy, pu, ku);
                            const bool data_sigma = sgi && !isnan(sgi[(size_t)it * ny + iy]);
                            if (data_sigma) sg = sgi[(size_t)it * ny + iy];
                            noise_jy(M::noise(iy), M::observable(iy, ys, pu, ku), mv, sg, rr[iy], rs[iy]);
                            if (data_sigma) rs[iy] = 0.0;  // a noise scale from the data is a constant
                        }
                    }
                }
#pragma unroll
                for (int s = 0; s < S; s++) {
                    if (!own(s)) continue;
                    double acc = 0.0;
#pragma unroll
                    for (int iy = 0; iy < ny; iy++)
                        for (int e = M::obs_begin(iy); e < M::obs_end(iy); e++)
                            if (M::obs_state(e) == idx(s)) acc = fma(rr[iy], M::obs_dydx(e, ys, pu, ku), acc);
                    st_dj[(size_t)it * N + idx(s)] = acc;
                }
                if constexpr (M::HAS_DYDP || M::HAS_DSIGMA) {
                    if (b.sllh)
                        for (int c = g.lane; c < b.nplist; c += G) {
                            const int pj = b.plist[c];
                            double acc = 0.0;
                            for (int iy = 0; iy < ny; iy++) {
                                if constexpr (M::HAS_DYDP) acc = fma(rr[iy], M::obs_dydp(iy, pj, ys, pu, ku), acc);
                                if constexpr (M::HAS_DSIGMA) acc = fma(rs[iy], M::dsigma_dp(iy, pj, pu, ku), acc);
                            }
                            b.sllh[(size_t)inst * b.nplist + c] -= acc;
                        }
                }
            }
            if constexpr (SENS) {
                // sx, sy (ReturnData::get_data_sensis_fsa) and sllh, chain rule
                // to the parameter scale (rdata.cpp:749-968); lane-own columns
                int m = 0;
                for (int c = g.lane; c < ns; c += G, m++) {
                    const int pj = plist[c];
                    const int scl = b.pscale ? b.pscale[pj] : 0;
                    const double fac = scl == 1 ? pu[pj] : (scl == 2 ? pu[pj] * 2.302585092994046 : 1.0);
                    if (b.sx)
                        for (int i = 0; i < N; i++)
                            b.sx[(((size_t)inst * nt + it) * ns + c) * N + i] = SV(0, i, c) * fac;
                    for (int iy = 0; iy < ny; iy++) {
                        double sy = 0.0;
                        for (int e = M::obs_begin(iy); e < M::obs_end(iy); e++)
                            sy = fma(M::obs_dydx(e, ys, pu, ku), SV(0, M::obs_state(e), c), sy);
                        if constexpr (M::HAS_DYDP) sy += M::obs_dydp(iy, pj, ys, pu, ku);
                        sy *= fac;
                        if (b.sy) b.sy[(((size_t)inst * nt + it) * ns + c) * ny + iy] = sy;
                        if (myi) {
                            const double mv = myi[(size_t)it * ny + iy];
                            if (!isnan(mv)) {
                                double sg = M::sigma(iy, pu, ku);
                                const bool data_sigma = sgi && !isnan(sgi[(size_t)it * ny + iy]);
                                if (data_sigma) sg = sgi[(size_t)it * ny + iy];
                                double djdy, djds;
                                noise_jy(M::noise(iy), M::observable(iy, ys, pu, ku), mv, sg, djdy, djds);
                                double d = djdy * sy;
                                if constexpr (M::HAS_DSIGMA)
                                    if (!data_sigma) d += djds * M::dsigma_dp(iy, pj, pu, ku) * fac;
                                if (m < NPS) sllh_part[m] -= d;
                            }
                        }
                    }
                }
            }
            if (g.lane == 0) b.numsteps[(size_t)inst * nt + it] = (POSTEQ && isinf(tout)) ? 0 : nst;
            g.sync();
        }
        double llh = g.sum(llh_part);
        if (no_steady_state) {
            status = -99;  // the steady-state failure is an AmiException: AMICI_ERROR
            it = 0;
        }
        if (status != 0) {  // ReturnData::invalidate (rdata.cpp:684-747)
            for (int jt = it; jt < nt; jt++) {
                if (b.x)
                    for (int i = g.lane; i < N; i += G) b.x[((size_t)inst * nt + jt) * N + i] = NAN;
                for (int iy = g.lane; iy < ny; iy += G) {
                    const size_t oi = ((size_t)inst * nt + jt) * ny + iy;
                    if (b.y) b.y[oi] = NAN;
                    if (b.sigmay) b.sigmay[oi] = NAN;
                }
                if (g.lane == 0) b.numsteps[(size_t)inst * nt + jt] = nst;
                if constexpr (SENS) {
                    for (int c = g.lane; c < ns; c += G) {
                        if (b.sx)
                            for (int i = 0; i < N; i++) b.sx[(((size_t)inst * nt + jt) * ns + c) * N + i] = NAN;
                        if (b.sy)
                            for (int iy = 0; iy < ny; iy++) b.sy[(((size_t)inst * nt + jt) * ns + c) * ny + iy] = NAN;
                    }
                }
            }
            llh = NAN;
        }
        if constexpr (SENS) {
            if (b.sllh) {
                int m = 0;
                for (int c = g.lane; c < ns; c += G, m++)
                    b.sllh[(size_t)inst * ns + c] = (status != 0 || !myi) ? NAN : (m < NPS ? sllh_part[m] : NAN);
            }
        }
        if (status == 0 && pe_status != 0 && pe_status != 1) status = -99;
        if (g.lane == 0) {
            b.llh[inst] = myi ? llh : NAN;
            b.status[inst] = status;
            if (b.diag) {
                int32_t* dg = b.diag + (size_t)inst * 8;
                dg[0] = nst;
                dg[1] = nfe;
                dg[2] = nni;
                dg[3] = nsetups;
                dg[4] = netf;
                dg[5] = ncfn;
                dg[6] = nje;
                dg[7] = 0;
            }
        }
        g.sync();
        return status;
    }
};

// Persistent kernel: each group pulls instance indices from the work queue.
// PREEQ: the pre-equilibration launch (simulation to steady state).
// POSTEQ: the main launch with post-equilibration outputs (t = inf).
template <class M, int G, class LUT, class R, bool SENS = false, bool PREEQ = false, bool POSTEQ = false>
__global__ void __launch_bounds__(128, 1) forward_kernel(Batch b, Opts o) {
    extern __shared__ __align__(16) unsigned char smem[];
    using LY = InstanceLayout<M, LUT, SENS>;
    const int gib = threadIdx.x / G;
    Integrator<M, G, LUT, R, SENS> I(smem + (size_t)gib * LY::bytes);
    I.o = &o;
    I.load_tables();
    if constexpr (SENS) {
        const long long gid = (long long)blockIdx.x * (blockDim.x / G) + gib;
        I.sb = b.sens_scratch + gid * b.sens_stride;
        I.nsp = b.nsp;
    }
    for (;;) {
        int idx = 0;
        if (I.g.lane == 0) idx = (int)atomicAdd(b.queue, 1u);
        idx = I.g.bcast(idx, 0);
        if (idx >= b.n) break;
        if constexpr (PREEQ) I.run_preeq(b, idx);
        else I.template run_instance<POSTEQ>(b, idx);
    }
}

// Persistent adjoint kernel: per instance the forward run (storing every step
// for the interpolant and dJy/dx at the outputs), then the backward problem
// with quadratures in the same group; groups pull instances from the queue.
template <class M, int G, class LUT, class R>
__global__ void __launch_bounds__(128, 1) adjoint_kernel(Batch b, Opts o) {
    extern __shared__ __align__(16) unsigned char smem[];
    using LY = InstanceLayout<M, LUT, false>;
    constexpr size_t stride = LY::bytes + BwdLayout<M>::bytes;
    constexpr size_t tb_bytes = ((sizeof(int) * (size_t)M::TB_TOTAL + 15) / 16) * 16;
    int* tbs = reinterpret_cast<int*>(smem);
    M::copy_tables(tbs, threadIdx.x, blockDim.x);
    __syncthreads();
    const int gib = threadIdx.x / G;
    unsigned char* base = smem + tb_bytes + (size_t)gib * stride;
    const long long gid = (long long)blockIdx.x * (blockDim.x / G) + gib;
    double* scr = b.adj_scratch + gid * b.adj_stride;
    const AdjLayout lay{b.adj_cap, b.nt, M::NX, b.nplist};
    const int lane = (threadIdx.x & 31) % G;
    for (;;) {
        int idx = 0;
        if (lane == 0) idx = (int)atomicAdd(b.queue, 1u);
        idx = Group<G>().bcast(idx, 0);
        if (idx >= b.n) break;
        long long npts = 0;
        int fstatus = 0;
        {
            Integrator<M, G, LUT, R, false, false> F(base);
            F.o = &o;
            F.load_tables();
            F.st_t = scr + lay.t_off();
            F.st_q = scr + lay.q_off();
            F.st_y = scr + lay.y_off();
            F.st_dj = scr + lay.dj_off();
            F.st_cap = b.adj_cap;
            fstatus = F.run_instance(b, idx);
            npts = F.st_n;
        }
        if (fstatus == 0 && b.my && b.nplist > 0) {
            Integrator<M, G, LUT, R, false, true> B(base);
            B.o = &o;
            B.plist = b.plist;
            B.nq = b.nplist;
            B.nqp = b.nplist;
            B.tb = tbs;
            int nstb = 0;
            const int bst = B.run_backward(b, idx, scr, npts, &nstb);
            if (lane == 0) {
                if (bst) {
                    b.status[idx] = bst;
                    b.llh[idx] = NAN;
                }
                if (b.diag) b.diag[(size_t)idx * 8 + 7] = nstb;
            }
        } else if (b.sllh) {
            for (int c = lane; c < b.nplist; c += G) b.sllh[(size_t)idx * b.nplist + c] = NAN;
        }
        Group<G>().sync();
    }
}

// Persistent adjoint kernel with forward check points every k steps (the
// reference's CVodeAdjInit(k, CV_HERMITE) scheme, cvodea.c:99-660,1365-1640):
// per instance the forward run saves its state before steps 0, k, 2k, ...
// and dJy/dx at the outputs; the backward problem then walks the segments
// from the last: each segment is replayed from its check point into (t, y,
// y') Hermite data, and the backward problem is resumed inside it until it
// reaches the segment's start or t0.
template <class M, int G, class LUT, class R>
__global__ void __launch_bounds__(128, 1) adjoint_ck_kernel(Batch b, Opts o) {
    extern __shared__ __align__(16) unsigned char smem[];
    using LY = InstanceLayout<M, LUT, false>;
    using FI = Integrator<M, G, LUT, R, false, false>;
    using BI = Integrator<M, G, LUT, R, false, true>;
    constexpr size_t stride = LY::bytes + BwdLayout<M>::bytes;
    constexpr size_t tb_bytes = ((sizeof(int) * (size_t)M::TB_TOTAL + 15) / 16) * 16;
    constexpr long long CKS = ck_stride_of<M>();
    int* tbs = reinterpret_cast<int*>(smem);
    M::copy_tables(tbs, threadIdx.x, blockDim.x);
    __syncthreads();
    const int gib = threadIdx.x / G;
    unsigned char* base = smem + tb_bytes + (size_t)gib * stride;
    const long long gid = (long long)blockIdx.x * (blockDim.x / G) + gib;
    double* scr = b.adj_scratch + gid * b.adj_stride;
    const AdjCkLayout lay{b.ck_k, b.ck_cap, b.nt, M::NX, b.nplist, CKS};
    double* cks = scr + lay.ck_off();
    double* seg_t = scr + lay.st_off();
    double* seg_y = scr + lay.sy_off();
    double* seg_yd = scr + lay.syd_off();
    double* dj = scr + lay.dj_off();
    double* bstate = scr + lay.bs_off(LMAX + 4);
    double* ctl = bstate + CKS;
    double* yBs = ctl + 8;
    const int lane = (threadIdx.x & 31) % G;
    for (;;) {
        int idx = 0;
        if (lane == 0) idx = (int)atomicAdd(b.queue, 1u);
        idx = Group<G>().bcast(idx, 0);
        if (idx >= b.n) break;
        int ck_n = 0, nst_final = 0, fstatus = 0;
        {
            FI F(base);
            F.o = &o;
            F.load_tables();
            F.ck_buf = cks;
            F.ck_k = b.ck_k;
            F.ck_next = 0;
            F.st_dj = dj;
            fstatus = F.run_instance(b, idx);
            ck_n = F.ck_n;
            nst_final = F.nst;
        }
        if (fstatus == 0 && b.my && b.nplist > 0 && ck_n > 0) {
            int seg = ck_n - 1, bst = 0, nstb = 0;
            bool first = true;
            for (;;) {
                long long np;
                {
                    FI F(base);
                    F.o = &o;
                    F.load_tables();
                    F.reload_coeffs();
                    F.load_state(cks + (size_t)seg * CKS);
                    const int nend = min((seg + 1) * b.ck_k, nst_final);
                    np = F.replay_segment(b, idx, nend, seg_t, seg_y, seg_yd);
                }
                if (np < 2) {
                    bst = np < 0 ? (int)np : -99;
                    break;
                }
                BI B(base);
                B.o = &o;
                B.plist = b.plist;
                B.nq = b.nplist;
                B.nqp = b.nplist;
                B.tb = tbs;
                B.qb = scr + lay.qv_off();
                B.pt_t = seg_t;
                B.pt_q = nullptr;
                B.pt_y = seg_y;
                B.pt_yd = seg_yd;
                B.npts = np;
                B.newdata = 1;
                B.dd_base = -1;
                B.dd_order = -1;
                B.t_interp = NAN;
                if (first) B.begin_backward(b, idx, dj, ctl, yBs);
                else B.load_state(bstate);
                const int need = B.resume_backward(b, idx, dj, ctl, yBs, seg_t[0], seg > 0);
                if (need) {
                    B.save_state(bstate);
                    seg--;
                    first = false;
                    continue;
                }
                bst = int(ctl[BI::BC_STATUS]);
                nstb = B.nst;
                B.write_gradient(b, idx, yBs, bst);
                break;
            }
            if (lane == 0) {
                if (bst) {
                    b.status[idx] = bst;
                    b.llh[idx] = NAN;
                }
                if (b.diag) b.diag[(size_t)idx * 8 + 7] = nstb;
            }
            if (bst && b.sllh)
                for (int c = lane; c < b.nplist; c += G) b.sllh[(size_t)idx * b.nplist + c] = NAN;
        } else if (b.sllh) {
            for (int c = lane; c < b.nplist; c += G) b.sllh[(size_t)idx * b.nplist + c] = NAN;
        }
        Group<G>().sync();
    }
}

}  // namespace agb
