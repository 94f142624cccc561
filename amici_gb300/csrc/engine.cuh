// GB300 (sm_103a) batched BDF engine: forward simulation of many model
// instances in one persistent kernel.
//
// Execution model.  A *group* of G consecutive lanes of a warp (G in
// {1,2,4,8,16,32}) integrates one instance; a warp holds 32/G instances.
// GB300 charges an FP64 warp instruction the same pipe time whatever its
// active mask, so packing several instances per warp (G < 32) amortises the
// group-uniform scalar step control over more instances, while G > 1 keeps
// enough warps in flight for small batches.  Groups take instances from a
// global work queue (atomicAdd), so instances with very different step counts
// keep every group busy until the batch drains.
//
// Per instance, all vectors live in shared memory: lane l of the group owns
// the elements i with i % G == l (Nordsieck history, error weights,
// corrections); the current iterate y and the fluxes w are read by all lanes
// of the group, and the iteration matrix M = I - gamma*J and its LU factors
// (column-major, FP32 by default, FP64 on request) are shared.
//
// Algorithm.  The integrator restates CVODES' variable-order BDF method as
// AMICI drives it (the reference's ThirdParty/sundials/src/cvodes/cvodes.c,
// cvodes_nls.c, cvodes_ls.c; src/solver.cpp:141-160): Nordsieck predictor
// (cvPredict, cvodes.c:6507), BDF coefficients (cvSetBDF/cvSetTqBDF :6788-6892),
// modified Newton with the linear-solver setup heuristics (cvNls :6894,
// cvNlsConvTest cvodes_nls.c:303, cvLsSetup cvodes_ls.c:1611, msbp=20,
// dgmax=0.3, msbj=51, dgmax_jbad=0.2), local error test (cvDoErrorTest :7461),
// history update and order/step selection (cvCompleteStep :7634,
// cvPrepareNextStep :7747, cvChooseEta :7935), initial step (cvHin :5436),
// and a stop time at every output (cvodes.c:3270-3330).  The state, residual,
// error norms and history are FP64; only M is factorised and solved in the
// LU precision (modified Newton tolerates an approximate M).
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
constexpr double ONEPSM = 1.000001, ADDON = 0.000001, BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0;
constexpr double CRDOWN = 0.3, RDIV = 2.0, FUZZ_FACTOR = 100.0, HLB_FACTOR = 100.0;
constexpr double HUB_FACTOR = 0.1, H_BIAS = 0.5, CORTES = 0.1, DGMAX_LSETUP = 0.3;
constexpr double DGMAX_JBAD = 0.2;
constexpr int MAX_ITERS = 4, MSBP = 20, MSBJ = 51;
constexpr double UROUND = 2.220446049250313e-16;

// internal flags (cvodes_impl.h:178-185)
constexpr int CV_SUCCESS = 0, CV_TSTOP_RETURN = 1, CV_TOO_MUCH_WORK = -1, CV_TOO_MUCH_ACC = -2,
              CV_ERR_FAILURE = -3, CV_CONV_FAILURE = -4, CV_ILL_INPUT = -22;
constexpr int DO_ERROR_TEST = 2, PREDICT_AGAIN = 3, TRY_AGAIN = 5, FIRST_CALL = 6,
              PREV_CONV_FAIL = 7, PREV_ERR_FAIL = 9, NLS_CONV_RECVR = 901, NLS_CONTINUE = 902;
constexpr int CV_NO_FAILURES = 0, CV_FAIL_BAD_J = 1, CV_FAIL_OTHER = 2;

struct Opts {
    double rtol, atol, rtolS, atolS;
    int64_t maxsteps;
    int maxcor, maxncf;
    double hmax_inv;
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
    unsigned int* queue;  // work-queue counter (scratch, zeroed before launch)
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
    __device__ __forceinline__ double sum(double v) const {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, G);
        return v;
    }
    __device__ __forceinline__ double max(double v) const {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(mask, v, o, G));
        return v;
    }
    __device__ __forceinline__ int bcast(int v, int src) const {
        return G > 1 ? __shfl_sync(mask, v, src, G) : v;
    }
};

__device__ __forceinline__ double powr(double base, double e) {  // SUNRpowerR
    return base <= 0.0 ? 0.0 : pow(base, e);
}
__device__ __forceinline__ double powi(double base, int e) {  // SUNRpowerI
    double prod = 1.0;
    for (int i = 1; i <= e; i++) prod *= base;
    return prod;
}

// Shared-memory layout of one instance.
template <class M, class LUT>
struct InstanceLayout {
    static constexpr int N = M::NX;
    static constexpr int NW = M::NW;
    static constexpr int NPK = M::NP + M::NK;
    // doubles
    static constexpr int off_zn = 0;                     // LMAX*N
    static constexpr int off_ewt = off_zn + LMAX * N;    // N
    static constexpr int off_acor = off_ewt + N;         // N
    static constexpr int off_tempv = off_acor + N;       // N
    static constexpr int off_ftemp = off_tempv + N;      // N
    static constexpr int off_y = off_ftemp + N;          // N
    static constexpr int off_w = off_y + N;              // NW
    static constexpr int off_c = off_w + NW;             // NW
    static constexpr int off_pk = off_c + NW;            // NP + NK (unscaled p, then k)
    static constexpr int n_double = off_pk + NPK;
    // LU-precision arrays
    static constexpr int n_lut = 2 * N * N + 2 * N;      // savedJ, M, bf, cf... (bf: N, spare N)
    static constexpr size_t bytes_double = sizeof(double) * n_double;
    static constexpr size_t bytes_lut = sizeof(LUT) * (size_t)n_lut;
    static constexpr size_t bytes_int = sizeof(int16_t) * (2 * N);  // perm, piv
    static constexpr size_t bytes = ((bytes_double + bytes_lut + bytes_int + 15) / 16) * 16;
};

template <class M, int G, class LUT>
struct Integrator {
    static constexpr int N = M::NX;
    static constexpr int NW = M::NW;
    using LY = InstanceLayout<M, LUT>;

    Group<G> g;
    double *zn, *ewt, *acor, *tempv, *ftemp, *y, *w, *c, *pu, *ku;
    LUT *Jsv, *Mm, *bf;
    int16_t *perm, *piv;

    const Opts* o;
    // group-uniform scalars (cvodes CVodeMemRec)
    double tn, h, hprime, hscale, eta, etamax;
    double tau[LMAX + 1], l[LMAX], tq[6];
    double rl1, gamma, gammap, gamrat, crate, delp, acnrm, saved_tq5, etaqm1, etaq, etaqp1, tstop;
    int q, qprime, qwait, L, indx_acor, convfail, jcur, jcur_nls, tstopset;
    int64_t nst, nstlp, nstlj;

    __device__ __forceinline__ Integrator(unsigned char* base) {
        double* d = reinterpret_cast<double*>(base);
        zn = d + LY::off_zn;
        ewt = d + LY::off_ewt;
        acor = d + LY::off_acor;
        tempv = d + LY::off_tempv;
        ftemp = d + LY::off_ftemp;
        y = d + LY::off_y;
        w = d + LY::off_w;
        c = d + LY::off_c;
        pu = d + LY::off_pk;
        ku = pu + M::NP;
        LUT* lb = reinterpret_cast<LUT*>(base + LY::bytes_double);
        Jsv = lb;
        Mm = lb + N * N;
        bf = lb + 2 * N * N;
        perm = reinterpret_cast<int16_t*>(base + LY::bytes_double + LY::bytes_lut);
        piv = perm + N;
    }

    __device__ __forceinline__ double* Z(int j) { return zn + j * N; }

    // ---------------- model evaluation ------------------------------------
    // f = S w(yv); yv must be complete in shared memory (callers sync first).
    __device__ void rhs(const double* yv, double* f) {
        for (int r = g.lane; r < NW; r += G) w[r] = c[r] * M::flux_monomial(r, yv);
        g.sync();
        for (int i = g.lane; i < N; i += G) f[i] = M::stoich_row_dot(i, w);
        g.sync();
    }

    __device__ double wrms(const double* v, const double* wt) {
        double s = 0.0;
        for (int i = g.lane; i < N; i += G) {
            double t = v[i] * wt[i];
            s += t * t;
        }
        s = g.sum(s);
        return sqrt(s / N);
    }

    __device__ int ewt_set(const double* yv, double* wt) {
        int bad = 0;
        for (int i = g.lane; i < N; i += G) {
            double t = o->rtol * fabs(yv[i]) + o->atol;
            if (t <= 0.0) bad = 1;
            wt[i] = 1.0 / t;
        }
        return (int)g.max((double)bad);
    }

    // ---------------- linear algebra: M = I - gamma*J, LU, solve -----------
    // Jacobian J = S * dw/dx at y (own rows), stored column-major in Jsv.
    __device__ void jac_eval() {
        for (int i = g.lane; i < N; i += G) {
            for (int j = 0; j < N; j++) Jsv[j * N + i] = LUT(0);
            M::template jac_row<LUT>(i, c, y, Jsv);
        }
        g.sync();
    }

    // cvLsSetup (cvodes_ls.c:1611) + dense GETRF (sundials_dense.c:82); returns 0 or 1 (singular)
    __device__ int lsetup() {
        double dgamma = fabs(gamma / gammap - 1.0);
        int jbad = (nst == 0) || (nst >= nstlj + MSBJ) ||
                   ((convfail == CV_FAIL_BAD_J) && (dgamma < DGMAX_JBAD)) || (convfail == CV_FAIL_OTHER);
        g.sync();  // y complete
        if (!jbad) {
            jcur = 0;
        } else {
            jac_eval();
            jcur = 1;
            nstlj = nst;
        }
        const LUT mg = LUT(-gamma);
        for (int i = g.lane; i < N; i += G)
            for (int j = 0; j < N; j++) Mm[j * N + i] = mg * Jsv[j * N + i] + (i == j ? LUT(1) : LUT(0));
        int ret = getrf();
        gamrat = 1.0;
        gammap = gamma;
        crate = 1.0;
        nstlp = nst;
        return ret;
    }

    __device__ int getrf() {
        g.sync();
        for (int k = 0; k < N; k++) {
            LUT* colk = Mm + k * N;
            // pivot: first row with maximal |a_ik|, i >= k
            LUT best = LUT(-1);
            int bi = N;
            for (int i = k + g.lane; i < N; i += G) {
                LUT v = fabs(colk[i]);
                if (v > best) { best = v; bi = i; }
            }
#pragma unroll
            for (int off = G / 2; off > 0; off >>= 1) {
                LUT ob = __shfl_xor_sync(g.mask, best, off, G);
                int oi = __shfl_xor_sync(g.mask, bi, off, G);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            const int lp = bi;
            if (g.lane == 0) piv[k] = (int16_t)lp;
            if (colk[lp] == LUT(0)) return 1;
            if (lp != k)
                for (int j = g.lane; j < N; j += G) {
                    LUT t = Mm[j * N + lp];
                    Mm[j * N + lp] = Mm[j * N + k];
                    Mm[j * N + k] = t;
                }
            g.sync();
            const LUT mult = LUT(1) / colk[k];
            for (int i = k + 1 + g.lane; i < N; i += G) {
                LUT lik = colk[i] * mult;
                colk[i] = lik;
                for (int j = k + 1; j < N; j++) {
                    LUT akj = Mm[j * N + k];
                    if (akj != LUT(0)) Mm[j * N + i] -= akj * lik;
                }
            }
            g.sync();
        }
        if (g.lane == 0) {
            for (int i = 0; i < N; i++) perm[i] = (int16_t)i;
            for (int k = 0; k < N; k++) {
                int pk = piv[k];
                int16_t t = perm[k];
                perm[k] = perm[pk];
                perm[pk] = t;
            }
        }
        g.sync();
        return 0;
    }

    // b <- M^{-1} b (cvLsSolve + GETRS, cvodes_ls.c:1720-1860), b in shared memory
    __device__ void lsolve(double* b) {
        g.sync();
        for (int i = g.lane; i < N; i += G) bf[i] = LUT(b[perm[i]]);
        g.sync();
        for (int k = 0; k < N - 1; k++) {
            const LUT bk = bf[k];
            const LUT* colk = Mm + k * N;
            for (int i = k + 1 + g.lane; i < N; i += G) bf[i] -= colk[i] * bk;
            g.sync();
        }
        const double sc = (gamrat != 1.0) ? 2.0 / (1.0 + gamrat) : 1.0;
        for (int k = N - 1; k >= 0; k--) {
            const LUT* colk = Mm + k * N;
            const LUT bk = bf[k] / colk[k];
            if (k % G == g.lane) b[k] = (gamrat != 1.0) ? double(bk) * sc : double(bk);
            for (int i = g.lane; i < k; i += G) bf[i] -= colk[i] * bk;
            g.sync();
        }
    }

    // ---------------- BDF bookkeeping (cvodes.c:6112-6894) ----------------
    __device__ void rescale() {
        double f = eta;
        for (int j = 1; j <= q; j++, f *= eta)
            for (int i = g.lane; i < N; i += G) Z(j)[i] *= f;
        h = hscale * eta;
        hscale = h;
    }

    __device__ void increase_bdf() {
        double alpha0, alpha1, prod, xi, xiold, hsum, A1;
        for (int i = 0; i <= QMAX; i++) l[i] = 0.0;
        l[2] = alpha1 = prod = xiold = 1.0;
        alpha0 = -1.0;
        hsum = hscale;
        if (q > 1) {
            for (int j = 1; j < q; j++) {
                hsum += tau[j + 1];
                xi = hsum / hscale;
                prod *= xi;
                alpha0 -= 1.0 / (j + 1);
                alpha1 += 1.0 / xi;
                for (int i = j + 2; i >= 2; i--) l[i] = l[i] * xiold + l[i - 1];
                xiold = xi;
            }
        }
        A1 = (-alpha0 - alpha1) / prod;
        for (int i = g.lane; i < N; i += G) {
            double zl = A1 * Z(indx_acor)[i];
            Z(L)[i] = zl;
            for (int j = 2; j <= q; j++) Z(j)[i] += l[j] * zl;
        }
    }

    __device__ void decrease_bdf() {
        double hsum, xi;
        for (int i = 0; i <= QMAX; i++) l[i] = 0.0;
        l[2] = 1.0;
        hsum = 0.0;
        for (int j = 1; j <= q - 2; j++) {
            hsum += tau[j];
            xi = hsum / hscale;
            for (int i = j + 2; i >= 2; i--) l[i] = l[i] * xi + l[i - 1];
        }
        for (int i = g.lane; i < N; i += G)
            for (int j = 2; j < q; j++) Z(j)[i] += -l[j] * Z(q)[i];
    }

    __device__ void adjust_order(int dq) {
        if (q == 2 && dq != 1) return;
        if (dq == 1) increase_bdf();
        else if (dq == -1) decrease_bdf();
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

    __device__ void predict() {
        tn += h;
        if (tstopset && (tn - tstop) * h > 0.0) tn = tstop;
        for (int i = g.lane; i < N; i += G)
            for (int k = 1; k <= q; k++)
                for (int j = q; j >= k; j--) Z(j - 1)[i] += Z(j)[i];
    }

    __device__ void restore(double saved_t) {
        tn = saved_t;
        for (int i = g.lane; i < N; i += G)
            for (int k = 1; k <= q; k++)
                for (int j = q; j >= k; j--) Z(j - 1)[i] -= Z(j)[i];
    }

    __device__ void set_bdf() {
        double alpha0, alpha0_hat, xi_inv, xistar_inv, hsum;
        l[0] = l[1] = xi_inv = xistar_inv = 1.0;
        for (int i = 2; i <= q; i++) l[i] = 0.0;
        alpha0 = alpha0_hat = -1.0;
        hsum = h;
        if (q > 1) {
            for (int j = 2; j < q; j++) {
                hsum += tau[j - 1];
                xi_inv = h / hsum;
                alpha0 -= 1.0 / j;
                for (int i = j; i >= 1; i--) l[i] += l[i - 1] * xi_inv;
            }
            alpha0 -= 1.0 / q;
            xistar_inv = -l[1] - alpha0;
            hsum += tau[q - 1];
            xi_inv = h / hsum;
            alpha0_hat = -l[1] - xi_inv;
            for (int i = q; i >= 1; i--) l[i] += l[i - 1] * xistar_inv;
        }
        double A1 = 1.0 - alpha0_hat + alpha0;
        double A2 = 1.0 + q * A1;
        tq[2] = fabs(A1 / (alpha0 * A2));
        tq[5] = fabs(A2 * xistar_inv / (l[q] * xi_inv));
        if (qwait == 1) {
            if (q > 1) {
                double C = xistar_inv / l[q];
                double A3 = alpha0 + 1.0 / q;
                double A4 = alpha0_hat + xi_inv;
                double Cpinv = (1.0 - A4 + A3) / A3;
                tq[1] = fabs(C * Cpinv);
            } else {
                tq[1] = 1.0;
            }
            hsum += tau[q];
            xi_inv = h / hsum;
            double A5 = alpha0 - (1.0 / (q + 1));
            double A6 = alpha0_hat - xi_inv;
            double Cppinv = (1.0 - A6 + A5) / A2;
            tq[3] = fabs(Cppinv / (xi_inv * (q + 2) * A5));
        }
        tq[4] = CORTES / tq[2];
    }

    __device__ void cv_set() {
        set_bdf();
        rl1 = 1.0 / l[1];
        gamma = h * rl1;
        if (nst == 0) gammap = gamma;
        gamrat = (nst > 0) ? gamma / gammap : 1.0;
    }

    // ---------------- Newton iteration (cvNls + SUNNonlinSolSolve_Newton) -
    // residual: delta = rl1*zn1 + ycor - gamma*f(zn0 + ycor)
    __device__ void nls_residual() {
        for (int i = g.lane; i < N; i += G) y[i] = Z(0)[i] + acor[i];
        g.sync();
        rhs(y, ftemp);
        for (int i = g.lane; i < N; i += G) tempv[i] = (rl1 * Z(1)[i] + acor[i]) + (-gamma) * ftemp[i];
    }

    __device__ int nls_convtest(int m) {
        double del = wrms(tempv, ewt);
        if (m > 0) crate = fmax(CRDOWN * crate, del / delp);
        double dcon = del * fmin(1.0, crate) / tq[4];
        if (dcon <= 1.0) {
            acnrm = (m == 0) ? del : wrms(acor, ewt);
            return CV_SUCCESS;
        }
        if (m >= 1 && del > RDIV * delp) return NLS_CONV_RECVR;
        delp = del;
        return NLS_CONTINUE;
    }

    __device__ int cv_nls(int nflag) {
        convfail = ((nflag == FIRST_CALL) || (nflag == PREV_ERR_FAIL)) ? CV_NO_FAILURES : CV_FAIL_OTHER;
        int callSetup = (nflag == PREV_CONV_FAIL) || (nflag == PREV_ERR_FAIL) || (nst == 0) ||
                        (nst >= nstlp + MSBP) || (fabs(gamrat - 1.0) > DGMAX_LSETUP);
        for (int i = g.lane; i < N; i += G) acor[i] = 0.0;
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
                for (int i = g.lane; i < N; i += G) tempv[i] = -tempv[i];
                lsolve(tempv);
                for (int i = g.lane; i < N; i += G) acor[i] += tempv[i];
                retval = nls_convtest(curiter);
                curiter++;
                if (retval == CV_SUCCESS) {
                    for (int i = g.lane; i < N; i += G) y[i] = Z(0)[i] + acor[i];
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
                for (int i = g.lane; i < N; i += G) acor[i] = 0.0;
                continue;
            }
            break;
        }
        return retval;
    }

    // ---------------- step control ----------------------------------------
    __device__ int handle_nflag(int* nflag, double saved_t, int* ncf) {
        if (*nflag == CV_SUCCESS) return DO_ERROR_TEST;
        restore(saved_t);
        (*ncf)++;
        etamax = 1.0;
        if (*ncf == o->maxncf) return CV_CONV_FAILURE;  // hmin = 0
        eta = ETA_CF;
        *nflag = PREV_CONV_FAIL;
        rescale();
        return PREDICT_AGAIN;
    }

    __device__ int do_error_test(int* nflag, double saved_t, double acor_nrm, int* nef, double* dsmp) {
        double dsm = acor_nrm * tq[2];
        *dsmp = dsm;
        if (dsm <= 1.0) return CV_SUCCESS;
        (*nef)++;
        *nflag = PREV_ERR_FAIL;
        restore(saved_t);
        if (*nef == MXNEF) return CV_ERR_FAILURE;
        etamax = 1.0;
        if (*nef <= MXNEF1) {
            eta = 1.0 / (powr(BIAS2 * dsm, 1.0 / L) + ADDON);
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
        g.sync();
        rhs(Z(0), tempv);
        for (int i = g.lane; i < N; i += G) Z(1)[i] = h * tempv[i];
        return TRY_AGAIN;
    }

    __device__ void complete_step() {
        nst++;
        for (int i = q; i >= 2; i--) tau[i] = tau[i - 1];
        if (q == 1 && nst > 1) tau[2] = tau[1];
        tau[1] = h;
        for (int i = g.lane; i < N; i += G) {
            double a = acor[i];
            for (int j = 0; j <= q; j++) Z(j)[i] += l[j] * a;
        }
        qwait--;
        if (qwait == 1 && q != QMAX) {
            for (int i = g.lane; i < N; i += G) Z(QMAX)[i] = acor[i];
            saved_tq5 = tq[5];
            indx_acor = QMAX;
        }
    }

    __device__ void set_eta() {
        if (eta > ETA_MIN_FX && eta < ETA_MAX_FX) {
            eta = 1.0;
            hprime = h;
        } else {
            if (eta >= ETA_MAX_FX) {
                eta = fmin(eta, etamax);
                eta /= fmax(1.0, fabs(h) * o->hmax_inv * eta);
            } else {
                eta = fmax(eta, ETA_MIN);
            }
            hprime = h * eta;
        }
    }

    __device__ void prepare_next_step(double dsm) {
        if (etamax == 1.0) {
            qwait = qwait > 2 ? qwait : 2;
            qprime = q;
            hprime = h;
            eta = 1.0;
            return;
        }
        etaq = 1.0 / (powr(BIAS2 * dsm, 1.0 / L) + ADDON);
        if (qwait != 0) {
            eta = etaq;
            qprime = q;
            set_eta();
            return;
        }
        qwait = 2;
        // cvComputeEtaqm1
        etaqm1 = 0.0;
        if (q > 1) {
            double ddn = wrms(Z(q), ewt) * tq[1];
            etaqm1 = 1.0 / (powr(BIAS1 * ddn, 1.0 / q) + ADDON);
        }
        // cvComputeEtaqp1
        etaqp1 = 0.0;
        if (q != QMAX && saved_tq5 != 0.0) {
            double cquot = (tq[5] / saved_tq5) * powi(h / tau[2], L);
            for (int i = g.lane; i < N; i += G) tempv[i] = -cquot * Z(QMAX)[i] + acor[i];
            double dup = wrms(tempv, ewt) * tq[3];
            etaqp1 = 1.0 / (powr(BIAS3 * dup, 1.0 / (L + 1)) + ADDON);
        }
        // cvChooseEta
        double etam = fmax(etaqm1, fmax(etaq, etaqp1));
        if (etam > ETA_MIN_FX && etam < ETA_MAX_FX) {
            eta = 1.0;
            qprime = q;
        } else if (etam == etaq) {
            eta = etaq;
            qprime = q;
        } else if (etam == etaqm1) {
            eta = etaqm1;
            qprime = q - 1;
        } else {
            eta = etaqp1;
            qprime = q + 1;
            for (int i = g.lane; i < N; i += G) Z(QMAX)[i] = acor[i];
        }
        set_eta();
    }

    __device__ int cv_step() {
        int ncf = 0, nef = 0, nflag, kflag, eflag;
        double dsm = 0.0;
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
            eflag = do_error_test(&nflag, saved_t, acnrm, &nef, &dsm);
            if (eflag == TRY_AGAIN) continue;
            if (eflag != CV_SUCCESS) return eflag;
            break;
        }
        complete_step();
        prepare_next_step(dsm);
        etamax = (nst <= SMALL_NST) ? ETA_MAX_ES : ETA_MAX_GS;
        return CV_SUCCESS;
    }

    // ---------------- initial step (cvHin, cvodes.c:5436-5798) ------------
    __device__ double upper_bound_h0(double tdist) {
        double hub_inv = 0.0;
        for (int i = g.lane; i < N; i += G) {
            double wv = 1.0 / ewt[i];
            double t = HUB_FACTOR * fabs(Z(0)[i]) + wv;
            double v = fabs(Z(1)[i]) / t;
            hub_inv = fmax(hub_inv, v);
        }
        hub_inv = g.max(hub_inv);
        double hub = HUB_FACTOR * tdist;
        if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
        return hub;
    }

    __device__ double ydd_norm(double hg) {
        for (int i = g.lane; i < N; i += G) y[i] = hg * Z(1)[i] + Z(0)[i];
        g.sync();
        rhs(y, tempv);
        for (int i = g.lane; i < N; i += G) tempv[i] = (1.0 / hg) * (tempv[i] - Z(1)[i]);
        return wrms(tempv, ewt);
    }

    __device__ int cv_hin(double tout) {
        double tdiff = tout - tn;
        if (tdiff == 0.0) return CV_ILL_INPUT;
        int sign = tdiff > 0.0 ? 1 : -1;
        double tdist = fabs(tdiff);
        double tround = UROUND * fmax(fabs(tn), fabs(tout));
        if (tdist < 2.0 * tround) return CV_ILL_INPUT;
        double hlb = HLB_FACTOR * tround;
        double hub = upper_bound_h0(tdist);
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
            double hrat = hnew / hg;
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

    // CVode(tout, NORMAL) with tstop = tout, as AMICI calls it
    __device__ int cv_solve(double tout, int64_t mxstep) {
        tstop = tout;
        tstopset = 1;
        if (nst == 0) {
            g.sync();
            if (ewt_set(Z(0), ewt)) return CV_ILL_INPUT;
            rhs(Z(0), Z(1));
            int hflag = cv_hin(tout);
            if (hflag != CV_SUCCESS) return CV_ILL_INPUT;
            double rh = fabs(h) * o->hmax_inv;
            if (rh > 1.0) h /= rh;
            if ((tn + h - tstop) * h > 0.0) h = (tstop - tn) * (1.0 - 4.0 * UROUND);
            hscale = h;
            hprime = h;
            for (int i = g.lane; i < N; i += G) Z(1)[i] *= h;
        } else {
            double troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
            if (fabs(tn - tstop) <= troundoff) return CV_TSTOP_RETURN;
            if ((tn + hprime - tstop) * h > 0.0) {
                hprime = (tstop - tn) * (1.0 - 4.0 * UROUND);
                eta = hprime / h;
            }
        }
        int64_t nstloc = 0;
        for (;;) {
            if (nst > 0 && ewt_set(Z(0), ewt)) return CV_ILL_INPUT;
            if (mxstep > 0 && nstloc >= mxstep) return CV_TOO_MUCH_WORK;
            double nrm = wrms(Z(0), ewt);
            if (UROUND * nrm > 1.0) return CV_TOO_MUCH_ACC;
            int kflag = cv_step();
            if (kflag != CV_SUCCESS) return kflag;
            nstloc++;
            double troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
            if (fabs(tn - tstop) <= troundoff) tn = tstop;
            troundoff = FUZZ_FACTOR * UROUND * (fabs(tn) + fabs(h));
            if (fabs(tn - tstop) <= troundoff) {
                tstopset = 0;
                return CV_TSTOP_RETURN;
            }
            if ((tn + hprime - tstop) * h > 0.0) {
                hprime = (tstop - tn) * (1.0 - 4.0 * UROUND);
                eta = hprime / h;
            }
        }
    }

    // ---------------- one instance through AMICI's output loop -------------
    __device__ void run_instance(const Batch& b, int inst) {
        const int ny = M::NY;
        const int nt = b.nt;
        // parameters: unscale (ParameterScaling), fixed parameters
        const double* pin = b.p + (size_t)inst * M::NP;
        for (int j = g.lane; j < M::NP; j += G) {
            double v = pin[j];
            int sc = b.pscale ? b.pscale[j] : 0;
            pu[j] = sc == 1 ? exp(v) : (sc == 2 ? exp10(v) : v);
        }
        for (int j = g.lane; j < M::NK; j += G) ku[j] = b.k[(size_t)inst * M::NK + j];
        g.sync();
        for (int r = g.lane; r < NW; r += G) c[r] = M::flux_coeff(r, pu, ku);
        for (int i = g.lane; i < N; i += G) {
            Z(0)[i] = M::x0(i, pu, ku);
            for (int j = 1; j < LMAX; j++) Z(j)[i] = 0.0;
            acor[i] = 0.0;
        }
        g.sync();
        // CVodeInit defaults
        q = 1;
        L = 2;
        qwait = L;
        etamax = ETA_MAX_FS;
        tn = 0.0;
        h = hprime = hscale = eta = 0.0;
        for (int j = 0; j <= LMAX; j++) tau[j] = 0.0;
        for (int j = 0; j < LMAX; j++) l[j] = 0.0;
        for (int j = 0; j < 6; j++) tq[j] = 0.0;
        rl1 = gamma = gammap = gamrat = crate = delp = acnrm = saved_tq5 = 0.0;
        etaqm1 = etaq = etaqp1 = 0.0;
        qprime = 1;
        indx_acor = 0;
        convfail = 0;
        jcur = jcur_nls = 0;
        tstopset = 0;
        nst = nstlp = nstlj = 0;

        const double t0 = 0.0;
        const double* tsi = b.ts + (size_t)inst * nt;
        const double* myi = b.my ? b.my + (size_t)inst * nt * ny : nullptr;
        const double* sgi = b.sigma_y ? b.sigma_y + (size_t)inst * nt * ny : nullptr;
        double llh_part = 0.0;
        int status = 0, it;
        double tcur = t0;
        for (it = 0; it < nt; it++) {
            const double tout = tsi[it];
            if (tout > t0) {
                while (tcur < tout) {
                    double tdiff = tout - tcur;
                    if (tdiff == 0.0 || fabs(tdiff) < 2.0 * UROUND * fmax(fabs(tcur), fabs(tout))) break;
                    int64_t remaining = o->maxsteps - nst;
                    if (remaining <= 0) {
                        status = -99;
                        break;
                    }
                    int flag = cv_solve(tout, remaining);
                    if (flag < 0) {
                        status = flag;
                        break;
                    }
                    // CV_TSTOP_RETURN reports tret = tstop (cvodes.c:3300-3306)
                    tcur = (flag == CV_TSTOP_RETURN) ? tout : tn;
                }
                if (status != 0) break;
            }
            g.sync();
            // outputs at this time point (ReturnData::get_data_output)
            if (b.x)
                for (int i = g.lane; i < N; i += G) b.x[((size_t)inst * nt + it) * N + i] = Z(0)[i];
            for (int iy = g.lane; iy < ny; iy += G) {
                double yv = M::observable(iy, Z(0), pu, ku);
                double s = M::sigma(iy, pu, ku);
                if (sgi && !isnan(sgi[(size_t)it * ny + iy])) s = sgi[(size_t)it * ny + iy];
                const size_t oi = ((size_t)inst * nt + it) * ny + iy;
                if (b.y) b.y[oi] = yv;
                if (b.sigmay) b.sigmay[oi] = s;
                if (myi) {
                    double mv = myi[(size_t)it * ny + iy];
                    if (!isnan(mv)) {
                        double r = (yv - mv) / s;
                        llh_part -= 0.5 * log(2.0 * 3.14159265358979323846 * s * s) + 0.5 * r * r;
                    }
                }
            }
            if (g.lane == 0) b.numsteps[(size_t)inst * nt + it] = (int32_t)nst;
        }
        double llh = g.sum(llh_part);
        if (status != 0) {
            for (int jt = it; jt < nt; jt++) {
                if (b.x)
                    for (int i = g.lane; i < N; i += G) b.x[((size_t)inst * nt + jt) * N + i] = NAN;
                for (int iy = g.lane; iy < ny; iy += G) {
                    const size_t oi = ((size_t)inst * nt + jt) * ny + iy;
                    if (b.y) b.y[oi] = NAN;
                    if (b.sigmay) b.sigmay[oi] = NAN;
                }
                if (g.lane == 0) b.numsteps[(size_t)inst * nt + jt] = (int32_t)nst;
            }
            llh = NAN;
        }
        if (g.lane == 0) {
            b.llh[inst] = myi ? llh : NAN;
            b.status[inst] = status;
        }
        g.sync();
    }
};

// Persistent kernel: each group pulls instance indices from the work queue.
template <class M, int G, class LUT>
__global__ void __launch_bounds__(128) forward_kernel(Batch b, Opts o) {
    extern __shared__ __align__(16) unsigned char smem[];
    using LY = InstanceLayout<M, LUT>;
    const int gib = threadIdx.x / G;
    Integrator<M, G, LUT> I(smem + (size_t)gib * LY::bytes);
    I.o = &o;
    for (;;) {
        int idx = 0;
        if (I.g.lane == 0) idx = (int)atomicAdd(b.queue, 1u);
        idx = I.g.bcast(idx, 0);
        if (idx >= b.n) break;
        I.run_instance(b, idx);
    }
}

}  // namespace agb
