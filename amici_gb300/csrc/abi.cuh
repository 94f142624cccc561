// Host side of one model library: the C ABI declared in include/amici_gb300.h,
// instantiated for a generated model type by AMICI_GB300_DEFINE_ABI(Model).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>

#include "../../include/amici_gb300.h"
#include "engine.cuh"

namespace agb {

inline thread_local char g_last_error[512] = "";

inline int set_error(int code, const char* msg) {
    snprintf(g_last_error, sizeof(g_last_error), "%s", msg);
    return code;
}

inline int cuda_check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return AMICI_GB300_OK;
    snprintf(g_last_error, sizeof(g_last_error), "%s: %s", what, cudaGetErrorString(e));
    return AMICI_GB300_ERR_CUDA;
}

inline void default_options(amici_gb300_solver_options* o) {
    memset(o, 0, sizeof(*o));
    o->rtol = 1e-8;            // solver.h:2060
    o->atol = 1e-16;           // solver.h:2057
    o->rtol_fsa = NAN;         // inherit (solver.h:2063-2072)
    o->atol_fsa = NAN;
    o->rtol_b = NAN;
    o->atol_b = NAN;
    o->rtol_quad = 1e-8;       // solver.h:2075-2078
    o->atol_quad = 1e-12;
    o->maxsteps = 10000;       // solver.h:1886
    o->max_step_size = INFINITY;
    o->sensi_order = 0;
    o->sensi_meth = AMICI_GB300_SENSI_FORWARD;
    o->max_nonlin_iters = 3;   // solver.h:2108
    o->max_conv_fails = 10;    // solver.h:2112
    o->lu_precision = 32;
    o->lanes_per_instance = 0;
    o->checkpoint_steps = 50;
    o->control_precision = 32;
    o->launch_mode = 0;
    o->instances_per_sm = 0;
    o->stldet = 1;             // solver.h:2037
}

inline Opts make_opts(const amici_gb300_solver_options* s) {
    Opts o;
    o.rtol = s->rtol;
    o.atol = s->atol;
    o.rtolS = isnan(s->rtol_fsa) ? s->rtol : s->rtol_fsa;
    o.atolS = isnan(s->atol_fsa) ? s->atol : s->atol_fsa;
    o.maxsteps = s->maxsteps;
    o.maxcor = s->max_nonlin_iters > 0 ? s->max_nonlin_iters : 3;
    o.maxncf = s->max_conv_fails > 0 ? s->max_conv_fails : 10;
    o.hmax_inv = (s->max_step_size > 0 && isfinite(s->max_step_size)) ? 1.0 / s->max_step_size : 0.0;
    // backward problem (Solver::apply_tolerances_asa / apply_quad_tolerances_asa,
    // solver.cpp:658-691; maxstepsB default 100 * maxsteps, solver.cpp:125)
    o.rtolB = isnan(s->rtol_b) ? s->rtol : s->rtol_b;
    o.atolB = isnan(s->atol_b) ? s->atol : s->atol_b;
    o.rtolQ = isnan(s->rtol_quad) ? s->rtol : s->rtol_quad;
    o.atolQ = isnan(s->atol_quad) ? s->atol : s->atol_quad;
    o.errconQ = !isinf(o.rtolQ) && !isinf(o.atolQ);
    o.maxstepsB = 100 * s->maxsteps;
    o.ipsm = s->instances_per_sm > 0 ? s->instances_per_sm : 0;
    o.stldet = s->stldet != 0;
    return o;
}

// With a cap on resident instances per SM, ask for no more shared memory per
// SM than those instances use, so that the rest serves as L1 cache (the
// driver rounds the carveout up to a supported size).
template <class K>
inline int apply_carveout(K kern, int per_sm, size_t smem, int dev) {
    int smem_sm = 0;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (smem_sm <= 0) return AMICI_GB300_OK;
    long pct = (100L * (long)per_sm * ((long)smem + 1024) + smem_sm - 1) / smem_sm;
    if (pct > 100) pct = 100;
    return cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)pct),
                      "cudaFuncSetAttribute(carveout)");
}

// The carveout is a lasting attribute of the kernel: an uncapped launch after
// a capped one of the same kernel puts the driver's default back (before the
// occupancy query, which takes the preference into account).  ``carved``
// records per kernel whether a cap set it.
template <class K>
inline void reset_carveout(K kern, std::atomic<bool>& carved) {
    if (!carved.exchange(false)) return;
    (void)cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutDefault);
    (void)cudaGetLastError();  // a refused hint leaves no error for the launch check
}

// Launch geometry for one (model, G, LU precision) choice.
struct Geometry {
    int threads;      // per block (multiple of 32)
    size_t smem;      // dynamic shared memory per block
    int blocks;       // grid size
};

template <class M, int G, class LUT, class R, bool SENS = false, bool PREEQ = false, bool POSTEQ = false>
int launch_forward(const Batch& b_in, const Opts& o, cudaStream_t stream) {
    using LY = InstanceLayout<M, LUT, SENS>;
    auto kern = forward_kernel<M, G, LUT, R, SENS, PREEQ, POSTEQ>;
    Batch b = b_in;
    int dev = 0;
    int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    int smem_max = 0, nsm = 0;
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // warps per block: spread the batch over every SM first, then pack up to 4
    const long inst_per_warp = 32 / G;
    const long warps_total = (b.n + inst_per_warp - 1) / inst_per_warp;
    long wpb = warps_total / nsm;
    if (wpb < 1) wpb = 1;
    if (wpb > 4) wpb = 4;
    const long max_inst = (long)smem_max / (long)LY::bytes;
    const long wpb_smem = (max_inst * G) / 32;
    if (wpb_smem < 1)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED,
                         "model too large for this lanes-per-instance choice: one warp of instances "
                         "does not fit in shared memory");
    if (wpb > wpb_smem) wpb = wpb_smem;
    if (o.ipsm > 0) {
        long cap_w = ((long)o.ipsm * G) / 32;
        if (cap_w < 1) cap_w = 1;
        if (wpb > cap_w) wpb = cap_w;
    }
    const int threads = (int)(32 * wpb);
    const size_t smem = (size_t)(threads / G) * LY::bytes;
    rc = cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "cudaFuncSetAttribute");
    if (rc) return rc;
    static std::atomic<bool> carved{false};
    if (o.ipsm <= 0) reset_carveout(kern, carved);
    int per_sm = 0;
    rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem),
                    "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if (rc) return rc;
    if (per_sm < 1) per_sm = 1;
    const long groups_per_block = threads / G;
    if (o.ipsm > 0) {
        const long cap_b = o.ipsm / groups_per_block;
        per_sm = (int)(cap_b < 1 ? 1 : (cap_b < per_sm ? cap_b : per_sm));
        rc = apply_carveout(kern, per_sm, smem, dev);
        if (rc) return rc;
        carved = true;
    }
    long blocks = (b.n + groups_per_block - 1) / groups_per_block;
    const long cap = (long)per_sm * nsm;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    void* sbuf = nullptr;
    if constexpr (SENS) {
        // sensitivity columns: Nordsieck history, weights, correction, residual, RHS per group
        b.nsp = ((b.nplist + G - 1) / G) * G;
        b.sens_stride = (long long)(LMAX + 4) * M::NX * b.nsp;
        const size_t groups = (size_t)blocks * (size_t)groups_per_block;
        rc = cuda_check(cudaMallocAsync(&sbuf, groups * (size_t)b.sens_stride * sizeof(double), stream),
                        "cudaMallocAsync(sensitivity scratch)");
        if (rc) return rc;
        b.sens_scratch = static_cast<double*>(sbuf);
    }
    kern<<<(unsigned)blocks, threads, smem, stream>>>(b, o);
    rc = cuda_check(cudaGetLastError(), "forward_kernel launch");
    if (sbuf) {
        const int rc2 = cuda_check(cudaFreeAsync(sbuf, stream), "cudaFreeAsync(sensitivity scratch)");
        if (!rc) rc = rc2;
    }
    return rc;
}

// Adjoint sensitivities: one warp per instance; per-group scratch holds every
// forward step (up to maxsteps + 2 points), dJy/dx per output and the
// quadrature history.  Shared memory per instance: the forward layout plus the
// backward problem's interpolant and flux work.
// CK: the check-point kernel (checkpoint_steps > 0), else the every-step
// kernel; the two are instantiated in separate translation units of a model
// library so that they compile in parallel.
template <class M, class LUT, class R, bool CK>
int launch_adjoint_v(const Batch& b_in, const Opts& o, cudaStream_t stream) {
    constexpr int G = 32;
    using LY = InstanceLayout<M, LUT, false>;
    constexpr size_t per_group = LY::bytes + BwdLayout<M>::bytes;
    constexpr size_t tb_bytes = ((sizeof(int) * (size_t)M::TB_TOTAL + 15) / 16) * 16;
    auto kern = [] {
        if constexpr (CK) return adjoint_ck_kernel<M, G, LUT, R>;
        else return adjoint_kernel<M, G, LUT, R>;
    }();
    Batch b = b_in;
    int dev = 0;
    int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    int smem_max = 0, nsm = 0;
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    long wpb = (long)b.n / nsm;
    if (wpb < 1) wpb = 1;
    if (wpb > 4) wpb = 4;
    const long wpb_smem = ((long)smem_max - (long)tb_bytes) / (long)per_group;
    if (wpb_smem < 1)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED,
                         "model too large for the adjoint kernel: one instance does not fit in shared memory");
    if (wpb > wpb_smem) wpb = wpb_smem;
    // automatic cap: instances of 48 KB or more run two per SM, and the on-chip
    // memory a third would take serves as L1 cache (spills, model tables); at
    // n = 100 that is 13% faster than three per SM
    const int ipsm = o.ipsm > 0 ? o.ipsm : (per_group >= 48 * 1024 ? 2 : 0);
    if (ipsm > 0 && wpb > ipsm) wpb = ipsm;
    const int threads = (int)(32 * wpb);
    const size_t smem = tb_bytes + (size_t)wpb * per_group;
    rc = cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "cudaFuncSetAttribute");
    if (rc) return rc;
    static std::atomic<bool> carved{false};
    if (ipsm <= 0) reset_carveout(kern, carved);
    int per_sm = 0;
    rc = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem),
                    "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if (rc) return rc;
    if (per_sm < 1) per_sm = 1;
    if (ipsm > 0) {
        const long cap_b = ipsm / wpb;
        per_sm = (int)(cap_b < 1 ? 1 : (cap_b < per_sm ? cap_b : per_sm));
        rc = apply_carveout(kern, per_sm, smem, dev);
        if (rc) return rc;
        carved = true;
    }
    long blocks = (b.n + wpb - 1) / wpb;
    if (blocks > (long)per_sm * nsm) blocks = (long)per_sm * nsm;
    if (blocks < 1) blocks = 1;
    long long stride_d;
    if (CK) {
        const AdjCkLayout lay{b.ck_k, (long long)o.maxsteps / b.ck_k + 2, b.nt, M::NX, b.nplist, ck_stride_of<M>()};
        b.ck_cap = lay.cap;
        stride_d = lay.stride(LMAX + 4);
    } else {
        const AdjLayout lay{(long long)o.maxsteps + 2, b.nt, M::NX, b.nplist};
        b.adj_cap = lay.cap;
        stride_d = lay.stride(LMAX + 4);
    }
    b.adj_stride = stride_d;
    const size_t groups = (size_t)blocks * (size_t)wpb;
    void* sbuf = nullptr;
    rc = cuda_check(cudaMallocAsync(&sbuf, groups * (size_t)b.adj_stride * sizeof(double), stream),
                    "cudaMallocAsync(adjoint scratch)");
    if (rc) return rc;
    b.adj_scratch = static_cast<double*>(sbuf);
    kern<<<(unsigned)blocks, threads, smem, stream>>>(b, o);
    rc = cuda_check(cudaGetLastError(), "adjoint_kernel launch");
    const int rc2 = cuda_check(cudaFreeAsync(sbuf, stream), "cudaFreeAsync(adjoint scratch)");
    return rc ? rc : rc2;
}

template <class M, class LUT, class R>
int launch_adjoint(const Batch& b, const Opts& o, cudaStream_t stream) {
    return b.ck_k > 0 ? launch_adjoint_v<M, LUT, R, true>(b, o, stream)
                      : launch_adjoint_v<M, LUT, R, false>(b, o, stream);
}

inline int lu_bits_of(const amici_gb300_solver_options* so) { return so->lu_precision == 64 ? 64 : 32; }
inline int ctl_bits_of(const amici_gb300_solver_options* so) { return so->control_precision == 64 ? 64 : 32; }

// adjoint kernel for the (LU, control) precision pair: both FP32 or both FP64
template <class M>
int launch_adjoint_bits(int bits, const Batch& b, const Opts& o, cudaStream_t stream) {
    if constexpr (M::HAS_ASA) {
        if (bits == 64) return launch_adjoint<M, double, double>(b, o, stream);
        return launch_adjoint<M, float, float>(b, o, stream);
    }
    return set_error(AMICI_GB300_ERR_UNSUPPORTED, "adjoint sensitivities are not compiled for this model");
}

// The pre-equilibration launch (one warp per instance): with sensitivities
// (forward sensitivities, or the adjoint's forward-sensitivity
// pre-equilibration) LU and control precision both 32 or both 64 bits
template <class M>
int launch_preeq(int lu_bits, int ctl_bits, bool sens, const Batch& b, const Opts& o, cudaStream_t s) {
    if constexpr (M::HAS_PREEQ) {
        if (sens) {
            if constexpr (M::HAS_FSA) {
                if (lu_bits == 64 && ctl_bits == 64) return launch_forward<M, 32, double, double, true, true>(b, o, s);
                if (lu_bits == 32 && ctl_bits == 32) return launch_forward<M, 32, float, float, true, true>(b, o, s);
                return set_error(AMICI_GB300_ERR_UNSUPPORTED,
                                 "pre-equilibration with sensitivities: lu_precision and control_precision are "
                                 "both 32 or both 64");
            }
            return set_error(AMICI_GB300_ERR_UNSUPPORTED,
                             "pre-equilibration with sensitivities needs the forward-sensitivity kernels, which "
                             "are not compiled for this model");
        }
        if (ctl_bits == 64) {
            if (lu_bits != 64)
                return set_error(AMICI_GB300_ERR_UNSUPPORTED, "FP64 control precision requires lu_precision 64");
            return launch_forward<M, 32, double, double, false, true>(b, o, s);
        }
        if (lu_bits == 64) return launch_forward<M, 32, double, float, false, true>(b, o, s);
        return launch_forward<M, 32, float, float, false, true>(b, o, s);
    }
    return set_error(AMICI_GB300_ERR_UNSUPPORTED, "pre-equilibration is not compiled for this model");
}

// The main launch with post-equilibration outputs (one warp per instance),
// in the precisions of the forward and forward-sensitivity kernels
template <class M>
int launch_posteq(int lu_bits, int ctl_bits, bool sens, const Batch& b, const Opts& o, cudaStream_t s) {
    if constexpr (M::HAS_POSTEQ) {
        if (sens) {
            if constexpr (M::HAS_FSA) {
                if (lu_bits == 64 && ctl_bits == 64)
                    return launch_forward<M, 32, double, double, true, false, true>(b, o, s);
                if (lu_bits == 32 && ctl_bits == 32)
                    return launch_forward<M, 32, float, float, true, false, true>(b, o, s);
                return set_error(AMICI_GB300_ERR_UNSUPPORTED,
                                 "forward sensitivities: lu_precision and control_precision are both 32 or both 64");
            }
            return set_error(AMICI_GB300_ERR_UNSUPPORTED, "forward sensitivities are not compiled for this model");
        }
        if (ctl_bits == 64) {
            if (lu_bits != 64)
                return set_error(AMICI_GB300_ERR_UNSUPPORTED, "FP64 control precision requires lu_precision 64");
            return launch_forward<M, 32, double, double, false, false, true>(b, o, s);
        }
        if (lu_bits == 64) return launch_forward<M, 32, double, float, false, false, true>(b, o, s);
        return launch_forward<M, 32, float, float, false, false, true>(b, o, s);
    }
    return set_error(AMICI_GB300_ERR_UNSUPPORTED, "post-equilibration is not compiled for this model");
}

template <class M, int G>
int launch_if_compiled(const Batch& b, const Opts& o, cudaStream_t s) {
    if constexpr ((M::LANE_MASK >> (G == 1 ? 0 : G == 2 ? 1 : G == 4 ? 2 : G == 8 ? 3 : G == 16 ? 4 : 5)) & 1)
        return launch_forward<M, G, float, float>(b, o, s);
    return set_error(AMICI_GB300_ERR_UNSUPPORTED,
                     "lanes_per_instance not compiled for this model (too many elements per lane)");
}

template <class M>
int dispatch_G(int G, const Batch& b, const Opts& o, cudaStream_t s) {
    switch (G) {
    case 1: return launch_if_compiled<M, 1>(b, o, s);
    case 2: return launch_if_compiled<M, 2>(b, o, s);
    case 4: return launch_if_compiled<M, 4>(b, o, s);
    case 8: return launch_if_compiled<M, 8>(b, o, s);
    case 16: return launch_if_compiled<M, 16>(b, o, s);
    case 32: return launch_forward<M, 32, float, float>(b, o, s);
    default: return set_error(AMICI_GB300_ERR_ARG, "lanes_per_instance must be 0,1,2,4,8,16,32");
    }
}

// FP32 LU with FP32 control (default, any compiled G), FP64 LU with FP32
// control or the all-FP64 variant (FP64 LU and FP64 control): one warp per
// instance.  Forward sensitivities: one warp per instance.
template <class M>
int dispatch(int G, int lu_bits, int ctl_bits, const Batch& b, const Opts& o, cudaStream_t s, bool sens = false) {
    if (sens) {
        if constexpr (M::HAS_FSA) {
            if (ctl_bits == 64 && lu_bits == 64) return launch_forward<M, 32, double, double, true>(b, o, s);
            if (ctl_bits == 64 || lu_bits == 64)
                return set_error(AMICI_GB300_ERR_UNSUPPORTED,
                                 "forward sensitivities: lu_precision and control_precision are both 32 or both 64");
            return launch_forward<M, 32, float, float, true>(b, o, s);
        }
        return set_error(AMICI_GB300_ERR_UNSUPPORTED, "forward sensitivities are not compiled for this model");
    }
    if (lu_bits == 64 || ctl_bits == 64) {
        if (G != 32)
            return set_error(AMICI_GB300_ERR_UNSUPPORTED, "FP64 LU or control precision requires 32 lanes per instance");
        if (ctl_bits == 64) {
            if (lu_bits != 64)
                return set_error(AMICI_GB300_ERR_UNSUPPORTED, "FP64 control precision requires lu_precision 64");
            return launch_forward<M, 32, double, double>(b, o, s);
        }
        return launch_forward<M, 32, double, float>(b, o, s);
    }
    return dispatch_G<M>(G, b, o, s);
}

// Lanes per instance when the caller leaves the choice to the library: the
// smallest G that still puts about four groups' worth of warps on every SM
// (FP64 issue is per warp instruction, so fewer lanes per instance is
// cheaper per instance as long as the SMs stay busy).
template <class M>
int pick_lanes(int n_instances, int nsm) {
    const long target_warps = 4L * nsm;
    int G = 1;
    while (G < 32 && ((long)n_instances * G) / 32 < target_warps) G *= 2;
    while (G < 32 && !((M::LANE_MASK >> (31 - __builtin_clz(G))) & 1)) G *= 2;  // compiled variants only
    return G;
}

template <class M>
int run_device(const amici_gb300_solver_options* so, const amici_gb300_batch* bb, cudaStream_t stream) {
    if (!so || !bb) return set_error(AMICI_GB300_ERR_ARG, "NULL options or batch");
    if (bb->n_instances < 0 || bb->nt < 0) return set_error(AMICI_GB300_ERR_ARG, "negative size");
    if (bb->n_instances == 0) return AMICI_GB300_OK;
    if (!bb->p && M::NP > 0) return set_error(AMICI_GB300_ERR_ARG, "p is NULL");
    if (!bb->k && M::NK > 0) return set_error(AMICI_GB300_ERR_ARG, "k is NULL");
    if (!bb->ts && bb->nt > 0) return set_error(AMICI_GB300_ERR_ARG, "ts is NULL");
    if (!bb->llh || !bb->numsteps || !bb->status) return set_error(AMICI_GB300_ERR_ARG, "llh/numsteps/status NULL");
    const bool sens = so->sensi_order > 0;
    const bool adj = sens && so->sensi_meth == AMICI_GB300_SENSI_ADJOINT;
    if (sens && so->sensi_meth != AMICI_GB300_SENSI_FORWARD && !adj)
        return set_error(AMICI_GB300_ERR_ARG, "sensi_meth must be forward or adjoint");
    if (sens && (bb->nplist <= 0 || bb->nplist > M::NP || !bb->plist))
        return set_error(AMICI_GB300_ERR_ARG, "sensitivities need plist with 1..np entries");
    if (sens && !adj && so->launch_mode == 1)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED, "forward sensitivities use the batched launch mode");
    if (adj && lu_bits_of(so) != ctl_bits_of(so))
        return set_error(AMICI_GB300_ERR_UNSUPPORTED,
                         "adjoint sensitivities: lu_precision and control_precision are both 32 or both 64");
    const bool preeq = bb->k_preeq != nullptr;
    if (preeq && so->launch_mode == 1)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED, "pre-equilibration uses the batched launch mode");
    // events are handled in the forward simulation (with or without forward
    // sensitivities) only
    if (M::NE > 0 && adj)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED, "adjoint sensitivities of a model with events are not available");
    if (M::NE > 0 && preeq)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED, "pre-equilibration of a model with events is not available");
    const bool posteq = bb->posteq != 0;
    if (posteq && adj)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED, "adjoint sensitivities with post-equilibration are not available");
    if (posteq && M::NE > 0)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED, "post-equilibration of a model with events is not available");
    if (posteq && so->launch_mode == 1)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED, "post-equilibration uses the batched launch mode");
    Batch b{};
    b.n = bb->n_instances;
    b.nt = bb->nt;
    b.nplist = bb->nplist;
    b.ck_k = so->checkpoint_steps > 0 ? so->checkpoint_steps : 0;
    b.p = bb->p;
    b.pscale = bb->pscale;
    b.k = bb->k;
    b.ts = bb->ts;
    b.my = bb->my;
    b.sigma_y = bb->sigma_y;
    b.plist = bb->plist;
    b.x = bb->x;
    b.y = bb->y;
    b.sigmay = bb->sigmay;
    b.llh = bb->llh;
    b.sx = bb->sx;
    b.sy = bb->sy;
    b.sllh = bb->sllh;
    b.numsteps = bb->numsteps;
    b.status = bb->status;
    b.diag = bb->diag;
    b.x0 = bb->x0;
    b.sx0 = sens ? bb->sx0 : nullptr;
    b.posteq_status = bb->posteq_status;
    b.posteq_numsteps = bb->posteq_numsteps;
    b.posteq_t = bb->posteq_t;
    b.posteq_wrms = bb->posteq_wrms;
    if (!sens) b.nplist = 0;
    Opts o = make_opts(so);
    int dev = 0, nsm = 0;
    int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int lu_bits = so->lu_precision == 64 ? 64 : 32;
    const int ctl_bits = so->control_precision == 64 ? 64 : 32;
    int G = so->lanes_per_instance > 0 ? so->lanes_per_instance : pick_lanes<M>(b.n, nsm);
    if ((ctl_bits == 64 || lu_bits == 64) && so->lanes_per_instance <= 0) G = 32;
    // scratch: work-queue counters (one per launch), stream-ordered
    const size_t nq = so->launch_mode == 1 ? (size_t)b.n : 1;
    void* q = nullptr;
    rc = cuda_check(cudaMallocAsync(&q, (nq + (preeq ? 1 : 0)) * sizeof(unsigned int) + 256, stream),
                    "cudaMallocAsync(queue)");
    if (rc) return rc;
    rc = cuda_check(cudaMemsetAsync(q, 0, (nq + (preeq ? 1 : 0)) * sizeof(unsigned int) + 256, stream),
                    "cudaMemsetAsync(queue)");
    void* pre = nullptr;  // steady-state results the caller does not take
    if (!rc && preeq) {
        // the pre-equilibration launch at k_preeq; the main launch starts from its steady state
        const size_t n = (size_t)b.n, npl = sens ? (size_t)b.nplist : 0;
        const size_t nd = (bb->x_ss ? 0 : n * M::NX) + (sens && !bb->sx_ss ? n * npl * M::NX : 0) +
                          (bb->preeq_t ? 0 : n) + (bb->preeq_wrms ? 0 : n),
                     ni = (bb->preeq_status ? 0 : n) + (bb->preeq_numsteps ? 0 : n);
        rc = cuda_check(cudaMallocAsync(&pre, nd * sizeof(double) + ni * sizeof(int32_t) + 256, stream),
                        "cudaMallocAsync(pre-equilibration results)");
        if (!rc) {
            double* d = static_cast<double*>(pre);
            auto take = [&](double* given, size_t cnt) {
                if (given) return given;
                double* r = d;
                d += cnt;
                return r;
            };
            Batch bp = b;
            bp.preeq = 1;
            bp.k = bb->k_preeq;
            bp.x = bp.y = bp.sigmay = bp.sx = bp.sy = bp.sllh = nullptr;
            bp.x_ss = take(bb->x_ss, n * M::NX);
            bp.sx_ss = sens ? take(bb->sx_ss, n * npl * M::NX) : nullptr;
            bp.preeq_t = take(bb->preeq_t, n);
            bp.preeq_wrms = take(bb->preeq_wrms, n);
            int32_t* di = reinterpret_cast<int32_t*>(d);
            bp.preeq_status = bb->preeq_status ? bb->preeq_status : di;
            di += bb->preeq_status ? 0 : n;
            bp.preeq_numsteps = bb->preeq_numsteps ? bb->preeq_numsteps : di;
            bp.queue = static_cast<unsigned int*>(q) + nq;
            rc = launch_preeq<M>(lu_bits, ctl_bits, sens, bp, o, stream);
            b.x0 = bp.x_ss;
            b.sx0 = bp.sx_ss;
            b.preeq_in = bp.preeq_status;
        }
    }
    if (!rc && so->launch_mode == 1) {
        // one launch per instance (the unbatched baseline): a one-instance view per launch
        for (int i = 0; i < b.n && !rc; i++) {
            Batch bi = b;
            bi.n = 1;
            bi.p = b.p + (size_t)i * M::NP;
            bi.k = b.k ? b.k + (size_t)i * M::NK : nullptr;
            bi.ts = b.ts + (size_t)i * b.nt;
            bi.my = b.my ? b.my + (size_t)i * b.nt * M::NY : nullptr;
            bi.sigma_y = b.sigma_y ? b.sigma_y + (size_t)i * b.nt * M::NY : nullptr;
            bi.x = b.x ? b.x + (size_t)i * b.nt * M::NX : nullptr;
            bi.y = b.y ? b.y + (size_t)i * b.nt * M::NY : nullptr;
            bi.sigmay = b.sigmay ? b.sigmay + (size_t)i * b.nt * M::NY : nullptr;
            bi.llh = b.llh + i;
            bi.numsteps = b.numsteps + (size_t)i * b.nt;
            bi.status = b.status + i;
            bi.diag = b.diag ? b.diag + (size_t)i * 8 : nullptr;
            bi.sllh = b.sllh ? b.sllh + (size_t)i * b.nplist : nullptr;
            bi.x0 = b.x0 ? b.x0 + (size_t)i * M::NX : nullptr;
            bi.sx0 = b.sx0 ? b.sx0 + (size_t)i * b.nplist * M::NX : nullptr;
            bi.queue = static_cast<unsigned int*>(q) + i;
            if (adj) rc = launch_adjoint_bits<M>(lu_bits, bi, o, stream);
            else rc = dispatch<M>(G, lu_bits, ctl_bits, bi, o, stream);
        }
    } else if (!rc && adj) {
        b.queue = static_cast<unsigned int*>(q);
        rc = launch_adjoint_bits<M>(lu_bits, b, o, stream);
    } else if (!rc && posteq) {
        b.queue = static_cast<unsigned int*>(q);
        rc = launch_posteq<M>(lu_bits, ctl_bits, sens, b, o, stream);
    } else if (!rc) {
        b.queue = static_cast<unsigned int*>(q);
        rc = dispatch<M>(G, lu_bits, ctl_bits, b, o, stream, sens);
    }
    if (pre) {
        const int rc3 = cuda_check(cudaFreeAsync(pre, stream), "cudaFreeAsync(pre-equilibration results)");
        if (!rc) rc = rc3;
    }
    const int rc2 = cuda_check(cudaFreeAsync(q, stream), "cudaFreeAsync(queue)");
    return rc ? rc : rc2;
}

// Host-buffer entry: device buffers cached per library (guarded by a mutex).
struct HostCache {
    std::mutex mu;
    void* dbuf = nullptr;
    size_t cap = 0;
};

inline HostCache& host_cache() {
    static HostCache c;
    return c;
}

template <class M>
int run_host(const amici_gb300_solver_options* so, const amici_gb300_batch* hb, cudaStream_t stream) {
    if (!so || !hb) return set_error(AMICI_GB300_ERR_ARG, "NULL options or batch");
    const size_t n = (size_t)hb->n_instances, nt = (size_t)hb->nt;
    if (hb->n_instances < 0 || hb->nt < 0) return set_error(AMICI_GB300_ERR_ARG, "negative size");
    if (n == 0) return AMICI_GB300_OK;
    const size_t sz_p = n * M::NP, sz_k = n * M::NK, sz_ts = n * nt, sz_my = hb->my ? n * nt * M::NY : 0,
                 sz_sg = hb->sigma_y ? n * nt * M::NY : 0, sz_x = hb->x ? n * nt * M::NX : 0,
                 sz_y = hb->y ? n * nt * M::NY : 0, sz_sgy = hb->sigmay ? n * nt * M::NY : 0;
    const bool sens = so->sensi_order > 0 && hb->nplist > 0;
    const size_t npl = sens ? (size_t)hb->nplist : 0;
    const bool fsa = sens && so->sensi_meth == AMICI_GB300_SENSI_FORWARD;
    const size_t sz_sx = (fsa && hb->sx) ? n * nt * npl * M::NX : 0, sz_sy = (fsa && hb->sy) ? n * nt * npl * M::NY : 0,
                 sz_sllh = (sens && hb->sllh) ? n * npl : 0;
    // initial-state overrides and pre-equilibration
    const bool pe = hb->k_preeq != nullptr;
    const size_t sz_kp = pe ? n * M::NK : 0, sz_x0 = hb->x0 ? n * M::NX : 0,
                 sz_sx0 = (sens && hb->sx0) ? n * npl * M::NX : 0, sz_xss = (pe && hb->x_ss) ? n * M::NX : 0,
                 sz_sxss = (pe && sens && hb->sx_ss) ? n * npl * M::NX : 0, sz_pt = (pe && hb->preeq_t) ? n : 0,
                 sz_pw = (pe && hb->preeq_wrms) ? n : 0, sz_ps = (pe && hb->preeq_status) ? n : 0,
                 sz_pn = (pe && hb->preeq_numsteps) ? n : 0;
    // post-equilibration: requested, or output times at inf
    bool po = hb->posteq != 0;
    for (size_t e = 0; e < n * nt && !po && hb->ts; e++) po = isinf(hb->ts[e]) != 0;
    const size_t sz_qt = (po && hb->posteq_t) ? n : 0, sz_qw = (po && hb->posteq_wrms) ? n : 0,
                 sz_qs = (po && hb->posteq_status) ? n : 0, sz_qn = (po && hb->posteq_numsteps) ? n : 0;
    const size_t n_dbl = sz_p + sz_k + sz_ts + sz_my + sz_sg + sz_x + sz_y + sz_sgy + n + sz_sx + sz_sy + sz_sllh +
                         sz_kp + sz_x0 + sz_sx0 + sz_xss + sz_sxss + sz_pt + sz_pw + sz_qt + sz_qw;
    const size_t n_int = M::NP + n * nt + n + (hb->diag ? 8 * n : 0) + npl + sz_ps + sz_pn + sz_qs + sz_qn;
    const size_t bytes = (n_dbl * sizeof(double) + n_int * sizeof(int32_t) + 4096);
    HostCache& hc = host_cache();
    std::lock_guard<std::mutex> lock(hc.mu);
    if (hc.cap < bytes) {
        if (hc.dbuf) cudaFree(hc.dbuf);
        hc.dbuf = nullptr;
        hc.cap = 0;
        int rc = cuda_check(cudaMalloc(&hc.dbuf, bytes), "cudaMalloc(host-path buffers)");
        if (rc) return rc;
        hc.cap = bytes;
    }
    double* d = static_cast<double*>(hc.dbuf);
    amici_gb300_batch db = *hb;
    auto put = [&](const double* src, size_t cnt) -> double* {
        if (!src || cnt == 0) return nullptr;
        double* dst = d;
        d += cnt;
        cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyHostToDevice, stream);
        return dst;
    };
    auto take = [&](double* src_host, size_t cnt) -> double* {
        if (!src_host || cnt == 0) return nullptr;
        double* dst = d;
        d += cnt;
        return dst;
    };
    db.p = put(hb->p, sz_p);
    db.k = put(hb->k, sz_k);
    db.ts = put(hb->ts, sz_ts);
    db.my = put(hb->my, sz_my);
    db.sigma_y = put(hb->sigma_y, sz_sg);
    db.x = take(hb->x, sz_x);
    db.y = take(hb->y, sz_y);
    db.sigmay = take(hb->sigmay, sz_sgy);
    db.llh = take(hb->llh, n);
    db.sx = take(hb->sx, sz_sx);
    db.sy = take(hb->sy, sz_sy);
    db.sllh = take(hb->sllh, sz_sllh);
    db.k_preeq = put(hb->k_preeq, sz_kp);
    if (pe && !db.k_preeq) db.k_preeq = d;  // a model without fixed parameters: any non-NULL pointer
    db.x0 = put(hb->x0, sz_x0);
    db.sx0 = put(hb->sx0, sz_sx0);
    db.x_ss = take(hb->x_ss, sz_xss);
    db.sx_ss = take(hb->sx_ss, sz_sxss);
    db.preeq_t = take(hb->preeq_t, sz_pt);
    db.preeq_wrms = take(hb->preeq_wrms, sz_pw);
    db.posteq = po ? 1 : 0;
    db.posteq_t = take(hb->posteq_t, sz_qt);
    db.posteq_wrms = take(hb->posteq_wrms, sz_qw);
    int32_t* di = reinterpret_cast<int32_t*>(d);
    if (hb->pscale) {
        cudaMemcpyAsync(di, hb->pscale, M::NP * sizeof(int32_t), cudaMemcpyHostToDevice, stream);
        db.pscale = di;
    }
    di += M::NP;
    db.numsteps = di;
    di += n * nt;
    db.status = di;
    di += n;
    db.diag = hb->diag ? di : nullptr;
    di += hb->diag ? 8 * n : 0;
    db.plist = nullptr;
    if (sens) {
        cudaMemcpyAsync(di, hb->plist, npl * sizeof(int32_t), cudaMemcpyHostToDevice, stream);
        db.plist = di;
        di += npl;
    }
    db.preeq_status = sz_ps ? di : nullptr;
    di += sz_ps;
    db.preeq_numsteps = sz_pn ? di : nullptr;
    di += sz_pn;
    db.posteq_status = sz_qs ? di : nullptr;
    di += sz_qs;
    db.posteq_numsteps = sz_qn ? di : nullptr;
    di += sz_qn;
    int rc = run_device<M>(so, &db, stream);
    if (rc) return rc;
    auto get = [&](double* dst, const double* src, size_t cnt) {
        if (dst && src && cnt) cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyDeviceToHost, stream);
    };
    get(hb->x, db.x, sz_x);
    get(hb->y, db.y, sz_y);
    get(hb->sigmay, db.sigmay, sz_sgy);
    get(hb->llh, db.llh, n);
    get(hb->sx, db.sx, sz_sx);
    get(hb->sy, db.sy, sz_sy);
    get(hb->sllh, db.sllh, sz_sllh);
    get(hb->x_ss, db.x_ss, sz_xss);
    get(hb->sx_ss, db.sx_ss, sz_sxss);
    get(hb->preeq_t, db.preeq_t, sz_pt);
    get(hb->preeq_wrms, db.preeq_wrms, sz_pw);
    if (sz_ps) cudaMemcpyAsync(hb->preeq_status, db.preeq_status, n * sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if (sz_pn) cudaMemcpyAsync(hb->preeq_numsteps, db.preeq_numsteps, n * sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    get(hb->posteq_t, db.posteq_t, sz_qt);
    get(hb->posteq_wrms, db.posteq_wrms, sz_qw);
    if (sz_qs) cudaMemcpyAsync(hb->posteq_status, db.posteq_status, n * sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if (sz_qn) cudaMemcpyAsync(hb->posteq_numsteps, db.posteq_numsteps, n * sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(hb->numsteps, db.numsteps, n * nt * sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(hb->status, db.status, n * sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if (hb->diag) cudaMemcpyAsync(hb->diag, db.diag, 8 * n * sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    return cuda_check(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
}

}  // namespace agb

#define AMICI_GB300_DEFINE_ABI(MODEL)                                                               \
    extern "C" {                                                                                    \
    int32_t amici_gb300_abi_version(void) { return AMICI_GB300_ABI_VERSION; }                      \
    const char* amici_gb300_model_name(void) { return MODEL::NAME; }                                \
    int32_t amici_gb300_model_dims_get(amici_gb300_model_dims* out) {                               \
        if (!out) return AMICI_GB300_ERR_ARG;                                                       \
        out->nx = MODEL::NX;                                                                        \
        out->np = MODEL::NP;                                                                        \
        out->nk = MODEL::NK;                                                                        \
        out->ny = MODEL::NY;                                                                        \
        out->nw = MODEL::NW;                                                                        \
        out->nnz_jac = MODEL::NNZ_J;                                                                \
        return AMICI_GB300_OK;                                                                      \
    }                                                                                               \
    void amici_gb300_default_options(amici_gb300_solver_options* out) {                            \
        if (out) agb::default_options(out);                                                         \
    }                                                                                               \
    int32_t amici_gb300_run_simulations_device(const amici_gb300_solver_options* opts,             \
                                               const amici_gb300_batch* batch, void* stream) {      \
        agb::g_last_error[0] = 0;                                                                   \
        return agb::run_device<MODEL>(opts, batch, static_cast<cudaStream_t>(stream));             \
    }                                                                                               \
    int32_t amici_gb300_run_simulations_host(const amici_gb300_solver_options* opts,               \
                                             const amici_gb300_batch* batch, void* stream) {        \
        agb::g_last_error[0] = 0;                                                                   \
        return agb::run_host<MODEL>(opts, batch, static_cast<cudaStream_t>(stream));               \
    }                                                                                               \
    const char* amici_gb300_last_error(void) { return agb::g_last_error; }                         \
    }
