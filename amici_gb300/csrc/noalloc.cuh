// Allocation-free variant of the batched device entry point.
//
// The regular device entry point takes a few bytes of scratch memory per call
// (the work-queue counters the persistent kernel's groups use to pull
// instances) from the stream-ordered allocator.  Some callers cannot let a
// library enter the CUDA allocator at all: applications that reserve all
// device memory up front in their own pool and treat any further allocation as
// an error, and latency-critical callers for which a pool growth inside
// cudaMallocAsync (which may have to map new memory) is an unbounded stall at
// an unpredictable point.  For them, this entry point keeps the counters in a
// fixed, file-scope device array instead and allocates nothing.
//
// This header is included by exactly one translation unit of a model library
// (the generated abi.cu), so the array, the symbol lookup and the entry point
// live in the same file.
#pragma once

#include <mutex>

#include "abi.cuh"

// Work-queue counters shared by every call of the allocation-free entry point
// on a device; every GPU that loads the library holds this array until exit.
static __device__ __align__(256) unsigned int amici_gb300_noalloc_queue[AMICI_GB300_NOALLOC_MAX_COUNTERS];

namespace agb {
namespace noalloc {

constexpr int kMaxDevices = 64;

// Device address of the counter array, looked up once per device with that
// device current (the symbol's host-side name is not a device address).
inline int queue_address(unsigned int** out) {
    static std::mutex mu;
    static unsigned int* addr[kMaxDevices] = {};
    int dev = 0;
    int rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= kMaxDevices) return set_error(AMICI_GB300_ERR_UNSUPPORTED, "device ordinal too large");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        rc = cuda_check(cudaGetSymbolAddress(&p, amici_gb300_noalloc_queue), "cudaGetSymbolAddress");
        if (rc) return rc;
        addr[dev] = static_cast<unsigned int*>(p);
    }
    *out = addr[dev];
    return AMICI_GB300_OK;
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
    if (so->sensi_order > 0)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED, "sensitivities are not available in this entry point");
    if (bb->k_preeq)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED,
                         "pre-equilibration is not available in this entry point (its steady states need scratch)");
    if (bb->posteq)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED, "post-equilibration is not available in this entry point");
    const long counters = so->launch_mode == 1 ? (long)bb->n_instances : 1L;
    if (counters > AMICI_GB300_NOALLOC_MAX_COUNTERS)
        return set_error(AMICI_GB300_ERR_UNSUPPORTED,
                         "allocation-free entry point: per-instance launch mode needs one work-queue counter "
                         "per instance and at most AMICI_GB300_NOALLOC_MAX_COUNTERS (4096) are available");
    unsigned int* q = nullptr;
    int rc = queue_address(&q);
    if (rc) return rc;
    Batch b{};
    b.n = bb->n_instances;
    b.nt = bb->nt;
    b.nplist = bb->nplist;
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
    const Opts o = make_opts(so);
    int dev = 0, nsm = 0;
    rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int lu_bits = so->lu_precision == 64 ? 64 : 32;
    const int ctl_bits = so->control_precision == 64 ? 64 : 32;
    int G = so->lanes_per_instance > 0 ? so->lanes_per_instance : pick_lanes<M>(b.n, nsm);
    if ((ctl_bits == 64 || lu_bits == 64) && so->lanes_per_instance <= 0) G = 32;
    // the counters keep the previous call's values: zero the ones this call uses
    rc = cuda_check(cudaMemsetAsync(q, 0, (size_t)counters * sizeof(unsigned int), stream), "cudaMemsetAsync");
    if (rc) return rc;
    if (so->launch_mode == 1) {
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
            bi.x0 = b.x0 ? b.x0 + (size_t)i * M::NX : nullptr;
            bi.queue = q + i;
            rc = dispatch<M>(G, lu_bits, ctl_bits, bi, o, stream);
        }
        return rc;
    }
    b.queue = q;
    return dispatch<M>(G, lu_bits, ctl_bits, b, o, stream);
}

}  // namespace noalloc
}  // namespace agb

#define AMICI_GB300_DEFINE_NOALLOC_ABI(MODEL)                                                    \
    extern "C" int32_t amici_gb300_run_simulations_device_noalloc(                               \
        const amici_gb300_solver_options* opts, const amici_gb300_batch* batch, void* stream) {  \
        agb::g_last_error[0] = 0;                                                                \
        return agb::noalloc::run_device<MODEL>(opts, batch, static_cast<cudaStream_t>(stream)); \
    }
