"""The allocation-free device entry point against the regular one.

``amici_gb300_run_simulations_device_noalloc`` is for callers that cannot let
a library allocate device memory (an application that owns all device memory
through its own pool, or a latency-critical caller that cannot afford an
allocator stall): it keeps the persistent kernel's work-queue counters in a
fixed device array of the library instead of allocating them per call, and
it runs forward simulation only.  It must produce what the regular device
entry point produces, bit for bit, on consecutive calls (the array keeps the
previous call's counters), allocate nothing (neither from the device's
stream-ordered pool nor through torch's allocator), and refuse what it cannot
do: sensitivities, and requests that need more counters than the array holds.

This file is collected last so that a run stopping at the first failure has
run every other test before it; it also passes on its own in a fresh process.
"""
import ctypes
import ctypes.util
import glob
import os

import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300 import _native
from amici_gb300.networks import net20_workload

pytestmark = pytest.mark.gpu

N = 256
# cudaMemPoolAttr values of the CUDA runtime API
_USED_MEM_CURRENT, _USED_MEM_HIGH, _RESERVED_MEM_HIGH = 0x7, 0x8, 0x6


def _cudart():
    """The CUDA runtime library, to read the device's default memory pool."""
    import torch
    names = [ctypes.util.find_library("cudart"), "/usr/local/cuda/lib64/libcudart.so"]
    names += sorted(glob.glob(os.path.join(os.path.dirname(torch.__file__), "lib", "libcudart*.so*")))
    for nm in names:
        if nm:
            try:
                return ctypes.CDLL(nm)
            except OSError:
                continue
    pytest.skip("libcudart not found")


class _PoolWatch:
    """High-water mark of the device's default stream-ordered memory pool
    (the pool cudaMallocAsync draws from), reset before a call."""

    def __init__(self, dev_index):
        self.rt = _cudart()
        self.pool = ctypes.c_void_p()
        assert self.rt.cudaDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev_index) == 0

    def _get(self, attr):
        v = ctypes.c_uint64()
        assert self.rt.cudaMemPoolGetAttribute(self.pool, attr, ctypes.byref(v)) == 0
        return v.value

    def reset(self):
        zero = ctypes.c_uint64(0)
        assert self.rt.cudaMemPoolSetAttribute(self.pool, _USED_MEM_HIGH, ctypes.byref(zero)) == 0
        return self._get(_USED_MEM_CURRENT)

    def high(self):
        return self._get(_USED_MEM_HIGH)


def _device_batch(torch, dev, w, n):
    nt, nx, ny = w.ts.shape[1], w.model.nx, w.model.ny
    T = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a)).to(dev, dt)
    bufs = dict(p=T(w.p[:n]), ts=T(w.ts[:n]), pscale=T(w.pscale, torch.int32),
                x=torch.full((n, nt, nx), float("nan"), dtype=torch.float64, device=dev),
                llh=torch.zeros(n, dtype=torch.float64, device=dev),
                numsteps=torch.zeros((n, nt), dtype=torch.int32, device=dev),
                status=torch.full((n,), -7, dtype=torch.int32, device=dev),
                sllh=torch.zeros((n, w.model.np), dtype=torch.float64, device=dev),
                plist=torch.arange(w.model.np, dtype=torch.int32, device=dev),
                my=torch.zeros((n, nt, ny), dtype=torch.float64, device=dev))
    b = _native.Batch()
    b.n_instances, b.nt, b.nplist = n, nt, 0
    b.p, b.pscale, b.ts = bufs["p"].data_ptr(), bufs["pscale"].data_ptr(), bufs["ts"].data_ptr()
    b.k = b.my = b.sigma_y = b.plist = None
    b.x, b.llh = bufs["x"].data_ptr(), bufs["llh"].data_ptr()
    b.y = b.sigmay = b.sx = b.sy = b.sllh = b.diag = None
    b.numsteps, b.status = bufs["numsteps"].data_ptr(), bufs["status"].data_ptr()
    return b, bufs


def _host(bufs):
    return {k: bufs[k].cpu().numpy() for k in ("x", "llh", "numsteps", "status")}


def _setup(torch):
    dev = torch.device("cuda", 0)
    w = net20_workload(1024)
    model = ag.Model(w.model)
    solver = ag.Solver()
    solver.set_relative_tolerance(w.rtol)
    solver.set_absolute_tolerance(w.atol)
    return dev, w, model, solver, torch.cuda.current_stream(dev).cuda_stream


@pytest.mark.parametrize("launch_mode,n", [(0, N), (1, 8)])
def test_noalloc_matches_allocating_entry_on_consecutive_calls(launch_mode, n):
    """Batched launch and one launch per instance (each with its own counter)."""
    torch = pytest.importorskip("torch")
    dev, w, model, solver, stream = _setup(torch)
    solver.set_launch_mode(launch_mode)
    opts = solver.to_options()
    lib = model.library
    pool = _PoolWatch(dev.index)

    b_ref, ref_bufs = _device_batch(torch, dev, w, n)
    pool.reset()
    lib.run_device(opts, b_ref, stream)
    torch.cuda.synchronize(dev)
    assert pool.high() > 0  # the regular entry point does draw scratch from the pool (the watch works)
    ref = _host(ref_bufs)
    assert (ref["status"] == 0).all()

    for call in range(2):  # consecutive calls reuse the library's counter array
        b, bufs = _device_batch(torch, dev, w, n)
        torch.cuda.synchronize(dev)
        torch_before = torch.cuda.memory_stats(dev).get("allocation.all.allocated", 0)
        used_before = pool.reset()
        lib.run_device_noalloc(opts, b, stream)
        torch.cuda.synchronize(dev)
        assert pool.high() <= used_before, f"call {call}: the stream-ordered pool grew"
        assert torch.cuda.memory_stats(dev).get("allocation.all.allocated", 0) == torch_before
        got = _host(bufs)
        # same kernel on the same inputs: bit-identical results
        for key in ("status", "numsteps", "x", "llh"):
            np.testing.assert_array_equal(got[key], ref[key], err_msg=f"call {call}: {key}")


def test_noalloc_refuses_sensitivities():
    """Forward simulation only: the sensitivity kernels need per-call scratch
    that this entry point does not allocate."""
    torch = pytest.importorskip("torch")
    dev, w, model, solver, stream = _setup(torch)
    b, bufs = _device_batch(torch, dev, w, 4)
    b.nplist, b.plist, b.sllh, b.my = w.model.np, bufs["plist"].data_ptr(), bufs["sllh"].data_ptr(), \
        bufs["my"].data_ptr()
    solver.set_sensitivity_order(ag.SensitivityOrder.first)
    for meth in (ag.SensitivityMethod.forward, ag.SensitivityMethod.adjoint):
        solver.set_sensitivity_method(meth)
        with pytest.raises(_native.EngineError, match="sensitivities are not available"):
            model.library.run_device_noalloc(solver.to_options(), b, stream)


def test_noalloc_rejects_more_counters_than_it_holds():
    torch = pytest.importorskip("torch")
    dev, w, model, solver, stream = _setup(torch)
    solver.set_launch_mode(1)  # one counter per instance
    n = 4097
    reps = int(np.ceil(n / w.n))
    big = w.subset(np.tile(np.arange(w.n), reps)[:n])
    b, _ = _device_batch(torch, dev, big, n)
    with pytest.raises(_native.EngineError, match="at most AMICI_GB300_NOALLOC_MAX_COUNTERS"):
        model.library.run_device_noalloc(solver.to_options(), b, stream)
