"""The allocation-free device entry point against the regular one.

``amici_gb300_run_simulations_device_noalloc`` is for callers that cannot let
a library allocate device memory (an application that owns all device memory
through its own pool, or a latency-critical caller that cannot afford an
allocator stall): it keeps the persistent kernel's work-queue counters in a
fixed device array of the library instead of allocating them per call.  It
must produce what the regular device entry point produces, on consecutive
calls (the array keeps the previous call's counters), and refuse requests
that need more counters than the array holds.

This file is collected last so that a run stopping at the first failure has
run every other test before it; it also passes on its own in a fresh process.
"""
import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300 import _native
from amici_gb300.networks import net20_workload

pytestmark = pytest.mark.gpu

N = 256


def _device_batch(torch, dev, w, n):
    nt, nx, ny = w.ts.shape[1], w.model.nx, w.model.ny
    T = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a)).to(dev, dt)
    bufs = dict(p=T(w.p[:n]), ts=T(w.ts[:n]), pscale=T(w.pscale, torch.int32),
                x=torch.full((n, nt, nx), float("nan"), dtype=torch.float64, device=dev),
                llh=torch.zeros(n, dtype=torch.float64, device=dev),
                numsteps=torch.zeros((n, nt), dtype=torch.int32, device=dev),
                status=torch.full((n,), -7, dtype=torch.int32, device=dev))
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


def test_noalloc_matches_allocating_entry_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    w = net20_workload(1024)
    model = ag.Model(w.model)
    solver = ag.Solver()
    solver.set_relative_tolerance(w.rtol)
    solver.set_absolute_tolerance(w.atol)
    opts = solver.to_options()
    lib = model.library
    stream = torch.cuda.current_stream(dev).cuda_stream

    b_ref, ref_bufs = _device_batch(torch, dev, w, N)
    lib.run_device(opts, b_ref, stream)
    torch.cuda.synchronize(dev)
    ref = _host(ref_bufs)
    assert (ref["status"] == 0).all()

    for call in range(2):  # consecutive calls reuse the library's counter array
        b, bufs = _device_batch(torch, dev, w, N)
        lib.run_device_noalloc(opts, b, stream)
        torch.cuda.synchronize(dev)
        got = _host(bufs)
        np.testing.assert_array_equal(got["status"], ref["status"], err_msg=f"call {call}")
        np.testing.assert_array_equal(got["numsteps"], ref["numsteps"], err_msg=f"call {call}")
        # same kernel on the same inputs: identical up to the tolerance of the parity tests
        tol = w.rtol * np.abs(ref["x"]) + w.atol
        assert np.all(np.abs(got["x"] - ref["x"]) <= tol), f"call {call}"
        np.testing.assert_allclose(got["llh"], ref["llh"], rtol=1e-12, equal_nan=True)


def test_noalloc_rejects_more_counters_than_it_holds():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    w = net20_workload(1024)
    model = ag.Model(w.model)
    solver = ag.Solver()
    solver.set_launch_mode(1)  # one counter per instance
    n = 4097
    reps = int(np.ceil(n / w.n))
    big = w.subset(np.tile(np.arange(w.n), reps)[:n])
    b, _ = _device_batch(torch, dev, big, n)
    with pytest.raises(_native.EngineError, match="at most AMICI_GB300_NOALLOC_MAX_COUNTERS"):
        model.library.run_device_noalloc(solver.to_options(), b, torch.cuda.current_stream(dev).cuda_stream)
