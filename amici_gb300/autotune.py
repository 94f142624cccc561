"""Autotuner for the launch shape of the batched forward kernel.

The engine compiles one forward kernel per lanes-per-instance choice G (the
group of lanes that integrates one instance; 32 / G instances per warp) that
keeps every lane at a few state elements (``codegen.lane_choices``).  Which G
is fastest depends on the model size, the batch size and the step counts
(fewer lanes per instance cost less FP64 issue per instance but leave the SMs
with fewer independent instruction streams when the batch is small).  The
library's built-in choice is a static rule (``pick_lanes`` in the C ABI);
``tune_lanes`` replaces it with a measurement: it times every compiled G on a
sample of the caller's batch with CUDA events on the device entry point and
returns the fastest, caching the result per (model, batch-size bucket,
precision).  ``Solver.set_lanes_per_instance`` applies it.
"""
from __future__ import annotations

import math

import numpy as np

from . import _native
from .codegen import lane_choices

_CACHE: dict[tuple, dict] = {}


def _bucket(n: int) -> int:
    return 1 << max(0, int(math.ceil(math.log2(max(n, 1)))))


def tune_lanes(model, solver, p, k, ts, *, pscale=None, sample: int | None = None, reps: int = 2,
               candidates=None) -> dict:
    """Time the forward kernel for each compiled lanes-per-instance choice.

    ``p, k, ts`` are the batch's host arrays (``[N, ...]``); the first
    ``sample`` rows (default: all) are timed ``reps`` times per candidate after
    one warm-up call.  Returns ``{"best": G, "ms": {G: ms}, "n": rows}`` and
    caches it per (model, batch-size bucket, LU and control precision).
    All-FP64 variants only exist for G = 32 and are not tuned.
    """
    import torch

    spec = model.spec
    p = np.atleast_2d(np.asarray(p, dtype=np.float64))
    n = p.shape[0] if sample is None else min(sample, p.shape[0])
    key = (spec.name, _bucket(n), solver.lu_precision, solver.control_precision)
    if key in _CACHE:
        return _CACHE[key]
    if solver.lu_precision == 64 or solver.control_precision == 64:
        res = {"best": 32, "ms": {}, "n": n}
        _CACHE[key] = res
        return res
    dev = torch.device("cuda", torch.cuda.current_device())
    ts = np.ascontiguousarray(np.broadcast_to(ts, (p.shape[0], np.shape(ts)[-1]))[:n])
    nt = ts.shape[1]
    T = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a)).to(dev, dt)
    dp = T(p[:n])
    dts = T(ts)
    dk = T(np.broadcast_to(k, (p.shape[0], spec.nk))[:n] if spec.nk else np.zeros((n, 0)))
    dps = T(model.get_parameter_scale() if pscale is None else pscale, torch.int32)
    dx = torch.empty((n, nt, spec.nx), dtype=torch.float64, device=dev)
    llh = torch.empty(n, dtype=torch.float64, device=dev)
    ns = torch.empty((n, nt), dtype=torch.int32, device=dev)
    st = torch.empty(n, dtype=torch.int32, device=dev)
    b = _native.Batch()
    b.n_instances, b.nt, b.nplist = n, nt, 0
    b.p, b.pscale, b.k, b.ts = dp.data_ptr(), dps.data_ptr(), dk.data_ptr() if spec.nk else None, dts.data_ptr()
    b.my = b.sigma_y = b.plist = None
    b.x, b.llh = dx.data_ptr(), llh.data_ptr()
    b.y = b.sigmay = b.sx = b.sy = b.sllh = b.diag = None
    b.numsteps, b.status = ns.data_ptr(), st.data_ptr()
    stream = torch.cuda.current_stream(dev)
    lib = model.library
    cands = tuple(candidates or lane_choices(spec))
    times = {}
    for G in cands:
        opts = solver.to_options()
        opts.sensi_order = 0
        opts.lanes_per_instance = G
        lib.run_device(opts, b, stream.cuda_stream)  # warm-up
        best = math.inf
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lib.run_device(opts, b, stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            best = min(best, e0.elapsed_time(e1))
        times[G] = best
    res = {"best": min(times, key=times.get), "ms": times, "n": n}
    _CACHE[key] = res
    return res
