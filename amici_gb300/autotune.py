"""Autotuners for the launch shape of the batched kernels.

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

``tune_instances_per_sm`` does the same for the sensitivity kernels' cap on
resident instances per SM (``Solver.set_instances_per_sm``).
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


def _time_sensitivity_call(model, solver, theta, k, ts, my, method, reps) -> float:
    """Best of ``reps`` CUDA-event times (ms) of one sensitivity call, after
    one untimed call."""
    import torch

    from .autograd import log_likelihood_and_gradient

    dev = theta.device
    stream = torch.cuda.current_stream(dev)
    log_likelihood_and_gradient(model, solver, theta, k, ts, my, method=method)
    best = math.inf
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        log_likelihood_and_gradient(model, solver, theta, k, ts, my, method=method)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        best = min(best, e0.elapsed_time(e1))
    return best


def tune_instances_per_sm(model, solver, theta, k, ts, my, *, candidates=(0, 1, 2, 3, 4), sample=None,
                          reps=1, method=None) -> dict:
    """Time the sensitivity kernels for each cap on resident instances per SM.

    The adjoint and forward-sensitivity kernels are latency-bound per
    instance; fewer resident instances leave more on-chip memory to L1 and
    run each instance faster, more resident instances hide more latency.
    Which wins depends on the model size and the batch (n = 100 adjoint: two
    per SM beat three by 13%; forward sensitivities at n = 50: uncapped
    beats every cap).  ``theta, k, ts, my`` are the batch's inputs (arrays or
    CUDA tensors); the first ``sample`` rows are timed.  0 stands for the
    library's automatic launch.  Returns ``{"best": cap, "ms": {cap: ms},
    "n": rows}``, cached per (model, batch-size bucket, precision, method);
    ``Solver.set_instances_per_sm(result["best"])`` applies it."""
    import torch

    from .simulation import SensitivityMethod, Solver

    method = SensitivityMethod.adjoint if method is None else method
    if any(int(c) < 0 for c in candidates) or not candidates:
        raise ValueError("candidates are caps >= 0 (0: automatic)")
    spec = model.spec
    dev = torch.device("cuda", torch.cuda.current_device())
    T = lambda a: torch.as_tensor(a, dtype=torch.float64).to(dev)  # noqa: E731
    theta = T(theta)
    theta = theta.unsqueeze(0) if theta.dim() == 1 else theta
    n = theta.shape[0] if sample is None else min(sample, theta.shape[0])
    key = ("ipsm", spec.name, _bucket(n), solver.lu_precision, solver.control_precision, int(method),
           tuple(int(c) for c in candidates))
    if key in _CACHE:
        return _CACHE[key]
    k = T(k if spec.nk else np.zeros((theta.shape[0], 0)))
    ts = T(ts)
    my = T(my)
    rows = slice(0, n)
    kk = k.expand(theta.shape[0], spec.nk)[rows]
    tt = ts.expand(theta.shape[0], ts.shape[-1])[rows]
    mm = my.expand(theta.shape[0], tt.shape[1], spec.ny)[rows]
    times = {}
    for c in candidates:
        s = Solver()
        s.__dict__.update(solver.__dict__)
        s.set_instances_per_sm(int(c))
        times[int(c)] = _time_sensitivity_call(model, s, theta[rows], kk, tt, mm, method, reps)
    res = {"best": min(times, key=times.get), "ms": times, "n": n}
    _CACHE[key] = res
    return res
