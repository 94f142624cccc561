"""PyTorch autograd boundary: the log-likelihood of a batch of conditions with
its gradient from the GPU adjoint.

``LogLikelihood.apply(theta, model, solver, k, ts, my)`` returns ``llh[N]``
for the parameter rows ``theta[N, np]`` (in the model's parameter scale) and
registers ``d llh / d theta`` for autograd.  One call of the engine's device
entry point on torch's current stream runs, per condition, the forward
problem (checkpoint data for the interpolant in the kernel's scratch) and the
backward problem with quadratures (AMICI's BackwardProblem,
``src/backwardproblem.cpp``); the autograd backward only scales the stored
gradient by the incoming ``grad_output``.  All tensors stay on the device; no
host copy is made.

The equivalent reference computation is ``run_simulations`` with
``SensitivityMethod.adjoint`` and the ReturnData fields ``llh`` and ``sllh``.
"""
from __future__ import annotations

import numpy as np

from . import _native
from .simulation import Model, SensitivityMethod, SensitivityOrder, Solver


def _dev(t, dtype, device):
    import torch
    if t is None:
        return None
    if isinstance(t, np.ndarray) and not t.flags.writeable:
        t = t.copy()  # torch does not wrap read-only arrays (np.broadcast_to views)
    return torch.as_tensor(t, dtype=dtype, device=device).contiguous()


def log_likelihood_and_gradient(model: Model, solver: Solver, theta, k, ts, my, sigma=None, *,
                                plist=None, stream=None, method=SensitivityMethod.adjoint, diag=None,
                                k_preeq=None, x0=None, sx0=None):
    """llh [N] and sllh [N, nplist] for device tensors (or arrays) on CUDA.

    Calls ``amici_gb300_run_simulations_device`` with adjoint (default) or
    forward sensitivities on ``stream`` (a ``torch.cuda.Stream`` or a raw
    ``cudaStream_t`` handle; default: torch's current stream); raises if the
    engine reports an error.  Per-instance failures give NaN llh/sllh and a
    nonzero status, returned as the third value.  The inputs are prepared and
    the outputs allocated on torch's current stream; with another stream the
    launch waits for that work, every tensor the kernel touches is marked as
    used on the launch stream (the caching allocator does not hand its memory
    out again before the kernel is done), and the current stream waits for the
    kernel before the results are returned, so they are safe to read there.
    ``diag``: an optional [N, 8] int32 CUDA tensor that receives the
    per-instance solver counters (``amici_gb300_batch.diag``).  ``k_preeq``
    [N, nk]: pre-equilibrate at these fixed parameters first (with forward
    sensitivities, whose steady-state sensitivities enter the gradient);
    ``x0`` [N, nx] / ``sx0`` [N, nplist, nx] (scaled parameters): given
    initial states and sensitivities."""
    import torch
    spec = model.spec
    dev = theta.device if isinstance(theta, torch.Tensor) else torch.device("cuda")
    theta = _dev(theta, torch.float64, dev)
    if theta.dim() == 1:
        theta = theta.unsqueeze(0)
    n = theta.shape[0]
    ts = _dev(ts, torch.float64, dev)
    ts = ts.expand(n, ts.shape[-1]).contiguous()
    nt = ts.shape[1]
    k = _dev(k if spec.nk else np.zeros((n, 0)), torch.float64, dev)
    k = k.expand(n, spec.nk).contiguous()
    my = _dev(my, torch.float64, dev).expand(n, nt, spec.ny).contiguous()
    sg = None if sigma is None else _dev(sigma, torch.float64, dev).expand(n, nt, spec.ny).contiguous()
    pscale = _dev(model.get_parameter_scale(), torch.int32, dev)
    pl = np.arange(spec.np) if plist is None else np.asarray(plist)
    plist_t = _dev(pl, torch.int32, dev)
    npl = len(pl)
    llh = torch.empty(n, dtype=torch.float64, device=dev)
    sllh = torch.empty((n, npl), dtype=torch.float64, device=dev)
    numsteps = torch.empty((n, nt), dtype=torch.int32, device=dev)
    status = torch.empty(n, dtype=torch.int32, device=dev)
    b = _native.Batch()
    b.n_instances, b.nt, b.nplist = n, nt, npl
    b.p, b.pscale, b.k, b.ts = theta.data_ptr(), pscale.data_ptr(), k.data_ptr(), ts.data_ptr()
    b.my, b.sigma_y, b.plist = my.data_ptr(), None if sg is None else sg.data_ptr(), plist_t.data_ptr()
    b.x = b.y = b.sigmay = b.sx = b.sy = None
    if diag is not None:
        if diag.shape != (n, 8) or diag.dtype != torch.int32 or not diag.is_cuda or not diag.is_contiguous():
            raise ValueError("diag must be a contiguous [N, 8] int32 CUDA tensor")
        b.diag = diag.data_ptr()
    else:
        b.diag = None
    b.llh, b.sllh = llh.data_ptr(), sllh.data_ptr()
    b.numsteps, b.status = numsteps.data_ptr(), status.data_ptr()
    extras = []
    if k_preeq is not None:
        kp = _dev(k_preeq if spec.nk else np.zeros((n, 1)), torch.float64, dev)
        kp = kp.expand(n, max(spec.nk, 1)).contiguous()
        extras.append(kp)
        b.k_preeq = kp.data_ptr()
    if x0 is not None:
        x0t = _dev(x0, torch.float64, dev).expand(n, spec.nx).contiguous()
        extras.append(x0t)
        b.x0 = x0t.data_ptr()
    if sx0 is not None:
        sx0t = _dev(sx0, torch.float64, dev).expand(n, npl, spec.nx).contiguous()
        extras.append(sx0t)
        b.sx0 = sx0t.data_ptr()
    s = Solver()
    s.__dict__.update(solver.__dict__)
    s.set_sensitivity_order(SensitivityOrder.first)
    s.set_sensitivity_method(method)
    cur = torch.cuda.current_stream(dev)
    if stream is None:
        st = cur
    elif isinstance(stream, torch.cuda.Stream):
        st = stream
    else:
        st = torch.cuda.ExternalStream(int(stream), device=dev)
    if st != cur:
        st.wait_stream(cur)
        for t in (theta, ts, k, my, sg, pscale, plist_t, llh, sllh, numsteps, status, diag, *extras):
            if t is not None:
                t.record_stream(st)
    model.library.run_device(s.to_options(), b, st.cuda_stream)
    if st != cur:
        cur.wait_stream(st)
    return llh, sllh, status


class LogLikelihood:
    """``torch.autograd.Function`` computing llh(theta) per condition with the
    adjoint gradient; see the module docstring."""

    _fn = None

    @classmethod
    def apply(cls, theta, model: Model, solver: Solver, k, ts, my, sigma=None):
        if cls._fn is None:
            cls._fn = _make_function()
        return cls._fn.apply(theta, model, solver, k, ts, my, sigma)


def _make_function():
    import torch

    class _LLH(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, model, solver, k, ts, my, sigma):
            llh, sllh, _ = log_likelihood_and_gradient(model, solver, theta.detach(), k, ts, my, sigma)
            ctx.save_for_backward(sllh)
            ctx.theta_shape = theta.shape
            return llh if theta.dim() > 1 else llh[0]

        @staticmethod
        def backward(ctx, grad_llh):
            (sllh,) = ctx.saved_tensors
            g = grad_llh.reshape(-1, 1).to(sllh.dtype) * sllh
            return g.reshape(ctx.theta_shape), None, None, None, None, None, None

    return _LLH
