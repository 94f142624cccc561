"""Objective over conditions: parameter mapping and llh/sllh aggregation.

In estimation workflows the simulation path is called through AMICI's PEtab
layer: one vector of problem parameters is mapped onto every condition's
model parameters (``ParameterMappingForCondition``,
``python/sdist/amici/sim/_parameter_mapping.py:18-107``;
``fill_in_parameters_for_condition``,
``python/sdist/amici/sim/sundials/petab/v1/_conditions.py:98-200``), all
conditions are simulated, the condition llh are summed and the condition
sllh are accumulated per problem parameter (``simulate_petab`` and
``aggregate_sllh``,
``python/sdist/amici/sim/sundials/petab/v1/_simulations.py:69-361``).

Here the mapping is a few tensor operations in front of one batched device
call: each model parameter of each condition is either gathered from the
problem vector or a constant, given on its mapping scale (lin, log, log10)
and converted to the model's parameter scale.  ``Objective.__call__`` runs
the device adjoint (``log_likelihood_and_gradient``) on every condition at
once and pulls the per-condition sllh back through the mapping (a
vector-Jacobian product, which is the accumulation of ``aggregate_sllh``);
``Objective.torch_llh`` puts the same mapping in front of ``LogLikelihood``
for use inside a larger autograd graph.

As in the reference: a problem parameter must be mapped on its own scale
(a different mapping scale is an error); a NaN constant is taken as 0; the
llh is the sum over conditions, and the gradient is None when a condition
failed; with ``scaled_gradients=False`` the gradient is rescaled to linear
parameters (``rescale_sensitivity``, ``_simulations.py:363-410``).  Problem
parameters that no condition uses get a zero gradient.
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, field

import numpy as np

from .autograd import LogLikelihood, log_likelihood_and_gradient
from .simulation import Model, Solver

SCALE_CODES = {"lin": 0, "log": 1, "ln": 1, "log10": 2}


def _scale_code(s) -> int:
    if isinstance(s, (int, np.integer)):
        if int(s) not in (0, 1, 2):
            raise ValueError(f"unknown parameter scale {s!r}")
        return int(s)
    try:
        return SCALE_CODES[str(s).lower()]
    except KeyError:
        raise ValueError(f"unknown parameter scale {s!r} (lin, log, log10)") from None


@dataclass
class ConditionMapping:
    """Mapping of one condition (``ParameterMappingForCondition``).

    ``map_sim_var``: model parameter id -> problem parameter id or a number;
    ``scale_map_sim_var``: model parameter id -> scale the value is given on
    (default lin); ``map_sim_fix``: fixed parameter id -> number or problem
    parameter id (linear value, a constant of the objective); fixed
    parameters not listed keep the model's nominal values."""

    map_sim_var: dict
    scale_map_sim_var: dict = field(default_factory=dict)
    map_sim_fix: dict = field(default_factory=dict)


class Objective:
    """Sum of the condition log-likelihoods as a function of the problem
    parameters, with its gradient from one batched adjoint call.

    ``ts`` is [C, nt] (or [nt]), ``my`` [C, nt, ny], ``sigma`` optional
    [C, nt, ny] (NaN: model value); ``problem_scales`` are the problem
    parameters' scales (lin, log, log10), on which ``theta`` is given."""

    def __init__(self, model: Model, solver: Solver, problem_parameter_ids, problem_scales,
                 mappings, ts, my, sigma=None):
        spec = model.spec
        self.model, self.solver = model, solver
        self.problem_ids = list(problem_parameter_ids)
        self.problem_scales = np.array([_scale_code(s) for s in problem_scales], dtype=np.int64)
        if len(self.problem_scales) != len(self.problem_ids):
            raise ValueError("one scale per problem parameter")
        index = {pid: i for i, pid in enumerate(self.problem_ids)}
        C = len(mappings)
        if C == 0:
            raise ValueError("no conditions")
        src = np.full((C, spec.np), -1, dtype=np.int64)
        val = np.zeros((C, spec.np))
        scale = np.zeros((C, spec.np), dtype=np.int64)
        kidx = np.full((C, spec.nk), -1, dtype=np.int64)
        kval = np.tile(np.asarray(spec.k_nominal if spec.k_nominal else np.zeros(spec.nk), dtype=float),
                       (C, 1)) if spec.nk else np.zeros((C, 0))
        for c, m in enumerate(mappings):
            for j, pid in enumerate(spec.parameter_ids):
                if pid not in m.map_sim_var:
                    raise ValueError(f"condition {c}: model parameter {pid!r} is not mapped")
                v = m.map_sim_var[pid]
                sc = _scale_code(m.scale_map_sim_var.get(pid, "lin"))
                scale[c, j] = sc
                if isinstance(v, str):
                    if v not in index:
                        raise ValueError(f"condition {c}: {pid!r} maps to unknown problem parameter {v!r}")
                    i = index[v]
                    if self.problem_scales[i] != sc:
                        raise ValueError(f"the scale of problem parameter {v!r} differs between its mapping "
                                         f"onto {pid!r} and the problem")
                    src[c, j] = i
                else:
                    val[c, j] = 0.0 if math.isnan(float(v)) else float(v)
            for j, kid in enumerate(spec.fixed_parameter_ids):
                if kid not in m.map_sim_fix:
                    continue
                v = m.map_sim_fix[kid]
                if isinstance(v, str):
                    if v not in index:
                        raise ValueError(f"condition {c}: fixed {kid!r} maps to unknown problem parameter {v!r}")
                    kidx[c, j] = index[v]
                else:
                    kval[c, j] = 0.0 if math.isnan(float(v)) else float(v)
        self.src, self.val, self.scale = src, val, scale
        self.kidx, self.kval = kidx, kval
        self.model_scale = np.asarray(model.get_parameter_scale(), dtype=np.int64)
        nt = np.shape(ts)[-1]
        self.ts = np.ascontiguousarray(np.broadcast_to(ts, (C, nt)), dtype=np.float64)
        self.my = np.ascontiguousarray(np.broadcast_to(my, (C, nt, spec.ny)), dtype=np.float64)
        self.sigma = None if sigma is None else np.ascontiguousarray(
            np.broadcast_to(sigma, (C, nt, spec.ny)), dtype=np.float64)
        self.n_conditions = C
        self.device = None  # device of the mapping when theta is not a CUDA tensor (default: current CUDA device)

    def shard(self, rank: int, world: int) -> "Objective":
        """The objective over this rank's contiguous share of the conditions
        (``replicas.shard_range``).  Every rank evaluates its shard at the
        same ``theta`` and ``allreduce`` combines the results."""
        from .replicas import shard_range

        a, b = shard_range(self.n_conditions, rank, world)
        if a == b:
            raise ValueError("more ranks than conditions")
        o = copy.copy(self)
        o.src, o.val, o.scale = self.src[a:b], self.val[a:b], self.scale[a:b]
        o.kidx, o.kval = self.kidx[a:b], self.kval[a:b]
        o.ts, o.my = self.ts[a:b], self.my[a:b]
        o.sigma = None if self.sigma is None else self.sigma[a:b]
        o.n_conditions = b - a
        o.condition_range = (a, b)
        return o

    # ---- mapping -----------------------------------------------------------
    def map_parameters(self, theta):
        """Model parameters [C, np] on the model's scale from the problem
        parameters ``theta`` (torch tensor on the problem scales); every
        operation is differentiable."""
        import torch

        dev, dt = theta.device, theta.dtype
        val = torch.as_tensor(self.val, device=dev, dtype=dt)
        if theta.numel() == 0:  # no problem parameters: constants only
            x = val
        else:
            src = torch.as_tensor(self.src, device=dev)
            x = torch.where(src >= 0, theta[src.clamp(min=0)], val)
        need = self.scale != self.model_scale[None, :]
        if not need.any():
            return x
        # only the entries whose mapping scale differs from the model's are converted
        mask = torch.as_tensor(need, device=dev)
        s_from = torch.as_tensor(self.scale[need], device=dev)
        s_to = torch.as_tensor(np.broadcast_to(self.model_scale, self.scale.shape)[need], device=dev)
        return x.masked_scatter(mask, _from_linear(_to_linear(x[mask], s_from), s_to))

    def fixed_parameters(self, theta_np):
        """Fixed parameters [C, nk] (linear) for problem parameters ``theta_np``."""
        k = self.kval.copy()
        if k.size:
            lin = _unscale(np.asarray(theta_np, dtype=float), self.problem_scales)
            sel = self.kidx >= 0
            k[sel] = lin[self.kidx[sel]]
        return k

    # ---- evaluation ----------------------------------------------------------
    def __call__(self, theta, *, scaled_gradients=True, stream=None):
        """``{"llh", "sllh", "llh_conditions", "status"}`` at ``theta`` (problem
        parameters on their scales; numpy or a CUDA tensor).  ``sllh`` is the
        gradient of the summed llh w.r.t. ``theta`` (None after a failed
        condition); with ``scaled_gradients=False`` w.r.t. the linear values."""
        import torch

        th = torch.as_tensor(np.asarray(theta, dtype=np.float64) if not isinstance(theta, torch.Tensor)
                             else theta.detach(), dtype=torch.float64)
        dev = th.device if th.is_cuda else (self.device or torch.device("cuda", torch.cuda.current_device()))
        th = th.to(dev).requires_grad_(True)
        p = self.map_parameters(th)
        k = self.fixed_parameters(th.detach().cpu().numpy())
        llh, sllh, status = log_likelihood_and_gradient(self.model, self.solver, p.detach(), k, self.ts, self.my,
                                                        self.sigma, stream=stream)
        st = status.cpu().numpy()
        llh_c = llh.cpu().numpy()
        out = {"llh": float(llh_c.sum()), "llh_conditions": llh_c, "status": st, "sllh": None}
        if (st == 0).all():
            if th.numel() == 0:
                g = np.zeros(0)
            else:
                (g,) = torch.autograd.grad(p, th, grad_outputs=sllh)
                g = g.cpu().numpy()
            if not scaled_gradients:
                g = _rescale_to_linear(g, th.detach().cpu().numpy(), self.problem_scales)
            out["sllh"] = g
        return out

    def torch_llh(self, theta):
        """Summed llh as a tensor in the autograd graph of ``theta`` (problem
        parameters on their scales, CUDA tensor): the mapping in front of
        ``LogLikelihood``."""
        p = self.map_parameters(theta)
        k = self.fixed_parameters(theta.detach().cpu().numpy())
        llh = LogLikelihood.apply(p, self.model, self.solver, k, self.ts, self.my, self.sigma)
        return llh.sum()


def allreduce(objective: Objective, result: dict, group=None) -> dict:
    """Combine the results of the shards of one objective across ranks: one
    all-reduce of llh, the count of failed conditions and the gradient
    (problem parameters + 2 doubles).  Returns ``{"llh", "sllh",
    "n_failed"}`` on every rank; ``sllh`` is None when a condition failed on
    any rank."""
    import torch
    import torch.distributed as dist

    buf = torch.zeros(2 + len(objective.problem_ids), dtype=torch.float64)
    buf[0] = result["llh"]
    buf[1] = float((np.asarray(result["status"]) != 0).sum())
    if result["sllh"] is not None:
        buf[2:] = torch.as_tensor(result["sllh"], dtype=torch.float64)
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    n_failed = int(buf[1].item())
    return {"llh": float(buf[0].item()), "n_failed": n_failed,
            "sllh": None if n_failed else buf[2:].numpy().copy()}


def _to_linear(x, s):
    """Linear values from values on scales ``s`` (torch); every branch is
    evaluated at a finite point so that unselected branches pass no NaN into
    the gradient."""
    import torch

    zero = torch.zeros_like(x)
    p10 = torch.pow(10.0, torch.where(s == 2, x, zero))
    pe = torch.exp(torch.where(s == 1, x, zero))
    return torch.where(s == 2, p10, torch.where(s == 1, pe, x))


def _from_linear(v, s):
    """Values on scales ``s`` from linear values (torch), branch-safe as
    ``_to_linear``."""
    import torch

    one = torch.ones_like(v)
    l10 = torch.log10(torch.where(s == 2, v, one))
    ln = torch.log(torch.where(s == 1, v, one))
    return torch.where(s == 2, l10, torch.where(s == 1, ln, v))


def _unscale(x, scales):
    return np.where(scales == 2, 10.0 ** x, np.where(scales == 1, np.exp(x), x))


def _rescale_to_linear(g, x, scales):
    """d/d(linear value) from d/d(scaled value) (``rescale_sensitivity`` to lin)."""
    lin = _unscale(x, scales)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(scales == 2, g / (lin * np.log(10.0)), np.where(scales == 1, g / lin, g))
