"""The objective over conditions on the GPU: one batched adjoint call, the
condition gradients pulled back through the parameter mapping, against a
hand-written chain rule over the per-condition sllh, and the same objective
through ``LogLikelihood`` and torch autograd."""
import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import robertson_workload
from amici_gb300.objective import ConditionMapping, Objective

pytestmark = pytest.mark.gpu


def _setup():
    w = robertson_workload()
    spec = w.model
    m = ag.Model(spec)
    m.set_parameter_scale(w.pscale)  # ln k
    s = ag.Solver()
    s.set_relative_tolerance(1e-8)
    s.set_absolute_tolerance(1e-12)
    p1, p2, p3 = spec.parameter_ids
    k = np.exp(w.p[0])
    maps = [
        ConditionMapping({p1: "k1", p2: "k2", p3: "k3"}, {p1: "log10", p2: "log", p3: "log"}),
        ConditionMapping({p1: "k1", p2: "k2", p3: float(np.log(2 * k[2]))}, {p1: "log10", p2: "log", p3: "log"}),
        ConditionMapping({p1: float(np.log10(0.5 * k[0])), p2: "k2", p3: "k3"}, {p1: "log10", p2: "log", p3: "log"}),
    ]
    theta = np.array([np.log10(k[0]), np.log(k[1]), np.log(k[2])])
    my = 0.5 + 0.01 * np.random.default_rng(3).normal(size=(3, len(w.ts[0]), 3))
    o = Objective(m, s, ["k1", "k2", "k3"], ["log10", "log", "log"], maps, w.ts[0], my)
    return o, theta, m, s, w, my


def test_objective_gradient_is_the_chain_rule_over_conditions():
    o, theta, m, s, w, my = _setup()
    r = o(theta)
    assert (r["status"] == 0).all() and r["sllh"] is not None
    # the same device call by hand: mapped model parameters (ln k) per condition
    ln10 = np.log(10.0)
    P = np.array([[theta[0] * ln10, theta[1], theta[2]],
                  [theta[0] * ln10, theta[1], o.val[1, 2]],
                  [o.val[2, 0] * ln10, theta[1], theta[2]]])
    import torch

    Pm = o.map_parameters(torch.tensor(theta, device="cuda")).cpu().numpy()
    np.testing.assert_allclose(Pm, P, rtol=1e-14)
    # the mapped values themselves (a last-bit change of a parameter can change the step sequence)
    llh, sllh, st = ag.log_likelihood_and_gradient(m, s, Pm, np.zeros((3, 0)), o.ts, my)
    assert (st.cpu().numpy() == 0).all()
    sl = sllh.cpu().numpy()
    np.testing.assert_allclose(r["llh"], llh.cpu().numpy().sum(), rtol=1e-12)
    # d p_c1/d k1 = ln 10 where k1 is mapped; k2, k3 enter on the model's ln scale
    g = np.array([ln10 * (sl[0, 0] + sl[1, 0]), sl[:, 1].sum(), sl[0, 2] + sl[2, 2]])
    np.testing.assert_allclose(r["sllh"], g, rtol=1e-10)
    # gradient w.r.t. linear values: divided by (value ln 10) for log10, by value for log
    lin = np.array([10 ** theta[0], np.exp(theta[1]), np.exp(theta[2])])
    rl = o(theta, scaled_gradients=False)
    np.testing.assert_allclose(rl["sllh"], g / np.array([lin[0] * ln10, lin[1], lin[2]]), rtol=1e-10)


def test_objective_through_autograd():
    import torch

    o, theta, *_ = _setup()
    th = torch.tensor(theta, device="cuda", requires_grad=True)
    total = o.torch_llh(th)
    total.backward()
    r = o(theta)
    np.testing.assert_allclose(total.item(), r["llh"], rtol=1e-12)
    np.testing.assert_allclose(th.grad.cpu().numpy(), r["sllh"], rtol=1e-10)
