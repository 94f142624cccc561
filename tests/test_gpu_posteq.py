"""GPU post-equilibration against the reference.

The preeq12 network with outputs at t = inf (golden vectors from the
reference's CVODES driven like AMICI): pre-equilibrated at basal inputs, the
stimulus response at ten finite outputs, then the main solver continues in
ONE_STEP mode to steady state and the two outputs at t = inf are taken
there.  Forward simulation and forward sensitivities (FP32 and FP64
iteration matrix).

Targets: the outputs at the finite times as for the other workloads (no
less accurate against the rtol = atol = 1e-12 reference than the reference
itself at the stated tolerances, a small multiple in tolerance units); the
steady state is only determined to the steady-state tolerances (100 x the
solver's, a residual norm below 1), so the outputs at t = inf are compared
at that level and llh within 1e-6 of the 1e-12 reference or within 10 x the
reference's own error; sllh within 1e-4 and the sensitivities at t = inf
within 1e-3 (relative to each instance's largest component); steps of the
post-equilibration within 20% of the reference's; no step count at the
outputs at t = inf, as in the reference."""
from pathlib import Path

import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300 import _native
from amici_gb300.networks import preeq_model

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _g(name):
    return dict(np.load(GOLD / f"{name}.npz"))


@pytest.fixture(scope="module")
def model():
    return ag.Model(preeq_model())


def _solver(g, method=None, lu=32):
    s = ag.Solver()
    s.set_relative_tolerance(float(g["rtol"]))
    s.set_absolute_tolerance(float(g["atol"]))
    s.set_max_steps(100000)
    s.set_lu_precision(lu)
    s.set_control_precision(lu)
    if method is not None:
        s.set_sensitivity_order(ag.SensitivityOrder.first)
        s.set_sensitivity_method(method)
    return s


def _tu(x, ref, g):
    return np.abs(x - ref) / (float(g["rtol"]) * np.abs(ref) + float(g["atol"]))


def _llh_ok(llh, ref_stated, tight):
    rel = lambda a: np.abs(a - tight) / np.abs(tight)
    tol = max(1e-6, 10 * rel(ref_stated).max())
    return np.all(rel(llh) <= tol), (rel(llh).max(), tol)


def _rel_to_max(a, ref):
    return np.max(np.abs(a - ref) / np.abs(ref).max(axis=1, keepdims=True))


def _check(r, g, t, x_ref, llh_ref, pre):
    assert (r["status"] == 0).all(), r["status"]
    assert (r["posteq_status"] == 1).all(), r["posteq_status"]
    assert (r["numsteps"][:, -2:] == 0).all()
    eg, er = _tu(r["x"][:, :-2], t["x"][:, :-2], g), _tu(x_ref[:, :-2], t["x"][:, :-2], g)
    assert eg.max() <= 3 * er.max() + 10, (eg.max(), er.max())
    ss_tol = 100 * (float(g["rtol"]) * np.abs(t["x"][:, -1]) + float(g["atol"]))
    dev = np.abs(r["x"][:, -1] - t["x"][:, -1]) / ss_tol
    assert dev.max() <= 100, dev.max()
    np.testing.assert_array_equal(r["x"][:, -1], r["x"][:, -2])
    ok, info = _llh_ok(r["llh"], llh_ref, t["llh"])
    assert ok, info
    ns, nr = r["posteq_numsteps"], g[pre + "posteq_numsteps"]
    assert np.all(np.abs(ns - nr) <= 0.2 * nr + 2), (ns, nr)
    assert np.all(r["posteq_wrms"] < 1.0) and np.all(r["posteq_t"] > g["ts"][:, -3])


@pytest.mark.parametrize("lu", [32, 64])
def test_posteq_forward(model, lu):
    g, t = _g("posteq"), _g("posteq_tight")
    r = ag.simulate_batch(model, _solver(g, lu=lu), g["p"], g["k"], g["ts"], g["my"], pscale=g["pscale"],
                          k_preeq=g["k_preeq"])
    _check(r, g, t, g["fwd_x"], g["fwd_llh"], "fwd_")


@pytest.mark.parametrize("lu", [32, 64])
def test_posteq_forward_sensitivities(model, lu):
    g, t = _g("posteq"), _g("posteq_tight")
    r = ag.simulate_batch(model, _solver(g, ag.SensitivityMethod.forward, lu), g["p"], g["k"], g["ts"], g["my"],
                          pscale=g["pscale"], k_preeq=g["k_preeq"])
    _check(r, g, t, g["x"], g["llh"], "")
    assert _rel_to_max(r["sllh"], t["sllh"]) <= 1e-4
    n = len(g["p"])
    assert _rel_to_max(r["sx"][:, -1].reshape(n, -1), t["sx_last"].reshape(n, -1)) <= 1e-3


def test_posteq_through_run_simulations(model):
    """ExpData with outputs at t = inf through run_simulations: the
    post-equilibration results land in each ReturnData."""
    g = _g("posteq")
    model.set_parameter_scale(g["pscale"])
    es = [ag.ExpData(ts=g["ts"][i], measurements=g["my"][i], parameters=g["p"][i], fixed_parameters=g["k"][i],
                     fixed_parameters_pre_equilibration=g["k_preeq"][i]) for i in range(4)]
    rs = ag.run_simulations(model, _solver(g), es)
    assert all(r.status == 0 and r.posteq_status == 1 and r.posteq_numsteps > 0 for r in rs)
    assert all(r.numsteps[-1] == 0 and np.isinf(r.ts[-1]) for r in rs)


def test_posteq_adjoint_refused(model):
    g = _g("posteq")
    with pytest.raises(_native.EngineError, match="post-equilibration"):
        ag.simulate_batch(model, _solver(g, ag.SensitivityMethod.adjoint), g["p"][:2], g["k"][:2], g["ts"][:2],
                          g["my"][:2], pscale=g["pscale"], k_preeq=g["k_preeq"][:2])


def test_failed_posteq_keeps_outputs():
    """A model without a steady state (exponential growth) with a step
    budget of 200: the post-equilibration runs out of steps (-2), the
    instance gets AMICI_ERROR and every output stays in place, the outputs
    at t = inf from the last state reached, as in the reference and the
    oracle."""
    import sympy as sp
    from amici_gb300.model_spec import ModelSpec
    from oracle.pyoracle import Oracle
    x, p = sp.symbols("x0:1", real=True), sp.symbols("p0:1", real=True)
    spec = ModelSpec(name="growth1", state_ids=["x"], parameter_ids=["r"], fixed_parameter_ids=[],
                     observable_ids=["x"], x0=[sp.Integer(1)], w=[p[0] * x[0]], stoich={(0, 0): 1}, y=[x[0]],
                     sigma_y=[sp.Float(0.1)], x=list(x), p=list(p), k=[], p_nominal=[0.1], k_nominal=[])
    spec.families = ("fwd", "posteq")
    s = ag.Solver()
    s.set_relative_tolerance(1e-8)
    s.set_absolute_tolerance(1e-10)
    s.set_max_steps(200)
    th, pscale = np.log([[0.1]] * 4), np.array([1], np.int32)
    ts, my = np.array([[0.5, 1.0, np.inf]] * 4), np.array([[[1.0], [1.1], [2.0]]] * 4)
    r = ag.simulate_batch(ag.Model(spec), s, th, np.zeros((4, 0)), ts, my, pscale=pscale)
    o = Oracle(spec).run(th, pscale, np.zeros((4, 0)), ts, my, rtol=1e-8, atol=1e-10, maxsteps=200)
    assert (r["status"] == -99).all() and (o["status"] == -99).all()
    np.testing.assert_array_equal(r["posteq_status"], o["posteq_status"])
    np.testing.assert_array_equal(r["numsteps"], o["numsteps"])
    assert np.isnan(r["posteq_t"]).all()
    np.testing.assert_allclose(r["x"][:, :2], o["x"][:, :2], rtol=1e-6)
    np.testing.assert_allclose(r["x"][:, 2], o["x"][:, 2], rtol=1e-2)
    assert np.isfinite(r["llh"]).all()
