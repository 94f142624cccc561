"""GPU pre-equilibration and initial-state overrides against the reference.

The preeq12 workload (golden vectors from the reference's CVODES driven
like AMICI): every instance is brought to steady state at basal input levels
(simulation to steady state, the reference's default), then simulated from
that state at its own stimulus levels, with forward sensitivities and with
adjoint sensitivities (whose pre-equilibration runs with forward
sensitivities, as the reference's default); and the same instances started
from given x0 / sx0 without pre-equilibration.

Targets as for the other workloads: states at the outputs no less accurate
against the rtol = atol = 1e-12 reference than the reference itself at the
stated tolerances (a small multiple, in tolerance units); sllh within 1e-4
(relative to the instance's largest component) of the 1e-12 reference; step
counts within 20% of the reference's.  The steady state itself is only
determined to the steady-state tolerances (100 x the solver's, a residual
norm below 1), so x_ss is compared at that level, and the llh of a
simulation that starts from it varies between any two integrations by more
than the solver's tolerances alone would give: llh within 1e-6 of the 1e-12
reference or within 10 x the reference's own error at the stated tolerances.
"""
from pathlib import Path

import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import preeq_model
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _g(name):
    return dict(np.load(GOLD / f"{name}.npz"))


@pytest.fixture(scope="module")
def model():
    return ag.Model(preeq_model())


def _solver(g, method=None):
    s = ag.Solver()
    s.set_relative_tolerance(float(g["rtol"]))
    s.set_absolute_tolerance(float(g["atol"]))
    s.set_max_steps(100000)
    if method is not None:
        s.set_sensitivity_order(ag.SensitivityOrder.first)
        s.set_sensitivity_method(method)
    return s


def _tu(x, ref, g):
    return np.abs(x - ref) / (float(g["rtol"]) * np.abs(ref) + float(g["atol"]))


def _llh_ok(llh, ref_stated, tight):
    """llh within max(1e-6, 10 x the reference's own largest relative error)."""
    rel = lambda a: np.abs(a - tight) / np.abs(tight)
    tol = max(1e-6, 10 * rel(ref_stated).max())
    return np.all(rel(llh) <= tol), (rel(llh).max(), tol)


def _rel_to_max(a, ref):
    return np.max(np.abs(a - ref) / np.abs(ref).max(axis=1, keepdims=True))


@pytest.mark.parametrize("lu", [32, 64])
def test_preeq_forward_sensitivities(model, lu):
    g, t = _g("preeq_fsa"), _g("preeq_fsa_tight")
    s = _solver(g, ag.SensitivityMethod.forward)
    s.set_lu_precision(lu)
    s.set_control_precision(lu)
    r = ag.simulate_batch(model, s, g["p"], g["k"], g["ts"], g["my"], pscale=g["pscale"], k_preeq=g["k_preeq"])
    assert (r["status"] == 0).all() and (r["preeq_status"] == 1).all(), (r["status"], r["preeq_status"])
    # the steady state, to the steady-state tolerances
    ss_tol = 100 * (float(g["rtol"]) * np.abs(g["x_ss"]) + float(g["atol"]))
    assert np.all(np.abs(r["x_ss"] - g["x_ss"]) <= 100 * ss_tol), np.max(np.abs(r["x_ss"] - g["x_ss"]) / ss_tol)
    assert np.all(np.abs(r["preeq_numsteps"] - g["preeq_numsteps"]) <= 0.2 * g["preeq_numsteps"])
    assert np.all(r["preeq_wrms"] < 1.0)
    # the response from the steady state
    eg, er = _tu(r["x"], t["x"], g), _tu(g["x"], t["x"], g)
    assert eg.max() <= 3 * er.max() + 10, (eg.max(), er.max())
    ok, info = _llh_ok(r["llh"], g["llh"], t["llh"])
    assert ok, info
    assert _rel_to_max(r["sllh"], t["sllh"]) <= 1e-4
    assert _rel_to_max(r["sx_ss"].reshape(len(g["p"]), -1), t["sx_ss"].reshape(len(g["p"]), -1)) <= 1e-3
    nf = r["numsteps"][:, -1]
    assert np.all(np.abs(nf - g["numsteps"][:, -1]) <= 0.2 * g["numsteps"][:, -1])


@pytest.mark.parametrize("lu", [32, 64])
def test_preeq_adjoint(model, lu):
    """The adjoint gradient with a pre-equilibration: sx_ss of the
    forward-sensitivity pre-equilibration enters through the initial-state
    term; it matches the reference's adjoint and forward-sensitivity
    gradients."""
    g, t = _g("preeq_fsa"), _g("preeq_fsa_tight")
    s = _solver(g, ag.SensitivityMethod.adjoint)
    s.set_lu_precision(lu)
    s.set_control_precision(lu)
    model.set_parameter_scale(g["pscale"])  # the device entry takes the model's scale
    llh, sllh, st = ag.log_likelihood_and_gradient(model, s, g["p"], g["k"], g["ts"], g["my"],
                                                   k_preeq=g["k_preeq"])
    llh, sllh, st = llh.cpu().numpy(), sllh.cpu().numpy(), st.cpu().numpy()
    assert (st == 0).all(), st
    ok, info = _llh_ok(llh, g["asa_llh"], t["asa_llh"])
    assert ok, info
    assert _rel_to_max(sllh, t["asa_sllh"]) <= 1e-4
    assert _rel_to_max(sllh, t["sllh"]) <= 1e-4


def test_initial_state_overrides(model):
    """ExpData x0 / sx0 without pre-equilibration, through run_simulations."""
    g, t = _g("preeq_fsa"), _g("preeq_fsa_tight")
    s = _solver(g, ag.SensitivityMethod.forward)
    model.set_parameter_scale(g["pscale"])
    es = [ag.ExpData(ts=g["ts"][i], measurements=g["my"][i], parameters=g["p"][i], fixed_parameters=g["k"][i],
                     x0=g["ov_x0"][i], sx0=g["ov_sx0"][i].ravel()) for i in range(len(g["p"]))]
    rs = ag.run_simulations(model, s, es)
    x = np.stack([r.x for r in rs])
    assert all(r.status == 0 and r.x_ss is None for r in rs)
    eg, er = _tu(x, t["ov_x"], g), _tu(g["ov_x"], t["ov_x"], g)
    assert eg.max() <= 3 * er.max() + 10, (eg.max(), er.max())
    llh = np.array([r.llh for r in rs])
    assert np.all(np.abs(llh - t["ov_llh"]) <= 1e-6 * np.abs(t["ov_llh"]))
    assert _rel_to_max(np.stack([r.sllh for r in rs]), t["ov_sllh"]) <= 1e-4
    sx_last = np.stack([r.sx[-1] for r in rs])
    assert _rel_to_max(sx_last.reshape(len(rs), -1), t["ov_sx_last"].reshape(len(rs), -1)) <= 1e-3


def test_failed_preequilibration_is_not_simulated(model):
    """A step budget too small for the steady state: the pre-equilibration
    fails with the step budget exhausted (-2) as in the reference, and the
    instance is not simulated (AMICI_ERROR, NaN outputs, no steps)."""
    g = _g("preeq_fsa")
    n = 4
    s = _solver(g)
    s.set_max_steps(50)
    r = ag.simulate_batch(model, s, g["p"][:n], g["k"][:n], g["ts"][:n], g["my"][:n], pscale=g["pscale"],
                          k_preeq=g["k_preeq"][:n])
    o = Oracle(model.spec).run(g["p"][:n], g["pscale"], g["k"][:n], g["ts"][:n], g["my"][:n],
                               rtol=float(g["rtol"]), atol=float(g["atol"]), maxsteps=50, k_preeq=g["k_preeq"][:n])
    np.testing.assert_array_equal(r["preeq_status"], o["preeq_status"])
    np.testing.assert_array_equal(r["status"], o["status"])
    assert (r["preeq_status"] == -2).all() and (r["status"] == -99).all()
    assert np.isnan(r["x"]).all() and np.isnan(r["llh"]).all() and not r["numsteps"].any()
    assert (r["preeq_numsteps"] == 50).all()
