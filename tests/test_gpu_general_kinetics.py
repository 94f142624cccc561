"""GPU general kinetics against the reference: the mapk9 workload, a MAPK
cascade whose fluxes are Michaelis-Menten, Hill-type feedback and
inhibition rate laws (plus one mass-action flux), with a nonlinear and a
parameter-dependent observable (golden vectors from the reference's CVODES
driven like AMICI; the reference evaluates the same symbolic right-hand side
through the oracle's generated C).  The engine evaluates the general rate
laws through generated code shared by fluxes of the same form.

Targets as for the other workloads: states no less accurate against the
rtol = atol = 1e-12 reference than the reference itself at the stated
tolerances (a small multiple, in tolerance units); llh within 1e-6 of the
1e-12 reference, or within twice the reference's own error at the stated
tolerances where that is larger (its adjoint reaches 9e-7 here); sllh within
1e-4 (relative to each instance's largest component); step counts within 20%
of the reference's."""
from pathlib import Path

import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import mapk_model

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _g(name):
    return dict(np.load(GOLD / f"{name}.npz"))


@pytest.fixture(scope="module")
def model():
    return ag.Model(mapk_model())


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
    """llh within max(1e-6, 2 x the reference's own largest relative error)."""
    rel = lambda a: np.abs(a - tight) / np.abs(tight)
    tol = max(1e-6, 2 * rel(ref_stated).max())
    return np.all(rel(llh) <= tol), (rel(llh).max(), tol)


def _rel_to_max(a, ref):
    return np.max(np.abs(a - ref) / np.abs(ref).max(axis=1, keepdims=True))


@pytest.mark.parametrize("lanes", [0, 32])
def test_general_kinetics_forward(model, lanes):
    g, t = _g("mapk9"), _g("mapk9_tight")
    s = _solver(g)
    s.set_lanes_per_instance(lanes)
    r = ag.simulate_batch(model, s, g["p"], g["k"], g["ts"], g["my"], pscale=g["pscale"])
    assert (r["status"] == 0).all(), r["status"]
    # against the reference's forward simulation (without sensitivities in
    # the error test) at the same tolerances
    eg, er = _tu(r["x"], t["x"], g), _tu(g["fwd_x"], t["x"], g)
    assert eg.max() <= 3 * er.max() + 10, (eg.max(), er.max())
    ok, info = _llh_ok(r["llh"], g["fwd_llh"], t["llh"])
    assert ok, info
    nf, nr = r["numsteps"][:, -1], g["fwd_numsteps"][:, -1]
    assert np.all(np.abs(nf - nr) <= 0.2 * nr), (nf, nr)


@pytest.mark.parametrize("lu", [32, 64])
def test_general_kinetics_forward_sensitivities(model, lu):
    g, t = _g("mapk9"), _g("mapk9_tight")
    r = ag.simulate_batch(model, _solver(g, ag.SensitivityMethod.forward, lu), g["p"], g["k"], g["ts"], g["my"],
                          pscale=g["pscale"])
    assert (r["status"] == 0).all(), r["status"]
    ok, info = _llh_ok(r["llh"], g["llh"], t["llh"])
    assert ok, info
    assert _rel_to_max(r["sllh"], t["sllh"]) <= 1e-4
    n = len(g["p"])
    assert _rel_to_max(r["sx"][:, -1].reshape(n, -1), t["sx_last"].reshape(n, -1)) <= 1e-3


@pytest.mark.parametrize("lu", [32, 64])
def test_general_kinetics_adjoint(model, lu):
    g, t = _g("mapk9"), _g("mapk9_tight")
    model.set_parameter_scale(g["pscale"])
    llh, sllh, st = ag.log_likelihood_and_gradient(model, _solver(g, ag.SensitivityMethod.adjoint, lu), g["p"],
                                                   g["k"], g["ts"], g["my"])
    llh, sllh, st = llh.cpu().numpy(), sllh.cpu().numpy(), st.cpu().numpy()
    assert (st == 0).all(), st
    ok, info = _llh_ok(llh, g["asa_llh"], t["asa_llh"])
    assert ok, info
    assert _rel_to_max(sllh, t["asa_sllh"]) <= 1e-4
    assert _rel_to_max(sllh, t["sllh"]) <= 1e-4
