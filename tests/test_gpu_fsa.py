"""GPU staggered forward sensitivities vs the reference (golden vectors).

Targets: llh within 1e-6 and sllh within 1e-4 relative of the reference at
rtol = atol = 1e-12; sensitivities as accurate as the reference's own at the
stated tolerances (distribution of errors, see tests/test_gpu_forward.py).
"""
from pathlib import Path

import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import net50_fsa_workload, robertson_workload

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _g(name):
    return dict(np.load(GOLD / f"{name}.npz"))


def _solver(rtol, atol, lu=32, ctl=32):
    s = ag.Solver()
    s.set_relative_tolerance(rtol)
    s.set_absolute_tolerance(atol)
    s.set_sensitivity_order(ag.SensitivityOrder.first)
    s.set_sensitivity_method(ag.SensitivityMethod.forward)
    s.set_lu_precision(lu)
    s.set_control_precision(ctl)
    s.set_max_steps(100000)
    return s


def _rel(a, b):
    return np.abs(a - b) / np.abs(b)


@pytest.mark.parametrize("lu,ctl", [(32, 32), (64, 64)])
def test_robertson_sllh(lu, ctl):
    g, gt = _g("robertson_fsa"), _g("robertson_fsa_tight")
    m = ag.Model(robertson_workload().model)
    r = ag.simulate_batch(m, _solver(1e-8, 1e-12, lu, ctl), g["p"], np.zeros((1, 0)), g["ts"], g["my"],
                          pscale=g["pscale"], plist=np.arange(3))
    assert r["status"][0] == 0
    assert _rel(r["llh"], gt["llh"]).max() <= 1e-6
    # the reference's own sllh error at rtol 1e-8 is ~8e-6 relative
    assert _rel(r["sllh"], gt["sllh"]).max() <= 1e-4, (r["sllh"], gt["sllh"])
    # sx: as accurate as the reference at the same tolerances
    tol = 1e-8 * np.abs(gt["sx"]) + 1e-12
    eg, er = np.abs(r["sx"] - gt["sx"]) / tol, np.abs(g["sx"] - gt["sx"]) / tol
    assert np.percentile(eg, 99) <= 2 * np.percentile(er, 99) + 10
    np.testing.assert_allclose(r["sx"].sum(-1), 0.0, atol=1e-6)  # mass conservation of sx


@pytest.mark.parametrize("lu", [32, 64])
def test_net50_sllh(lu):
    g, gt = _g("net50_fsa"), _g("net50_fsa_tight")
    m = ag.Model(net50_fsa_workload(1).model)
    r = ag.simulate_batch(m, _solver(float(g["rtol"]), float(g["atol"]), lu, lu), g["p"],
                          np.zeros((len(g["p"]), 0)), g["ts"], g["my"], pscale=g["pscale"],
                          plist=np.arange(100))
    assert (r["status"] == 0).all()
    assert _rel(r["llh"], gt["llh"]).max() <= 1e-6
    # sllh: as accurate as the reference at the same tolerances, within 1e-4 where
    # the reference is (tiny components are compared in absolute terms)
    scale = np.abs(gt["sllh"]) + 1e-3 * np.abs(gt["sllh"]).max(axis=1, keepdims=True)
    eg = np.abs(r["sllh"] - gt["sllh"]) / scale
    er = np.abs(g["sllh"] - gt["sllh"]) / scale
    assert eg.max() <= max(1e-4, 3 * er.max()), (eg.max(), er.max())
    rel = np.abs(r["numsteps"][:, -1] - g["numsteps"][:, -1]) / g["numsteps"][:, -1]
    assert np.median(rel) <= 0.1 and rel.max() <= 0.3


def test_fsa_through_run_simulations():
    g = _g("robertson_fsa")
    m = ag.Model(robertson_workload().model)
    m.set_parameter_scale(1)
    m.set_parameters(g["p"][0])
    s = _solver(1e-8, 1e-12)
    rd = ag.run_simulations(m, s, [ag.ExpData(ts=g["ts"][0], measurements=g["my"][0])])[0]
    assert rd.status == 0 and rd.sx.shape == (40, 3, 3) and rd.sy.shape == (40, 3, 3)
    assert rd.sllh.shape == (3,)
    assert _rel(rd.sllh, g["sllh"][0]).max() <= 1e-3
