"""GPU adjoint sensitivities vs the reference (golden vectors) and finite differences.

Targets: llh within 1e-6 and sllh within 1e-4 of the reference at
rtol = atol = 1e-12 (sllh relative to the instance's largest component);
the GPU's error no larger than a small multiple of the reference's own at
the same tolerances; backward step counts within 20% of the reference's.
"""
from pathlib import Path

import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import net20_workload, net100_adjoint_workload, robertson_workload

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _g(name):
    return dict(np.load(GOLD / f"{name}.npz"))


def _solver(rtol, atol, lu=32, ck=50):
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


def _spec(name):
    return {"robertson": robertson_workload().model, "net20": net20_workload(16).model,
            "net100": net100_adjoint_workload(1).model}[name]


def _norm_err(a, b):
    """|a - b| relative to the largest |b| component of each instance."""
    return np.abs(a - b) / np.abs(b).max(axis=1, keepdims=True)


@pytest.mark.parametrize("name", ["robertson", "net20", "net100"])
@pytest.mark.parametrize("lu", [32, 64])
@pytest.mark.parametrize("ck", [0, 50, 7])
def test_asa_vs_reference(name, lu, ck):
    """ck = 0: every forward step stored, polynomial interpolation (the
    reference's scheme as AMICI configures it); ck > 0: forward check points
    every ck steps, each segment replayed into cubic Hermite data."""
    if ck == 7 and (name == "net100" or lu == 64):
        pytest.skip("many-segment case covered on the smaller models in FP32")
    g, t = _g(f"{name}_asa"), _g(f"{name}_asa_tight")
    n = len(g["p"])
    k = g["k"] if "k" in g else np.zeros((n, 0))
    m = ag.Model(_spec(name))
    r = ag.simulate_batch(m, _solver(float(g["rtol"]), float(g["atol"]), lu, ck), g["p"], k, g["ts"],
                          g["my"], pscale=g["pscale"])
    assert (r["status"] == 0).all(), r["status"]
    # accuracy targets against the reference at 1e-12
    assert np.all(np.abs(r["llh"] - t["llh"]) <= 1e-6 * np.abs(t["llh"]))
    e_gpu = _norm_err(r["sllh"], t["sllh"])
    e_ref = _norm_err(g["sllh"], t["sllh"])
    assert e_gpu.max() <= 1e-4, e_gpu.max()
    assert e_gpu.max() <= max(20 * e_ref.max(), 1e-5), (e_gpu.max(), e_ref.max())
    # the same amount of backward work as the reference (step sequences differ at O(tol))
    nb = r["diag"][:, 7]
    assert np.all(np.abs(nb - g["nst_b"]) <= 0.2 * g["nst_b"]), (nb, g["nst_b"])


def test_asa_without_data_is_nan():
    w = robertson_workload()
    m = ag.Model(w.model)
    r = ag.simulate_batch(m, _solver(1e-8, 1e-12), w.p, w.k, w.ts, pscale=w.pscale)
    assert r["status"][0] == 0 and np.isnan(r["llh"][0]) and np.isnan(r["sllh"]).all()


def test_asa_against_central_differences_16_conditions():
    """The n=100 adjoint workload: gradients of 16 conditions against central finite
    differences (h = 1e-5 in ln k) of the GPU's own llh at tight tolerances,
    all 2 * 256 * 16 perturbed solves in one batch."""
    from oracle.pyoracle import Oracle

    def simulate(mdl, p, pscale, k, ts):
        return Oracle(mdl).run(p, pscale, k, ts, rtol=1e-10, atol=1e-12, nthreads=0)["y"]

    w = net100_adjoint_workload(16, simulate=simulate)
    m = ag.Model(w.model)
    r = ag.simulate_batch(m, _solver(w.rtol, w.atol), w.p, w.k, w.ts, w.my, pscale=w.pscale)
    assert (r["status"] == 0).all()
    h = 1e-5
    npar = w.p.shape[1]
    P = np.repeat(w.p, 2 * npar, axis=0).reshape(16, 2 * npar, npar)
    j = np.arange(npar)
    P[:, 2 * j, j] += h
    P[:, 2 * j + 1, j] -= h
    s = ag.Solver()
    s.set_relative_tolerance(1e-12)
    s.set_absolute_tolerance(1e-14)
    s.set_max_steps(100000)
    s.set_lu_precision(64)
    s.set_control_precision(64)
    K = np.repeat(w.k, 2 * npar, axis=0)
    TS = np.repeat(w.ts, 2 * npar, axis=0)
    MY = np.repeat(w.my, 2 * npar, axis=0)
    f = ag.simulate_batch(m, s, P.reshape(-1, npar), K, TS, MY, pscale=w.pscale)
    assert (f["status"] == 0).all()
    llh = f["llh"].reshape(16, npar, 2)
    fd = (llh[:, :, 0] - llh[:, :, 1]) / (2 * h)
    err = _norm_err(r["sllh"], fd)
    assert err.max() <= 1e-3, err.max()
    assert np.median(err) <= 1e-5, np.median(err)


@pytest.mark.parametrize("ck", [0, 50])
def test_asa_missing_data_and_sigma_overrides(ck):
    """Measurements partly missing (NaN: no jump, no llh term) and noise
    scales partly given per data point (NaN: the model's sigma), as ExpData
    allows; against the oracle's adjoint at 1e-12 on the same inputs."""
    from oracle.pyoracle import Oracle

    g = _g("robertson_asa")
    rng = np.random.default_rng(11)
    my = g["my"].copy()
    my[rng.random(my.shape) < 0.3] = np.nan
    sigma = np.full_like(my, np.nan)
    pick = rng.random(sigma.shape) < 0.4
    sigma[pick] = rng.uniform(0.005, 0.05, pick.sum())
    w = robertson_workload()
    o = Oracle(w.model)
    tight = o.run_asa(g["p"], g["pscale"], w.k, g["ts"], my, sigma, rtol=1e-12, atol=1e-12, maxsteps=100000)
    own = o.run_asa(g["p"], g["pscale"], w.k, g["ts"], my, sigma, rtol=1e-8, atol=1e-12, maxsteps=100000)
    m = ag.Model(w.model)
    r = ag.simulate_batch(m, _solver(1e-8, 1e-12, 32, ck), g["p"], w.k, g["ts"], my, sigma, pscale=g["pscale"])
    assert r["status"][0] == 0 and tight["status"][0] == 0
    assert abs(r["llh"][0] - tight["llh"][0]) <= 1e-6 * abs(tight["llh"][0])
    e_gpu = _norm_err(r["sllh"], tight["sllh"])
    e_ref = _norm_err(own["sllh"], tight["sllh"])
    assert e_gpu.max() <= max(20 * e_ref.max(), 1e-5), (e_gpu.max(), e_ref.max())
    # the noise scales reported are the overrides where given, the model's elsewhere
    np.testing.assert_array_equal(r["sigmay"][0], np.where(np.isnan(sigma[0]), 0.01, sigma[0]))
