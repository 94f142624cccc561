"""GPU forward simulation vs the reference (golden vectors) and the CPU oracle.

Parity criteria (the reference's own global error at rtol=1e-8 is tens of
tolerance units, so both are needed):
  * agreement: |gpu - ref| <= 10*(rtol*|ref| + atol) for >= 99% of entries,
    with ref the reference at the same tolerances;
  * accuracy: |gpu - tight| <= 3*|ref - tight| + 10*(rtol*|tight| + atol)
    for every entry, with tight the reference at rtol = atol = 1e-12;
  * llh within 1e-6 relative of the 1e-12 reference.
"""
from pathlib import Path

import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import config2_workload, robertson_workload
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
LANES = (1, 2, 4, 8, 16, 32)


def _g(name):
    return dict(np.load(GOLD / f"{name}.npz"))


def _solver(rtol, atol, G=0, lu=32, maxsteps=10000):
    s = ag.Solver()
    s.set_relative_tolerance(rtol)
    s.set_absolute_tolerance(atol)
    s.set_max_steps(maxsteps)
    s.set_lanes_per_instance(G)
    s.set_lu_precision(lu)
    return s


def assert_parity(gpu, ref, tight, rtol, atol, frac=0.99):
    tol = rtol * np.abs(ref) + atol
    within = np.abs(gpu - ref) <= 10 * tol
    assert within.mean() >= frac, f"only {within.mean():.4f} of entries within 10x tolerance"
    if tight is not None:
        bound = 3 * np.abs(ref - tight) + 10 * (rtol * np.abs(tight) + atol)
        bad = np.abs(gpu - tight) > bound
        assert not bad.any(), f"{bad.sum()} entries less accurate than the reference"


@pytest.fixture(scope="module")
def rob_model():
    return ag.Model(robertson_workload().model)


@pytest.fixture(scope="module")
def net20():
    w = config2_workload(1024)
    m = ag.Model(w.model)
    m.set_parameter_scale(2)
    return w, m


@pytest.mark.parametrize("lu", [32, 64])
@pytest.mark.parametrize("G", LANES)
def test_robertson_llh_and_states(rob_model, G, lu):
    g, gt = _g("robertson_fsa"), _g("robertson_fsa_tight")
    r = ag.simulate_batch(rob_model, _solver(1e-8, 1e-12, G, lu), g["p"], np.zeros((1, 0)), g["ts"],
                          g["my"], pscale=g["pscale"])
    assert r["status"][0] == 0
    assert_parity(r["x"], g["x"], gt["x"], 1e-8, 1e-12)
    assert abs(r["llh"][0] - gt["llh"][0]) <= 1e-6 * abs(gt["llh"][0])
    np.testing.assert_allclose(r["x"].sum(-1), 1.0, atol=1e-8)
    # forward-only run of the reference takes 1141 steps; step counts track it
    assert abs(int(r["numsteps"][0, -1]) - 1141) <= 0.2 * 1141


@pytest.mark.parametrize("lu", [32, 64])
@pytest.mark.parametrize("G", LANES)
def test_net20_subset_vs_reference(net20, G, lu):
    w, m = net20
    g, gt = _g("net20_fwd"), _g("net20_fwd_tight")
    r = ag.simulate_batch(m, _solver(w.rtol, w.atol, G, lu), g["p"], np.zeros((len(g["p"]), 0)),
                          g["ts"], pscale=g["pscale"])
    assert (r["status"] == 0).all()
    assert_parity(r["x"], g["x"], gt["x"], w.rtol, w.atol)
    rel = np.abs(r["numsteps"][:, -1] - g["numsteps"][:, -1]) / g["numsteps"][:, -1]
    assert np.median(rel) <= 0.05 and rel.max() <= 0.2


def test_net20_full_batch_vs_oracle(net20):
    w, m = net20
    r = ag.simulate_batch(m, _solver(w.rtol, w.atol), w.p, w.k, w.ts, pscale=w.pscale)
    o = Oracle(w.model).run(w.p, w.pscale, w.k, w.ts, rtol=w.rtol, atol=w.atol, nthreads=0)
    assert (r["status"] == 0).all() and (o["status"] == 0).all()
    assert_parity(r["x"], o["x"], None, w.rtol, w.atol, frac=0.99)
    assert np.all(np.abs(r["x"] - o["x"]) <= 1000 * (w.rtol * np.abs(o["x"]) + w.atol))


def test_run_simulations_api(rob_model):
    """The AMICI-style entry: ExpData list in, ReturnDataView list out."""
    g = _g("robertson_fsa")
    rob_model.set_parameter_scale(1)
    rob_model.set_parameters(g["p"][0])
    solver = rob_model.create_solver()
    solver.set_relative_tolerance(1e-8)
    solver.set_absolute_tolerance(1e-12)
    edatas = [ag.ExpData(ts=g["ts"][0], measurements=g["my"][0]) for _ in range(3)]
    edatas.append(ag.ExpData(ts=g["ts"][0][:10]))  # different grid -> separate batch
    rdatas = ag.run_simulations(rob_model, solver, edatas)
    assert len(rdatas) == 4
    for rd in rdatas[:3]:
        assert rd.status == ag.AMICI_SUCCESS
        assert rd.x.shape == (40, 3) and rd.y.shape == (40, 3) and rd.sigmay.shape == (40, 3)
        assert abs(rd.llh - g["llh"][0]) <= 1e-6 * abs(g["llh"][0])
    assert np.isnan(rdatas[3].llh) and rdatas[3].x.shape == (10, 3)
    np.testing.assert_allclose(rdatas[3].x, rdatas[0].x[:10], rtol=1e-6, atol=1e-12)
    rd = ag.run_simulation(rob_model, solver, edatas[0])
    assert rd.status == 0 and ag.runAmiciSimulations is ag.run_simulations


def test_too_much_work_status_matches_reference(rob_model):
    """maxsteps exhausted: AMICI_TOO_MUCH_WORK, outputs after the failure NaN,
    llh NaN, at the output where the reference fails."""
    w = robertson_workload()
    o = Oracle(w.model).run(w.p, w.pscale, w.k, w.ts, rtol=1e-8, atol=1e-12, maxsteps=300)
    r = ag.simulate_batch(rob_model, _solver(1e-8, 1e-12, 32, 64, maxsteps=300), w.p, w.k, w.ts,
                          np.zeros((1, 40, 3)), pscale=w.pscale)
    assert r["status"][0] == o["status"][0] == ag.simulation.AMICI_TOO_MUCH_WORK
    first_nan = np.argmax(np.isnan(r["x"][0, :, 0]))
    assert first_nan == np.argmax(np.isnan(o["x"][0, :, 0])) > 0
    assert np.isnan(r["llh"][0])


def test_edge_cases(rob_model):
    w = robertson_workload()
    s = _solver(1e-8, 1e-12)
    # empty batch
    r = ag.simulate_batch(rob_model, s, np.zeros((0, 3)), np.zeros((0, 0)), np.zeros((0, 5)),
                          pscale=w.pscale)
    assert r["x"].shape == (0, 5, 3)
    # outputs at t0 and repeated timepoints; NaN measurements are skipped
    ts = np.array([[0.0, 0.0, 1.0, 1.0, 10.0]])
    my = np.full((1, 5, 3), np.nan)
    my[0, 2, 0] = 0.97
    r = ag.simulate_batch(rob_model, s, w.p, np.zeros((1, 0)), ts, my, pscale=w.pscale)
    o = Oracle(w.model).run(w.p, w.pscale, w.k, ts, my, rtol=1e-8, atol=1e-12)
    assert r["status"][0] == 0
    np.testing.assert_array_equal(r["x"][0, 0], [1.0, 0.0, 0.0])
    np.testing.assert_array_equal(r["x"][0, 2], r["x"][0, 3])
    np.testing.assert_allclose(r["x"], o["x"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(r["llh"], o["llh"], rtol=1e-8)
    # data-provided noise scales override the model's sigma
    sg = np.full((1, 5, 3), np.nan)
    sg[0, 2, 0] = 0.5
    r2 = ag.simulate_batch(rob_model, s, w.p, np.zeros((1, 0)), ts, my, sg, pscale=w.pscale)
    assert r2["sigmay"][0, 2, 0] == 0.5 and r2["sigmay"][0, 2, 1] == 0.01
