"""GPU forward simulation vs the reference (golden vectors) and the CPU oracle.

A variable-step integrator's output is sensitive at the level of its global
error to any rounding difference: the reference itself, with its parameters
perturbed by 1e-15 relative, moves by up to ~45 (Robertson) and ~185 (n=20
network) tolerance units at single outputs, with 91% / 97% of entries within
10x the tolerance and step counts within 12% (tests/test_oracle.py measures
this envelope).  Parity is therefore asserted as:
  * agreement with the reference at the same tolerances inside that envelope
    (fraction of entries within 10x tolerance, maximal deviation);
  * accuracy against the reference at rtol = atol = 1e-12 no worse than the
    reference's own (99th percentile and maximum, in tolerance units);
  * llh within 1e-6 relative of the 1e-12 reference; steps within 20%.
"""
from pathlib import Path

import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import net20_workload, robertson_workload
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


def tol_units(a, ref, rtol, atol):
    return np.abs(a - ref) / (rtol * np.abs(ref) + atol)


def assert_parity(gpu, ref, tight, rtol, atol, *, frac=0.95, max_dev=400.0):
    e = tol_units(gpu, ref, rtol, atol)
    assert np.mean(e <= 10) >= frac, f"only {np.mean(e <= 10):.4f} of entries within 10x tolerance"
    assert e.max() <= max_dev, f"deviation {e.max():.1f} tolerance units"
    if tight is not None:
        eg, er = tol_units(gpu, tight, rtol, atol), tol_units(ref, tight, rtol, atol)
        assert np.percentile(eg, 99) <= 2 * np.percentile(er, 99) + 10, (np.percentile(eg, 99), np.percentile(er, 99))
        assert eg.max() <= 3 * er.max() + 10, (eg.max(), er.max())


@pytest.fixture(scope="module")
def rob_model():
    return ag.Model(robertson_workload().model)


@pytest.fixture(scope="module")
def net20():
    w = net20_workload(1024)
    m = ag.Model(w.model)
    m.set_parameter_scale(2)
    return w, m


@pytest.mark.parametrize("G,lu", [(G, 32) for G in LANES] + [(32, 64)])
def test_robertson_llh_and_states(rob_model, G, lu):
    g, gt = _g("robertson_fsa"), _g("robertson_fsa_tight")
    r = ag.simulate_batch(rob_model, _solver(1e-8, 1e-12, G, lu), g["p"], np.zeros((1, 0)), g["ts"],
                          g["my"], pscale=g["pscale"])
    assert r["status"][0] == 0
    assert_parity(r["x"], g["x"], gt["x"], 1e-8, 1e-12, frac=0.85, max_dev=100.0)
    assert abs(r["llh"][0] - gt["llh"][0]) <= 1e-6 * abs(gt["llh"][0])
    np.testing.assert_allclose(r["x"].sum(-1), 1.0, atol=1e-8)
    # forward-only run of the reference takes 1141 steps; step counts track it
    assert abs(int(r["numsteps"][0, -1]) - 1141) <= 0.2 * 1141


@pytest.mark.parametrize("G,lu", [(8, 32), (16, 32), (32, 32), (32, 64)])
def test_net20_subset_vs_reference(net20, G, lu):
    w, m = net20
    g, gt = _g("net20_fwd"), _g("net20_fwd_tight")
    r = ag.simulate_batch(m, _solver(w.rtol, w.atol, G, lu), g["p"], np.zeros((len(g["p"]), 0)),
                          g["ts"], pscale=g["pscale"])
    assert (r["status"] == 0).all()
    assert_parity(r["x"], g["x"], gt["x"], w.rtol, w.atol)
    rel = np.abs(r["numsteps"][:, -1] - g["numsteps"][:, -1]) / g["numsteps"][:, -1]
    total = abs(r["numsteps"][:, -1].sum() / g["numsteps"][:, -1].sum() - 1)
    assert total <= 0.05 and np.median(rel) <= 0.05 and rel.max() <= 0.3


def test_uncompiled_variants_are_rejected(net20):
    """Lane counts that would put more than 4 states on a lane are not compiled
    for the n=20 model, and FP64 LU runs one warp per instance."""
    w, m = net20
    for G, lu in ((2, 32), (8, 64)):
        with pytest.raises(ag._native.EngineError):
            ag.simulate_batch(m, _solver(w.rtol, w.atol, G, lu), w.p[:4], w.k[:4], w.ts[:4], pscale=w.pscale)


def test_net20_full_batch_vs_oracle(net20):
    w, m = net20
    r = ag.simulate_batch(m, _solver(w.rtol, w.atol), w.p, w.k, w.ts, pscale=w.pscale)
    o = Oracle(w.model).run(w.p, w.pscale, w.k, w.ts, rtol=w.rtol, atol=w.atol, nthreads=0)
    assert (r["status"] == 0).all() and (o["status"] == 0).all()
    assert_parity(r["x"], o["x"], None, w.rtol, w.atol, frac=0.95, max_dev=1000.0)


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
    # the 300th step falls into the same output interval, up to one interval
    # of step-sequence difference
    assert first_nan > 0 and abs(first_nan - np.argmax(np.isnan(o["x"][0, :, 0]))) <= 1
    assert np.isfinite(r["x"][0, :first_nan]).all() and np.isnan(r["x"][0, first_nan:]).all()
    assert r["numsteps"][0, first_nan - 1] < 300
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
    np.testing.assert_allclose(r["llh"], o["llh"], rtol=1e-6)  # llh target: 1e-6 relative
    # data-provided noise scales override the model's sigma
    sg = np.full((1, 5, 3), np.nan)
    sg[0, 2, 0] = 0.5
    r2 = ag.simulate_batch(rob_model, s, w.p, np.zeros((1, 0)), ts, my, sg, pscale=w.pscale)
    assert r2["sigmay"][0, 2, 0] == 0.5 and r2["sigmay"][0, 2, 1] == 0.01
