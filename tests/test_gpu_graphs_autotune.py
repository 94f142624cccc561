"""CUDA-graph-captured launches and the lanes-per-instance autotuner."""
import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.autotune import tune_lanes
from amici_gb300.codegen import lane_choices
from amici_gb300.graphs import GraphedSimulation
from amici_gb300.networks import net20_workload, robertson_workload

pytestmark = pytest.mark.gpu


def test_graph_replay_matches_direct_calls():
    torch = pytest.importorskip("torch")
    w = net20_workload(64)
    m = ag.Model(w.model)
    m.set_parameter_scale(w.pscale)
    s = ag.Solver()
    s.set_relative_tolerance(w.rtol)
    s.set_absolute_tolerance(w.atol)
    gs = GraphedSimulation(m, s, 64, w.ts.shape[1], with_data=False, want_x=True)
    for shift in (0.0, 0.1):  # two replays with different parameters
        p = w.p + shift
        gs.run(p=torch.tensor(p, device="cuda"), ts=torch.tensor(w.ts, device="cuda"))
        torch.cuda.synchronize()
        ref = ag.simulate_batch(m, s, p, w.k, w.ts, pscale=w.pscale)
        np.testing.assert_array_equal(gs.status.cpu().numpy(), ref["status"])
        np.testing.assert_array_equal(gs.x.cpu().numpy(), ref["x"])
        np.testing.assert_array_equal(gs.numsteps.cpu().numpy(), ref["numsteps"])


def test_graph_replay_adjoint():
    torch = pytest.importorskip("torch")
    g = dict(np.load(__import__("pathlib").Path(__file__).resolve().parent / "golden" / "robertson_asa.npz"))
    m = ag.Model(robertson_workload().model)
    m.set_parameter_scale(g["pscale"])
    s = ag.Solver()
    s.set_relative_tolerance(1e-8)
    s.set_absolute_tolerance(1e-12)
    s.set_sensitivity_order(ag.SensitivityOrder.first)
    s.set_sensitivity_method(ag.SensitivityMethod.adjoint)
    gs = GraphedSimulation(m, s, 1, g["ts"].shape[1])
    gs.run(p=torch.tensor(g["p"], device="cuda"), ts=torch.tensor(g["ts"], device="cuda"),
           my=torch.tensor(g["my"], device="cuda"))
    torch.cuda.synchronize()
    ref = ag.simulate_batch(m, s, g["p"], np.zeros((1, 0)), g["ts"], g["my"], pscale=g["pscale"])
    np.testing.assert_array_equal(gs.llh.cpu().numpy(), ref["llh"])
    np.testing.assert_array_equal(gs.sllh.cpu().numpy(), ref["sllh"])


def test_autotuner_picks_a_compiled_variant():
    w = net20_workload(256)
    m = ag.Model(w.model)
    m.set_parameter_scale(w.pscale)
    s = ag.Solver()
    s.set_relative_tolerance(w.rtol)
    s.set_absolute_tolerance(w.atol)
    res = tune_lanes(m, s, w.p, w.k, w.ts, reps=1)
    assert res["best"] in lane_choices(w.model)
    assert set(res["ms"]) == set(lane_choices(w.model))
    assert res["ms"][res["best"]] == min(res["ms"].values())
    # the tuned variant integrates the batch like the default one (same tolerances)
    s.set_lanes_per_instance(res["best"])
    r = ag.simulate_batch(m, s, w.p, w.k, w.ts, pscale=w.pscale)
    assert (r["status"] == 0).all()
