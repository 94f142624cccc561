"""The torch.autograd boundary: llh(theta) with the GPU adjoint gradient."""
from pathlib import Path

import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import net100_adjoint_workload, robertson_workload

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _solver(rtol, atol):
    s = ag.Solver()
    s.set_relative_tolerance(rtol)
    s.set_absolute_tolerance(atol)
    s.set_max_steps(100000)
    return s


def test_robertson_grad_matches_reference():
    torch = pytest.importorskip("torch")
    g, t = dict(np.load(GOLD / "robertson_asa.npz")), dict(np.load(GOLD / "robertson_asa_tight.npz"))
    m = ag.Model(robertson_workload().model)
    m.set_parameter_scale(g["pscale"])
    theta = torch.tensor(g["p"][0], dtype=torch.float64, device="cuda", requires_grad=True)
    llh = ag.LogLikelihood.apply(theta, m, _solver(1e-8, 1e-12), None, g["ts"][0], g["my"][0])
    (-llh).backward()  # a negative log-likelihood objective
    torch.cuda.synchronize()
    assert abs(float(llh) - t["llh"][0]) <= 1e-6 * abs(t["llh"][0])
    grad = -theta.grad.cpu().numpy()
    assert np.all(np.abs(grad - t["sllh"][0]) <= 1e-4 * np.abs(t["sllh"][0]).max())


def test_batched_grad_is_the_adjoint_sllh():
    """Per-condition gradients of sum(w_i * llh_i) through autograd equal w_i times
    the engine's sllh of the same conditions (same kernel, same inputs)."""
    torch = pytest.importorskip("torch")
    g = dict(np.load(GOLD / "net100_asa.npz"))
    m = ag.Model(net100_adjoint_workload(1).model)
    m.set_parameter_scale(g["pscale"])
    s = _solver(float(g["rtol"]), float(g["atol"]))
    theta = torch.tensor(g["p"], dtype=torch.float64, device="cuda", requires_grad=True)
    llh = ag.LogLikelihood.apply(theta, m, s, g["k"], g["ts"], g["my"])
    wts = torch.arange(1, 5, dtype=torch.float64, device="cuda")
    (wts * llh).sum().backward()
    s2 = _solver(float(g["rtol"]), float(g["atol"]))
    s2.set_sensitivity_order(ag.SensitivityOrder.first)
    s2.set_sensitivity_method(ag.SensitivityMethod.adjoint)
    r = ag.simulate_batch(m, s2, g["p"], g["k"], g["ts"], g["my"], pscale=g["pscale"])
    np.testing.assert_array_equal(llh.detach().cpu().numpy(), r["llh"])
    np.testing.assert_array_equal(theta.grad.cpu().numpy(), np.arange(1, 5)[:, None] * r["sllh"])


def test_side_stream_results_match_the_current_stream():
    """log_likelihood_and_gradient on a side stream (a torch stream or a raw
    cudaStream_t handle): the results are ordered before torch's current
    stream reads them and equal those of a launch on the current stream."""
    torch = pytest.importorskip("torch")
    g = dict(np.load(GOLD / "robertson_asa.npz"))
    m = ag.Model(robertson_workload().model)
    m.set_parameter_scale(g["pscale"])
    s = _solver(float(g["rtol"]), float(g["atol"]))
    ref = ag.log_likelihood_and_gradient(m, s, g["p"], None, g["ts"], g["my"])
    side = torch.cuda.Stream()
    for stream in (side, side.cuda_stream):
        llh, sllh, st = ag.log_likelihood_and_gradient(m, s, g["p"], None, g["ts"], g["my"], stream=stream)
        # read on the current stream without an explicit synchronisation of the side stream
        np.testing.assert_array_equal(llh.cpu().numpy(), ref[0].cpu().numpy())
        np.testing.assert_array_equal(sllh.cpu().numpy(), ref[1].cpu().numpy())
        assert int(st.cpu()[0]) == 0
