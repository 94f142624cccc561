"""Objective over conditions (parameter mapping and llh/sllh aggregation) on
the CPU, with the device call replaced by an analytic log-likelihood: the
mapping, its scale conversions and the pull-back of the condition gradients
against finite differences, and the reference's error and failure rules."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import amici_gb300 as ag  # noqa: E402
from amici_gb300 import objective as objmod  # noqa: E402
from amici_gb300.networks import robertson_model  # noqa: E402
from amici_gb300.objective import ConditionMapping, Objective  # noqa: E402

A = np.array([[0.3, -1.2, 0.7], [1.1, 0.2, -0.4], [-0.5, 0.9, 0.1]])


def _fake_engine(status=None):
    """llh_c = -1/2 sum_j (j+1) (p_cj - A_cj)^2 on the model scale; sllh its gradient."""
    def f(model, solver, p, k, ts, my, sigma=None, *, stream=None, **kw):
        w = torch.arange(1, p.shape[1] + 1, dtype=p.dtype)
        d = p - torch.as_tensor(A[:p.shape[0], :p.shape[1]])
        llh = -0.5 * (w * d * d).sum(1)
        st = torch.zeros(p.shape[0], dtype=torch.int32) if status is None else torch.as_tensor(status)
        return llh, -(w * d), st
    return f


def _objective(monkeypatch, status=None):
    monkeypatch.setattr(objmod, "log_likelihood_and_gradient", _fake_engine(status))
    spec = robertson_model()
    m = ag.Model(spec)
    m.set_parameter_scale([ag.ParameterScaling.ln, ag.ParameterScaling.log10, ag.ParameterScaling.none])
    p1, p2, p3 = spec.parameter_ids
    maps = [
        ConditionMapping({p1: "a", p2: "b", p3: 2.5}, {p1: "log10", p2: "log", p3: "lin"}),
        ConditionMapping({p1: "a", p2: -0.3, p3: "c"}, {p1: "log10", p2: "log10", p3: "lin"}),
        ConditionMapping({p1: "b", p2: "a", p3: float("nan")}, {p1: "log", p2: "log10"}),
    ]
    ts = np.linspace(0.1, 1.0, 4)
    o = Objective(m, ag.Solver(), ["a", "b", "c", "unused"], ["log10", "log", "lin", "lin"], maps, ts,
                  np.zeros((3, 4, 3)))
    o.device = torch.device("cpu")
    return o


def _llh_at(o, theta):
    return o(theta)["llh"]


def test_mapping_values(monkeypatch):
    o = _objective(monkeypatch)
    th = torch.tensor([0.5, -0.7, 3.0, 9.0], dtype=torch.float64)
    p = o.map_parameters(th).numpy()
    # condition 0: a on log10 -> model ln; b on ln -> model log10; 2.5 lin -> lin
    np.testing.assert_allclose(p[0], [0.5 * np.log(10), -0.7 / np.log(10), 2.5], rtol=1e-14)
    # condition 1: the constant -0.3 on log10 is the model's scale already
    np.testing.assert_allclose(p[1], [0.5 * np.log(10), -0.3, 3.0], rtol=1e-14)
    # condition 2: b (ln) onto the model's ln untouched, a (log10) onto log10, NaN constant -> 0
    assert p[2, 0] == -0.7 and p[2, 1] == 0.5 and p[2, 2] == 0.0


@pytest.mark.parametrize("scaled", [True, False])
def test_gradient_matches_finite_differences(monkeypatch, scaled):
    o = _objective(monkeypatch)
    th = np.array([0.5, -0.7, 3.0, 9.0])
    r = o(th, scaled_gradients=scaled)
    assert r["llh"] == pytest.approx(r["llh_conditions"].sum())
    fd = np.zeros(4)
    for i in range(4):
        h = 1e-6
        if scaled:
            e = np.zeros(4)
            e[i] = h
            fd[i] = (_llh_at(o, th + e) - _llh_at(o, th - e)) / (2 * h)
        else:
            # perturb the linear value of parameter i
            lin = objmod._unscale(th, o.problem_scales)

            def scaled_of(v):
                out = th.copy()
                s = o.problem_scales[i]
                out[i] = np.log10(v) if s == 2 else (np.log(v) if s == 1 else v)
                return out
            hh = h * max(1.0, abs(lin[i]))
            fd[i] = (_llh_at(o, scaled_of(lin[i] + hh)) - _llh_at(o, scaled_of(lin[i] - hh))) / (2 * hh)
    np.testing.assert_allclose(r["sllh"], fd, rtol=1e-6, atol=1e-8)
    assert r["sllh"][3] == 0.0  # used by no condition


def test_failed_condition_gives_no_gradient(monkeypatch):
    o = _objective(monkeypatch, status=[0, -1, 0])
    r = o(np.array([0.5, -0.7, 3.0, 9.0]))
    assert r["sllh"] is None and list(r["status"]) == [0, -1, 0]


def test_mapping_errors(monkeypatch):
    monkeypatch.setattr(objmod, "log_likelihood_and_gradient", _fake_engine())
    spec = robertson_model()
    m = ag.Model(spec)
    p1, p2, p3 = spec.parameter_ids
    ts, my = np.ones(2), np.zeros((1, 2, 3))
    with pytest.raises(ValueError, match="not mapped"):
        Objective(m, ag.Solver(), ["a"], ["lin"], [ConditionMapping({p1: "a", p2: 1.0})], ts, my)
    with pytest.raises(ValueError, match="unknown problem parameter"):
        Objective(m, ag.Solver(), ["a"], ["lin"], [ConditionMapping({p1: "a", p2: "zz", p3: 1.0})], ts, my)
    with pytest.raises(ValueError, match="differs"):
        Objective(m, ag.Solver(), ["a"], ["log10"],
                  [ConditionMapping({p1: "a", p2: 1.0, p3: 1.0}, {p1: "log"})], ts, my)
    with pytest.raises(ValueError, match="unknown parameter scale"):
        Objective(m, ag.Solver(), ["a"], ["log2"], [ConditionMapping({p1: "a", p2: 1.0, p3: 1.0})], ts, my)


def test_fixed_parameters_from_constants_and_problem_parameters(monkeypatch):
    monkeypatch.setattr(objmod, "log_likelihood_and_gradient", _fake_engine())
    from amici_gb300.networks import net100_adjoint_workload

    spec = net100_adjoint_workload(1).model
    m = ag.Model(spec)
    pm = {pid: 0.0 for pid in spec.parameter_ids}
    k0, k1 = spec.fixed_parameter_ids[:2]
    maps = [ConditionMapping(dict(pm), map_sim_fix={k0: 2.0, k1: "s"}), ConditionMapping(dict(pm))]
    o = Objective(m, ag.Solver(), ["s"], ["log10"], maps, np.ones(3), np.zeros((2, 3, spec.ny)))
    k = o.fixed_parameters(np.array([0.5]))
    nominal = np.asarray(spec.k_nominal) if spec.k_nominal else np.zeros(spec.nk)
    np.testing.assert_allclose(k[0, :2], [2.0, 10 ** 0.5])  # problem parameters enter unscaled
    np.testing.assert_allclose(k[0, 2:], nominal[2:])
    np.testing.assert_allclose(k[1], nominal)


def _fake_by_time():
    """As ``_fake_engine``, with the condition read from ts[c, 0] (so that a
    shard of the conditions sees its own targets)."""
    def f(model, solver, p, k, ts, my, sigma=None, *, stream=None, **kw):
        c = np.asarray(ts)[:, 0].astype(int)
        w = torch.arange(1, p.shape[1] + 1, dtype=p.dtype)
        d = p - torch.as_tensor(A[c][:, :p.shape[1]])
        st = torch.zeros(p.shape[0], dtype=torch.int32)
        return -0.5 * (w * d * d).sum(1), -(w * d), st
    return f


def _sharded_objective():
    spec = robertson_model()
    m = ag.Model(spec)
    m.set_parameter_scale([ag.ParameterScaling.ln, ag.ParameterScaling.log10, ag.ParameterScaling.none])
    p1, p2, p3 = spec.parameter_ids
    maps = [ConditionMapping({p1: "a", p2: "b", p3: 2.5}, {p1: "log10", p2: "log"}),
            ConditionMapping({p1: "a", p2: -0.3, p3: "c"}, {p1: "log10", p2: "log10"}),
            ConditionMapping({p1: "b", p2: "a", p3: "c"}, {p1: "log", p2: "log10"})]
    ts = np.array([[float(c), 1.0, 2.0] for c in range(3)])
    o = Objective(m, ag.Solver(), ["a", "b", "c"], ["log10", "log", "lin"], maps, ts, np.zeros((3, 3, 3)))
    o.device = torch.device("cpu")
    return o


def _objective_worker(rank, world, port, out_path):
    import os

    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    objmod.log_likelihood_and_gradient = _fake_by_time()  # this child process only
    o = _sharded_objective()
    th = np.array([0.4, -0.2, 1.5])
    tot = objmod.allreduce(o, o.shard(rank, world)(th))
    if rank == 0:
        np.savez(out_path, llh=tot["llh"], sllh=tot["sllh"], n_failed=tot["n_failed"])
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_objective_allreduce_equals_single_process(tmp_path, monkeypatch):
    """Two gloo ranks, each evaluating its shard of the conditions, combine to
    the single-process objective."""
    import socket

    import torch.multiprocessing as mp

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    out = tmp_path / "obj.npz"
    mp.spawn(_objective_worker, args=(2, port, str(out)), nprocs=2, join=True)
    got = np.load(out)
    monkeypatch.setattr(objmod, "log_likelihood_and_gradient", _fake_by_time())
    ref = _sharded_objective()(np.array([0.4, -0.2, 1.5]))
    assert int(got["n_failed"]) == 0
    np.testing.assert_allclose(float(got["llh"]), ref["llh"], rtol=1e-14)
    np.testing.assert_allclose(got["sllh"], ref["sllh"], rtol=1e-14)
    with pytest.raises(ValueError, match="more ranks"):
        _sharded_objective().shard(3, 4)


def test_objective_without_problem_parameters(monkeypatch):
    monkeypatch.setattr(objmod, "log_likelihood_and_gradient", _fake_engine())
    spec = robertson_model()
    m = ag.Model(spec)
    p1, p2, p3 = spec.parameter_ids
    o = Objective(m, ag.Solver(), [], [], [ConditionMapping({p1: 0.3, p2: -1.2, p3: 0.7})], np.ones(2),
                  np.zeros((1, 2, 3)))
    o.device = torch.device("cpu")
    r = o(np.zeros(0))
    assert r["llh"] == 0.0 and r["sllh"].shape == (0,)
