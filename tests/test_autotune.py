"""Residency-cap autotuner: candidate handling, selection and caching, with
the timed device call replaced by a table of times (host logic on the CPU)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import amici_gb300 as ag  # noqa: E402
from amici_gb300 import autotune  # noqa: E402
from amici_gb300.networks import robertson_model  # noqa: E402


def test_tune_instances_per_sm_picks_the_fastest_and_caches(monkeypatch):
    calls = []

    def fake(model, solver, theta, k, ts, my, method, reps):
        calls.append((solver.instances_per_sm, theta.shape[0], ts.shape, my.shape))
        return {0: 10.0, 1: 30.0, 2: 7.5, 3: 9.0}[solver.instances_per_sm]

    monkeypatch.setattr(autotune, "_time_sensitivity_call", fake)
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    monkeypatch.setattr(autotune, "_CACHE", {})
    real_as_tensor = torch.as_tensor
    monkeypatch.setattr(torch, "as_tensor", lambda a, dtype=None, device=None: real_as_tensor(a, dtype=dtype))
    monkeypatch.setattr(torch.Tensor, "to", lambda self, *a, **k: self)
    m = ag.Model(robertson_model())
    s = ag.Solver()
    theta = np.zeros((10, 3))
    r = autotune.tune_instances_per_sm(m, s, theta, None, np.linspace(1, 2, 4), np.zeros((10, 4, 3)),
                                       candidates=(0, 1, 2, 3), sample=8)
    assert r["best"] == 2 and r["n"] == 8 and set(r["ms"]) == {0, 1, 2, 3}
    assert [c[0] for c in calls] == [0, 1, 2, 3]
    assert all(c[1] == 8 and c[2] == (8, 4) and c[3] == (8, 4, 3) for c in calls)
    assert s.instances_per_sm == 0  # the caller's solver is left alone
    autotune.tune_instances_per_sm(m, s, theta, None, np.linspace(1, 2, 4), np.zeros((10, 4, 3)),
                                   candidates=(0, 1, 2, 3), sample=8)
    assert len(calls) == 4  # cached
    with pytest.raises(ValueError):
        autotune.tune_instances_per_sm(m, s, theta, None, np.ones(4), np.zeros((10, 4, 3)), candidates=(-1,))
