"""ExpData: the reference fields this engine does not implement make the
simulation call raise rather than being ignored, and unknown attributes are
refused (host logic, no GPU)."""
import numpy as np
import pytest

import amici_gb300 as ag
from amici_gb300.networks import robertson_model
from amici_gb300.simulation import _stack_inputs


@pytest.mark.parametrize("field,value", [("fixed_parameters_presimulation", [1.0]), ("t_presim", 5.0),
                                         ("reinitialize_fixed_parameter_initial_states", True)])
def test_unsupported_fields_raise(field, value):
    m = ag.Model(robertson_model())
    e = ag.ExpData(ts=np.linspace(0, 1, 3))
    setattr(e, field, value)
    with pytest.raises(NotImplementedError, match=field):
        _stack_inputs(m, [e])


def test_post_equilibration_output_times():
    """Outputs at t = inf (post-equilibration) are accepted after the finite
    ones and refused anywhere else."""
    m = ag.Model(robertson_model())
    e = ag.ExpData(ts=np.array([0.0, 1.0, np.inf, np.inf]))
    _stack_inputs(m, [e])
    for bad in ([0.0, np.inf, 1.0], [-np.inf, 1.0]):
        e.ts = np.array(bad)
        with pytest.raises(ValueError, match="ts"):
            _stack_inputs(m, [e])


def test_supported_batch_and_unknown_attribute():
    m = ag.Model(robertson_model())
    e = ag.ExpData(ts=np.linspace(0, 1, 3), measurements=np.zeros((3, 3)))
    p, pscale, k, ts, my, sg, plist, extra = _stack_inputs(m, [e, e])
    assert p.shape == (2, 3) and ts.shape == (2, 3) and my.shape == (2, 3, 3) and sg is None and plist is None
    assert extra == {"k_preeq": None, "x0": None, "sx0": None}
    with pytest.raises(AttributeError):
        e.fixed_parameters_preequilibration = [1.0]  # misspelt: refused instead of ignored


def test_parameter_list_reaches_the_batch():
    """ExpData.plist selects the sensitivity parameters (as edata.plist in the
    reference); one batch shares one list."""
    m = ag.Model(robertson_model())
    e1 = ag.ExpData(ts=np.linspace(0, 1, 3), plist=np.array([2, 0]))
    e2 = ag.ExpData(ts=np.linspace(0, 1, 3), plist=np.array([2, 0]))
    *_, plist, _ = _stack_inputs(m, [e1, e2])
    assert plist.tolist() == [2, 0] and plist.dtype == np.int32
    with pytest.raises(ValueError, match="parameter list"):
        _stack_inputs(m, [e1, ag.ExpData(ts=np.linspace(0, 1, 3))])


def test_expdata_parameter_scale_overrides_the_models():
    m = ag.Model(robertson_model())
    m.set_unscaled_parameters([0.04, 3e7, 1e4])
    m.set_parameter_scale(ag.ParameterScaling.ln)
    e = ag.ExpData(ts=np.linspace(0, 1, 3), pscale=np.full(3, int(ag.ParameterScaling.log10)))
    p, pscale, *_ = _stack_inputs(m, [e])
    assert pscale.tolist() == [2, 2, 2]
    np.testing.assert_allclose(p[0], np.log10([0.04, 3e7, 1e4]), rtol=1e-14)
    p, pscale, *_ = _stack_inputs(m, [ag.ExpData(ts=np.linspace(0, 1, 3))])
    assert pscale.tolist() == [1, 1, 1]
    np.testing.assert_allclose(p[0], np.log([0.04, 3e7, 1e4]), rtol=1e-14)


def test_run_simulations_groups_batches_and_fills_results(monkeypatch):
    """run_simulations splits the ExpData list into batches by output grid,
    parameter list and parameter scale, hands each batch's list to the
    engine, and returns results in the caller's order with the counters."""
    from amici_gb300 import simulation as sim

    calls = []

    def fake(model, solver, p, k, ts, my=None, sigma=None, *, pscale=None, plist=None, stream=0, **kw):
        n, nt = ts.shape
        calls.append((n, nt, None if plist is None else plist.tolist(), pscale.tolist()))
        diag = np.tile(np.arange(8, dtype=np.int32), (n, 1)) + 100 * nt
        return dict(x=np.zeros((n, nt, 3)), y=np.zeros((n, nt, 3)), sigmay=np.zeros((n, nt, 3)),
                    llh=np.arange(n, dtype=float) + nt, numsteps=np.zeros((n, nt), np.int32),
                    status=np.zeros(n, np.int32), diag=diag, sx=None, sy=None, sllh=None)

    monkeypatch.setattr(sim, "simulate_batch", fake)
    m = ag.Model(robertson_model())
    E = ag.ExpData
    eds = [E(ts=np.linspace(0, 1, 3)), E(ts=np.linspace(0, 1, 4)), E(ts=np.linspace(0, 1, 3), plist=[1]),
           E(ts=np.linspace(0, 1, 3)), E(ts=np.linspace(0, 1, 3), pscale=[2, 2, 2])]
    rs = ag.run_simulations(m, ag.Solver(), eds)
    assert sorted(map(repr, calls)) == sorted(map(repr, [(2, 3, None, [0, 0, 0]), (1, 4, None, [0, 0, 0]),
                                                         (1, 3, [1], [0, 0, 0]), (1, 3, None, [2, 2, 2])]))
    assert [r.ts.size for r in rs] == [3, 4, 3, 3, 3]
    assert rs[3].llh == 4.0 and rs[0].llh == 3.0  # second of its batch / first of its batch
    assert rs[1].diagnostics["steps"] == 400 and rs[1].diagnostics["backward_steps"] == 407
    assert set(rs[0].diagnostics) == set(sim.DIAGNOSTIC_NAMES) and rs[0].cpu_time >= 0.0


@pytest.mark.parametrize("failfast", [True, False])
def test_failfast_skips_every_instance_after_the_first_failure(monkeypatch, failfast):
    """With failfast, every ExpData after the first failed one (list order)
    gets the reference's empty ReturnData: status AMICI_NOT_RUN, NaN llh and
    sllh, zero states and step counts (src/amici.cpp:245-260,
    src/rdata.cpp:104-200); without it every result is kept."""
    from amici_gb300 import simulation as sim

    def fake(model, solver, p, k, ts, my=None, sigma=None, *, pscale=None, plist=None, stream=0, **kw):
        n, nt = ts.shape
        status = np.zeros(n, np.int32)
        status[1] = -1  # the second instance of the batch runs out of steps
        return dict(x=np.ones((n, nt, 3)), y=np.ones((n, nt, 3)), sigmay=np.ones((n, nt, 3)),
                    llh=np.arange(n, dtype=float), numsteps=np.ones((n, nt), np.int32), status=status,
                    diag=np.ones((n, 8), np.int32), sx=None, sy=None, sllh=np.ones((n, 3)))

    monkeypatch.setattr(sim, "simulate_batch", fake)
    m = ag.Model(robertson_model())
    s = ag.Solver()
    s.set_sensitivity_order(ag.SensitivityOrder.first)
    s.set_sensitivity_method(ag.SensitivityMethod.adjoint)
    eds = [ag.ExpData(ts=np.linspace(0, 1, 3)) for _ in range(4)]
    rs = ag.run_simulations(m, s, eds, failfast=failfast)
    assert [r.status for r in rs[:2]] == [0, -1] and rs[0].llh == 0.0
    if failfast:
        for r in rs[2:]:
            assert r.status == sim.AMICI_NOT_RUN and np.isnan(r.llh) and np.isnan(r.sllh).all()
            assert not r.x.any() and not r.numsteps.any() and r.x.shape == (3, 3)
    else:
        assert [r.status for r in rs[2:]] == [0, 0] and rs[3].llh == 3.0


def test_preequilibration_and_initial_states_reach_the_batch():
    """ExpData's pre-equilibration parameters and x0 / sx0 overrides are
    stacked per batch (sx0 parameter-major, as edata.sx0); a batch gives them
    for all of its ExpData or for none."""
    from amici_gb300.networks import preeq_model
    m = ag.Model(preeq_model())
    m.set_parameter_list([3, 1])
    ts = np.linspace(0, 1, 3)
    es = [ag.ExpData(ts=ts, fixed_parameters=[1.0, 2.0], fixed_parameters_pre_equilibration=[0.1, 0.2],
                     x0=np.arange(12.0) + i, sx0=np.arange(24.0) * (i + 1)) for i in range(2)]
    *_, plist, extra = _stack_inputs(m, es)
    assert extra["k_preeq"].tolist() == [[0.1, 0.2]] * 2
    assert extra["x0"].shape == (2, 12) and extra["x0"][1, 0] == 1.0
    assert extra["sx0"].shape == (2, 2, 12) and extra["sx0"][1, 1, 0] == 24.0
    with pytest.raises(ValueError, match="fixed_parameters_pre_equilibration"):
        _stack_inputs(m, [es[0], ag.ExpData(ts=ts, fixed_parameters=[1.0, 2.0], x0=np.zeros(12),
                                            sx0=np.zeros(24))])
