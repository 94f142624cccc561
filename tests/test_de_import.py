"""The DEExporter hook: ``model_spec_from_de_model`` on the reference's own
``DEModel`` (``python/sdist/amici/_symbolic/de_model.py``), filled with the
reference's components the way its importers fill it: fluxes as
``Expression`` components, each state's ``dt`` the stoichiometric sum over
flux symbols divided by a compartment volume, observables with ``SigmaY``
noise scales and ``LogLikelihoodY`` cost functions made by the reference's
``noise_distribution_to_cost_function``, events with assignments.  The
ModelSpec read back must simulate (oracle) to the same results as the
workload models it was built from: mass action (net20), general rate laws
and a log-normal observable (mapk9), all six noise distributions and
nonlinear observables (obs6), explicit trigger times with a loading dose at
t0 (dose4), a trigger function with state resets (fire3), Heaviside
switches of the states and of time (switch3, raw and as the event symbols
the reference's importer leaves in the expressions).

The reference package's ``__init__`` needs libsbml, absent here, so its
``amici`` package is entered without it, and its ``toposort`` dependency
(not installed) is stood in for by Kahn's algorithm; the test is skipped
where the reference tree is absent."""
import sys
import types

import numpy as np
import pytest
import sympy as sp

from amici_gb300.de_import import model_spec_from_de_model, noise_distribution_of_cost
from amici_gb300.model_spec import TIME
from amici_gb300.networks import (PSCALE_LN, dosing_workload, fire_workload, mapk_workload, net20_workload,
                                  obs_workload, switch_workload)
from oracle.pyoracle import REF_ROOT, Oracle

REF = REF_ROOT / "python" / "sdist" / "amici"
pytestmark = pytest.mark.skipif(not REF.is_dir(), reason="reference tree absent")


def _toposort(data):
    """Kahn's algorithm as the toposort package publishes it: sets of items
    whose dependencies all came in earlier sets."""
    data = {key: set(v) - {key} for key, v in data.items()}
    for item in set().union(*data.values()) - set(data) if data else set():
        data[item] = set()
    while data:
        ready = {key for key, v in data.items() if not v}
        if not ready:
            raise ValueError("cyclic dependencies")
        yield ready
        data = {key: v - ready for key, v in data.items() if key not in ready}


@pytest.fixture(scope="module")
def ref():
    saved = {k: v for k, v in sys.modules.items() if k == "amici" or k.startswith("amici.") or k == "toposort"}
    pkg = types.ModuleType("amici")
    pkg.__path__ = [str(REF)]
    pkg.__version__ = "reference"
    tp = types.ModuleType("toposort")
    tp.toposort = _toposort
    tp.toposort_flatten = lambda d, sort=True: [x for s in _toposort(d) for x in (sorted(s, key=str) if sort else s)]
    sys.modules["amici"] = pkg
    sys.modules["toposort"] = tp
    try:
        import amici._symbolic.de_model as dm
        import amici._symbolic.de_model_components as dc
        from amici.importers.utils import noise_distribution_to_cost_function
        yield types.SimpleNamespace(DEModel=dm.DEModel, c=dc, cost=noise_distribution_to_cost_function)
    finally:
        for k in [k for k in sys.modules if k == "amici" or k.startswith("amici.") or k == "toposort"]:
            del sys.modules[k]
        sys.modules.update(saved)


def de_model_of(ref, spec, volumes=None):
    """A DEModel of ``spec`` as the reference's SBML importer would build it
    (fluxes as expressions, dt = sum_r S_ir flux_r / V_i)."""
    c = ref.c
    de = ref.DEModel()
    t = sp.Symbol("t", real=True)
    tmap = {TIME: t}
    for j, (pj, v) in enumerate(zip(spec.p, spec.p_nominal)):
        de.add_component(c.FreeParameter(pj, spec.parameter_ids[j], v))
    for j, (kj, v) in enumerate(zip(spec.k, spec.k_nominal)):
        de.add_component(c.FixedParameter(kj, spec.fixed_parameter_ids[j], v))
    fsym = [sp.Symbol(f"flux_r{r}", real=True) for r in range(spec.nw)]
    for r, w in enumerate(spec.w):
        de.add_component(c.Expression(fsym[r], f"flux_r{r}", sp.sympify(w).xreplace(tmap)))
    vol = volumes or [1] * spec.nx
    for i, xi in enumerate(spec.x):
        dt = sum((sp.Integer(s) * fsym[r] for (ii, r), s in sorted(spec.stoich.items()) if ii == i), sp.Integer(0))
        de.add_component(c.DifferentialState(xi, spec.state_ids[i], sp.sympify(spec.x0[i]), dt / vol[i]))
    noise = spec.noise_distributions or ["normal"] * spec.ny
    for iy, yv in enumerate(spec.y):
        oid = spec.observable_ids[iy]
        ysym = sp.Symbol(oid, real=True)
        ob = c.Observable(ysym, oid, sp.sympify(yv))
        de.add_component(ob)
        ssym = sp.Symbol(f"sigma{oid}", real=True)
        de.add_component(c.SigmaY(ssym, f"sigma{oid}", sp.sympify(spec.sigma_y[iy])))
        names = (oid, f"m{oid}", f"sigma{oid}")
        cost = sp.sympify(ref.cost(noise[iy])(oid), locals=dict(zip(names, (ysym, ob.get_measurement_symbol(), ssym))))
        de.add_component(c.LogLikelihoodY(sp.Symbol(f"J{oid}", real=True), f"J{oid}", cost))
    for ie, ev in enumerate(spec.events):
        trig = (ev.direction * (t - sp.sympify(ev.time))) if ev.time is not None else sp.sympify(ev.trigger).xreplace(tmap)
        assign = {spec.x[i]: spec.x[i] + sp.sympify(b) for i, b in ev.bolus.items()}
        de.add_component(c.Event(sp.Symbol(f"event{ie}", real=True), f"event{ie}", trig,
                                 use_values_from_trigger_time=True, assignments=assign,
                                 initial_value=ev.initial_value))
    return de


def _run(spec, w, sensi, n=4):
    o = Oracle(spec)
    kw = dict(rtol=1e-10, atol=1e-12, maxsteps=100000, nthreads=0)
    k = w.k[:n] if w.k is not None else np.zeros((n, spec.nk))
    return o.run(w.p[:n], w.pscale, k, w.ts[:n], w.my[:n] if w.my is not None else None, sensi=sensi, **kw)


def _synthetic_my(w):
    if w.my is None:
        w.my = np.exp(np.random.default_rng(0).normal(0.0, 0.3, (w.p.shape[0], w.ts.shape[1], w.model.ny)))
    return w


WORKLOADS = {
    "net20": lambda: net20_workload(4),
    "mapk9": lambda: mapk_workload(4),
    "obs6": lambda: obs_workload(4),
    "dose4": lambda: dosing_workload(4),
    "fire3": lambda: fire_workload(4),
    "switch3": lambda: switch_workload(4),
}


@pytest.mark.parametrize("name", list(WORKLOADS))
def test_de_model_round_trip(ref, name):
    w = _synthetic_my(WORKLOADS[name]())
    spec = w.model
    got = model_spec_from_de_model(de_model_of(ref, spec), name + "_de")
    assert (got.nx, got.np, got.nk, got.ny, got.ne) == (spec.nx, spec.np, spec.nk, spec.ny, spec.ne)
    assert got.noise_distributions == (spec.noise_distributions or ["normal"] * spec.ny)
    assert [e.trigger is None for e in got.events] == [e.trigger is None for e in spec.events]
    for sensi in (0, 1):
        a, b = _run(spec, w, sensi), _run(got, w, sensi)
        assert (a["status"] == 0).all() and (b["status"] == 0).all()
        for key in ("x", "y", "llh") + (("sx", "sllh") if sensi else ()):
            np.testing.assert_allclose(b[key], a[key], rtol=1e-6, atol=1e-9, err_msg=f"{name} {key}")


def test_de_model_compartment_volumes(ref):
    """dt = S w / V with V not 1: each flux with a non-integer coefficient
    becomes |c| w with an integer stoichiometry; results equal a model
    written with the volumes in the fluxes."""
    w = net20_workload(4)
    spec = w.model
    vols = [sp.Rational(1, 2) if i % 3 == 0 else (sp.Integer(3) if i % 3 == 1 else sp.Integer(1))
            for i in range(spec.nx)]
    got = model_spec_from_de_model(de_model_of(ref, spec, vols), "net20_vol")
    assert all(isinstance(v, int) for v in got.stoich.values())
    # the same model written directly: species i's rows divided by V_i
    direct_w, direct_s = [], {}
    for (i, r), s in sorted(spec.stoich.items()):
        direct_s[(i, len(direct_w))] = 1 if s > 0 else -1
        direct_w.append(abs(sp.Integer(s)) / vols[i] * spec.w[r])
    direct = type(spec)(**{**spec.__dict__, "name": "net20_vol_direct", "w": direct_w, "stoich": direct_s})
    a, b = _run(direct, w, 0), _run(got, w, 0)
    np.testing.assert_allclose(b["x"], a["x"], rtol=1e-6, atol=1e-9)


def test_noise_recognition_matches_reference_costs(ref):
    y, m, s = sp.symbols("obs mobs sigmaobs", real=True)
    for dist in ("normal", "log-normal", "log10-normal", "laplace", "log-laplace", "log10-laplace"):
        cost = sp.sympify(ref.cost(dist)("obs"), locals={"obs": y, "mobs": m, "sigmaobs": s})
        assert noise_distribution_of_cost(cost, y, m, s) == dist
    with pytest.raises(ValueError):
        noise_distribution_of_cost((y - m) ** 4 / s, y, m, s)


def test_de_model_refusals(ref):
    c = ref.c
    spec = fire_workload(2).model
    de = de_model_of(ref, spec)
    de._events[0]._priority = sp.Integer(1)
    with pytest.raises(NotImplementedError, match="priorit"):
        model_spec_from_de_model(de, "x")
    de = de_model_of(ref, spec)
    de.add_component(c.AlgebraicState(sp.Symbol("z", real=True), "z", sp.Integer(0)))
    with pytest.raises(NotImplementedError, match="algebraic"):
        model_spec_from_de_model(de, "x")


def test_explicit_trigger_time_detected(ref):
    """a (t - te(p, k)) becomes an explicit trigger time with direction
    sign(a) (also te - t, which crosses downwards); a state trigger stays a
    trigger function."""
    c = ref.c
    spec = dosing_workload(2).model
    de = de_model_of(ref, spec)
    got = model_spec_from_de_model(de, "d")
    assert all(e.time is not None and e.trigger is None and e.direction == 1 for e in got.events)
    assert sp.simplify(got.events[2].time - spec.events[2].time) == 0
    t = sp.Symbol("t", real=True)
    de._events = [c.Event(sp.Symbol("e", real=True), "e", spec.p[0] - t, use_values_from_trigger_time=True,
                          assignments={spec.x[0]: spec.x[0] + 1}),
                  c.Event(sp.Symbol("f", real=True), "f", spec.x[0] - spec.p[1], use_values_from_trigger_time=True,
                          assignments={spec.x[1]: spec.x[1] + 1})]
    got = model_spec_from_de_model(de, "d2")
    assert got.events[0].time == spec.p[0] and got.events[0].direction == -1 and got.events[0].trigger is None
    assert got.events[1].time is None and got.events[1].trigger is not None
    assert PSCALE_LN == 1


def test_de_model_processed_heavisides(ref):
    """A DEModel whose importer already replaced every Heaviside(g) by the
    symbol of an event on g (with the event on -g beside it), as
    DEModel._process_heavisides does: the hook turns the symbols back into
    Heavisides and the model simulates as switch3 itself."""
    from amici_gb300.model_spec import TIME, expand_heavisides
    w = _synthetic_my(switch_workload(4))
    spec = w.model
    c = ref.c
    t = sp.Symbol("t", real=True)
    expanded = expand_heavisides(spec)
    # switch3 with its Heavisides as event symbols, the events of the pairs in order
    de = de_model_of(ref, type(spec)(**{**spec.__dict__, "w": [sp.Integer(0)] * spec.nw}))
    esym = [sp.Symbol(f"Heaviside_{ie}", real=True) for ie in range(expanded.ne)]
    hmap = {expanded.k[spec.nk + j]: esym[ie] for j, ie in enumerate(expanded.heaviside_events)}
    de._expressions = [c.Expression(e.get_sym(), e.get_name(), sp.sympify(wr).xreplace(hmap).xreplace({TIME: t}))
                       for e, wr in zip(de._expressions, expanded.w)]
    de._events = []
    for ie, ev in enumerate(expanded.events):
        trig = ev.direction * (t - ev.time) if ev.time is not None else ev.trigger
        de.add_component(c.Event(esym[ie], esym[ie].name, trig, use_values_from_trigger_time=True))
    got = model_spec_from_de_model(de, "switch3_processed")
    a, b = _run(spec, w, 1), _run(got, w, 1)
    assert (a["status"] == 0).all() and (b["status"] == 0).all()
    for key in ("x", "llh", "sx"):
        np.testing.assert_allclose(b[key], a[key], rtol=1e-6, atol=1e-9, err_msg=key)
