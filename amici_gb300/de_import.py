"""ModelSpec from the reference's symbolic model (the ``DEExporter`` hook).

The reference's importers (SBML, PySB) fill a ``DEModel``
(``python/sdist/amici/_symbolic/de_model.py:79``) with components
(``de_model_components.py``): differential states with their initial value
and time derivative, free and fixed parameters, expressions (fluxes and
assignment rules), observables with noise scales and cost functions, and
events.  ``DEExporter`` (``python/sdist/amici/exporters/sundials/
de_export.py:90-510``) writes the C++ model from it; ``model_spec_from_de_model``
is the GB300 counterpart's entry: it reads the same components, through the
``DEModel`` methods only (no import of the reference package), and returns
the ``ModelSpec`` from which ``amici_gb300.Model`` generates and compiles the
``__device__`` model code.

Mapping:

* states ``differential_states()``: symbol, ``get_val()`` (x0), ``get_dt()``
  (xdot); parameters ``free_parameters()``, ``fixed_parameters()`` with their
  nominal values; expressions ``expressions()`` are substituted (in
  dependency order) into everything that uses them.
* fluxes: each state's ``get_dt()`` is, as the importers write it, a sum of
  expression symbols times constant coefficients (the stoichiometry, divided
  by compartment volumes).  Every expression with a nonzero coefficient
  becomes a flux; a coefficient c that is not an integer becomes a flux
  |c| w with stoichiometry sign(c) (one flux per distinct |c| of the same
  expression, so the integer stoichiometry tables hold); a remainder of
  ``get_dt()`` that is not of that form becomes a flux of its own.
* observables ``observables()``, noise scales ``sigma_ys()`` (same order),
  noise distributions recognised from the cost functions
  ``log_likelihood_ys()`` (each evaluated at sample points against the six
  distributions of ``importers/utils.py:110-130``).
* events ``events()``: the trigger ``get_val()``; a trigger of the form
  a (t - te(p, k)) with a constant a becomes an explicit trigger time with
  direction sign(a) (the roots the reference solves for t), any other a
  trigger function for root finding; the bolus ``get_state_update(x, x)``;
  ``get_initial_value()``.  An event's symbol inside an expression is the
  Heaviside indicator of its trigger (``DEModel._process_heavisides``
  replaced Heaviside(g) by it): it is turned back into Heaviside(g), which
  the code generator keeps with the same pair of events.

Refused with ``NotImplementedError``: algebraic states (DAEs), conservation
laws (import with ``compute_conservation_laws=False``), event priorities,
event observables, splines.  The bolus is evaluated at the state when it is
applied: for events that fire alone this is the reference's result for
either ``use_values_from_trigger_time``.
"""
from __future__ import annotations

import math

import sympy as sp

from .model_spec import NOISE_DISTRIBUTIONS, TIME, Event, ModelSpec

__all__ = ["model_spec_from_de_model", "noise_distribution_of_cost"]


def _components(de, name):
    f = getattr(de, name, None)
    return list(f()) if callable(f) else []


def _flatten(exprs, defs):
    """Substitute the expression definitions ``defs`` (symbol -> value) into
    ``exprs`` until no defined symbol remains (dependency order; a cycle is
    an error)."""
    out = [sp.sympify(e) for e in exprs]
    for _ in range(len(defs) + 1):
        if not any(e.free_symbols & defs.keys() for e in out):
            return out
        out = [e.xreplace(defs) if e.free_symbols & defs.keys() else e for e in out]
    raise ValueError("cyclic expression definitions in the model")


def _jy_forms(y, m, s):
    ln10 = math.log(10.0)
    lg = math.log10
    return {
        "normal": 0.5 * math.log(2 * math.pi * s * s) + 0.5 * ((y - m) / s) ** 2,
        "log-normal": 0.5 * math.log(2 * math.pi * s * s * m * m) + 0.5 * ((math.log(y) - math.log(m)) / s) ** 2,
        "log10-normal": 0.5 * math.log(2 * math.pi * s * s * m * m * ln10 * ln10) + 0.5 * ((lg(y) - lg(m)) / s) ** 2,
        "laplace": math.log(2 * s) + abs(y - m) / s,
        "log-laplace": math.log(2 * s * m) + abs(math.log(y) - math.log(m)) / s,
        "log10-laplace": math.log(2 * s * m * ln10) + abs(lg(y) - lg(m)) / s,
    }


def noise_distribution_of_cost(cost, y, m, sigma) -> str:
    """The noise distribution (one of NOISE_DISTRIBUTIONS) whose negative
    log-likelihood the cost function ``cost(y, m, sigma)`` is, recognised by
    its values at sample points; ``ValueError`` when it is none of them."""
    f = sp.lambdify((y, m, sigma), sp.sympify(cost), "math")
    samples = [(1.3, 0.7, 0.2), (0.4, 2.5, 1.1), (3.0, 3.5, 0.05), (0.9, 0.2, 2.0)]
    for name in NOISE_DISTRIBUTIONS:
        ok = True
        for yv, mv, sv in samples:
            ref = _jy_forms(yv, mv, sv)[name]
            try:
                v = float(f(yv, mv, sv))
            except (ValueError, ZeroDivisionError, OverflowError):
                ok = False
                break
            if not abs(v - ref) <= 1e-9 * max(1.0, abs(ref)):
                ok = False
                break
        if ok:
            return name
    raise ValueError(f"cost function {cost} is none of the supported noise distributions "
                     f"({', '.join(NOISE_DISTRIBUTIONS)})")


def _split_fluxes(dts, wsyms):
    """Fluxes and integer stoichiometry from the states' time derivatives
    ``dts`` written over the expression symbols ``wsyms``: returns
    (list of (expression or symbol, factor), {(i, r): s_ir})."""
    fluxes, index, stoich = [], {}, {}
    for i, dt in enumerate(dts):
        dt = sp.expand(sp.sympify(dt)) if any(dt.has(w) for w in wsyms) else sp.sympify(dt)
        rest = dt
        for w in wsyms:
            if not dt.has(w):
                continue
            c = sp.diff(dt, w)
            if not c.is_Number or sp.diff(c, w) != 0:
                continue  # not linear with a constant coefficient: left in the remainder
            rest = sp.expand(rest - c * w)
            if c == 0:
                continue
            mag = abs(c)
            if mag.is_Integer:
                key, s = (w, sp.Integer(1)), int(c)
            else:
                key, s = (w, mag), 1 if c > 0 else -1
            if key not in index:
                index[key] = len(fluxes)
                fluxes.append(key)
            r = index[key]
            stoich[(i, r)] = stoich.get((i, r), 0) + s
        rest = sp.simplify(rest) if rest != 0 else rest
        if rest != 0:
            key = (rest, sp.Integer(1))
            index[key] = len(fluxes)
            fluxes.append(key)
            stoich[(i, index[key])] = 1
    stoich = {ir: v for ir, v in stoich.items() if v != 0}
    return fluxes, stoich


def model_spec_from_de_model(de, name: str, families=("fwd", "fsa", "asa")) -> ModelSpec:
    """The ModelSpec of the reference's ``DEModel`` ``de`` (see the module
    docstring for the mapping and what is refused)."""
    if _components(de, "algebraic_states") or _components(de, "algebraic_equations"):
        raise NotImplementedError("algebraic states (DAE models) are not on the GB300 path")
    if _components(de, "conservation_laws"):
        raise NotImplementedError("conservation laws: import the model with compute_conservation_laws=False")
    if _components(de, "event_observables"):
        raise NotImplementedError("event observables are not built")
    if getattr(de, "_splines", None):
        raise NotImplementedError("splines are not built")

    states = _components(de, "differential_states")
    pars = _components(de, "free_parameters")
    fixed = _components(de, "fixed_parameters")
    exprs = _components(de, "expressions")
    obs = _components(de, "observables")
    sigmas = _components(de, "sigma_ys")
    costs = _components(de, "log_likelihood_ys")
    events = _components(de, "events")

    x = [s.get_sym() for s in states]
    p = [c.get_sym() for c in pars]
    k = [c.get_sym() for c in fixed]
    # the reference's time symbol is "t"; map it onto the engine's
    tsyms = {s for c in states + exprs + obs + events for s in sp.sympify(
        c.get_dt() if hasattr(c, "get_dt") else c.get_val()).free_symbols if s.name == "t"}
    tmap = {s: TIME for s in tsyms}
    defs = {c.get_sym(): sp.sympify(c.get_val()).xreplace(tmap) for c in exprs}
    # an event's symbol in an expression: the Heaviside of its trigger
    for ev in events:
        defs.setdefault(ev.get_sym(), sp.Heaviside(sp.sympify(ev.get_val()).xreplace(tmap)))
    wsyms = [c.get_sym() for c in exprs]

    dts = [sp.sympify(s.get_dt()).xreplace(tmap) for s in states]
    fl, stoich = _split_fluxes(dts, wsyms)
    w = _flatten([e * f for e, f in fl], defs)
    x0 = _flatten([sp.sympify(s.get_val()).xreplace(tmap) for s in states], defs)

    if len(sigmas) != len(obs):
        raise ValueError(f"{len(obs)} observables but {len(sigmas)} noise scales")
    y = _flatten([sp.sympify(o.get_val()).xreplace(tmap) for o in obs], defs)
    sigma_y = _flatten([sp.sympify(s.get_val()) for s in sigmas], defs)
    noise = []
    for i, o in enumerate(obs):
        if i < len(costs):
            noise.append(noise_distribution_of_cost(costs[i].get_val(), o.get_sym(), o.get_measurement_symbol(),
                                                    sigmas[i].get_sym()))
        else:
            noise.append("normal")

    allowed = set(p) | set(k)
    evs = []
    for ev in events:
        if getattr(ev, "get_priority", lambda: None)() is not None:
            raise NotImplementedError(f"event {ev.get_name()}: event priorities are not built")
        trig = _flatten([sp.sympify(ev.get_val()).xreplace(tmap)], defs)[0]
        upd = ev.get_state_update(sp.Matrix(x), sp.Matrix(x))
        bolus = {}
        if upd is not None:
            for i, b in enumerate(_flatten(list(upd), defs)):
                if b != 0:
                    bolus[i] = b
        init = bool(ev.get_initial_value())
        te, direction = None, 1
        if not (trig.free_symbols & set(x)):
            roots = sp.solve(trig, TIME) if trig.has(TIME) else []
            dtr = sp.diff(trig, TIME)
            if len(roots) == 1 and not (roots[0].free_symbols - allowed) and dtr.is_Number and dtr != 0:
                te, direction = roots[0], (1 if dtr > 0 else -1)
        evs.append(Event(time=te, bolus=bolus, initial_value=init, direction=direction) if te is not None
                   else Event(trigger=trig, bolus=bolus, initial_value=init))

    spec = ModelSpec(
        name=name,
        state_ids=[s.get_id() if isinstance(s.get_id(), str) else str(s.get_sym()) for s in states],
        parameter_ids=[str(c.get_sym()) for c in pars],
        fixed_parameter_ids=[str(c.get_sym()) for c in fixed],
        observable_ids=[str(o.get_sym()) for o in obs],
        x0=x0, w=w, stoich=stoich, y=y, sigma_y=sigma_y, x=x, p=p, k=k,
        p_nominal=[float(c.get_val()) for c in pars], k_nominal=[float(c.get_val()) for c in fixed],
        noise_distributions=noise, events=evs)
    spec.families = tuple(families) if not evs else tuple(f for f in families if f != "asa")
    if evs:
        spec.check_events()
    return spec
