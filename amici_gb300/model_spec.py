"""Symbolic model description consumed by the code generator.

A model is the ODE system ``dx/dt = S · w(x, p, k)`` that AMICI's ``DEModel``
builds from SBML/PySB (``python/sdist/amici/_symbolic/de_model.py``): states
``x``, free parameters ``p``, fixed parameters ``k``, flux expressions ``w``
(AMICI's "expressions"), a constant stoichiometric matrix ``S`` (AMICI's
``dxdotdw``, ``src/model_ode.cpp:47-57``), observables ``y = h(x, p, k)``, noise
scales ``sigma_y(p, k)`` and initial states ``x0(p, k)``.

Observables may be any expressions of ``x, p, k``; noise scales any
expressions of ``p, k``; each observable has a noise distribution of the
reference's list (``python/sdist/amici/importers/utils.py:110-130``):
normal, log-normal, log10-normal, laplace, log-laplace, log10-laplace.

The GPU engine evaluates a flux that is a *monomial* in the states,
``w_r = c_r(p, k) · Π_j x_j^{e_rj}`` with total degree ≤ 2 (mass-action
kinetics, all benchmark workloads), from tables; the coefficient ``c_r`` may
be any sympy expression of ``p`` and ``k`` and is evaluated once per instance.
Any other flux (Michaelis–Menten, Hill, inhibition terms, …) may be any
expression of at most two states and of ``p`` and ``k``: it becomes a *rate
law* — the expression with its states replaced by ``X0``/``X1`` and its
maximal state-free subexpressions by per-instance coefficients ``C0, C1, …``
— and fluxes with the same rate law share one piece of generated code.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import sympy as sp


# noise distributions (python/sdist/amici/importers/utils.py:110-130); the
# index is the code the generated model and the oracle use
NOISE_DISTRIBUTIONS = ("normal", "log-normal", "log10-normal", "laplace", "log-laplace", "log10-laplace")


@dataclass
class FluxMonomial:
    """``w = coeff(p, k) * x[a] * x[b]`` (``a``/``b`` = -1 mean "absent")."""

    coeff: sp.Expr
    a: int
    b: int


@dataclass
class FluxForm:
    """How the engine evaluates flux r: it depends on the states ``a`` and
    ``b`` (-1: absent) through rate law ``template`` with the per-instance
    coefficients ``coeffs`` (expressions of p and k).  Rate law 0 is the
    monomial ``C0 * x_a * x_b`` (``C0 * x_a``, ``C0 * x_a**2`` when a == b,
    ``C0``); rate law t > 0 is the t-th entry of the rate-law list that
    :meth:`ModelSpec.flux_forms` returns, an expression of ``RATE_X`` and
    ``rate_coefficient(i)``."""

    a: int
    b: int
    coeffs: list
    template: int


# time, in event triggers
TIME = sp.Symbol("t", real=True)

# the symbols of a rate law: its first and second state, its coefficients
RATE_X = (sp.Symbol("X0", real=True), sp.Symbol("X1", real=True))


def rate_coefficient(i: int) -> sp.Symbol:
    return sp.Symbol(f"C{i}", real=True)


def _rate_law(expr, xa, xb):
    """``expr`` with the states ``xa``/``xb`` replaced by ``RATE_X`` and its
    maximal state-free subexpressions (the state-free arguments of a sum or a
    product taken together) by coefficients, numbered in order of appearance;
    returns the rate law and the coefficient expressions."""
    xs = {v for v in (xa, xb) if v is not None}
    coeffs, cmap = [], {}

    def coef(e):
        if not e.free_symbols:
            return e
        if e not in cmap:
            cmap[e] = rate_coefficient(len(coeffs))
            coeffs.append(e)
        return cmap[e]

    def walk(e):
        if not (e.free_symbols & xs):
            return coef(e)
        if e == xa:
            return RATE_X[0]
        if e == xb:
            return RATE_X[1]
        if isinstance(e, (sp.Add, sp.Mul)):
            free = [a for a in e.args if not (a.free_symbols & xs)]
            parts = [walk(a) for a in e.args if a.free_symbols & xs]
            if free:
                parts.insert(0, coef(e.func(*free)))
            return e.func(*parts)
        return e.func(*[walk(a) for a in e.args])

    return walk(expr), coeffs


@dataclass
class Event:
    """An event and the jump of the states it causes.

    Its trigger is either explicit in time, ``time`` (an expression of p and
    k; AMICI's explicit roots, ``model.cpp:444-470``: the event fires when t
    reaches it), or a root function ``trigger`` of x, p, k and t (the event
    fires where it crosses zero upwards, located by CVODES' root finding).
    The states then jump by ``bolus`` (state index -> expression of x, p and
    k; the reference's ``deltax``).  A bolus must be affine in the states
    with constant coefficients (a dose ``x_i += d(p)``, a reset ``x_i := 0``
    written as ``-x_i``, a scaling ``x_i := c x_i``).  ``initial_value`` is
    the trigger's value before t0 (the reference's default, True): with
    False, an event whose trigger holds at t0 fires at t0
    (``Model::initialize_events``, ``model.cpp:407-440``).  ``direction``
    (explicit trigger times only) is the sign of the trigger's time
    derivative: the trigger is direction * (t - time), so an event with
    direction -1 crosses downwards at its time (the negative of a Heaviside
    of time)."""

    time: sp.Expr | None = None
    bolus: dict = field(default_factory=dict)
    initial_value: bool = True
    trigger: sp.Expr | None = None
    direction: int = 1


@dataclass
class ModelSpec:
    name: str
    state_ids: list[str]
    parameter_ids: list[str]
    fixed_parameter_ids: list[str]
    observable_ids: list[str]
    # symbolic pieces, all in terms of ``self.x``, ``self.p``, ``self.k``
    x0: list[sp.Expr]
    w: list[sp.Expr]
    stoich: dict[tuple[int, int], int]  # (species i, flux r) -> S_ir
    y: list[sp.Expr]
    sigma_y: list[sp.Expr]
    x: list[sp.Symbol] = field(default_factory=list)
    p: list[sp.Symbol] = field(default_factory=list)
    k: list[sp.Symbol] = field(default_factory=list)
    # default nominal values (the model's own parameter values)
    p_nominal: list[float] = field(default_factory=list)
    k_nominal: list[float] = field(default_factory=list)
    # kernel families compiled into the model's engine library: forward
    # simulation, forward sensitivities, adjoint sensitivities
    families: tuple = ("fwd", "fsa", "asa")
    # noise distribution per observable (NOISE_DISTRIBUTIONS; empty: all normal)
    noise_distributions: list[str] = field(default_factory=list)
    # storage of the iteration matrix's factors for models with a sparse LU:
    # "dense" (N x N array), "packed" (compressed rows of the factor pattern)
    # or "auto" (packed when the dense array would exceed 48 KB in FP32)
    lu_storage: str = "auto"
    # events (Event); none by default
    events: list = field(default_factory=list)
    # after expand_heavisides: the event whose Heaviside indicator h_j is
    # fixed parameter nk + j of the generated code (k holds nk + nh symbols)
    heaviside_events: list = field(default_factory=list)

    @property
    def nx(self) -> int:
        return len(self.state_ids)

    @property
    def np(self) -> int:
        return len(self.parameter_ids)

    @property
    def nk(self) -> int:
        return len(self.fixed_parameter_ids)

    @property
    def ny(self) -> int:
        return len(self.observable_ids)

    @property
    def nw(self) -> int:
        return len(self.w)

    @property
    def ne(self) -> int:
        return len(self.events)

    def root_events(self) -> list[int]:
        """Indices of the events with a trigger function (root finding)."""
        return [ie for ie, ev in enumerate(self.events) if ev.trigger is not None]

    def check_events(self) -> None:
        """Raises ``ValueError`` for an event the engine cannot run: a trigger
        time that depends on the states, or a bolus that is not affine in the
        states with constant coefficients."""
        xs, pk = set(self.x), set(self.p) | set(self.k)
        for ie, ev in enumerate(self.events):
            if (ev.time is None) == (ev.trigger is None):
                raise ValueError(f"event {ie}: give either a trigger time or a trigger function")
            if ev.trigger is not None:
                if not sp.sympify(ev.trigger).free_symbols <= xs | pk | {TIME}:
                    raise ValueError(f"event {ie}: the trigger may depend on x, p, k and t only")
            elif not sp.sympify(ev.time).free_symbols <= pk:
                raise ValueError(f"event {ie}: the trigger time may depend on p and k only")
            for i, d in ev.bolus.items():
                if not 0 <= i < self.nx:
                    raise ValueError(f"event {ie}: bolus on unknown state {i}")
                d = sp.sympify(d)
                if not d.free_symbols <= xs | pk:
                    raise ValueError(f"event {ie}: bolus of state {i} depends on unknown symbols")
                for xj in self.x:
                    if sp.diff(d, xj).free_symbols:
                        raise ValueError(f"event {ie}: the bolus of state {i} must be affine in the states "
                                         "with constant coefficients")

    def noise_codes(self) -> list[int]:
        """Noise distribution of every observable as its index in
        NOISE_DISTRIBUTIONS (normal when none is given)."""
        names = self.noise_distributions or ["normal"] * self.ny
        if len(names) != self.ny:
            raise ValueError("one noise distribution per observable")
        out = []
        for nm in names:
            key = {"lin-normal": "normal", "lin-laplace": "laplace"}.get(nm, nm)
            if key not in NOISE_DISTRIBUTIONS:
                raise ValueError(f"noise distribution {nm!r} is not supported "
                                 f"(supported: {', '.join(NOISE_DISTRIBUTIONS)})")
            out.append(NOISE_DISTRIBUTIONS.index(key))
        return out

    def xdot(self) -> list[sp.Expr]:
        out = [sp.Integer(0)] * self.nx
        for (i, r), s in sorted(self.stoich.items()):
            out[i] = out[i] + s * self.w[r]
        return out

    def _monomial(self, r: int):
        """Flux r as ``coeff(p,k) * x_a * x_b``, or the reason it is not one."""
        xs = set(self.x)
        wr = sp.expand(self.w[r])
        coeff, xpart = sp.S.One, []
        for fac in sp.Mul.make_args(wr):
            base, exp = fac.as_base_exp()
            if base in xs:
                if not (exp.is_Integer and exp > 0):
                    return f"flux {r}: non-integer power of a state: {wr}"
                xpart += [self.x.index(base)] * int(exp)
            else:
                if fac.free_symbols & xs:
                    return f"flux {r} is not a monomial in the states: {wr}"
                coeff = coeff * fac
        if len(xpart) > 2:
            return f"flux {r} has state degree {len(xpart)} > 2"
        xpart += [-1] * (2 - len(xpart))
        return FluxMonomial(coeff=coeff, a=xpart[0], b=xpart[1])

    def flux_monomials(self) -> list[FluxMonomial]:
        """Decompose every flux into ``coeff(p,k) * x_a * x_b``.

        Raises ``ValueError`` for a flux that is not such a monomial (see
        :meth:`flux_forms` for the general decomposition).
        """
        out = []
        for r in range(self.nw):
            m = self._monomial(r)
            if isinstance(m, str):
                raise ValueError(m)
            out.append(m)
        return out

    def flux_forms(self) -> tuple[list[FluxForm], list[sp.Expr]]:
        """Every flux as a monomial (rate law 0) or a general rate law of at
        most two states; returns the forms and the list of general rate laws
        (rate law t is entry t - 1).  Fluxes whose rate laws coincide after
        the renaming share an entry.  Raises ``ValueError`` for a flux of
        more than two states."""
        forms, laws, index = [], [], {}
        for r, wr in enumerate(self.w):
            m = self._monomial(r)
            if not isinstance(m, str):
                forms.append(FluxForm(a=m.a, b=m.b, coeffs=[m.coeff], template=0))
                continue
            deps = sorted(self.x.index(v) for v in wr.free_symbols & set(self.x))
            if len(deps) > 2:
                raise ValueError(f"flux {r} depends on {len(deps)} states; the GPU engine evaluates "
                                 f"fluxes of at most two states: {wr}")
            a = deps[0]
            b = deps[1] if len(deps) > 1 else -1
            law, coeffs = _rate_law(wr, self.x[a], self.x[b] if b >= 0 else None)
            key = sp.srepr(law)
            if key not in index:
                laws.append(law)
                index[key] = len(laws)
            forms.append(FluxForm(a=a, b=b, coeffs=coeffs, template=index[key]))
        return forms, laws

    def observable_matrix(self):
        """Return ``(H, h0)`` with ``y = H x + h0`` if all observables are
        affine in ``x`` with state-independent coefficients, else ``None``."""
        H = [[sp.Integer(0)] * self.nx for _ in range(self.ny)]
        h0 = []
        xs = set(self.x)
        for iy, yexpr in enumerate(self.y):
            yexpr = sp.expand(yexpr)
            rest = yexpr
            for j, xj in enumerate(self.x):
                c = sp.diff(yexpr, xj)
                if c.free_symbols & xs:
                    return None
                H[iy][j] = c
                rest = rest - c * xj
            rest = sp.simplify(rest)
            if rest.free_symbols & xs:
                return None
            h0.append(rest)
        return H, h0


def mass_action_model(name, nx, reactions, rate_param_index, np_, *, nk=0,
                      x0=None, observables=None, sigma=None, p_nominal=None,
                      k_nominal=None, state_prefix="x", fixed_x0_scale=None):
    """Build a :class:`ModelSpec` for a mass-action network.

    ``reactions`` is a list of ``(reactants, products)`` species-index lists;
    reaction ``r`` has rate constant ``p[rate_param_index[r]]`` and flux
    ``p * Π x_reactant``.  ``x0`` is a list of floats or sympy expressions;
    ``fixed_x0_scale`` maps a species to the fixed-parameter index that
    multiplies its initial value (condition-specific inputs).
    ``observables`` is a list of ``{species: weight}`` dicts.
    """
    xs = sp.symbols(f"{state_prefix}0:{nx}", real=True)
    ps = sp.symbols(f"p0:{np_}", real=True)
    ks = sp.symbols(f"k0:{nk}", real=True) if nk else ()
    w, stoich = [], {}
    for r, (reac, prod) in enumerate(reactions):
        flux = ps[rate_param_index[r]]
        for s in reac:
            flux = flux * xs[s]
        w.append(flux)
        for s in reac:
            stoich[(s, r)] = stoich.get((s, r), 0) - 1
        for s in prod:
            stoich[(s, r)] = stoich.get((s, r), 0) + 1
    stoich = {key: v for key, v in stoich.items() if v != 0}
    x0_exprs = []
    for i in range(nx):
        v = sp.Float(x0[i]) if x0 is not None and not isinstance(x0[i], sp.Basic) else (
            x0[i] if x0 is not None else sp.Integer(0))
        if fixed_x0_scale and i in fixed_x0_scale:
            v = v * ks[fixed_x0_scale[i]]
        x0_exprs.append(v)
    if observables is None:
        observables = [{i: 1.0} for i in range(nx)]
    y = []
    for obs in observables:
        e = sp.Integer(0)
        for s, wgt in obs.items():
            e = e + sp.Float(wgt) * xs[s]
        y.append(e)
    if sigma is None:
        sigma = 1.0
    sig = [sp.Float(sigma)] * len(y) if not isinstance(sigma, (list, tuple)) else [sp.Float(s) for s in sigma]
    return ModelSpec(
        name=name,
        state_ids=[f"{state_prefix}{i}" for i in range(nx)],
        parameter_ids=[f"p{i}" for i in range(np_)],
        fixed_parameter_ids=[f"k{i}" for i in range(nk)],
        observable_ids=[f"y{i}" for i in range(len(y))],
        x0=x0_exprs, w=w, stoich=stoich, y=y, sigma_y=sig,
        x=list(xs), p=list(ps), k=list(ks),
        p_nominal=list(p_nominal) if p_nominal is not None else [1.0] * np_,
        k_nominal=list(k_nominal) if k_nominal is not None else [1.0] * nk,
    )


def expand_heavisides(spec: ModelSpec) -> ModelSpec:
    """The model with every ``Heaviside(g)`` of a flux replaced by an
    indicator h_j that the event handling keeps (the reference's
    ``DEModel._process_heavisides``, de_model.py:2432-2470, and
    ``Model::update_heaviside``, model.cpp:1588-1592): g becomes the trigger
    function of an event without a bolus, and so does -g, so that a crossing
    in either direction is an upward crossing of one of them; an existing
    event with the same trigger is reused.  h_j is 1 where g >= 0 at t0
    (``Model::reinit_events``) and changes by the root direction at every
    crossing.  The indicators are appended to ``k`` (not to the model's
    inputs: ``nk`` is unchanged) and ``heaviside_events`` names the event of
    each.  A Heaviside of time, a (t - te(p, k)) with a constant a, becomes a
    pair of events with the explicit trigger time te (directions sign(a) and
    -sign(a)), as the reference treats roots it can solve for t; any other
    Heaviside of p, k and t only is refused.  Returns ``spec`` itself when
    no flux has a Heaviside."""
    import dataclasses
    hv = []
    for w in spec.w:
        for node in sp.preorder_traversal(sp.sympify(w)):
            if isinstance(node, sp.Heaviside) and node not in hv:
                hv.append(node)
    if not hv:
        return spec
    xs = set(spec.x)
    events = list(spec.events)

    def root_event(g):
        if not g.free_symbols & xs:  # a (t - te): an explicit trigger time
            a = sp.diff(g, TIME)
            te = sp.solve(g, TIME)
            if not (a.is_Number and a != 0 and len(te) == 1 and not sp.diff(a, TIME)):
                raise ValueError(f"Heaviside({g}) depends on p, k and t only and is not a (t - te(p, k)): write it "
                                 "as an event with an explicit trigger time")
            d = 1 if a > 0 else -1
            for ie, ev in enumerate(events):
                if ev.time is not None and ev.direction == d and sp.simplify(sp.sympify(ev.time) - te[0]) == 0:
                    return ie
            events.append(Event(time=te[0], direction=d))
            return len(events) - 1
        for ie, ev in enumerate(events):
            if ev.trigger is not None and sp.simplify(sp.sympify(ev.trigger) - g) == 0:
                return ie
        events.append(Event(trigger=g))
        return len(events) - 1

    hsyms, hev, repl = [], [], {}
    for node in hv:
        g = sp.sympify(node.args[0])
        ie = root_event(g)
        root_event(-g)
        if ie not in hev:
            hev.append(ie)
            hsyms.append(sp.Symbol(f"heaviside_{ie}", real=True))
        repl[node] = hsyms[hev.index(ie)]
    w = [sp.sympify(e).xreplace(repl) for e in spec.w]
    out = dataclasses.replace(spec, w=w, k=list(spec.k) + hsyms, events=events, heaviside_events=hev)
    out.families = getattr(spec, "families", out.families)
    return out
