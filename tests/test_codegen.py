"""Code generator: symbolic derivatives, engine tables and model structure."""
import ctypes

import numpy as np
import pytest
import sympy as sp

from amici_gb300.codegen import emit_engine_units
from amici_gb300.networks import net20_workload, robertson_model
from oracle.pyoracle import Oracle


def _oracle_fns(spec):
    o = Oracle(spec)

    class M(ctypes.Structure):
        _fields_ = [("name", ctypes.c_char_p)] + [(n, ctypes.c_int) for n in ("nx", "np", "nk", "ny")] + [
            (n, ctypes.c_void_p) for n in ("x0", "dx0dp", "xdot", "jac", "dxdotdp", "y", "dydx", "dydp", "sigmay")]

    m = M.from_address(o.lib.oracle_get_model())
    proto = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)
    return m, {n: proto(getattr(m, n)) for n in ("xdot", "jac", "dxdotdp")}


def _call(f, out, x, p, k):
    f(out.ctypes.data, 0.0, x.ctypes.data, p.ctypes.data, k.ctypes.data if k.size else None)


def test_jacobian_matches_finite_differences():
    spec = net20_workload(4).model
    _, F = _oracle_fns(spec)
    rng = np.random.default_rng(0)
    x = rng.uniform(0.1, 1.0, spec.nx)
    p = 10 ** rng.uniform(-1, 1, spec.np)
    k = np.zeros(1)
    J = np.zeros(spec.nx * spec.nx)
    _call(F["jac"], J, x, p, k)
    J = J.reshape(spec.nx, spec.nx).T  # column-major -> J[i, j]
    f0 = np.zeros(spec.nx)
    for j in range(spec.nx):
        h = 1e-6 * max(1.0, abs(x[j]))
        xp, xm = x.copy(), x.copy()
        xp[j] += h
        xm[j] -= h
        fp, fm = np.zeros(spec.nx), np.zeros(spec.nx)
        _call(F["xdot"], fp, xp, p, k)
        _call(F["xdot"], fm, xm, p, k)
        np.testing.assert_allclose(J[:, j], (fp - fm) / (2 * h), rtol=1e-6, atol=1e-8)
    del f0


def test_engine_tables_reproduce_rhs():
    """The flux-monomial / stoichiometry decomposition used on the GPU
    evaluates the same right-hand side as the symbolic C code."""
    spec = net20_workload(4).model
    _, F = _oracle_fns(spec)
    mono = spec.flux_monomials()
    rng = np.random.default_rng(1)
    x = rng.uniform(0.1, 1.0, spec.nx)
    p = 10 ** rng.uniform(-1, 1, spec.np)
    subs = {**dict(zip(spec.p, p))}
    c = np.array([float(m.coeff.xreplace(subs)) for m in mono])
    w = np.array([c[r] * (x[m.a] if m.a >= 0 else 1) * (x[m.b] if m.b >= 0 else 1)
                  for r, m in enumerate(mono)])
    f_tab = np.zeros(spec.nx)
    for (i, r), s in spec.stoich.items():
        f_tab[i] += s * w[r]
    f_c = np.zeros(spec.nx)
    _call(F["xdot"], f_c, x, p, np.zeros(1))
    np.testing.assert_allclose(f_tab, f_c, rtol=1e-13, atol=1e-15)


def test_robertson_structure():
    spec = robertson_model()
    xs, ps = spec.x, spec.p
    xdot = spec.xdot()
    assert sp.simplify(xdot[0] - (-ps[0] * xs[0] + ps[2] * xs[1] * xs[2])) == 0
    assert sp.simplify(xdot[1] - (ps[0] * xs[0] - ps[1] * xs[1] ** 2 - ps[2] * xs[1] * xs[2])) == 0
    assert sp.simplify(xdot[2] - ps[1] * xs[1] ** 2) == 0
    units = emit_engine_units(spec)
    assert "model.cuh" in units and "abi.cu" in units
    assert "NNZ_J = 7" in units["model.cuh"]


def test_compact_jacobian_reproduces_dense_jacobian():
    """The engine's compact Jacobian (pattern positions per stoichiometry
    entry, accumulated as jac_row_sparse does) equals the symbolic Jacobian."""
    from amici_gb300.codegen import compact_jacobian
    from amici_gb300.networks import net100_adjoint_workload

    spec = net100_adjoint_workload(1).model
    _, F = _oracle_fns(spec)
    mono = spec.flux_monomials()
    entries, row_ptr, pos_a, pos_b = compact_jacobian(spec)
    rng = np.random.default_rng(2)
    x = rng.uniform(0.1, 1.0, spec.nx)
    p = 10 ** rng.uniform(-1, 1, spec.np)
    c = np.array([float(m.coeff.xreplace(dict(zip(spec.p, p)))) for m in mono])
    Jc = np.zeros(len(entries))
    e = 0
    for i in range(spec.nx):
        for (ii, r), sv in sorted(spec.stoich.items()):
            if ii != i:
                continue
            a, b, sc = mono[r].a, mono[r].b, sv * c[r]
            if a >= 0:
                if b < 0:
                    Jc[pos_a[e]] += sc
                elif a == b:
                    Jc[pos_a[e]] += 2 * sc * x[a]
                else:
                    Jc[pos_a[e]] += sc * x[b]
                    Jc[pos_b[e]] += sc * x[a]
            e += 1
    J = np.zeros(spec.nx * spec.nx)
    _call(F["jac"], J, x, p, np.ones(spec.nk))
    J = J.reshape(spec.nx, spec.nx).T
    Jd = np.zeros_like(J)
    for q, (i, j) in enumerate(entries):
        Jd[i, j] = Jc[q]
    np.testing.assert_allclose(Jd, J, rtol=1e-13, atol=1e-14)
    assert all(row_ptr[i] <= row_ptr[i + 1] for i in range(spec.nx))


def test_sparse_lu_plan_is_closed_and_factorises():
    """The static order's symbolic fill contains every update of the
    elimination, and LU without row exchanges on that pattern reproduces a
    diagonally dominant matrix with the Jacobian's pattern."""
    from amici_gb300.codegen import compact_jacobian, sparse_lu_plan
    from amici_gb300.networks import net50_fsa_workload

    spec = net50_fsa_workload(1).model
    order, rows, cols, dflops, sflops = sparse_lu_plan(spec)
    assert sorted(order) == list(range(spec.nx)) and sflops < 0.2 * dflops
    entries, *_ = compact_jacobian(spec)
    n = spec.nx
    rng = np.random.default_rng(3)
    A = np.eye(n) * n
    for (i, j) in entries:
        A[i, j] += rng.uniform(-1, 1)
    iord = np.argsort(order)
    P = A[np.ix_(order, order)].copy()
    pattern = P != 0
    for k in range(n):
        for i in rows[k]:
            P[i, k] /= P[k, k]
        for i in rows[k]:
            for j in cols[k]:
                P[i, j] -= P[i, k] * P[k, j]
        pattern[np.ix_(rows[k], cols[k])] = True
        # nothing outside the planned rows/columns is touched
        assert np.all(P[k + 1:, k][~np.isin(np.arange(k + 1, n), rows[k])] == 0)
    L = np.tril(P, -1) + np.eye(n)
    U = np.triu(P)
    np.testing.assert_allclose((L @ U)[np.ix_(iord, iord)], A, rtol=1e-12, atol=1e-12)


def _restricted_lu(P, rows, cols):
    P = P.copy()
    for k in range(len(P)):
        for i in rows[k]:
            P[i, k] /= P[k, k]
            for j in cols[k]:
                P[i, j] -= P[i, k] * P[k, j]
    return np.tril(P, -1) + np.eye(len(P)), np.triu(P)


def test_sparse_lu_plan_transposed_for_the_backward_problem():
    """The backward problem's iteration matrix I + gamma*J^T has the transposed
    pattern: with the forward plan's row and column lists trading places the
    restricted elimination is exact, with them unchanged it is not (the plan
    of an unsymmetric pattern misses fill of the transpose)."""
    from amici_gb300.codegen import compact_jacobian, sparse_lu_plan
    from amici_gb300.networks import net100_adjoint_workload

    spec = net100_adjoint_workload(1).model
    order, rows, cols, _, _ = sparse_lu_plan(spec)
    entries, *_ = compact_jacobian(spec)
    n = spec.nx
    rng = np.random.default_rng(5)
    J = np.zeros((n, n))
    for (i, j) in entries:
        J[i, j] = rng.normal()
    B = (np.eye(n) + 0.1 * J.T)[np.ix_(order, order)]
    L, U = _restricted_lu(B, cols, rows)
    np.testing.assert_allclose(L @ U, B, rtol=0, atol=1e-12)
    L, U = _restricted_lu(B, rows, cols)
    assert np.abs(L @ U - B).max() > 1e-3


def _packed_factor_and_solve(n, tab, lrows, b, vals, tr):
    """The engine's packed factorisation and solves, step by step: per pivot
    the U row is scattered into a dense row and every L row of the pivot
    sweeps its compressed stretch against it; the solves walk each row's
    entries with one pointer forward (L) and one backward (U)."""
    rptr, col, diag, lpos, span, _ = tab
    val = vals.copy()
    urow = np.zeros(n)
    dinv = np.zeros(n)
    e = 0
    for k in range(n):
        dinv[k] = 1.0 / val[diag[k]]
        for q in range(diag[k] + 1, rptr[k + 1]):
            urow[col[q]] = val[q]
        for _i in lrows[k]:
            p = lpos[e]
            lik = val[p] * dinv[k]
            val[p] = lik
            for pp in range(p + 1, p + 1 + span[e]):
                val[pp] -= lik * urow[col[pp]]
            e += 1
        for q in range(diag[k] + 1, rptr[k + 1]):
            urow[col[q]] = 0.0
    x = b.copy()
    ptr = [rptr[i] for i in range(n)]
    for k in range(n - 1):
        for i in range(k + 1, n):
            if ptr[i] < diag[i] and col[ptr[i]] == k:
                x[i] -= val[ptr[i]] * x[k]
                ptr[i] += 1
    ptr = [rptr[i + 1] - 1 for i in range(n)]
    for k in range(n - 1, -1, -1):
        x[k] *= dinv[k]
        for i in range(k):
            if ptr[i] > diag[i] and col[ptr[i]] == k:
                x[i] -= val[ptr[i]] * x[k]
                ptr[i] -= 1
    return x


def test_packed_factor_tables_solve_both_problems():
    """The compressed-row factor tables of the n = 200 network (forward plan
    for I - gamma*J, transposed plan for the backward problem's
    I + gamma*J^T) reproduce the dense solution of both systems."""
    from amici_gb300.codegen import compact_jacobian, packed_lu_tables, sparse_lu_plan
    from amici_gb300.networks import net200_workload

    spec = net200_workload(1).model
    n = spec.nx
    order, rows, cols, _, _ = sparse_lu_plan(spec)
    iorder = np.argsort(order)
    jent, *_ = compact_jacobian(spec)
    rng = np.random.default_rng(11)
    Jv = rng.normal(size=len(jent))
    J = np.zeros((n, n))
    for (i, a), v in zip(jent, Jv):
        J[i, a] = v
    b = rng.normal(size=n)
    for tr, (R, C) in ((False, (rows, cols)), (True, (cols, rows))):
        tab = packed_lu_tables(n, R, C, jent, list(iorder), transposed=tr)
        rptr, col, diag, lpos, span, jpos = tab
        assert len(set(jpos)) == len(jpos) and len(lpos) == sum(len(r) for r in R)
        vals = np.zeros(rptr[-1])
        for p, v in enumerate(Jv):
            vals[jpos[p]] = (0.05 if tr else -0.05) * v
        for i in range(n):
            vals[diag[i]] += 1.0
        A = np.eye(n) + (0.05 * J.T if tr else -0.05 * J)
        Ap = A[np.ix_(order, order)]
        x = _packed_factor_and_solve(n, tab, R, b[order], vals, tr)
        np.testing.assert_allclose(x, np.linalg.solve(Ap, b[order]), rtol=1e-10, atol=1e-12)


def test_lu_storage_choice():
    """Factor storage per model: dense N x N up to 48 KB in FP32, compressed
    rows above (or on request); forward sensitivities need the dense form."""
    import dataclasses

    from amici_gb300.codegen import emit_engine_cuda, emit_engine_units
    from amici_gb300.networks import net100_adjoint_workload, net200_workload

    m100 = net100_adjoint_workload(1).model
    assert "PACKED_LU = false" in emit_engine_cuda(m100)
    assert "PACKED_LU = true" in emit_engine_cuda(dataclasses.replace(m100, lu_storage="packed"))
    m200 = net200_workload(1).model
    assert "PACKED_LU = true" in emit_engine_cuda(m200)
    with pytest.raises(ValueError, match="dense factor storage"):
        emit_engine_units(dataclasses.replace(m200, families=("fwd", "fsa")))
    with pytest.raises(ValueError, match="lu_storage"):
        emit_engine_cuda(dataclasses.replace(m100, lu_storage="banded"))


def _rate_law_value(spec, forms, laws, r, x, subs):
    """Flux r rebuilt from its engine form: the rate law with its states and
    coefficients put back, as the generated device code evaluates it."""
    from amici_gb300.model_spec import RATE_X, rate_coefficient

    f = forms[r]
    c = [float(ce.xreplace(subs)) for ce in f.coeffs]
    if f.template == 0:
        return c[0] * (x[f.a] if f.a >= 0 else 1.0) * (x[f.b] if f.b >= 0 else 1.0), None
    law = laws[f.template - 1]
    rep = {RATE_X[0]: x[f.a], RATE_X[1]: x[f.b] if f.b >= 0 else 0.0}
    rep.update({rate_coefficient(i): v for i, v in enumerate(c)})
    da = float(sp.diff(law, RATE_X[0]).xreplace(rep))
    return float(law.xreplace(rep)), da


def test_general_rate_laws_reproduce_the_fluxes():
    """Every flux of the MAPK cascade (Michaelis-Menten, Hill feedback,
    inhibition, one mass-action flux) rebuilt from its rate law and
    per-instance coefficients equals the flux and its state derivative;
    fluxes of the same form share a rate law; S * w from the rate laws equals
    the oracle's symbolic right-hand side."""
    from amici_gb300.networks import MAPK_NOMINAL, mapk_model

    spec = mapk_model()
    forms, laws = spec.flux_forms()
    assert len(laws) == 5 and forms[11].template == 0
    assert forms[1].template == forms[4].template == forms[5].template == forms[9].template
    assert forms[2].template == forms[3].template == forms[6].template == forms[7].template
    rng = np.random.default_rng(3)
    x = rng.uniform(1.0, 100.0, spec.nx)
    p = np.array(MAPK_NOMINAL) * 10 ** rng.uniform(-0.3, 0.3, spec.np)
    k = np.array([1.3])
    subs = {**dict(zip(spec.x, x)), **dict(zip(spec.p, p)), **dict(zip(spec.k, k))}
    w = np.zeros(spec.nw)
    for r in range(spec.nw):
        w[r], da = _rate_law_value(spec, forms, laws, r, x, subs)
        assert w[r] == pytest.approx(float(spec.w[r].xreplace(subs)), rel=1e-13)
        if da is not None:
            assert da == pytest.approx(float(sp.diff(spec.w[r], spec.x[forms[r].a]).xreplace(subs)), rel=1e-12)
    f_tab = np.zeros(spec.nx)
    for (i, r), sv in spec.stoich.items():
        f_tab[i] += sv * w[r]
    _, F = _oracle_fns(spec)
    f_c = np.zeros(spec.nx)
    _call(F["xdot"], f_c, x, p, k)
    np.testing.assert_allclose(f_tab, f_c, rtol=1e-12, atol=1e-12)
    units = emit_engine_units(spec)
    assert "GENERAL = true" in units["model.cuh"] and "NC = 24" in units["model.cuh"]


def test_flux_of_three_states_is_refused():
    spec = robertson_model()
    x, p = spec.x, spec.p
    spec.w[0] = p[0] * x[0] * x[1] / (1 + x[2])
    with pytest.raises(ValueError, match="at most two states"):
        spec.flux_forms()


def test_model_definition_example():
    """The model of the integration guide (a Michaelis-Menten flux, a
    mass-action flux and a dose event): it generates, and the oracle's
    forward sensitivities agree with finite differences."""
    from amici_gb300 import Event, ModelSpec

    x, p, k = sp.symbols("x0:2", real=True), sp.symbols("p0:4", real=True), sp.symbols("k0:1", real=True)
    spec = ModelSpec(name="mm", state_ids=["S", "P"], parameter_ids=["Vmax", "Km", "kdeg", "dose"],
                     fixed_parameter_ids=["t_dose"], observable_ids=["P"],
                     x0=[sp.Integer(1), sp.Integer(0)],
                     w=[p[0] * x[0] / (p[1] + x[0]), p[2] * x[1]],
                     stoich={(0, 0): -1, (1, 0): 1, (1, 1): -1},
                     y=[x[1]], sigma_y=[sp.Float(0.1)], x=list(x), p=list(p), k=list(k),
                     events=[Event(time=k[0], bolus={0: p[3]})])
    units = emit_engine_units(spec)
    assert "NE = 1" in units["model.cuh"] and "GENERAL = true" in units["model.cuh"]
    o = Oracle(spec)
    th = np.log(np.array([[1.0, 0.5, 0.2, 2.0]]))
    pscale = np.full(4, 1, np.int32)
    ts = np.linspace(0.5, 10.0, 20)[None, :]
    kk = np.array([[4.0]])
    kw = dict(rtol=1e-12, atol=1e-12, maxsteps=100000, nthreads=0)
    r = o.run(th, pscale, kk, ts, sensi=1, **kw)
    assert r["status"][0] == 0
    # the dose at t = 4 (output 7, taken after the event) shows in S
    assert r["x"][0, 7, 0] > r["x"][0, 6, 0] + 1.5
    h = 1e-4
    P = np.repeat(th, 8, axis=0)
    for j in range(4):
        P[2 * j, j] += h
        P[2 * j + 1, j] -= h
    f = o.run(P, pscale, np.repeat(kk, 8, 0), np.repeat(ts, 8, 0), **kw)
    fd = ((f["x"][0::2] - f["x"][1::2]) / (2 * h)).transpose(1, 0, 2)
    np.testing.assert_allclose(fd, r["sx"][0], rtol=0, atol=1e-6 * np.abs(r["sx"][0]).max())


def test_heaviside_expansion():
    """Heaviside functions of a flux become indicators appended to the fixed
    parameters, each with an event on its argument and one on its negative
    (shared between Heavisides of the same argument; an existing trigger
    function is reused); a Heaviside of time becomes a pair of explicit
    trigger times with opposite directions; the inputs (nk) are unchanged."""
    from amici_gb300.model_spec import TIME, Event, ModelSpec, expand_heavisides

    x, p, k = sp.symbols("x0:2", real=True), sp.symbols("p0:4", real=True), sp.symbols("k0:1", real=True)
    spec = ModelSpec(name="hv", state_ids=["a", "b"], parameter_ids=[f"p{i}" for i in range(4)],
                     fixed_parameter_ids=["k0"], observable_ids=["a"], x0=[sp.Integer(1), sp.Integer(0)],
                     w=[p[0] * sp.Heaviside(x[0] - p[1]), p[2] * x[1] * sp.Heaviside(x[0] - p[1]),
                        p[3] * sp.Heaviside(k[0] - TIME)],
                     stoich={(1, 0): 1, (1, 1): -1, (0, 2): 1}, y=[x[0]], sigma_y=[sp.Float(0.1)],
                     x=list(x), p=list(p), k=list(k), events=[Event(trigger=p[1] - x[0], bolus={1: sp.Integer(1)})])
    out = expand_heavisides(spec)
    assert out.nk == 1 and len(out.k) == 3 and out.heaviside_events == [1, 2]
    # the user's event (trigger p1 - x0) serves as the negative of x0 - p1
    assert [e.trigger for e in out.events[:2]] == [p[1] - x[0], x[0] - p[1]]
    assert out.events[2].time == k[0] and out.events[2].direction == -1
    assert out.events[3].time == k[0] and out.events[3].direction == 1
    h1, h2 = out.k[1], out.k[2]
    assert out.w == [p[0] * h1, p[2] * x[1] * h1, p[3] * h2]
    assert expand_heavisides(out) is out  # nothing left to expand
    units = emit_engine_units(spec)
    model = units["model.cuh"]
    assert "NH = 2" in model
    direction = model[model.index("event_direction"):]
    assert "case 2: return -1;" in direction[:direction.index("default")]
    bad = ModelSpec(**{**spec.__dict__, "w": [p[0] * sp.Heaviside(p[1] - 1), p[2] * x[1], p[3]]})
    with pytest.raises(ValueError, match="explicit trigger time"):
        expand_heavisides(bad)
