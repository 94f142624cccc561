"""Code generator: symbolic derivatives, engine tables and model structure."""
import ctypes

import numpy as np
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
