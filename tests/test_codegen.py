"""Code generator: symbolic derivatives, engine tables and model structure."""
import ctypes

import numpy as np
import sympy as sp

from amici_gb300.codegen import emit_engine_units
from amici_gb300.networks import config2_workload, robertson_model
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
    spec = config2_workload(4).model
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
    spec = config2_workload(4).model
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
