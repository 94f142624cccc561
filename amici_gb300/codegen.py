"""Model code generator: sympy model -> C (oracle ABI) and CUDA (engine).

This is the build's counterpart of AMICI's exporter
(``python/sdist/amici/exporters/sundials/de_export.py:267-510`` writes one C++
file per entry of the function table ``cxx_functions.py:102-410``).  Two
emitters share one symbolic model (:class:`~amici_gb300.model_spec.ModelSpec`):

* :func:`emit_oracle_c` — straight-line C for the CPU oracle's model ABI
  (``oracle/oracle_model.h``): ``x0``, ``dx0dp``, ``xdot``, dense ``jac``,
  ``dxdotdp``, ``y``, ``dydx``, ``dydp``, ``sigmay``; derivatives are taken
  symbolically, as AMICI does (``_symbolic/de_model.py:1975,2058``).
* :func:`emit_engine_cuda` — the GPU engine's model: per-instance
  coefficient/initial-state code (straight-line ``__device__`` code over the
  parameters) plus constant tables that let a group of lanes evaluate the
  fluxes ``w``, the right-hand side ``S·w``, the Jacobian ``S·dw/dx`` and the
  parameter derivative ``S·dw/dp`` lane-parallel.
"""
from __future__ import annotations

import hashlib
import math

import numpy as np
import sympy as sp

from .model_spec import ModelSpec


def _c_printer(spec: ModelSpec):
    """Return a function printing a sympy expression as C with array names."""
    repl = {}
    for i, s in enumerate(spec.x):
        repl[s] = sp.Symbol(f"x[{i}]")
    for i, s in enumerate(spec.p):
        repl[s] = sp.Symbol(f"p[{i}]")
    for i, s in enumerate(spec.k):
        repl[s] = sp.Symbol(f"k[{i}]")

    def pr(expr):
        e = sp.sympify(expr).xreplace(repl)
        return sp.ccode(sp.N(e, 17) if e.has(sp.Rational) and not e.is_Integer else e)

    return pr


def _assign_block(lines, target, exprs, pr, *, dense_len=None, index=lambda i: str(i)):
    """Append ``target[idx] = expr;`` for nonzero expressions (zero-filling a
    dense output first if ``dense_len`` is given)."""
    if dense_len is not None:
        lines.append(f"    memset({target}, 0, sizeof(double) * {max(dense_len, 1)});")
    for i, e in exprs:
        if e == 0:
            continue
        lines.append(f"    {target}[{index(i)}] = {pr(e)};")


def emit_oracle_c(spec: ModelSpec) -> str:
    """C source implementing ``oracle_get_model()`` for this model."""
    pr = _c_printer(spec)
    nx, np_, nk, ny = spec.nx, spec.np, spec.nk, spec.ny
    xdot = spec.xdot()
    L = [
        "/* Generated by amici_gb300.codegen.emit_oracle_c — model "
        f"{spec.name}; do not edit. */",
        "#include <math.h>",
        "#include <string.h>",
        '#include "oracle_model.h"',
        "",
    ]
    # x0
    L.append("static void m_x0(double* x0, const double* p, const double* k) {")
    L.append("    (void)p; (void)k;")
    _assign_block(L, "x0", list(enumerate(spec.x0)), pr, dense_len=nx)
    L.append("}")
    # dx0dp [np][nx]
    L.append("static void m_dx0dp(double* s, const double* p, const double* k) {")
    L.append("    (void)p; (void)k;")
    ent = []
    for j, pj in enumerate(spec.p):
        for i, e in enumerate(spec.x0):
            if pj in e.free_symbols:
                ent.append((j * nx + i, sp.diff(e, pj)))
    _assign_block(L, "s", ent, pr, dense_len=np_ * nx)
    L.append("}")
    # xdot
    L.append("static void m_xdot(double* f, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)t; (void)x; (void)p; (void)k;")
    _assign_block(L, "f", list(enumerate(xdot)), pr, dense_len=nx)
    L.append("}")
    # dense Jacobian, column-major
    L.append("static void m_jac(double* J, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)t; (void)x; (void)p; (void)k;")
    ent = []
    for i, fi in enumerate(xdot):
        fs = fi.free_symbols
        for j, xj in enumerate(spec.x):
            if xj in fs:
                ent.append((j * nx + i, sp.diff(fi, xj)))
    _assign_block(L, "J", ent, pr, dense_len=nx * nx)
    L.append("}")
    # dxdotdp [np][nx]
    L.append("static void m_dxdotdp(double* d, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)t; (void)x; (void)p; (void)k;")
    ent = []
    for i, fi in enumerate(xdot):
        fs = fi.free_symbols
        for j, pj in enumerate(spec.p):
            if pj in fs:
                ent.append((j * nx + i, sp.diff(fi, pj)))
    _assign_block(L, "d", ent, pr, dense_len=np_ * nx)
    L.append("}")
    # observables
    L.append("static void m_y(double* y, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)t; (void)x; (void)p; (void)k;")
    _assign_block(L, "y", list(enumerate(spec.y)), pr, dense_len=ny)
    L.append("}")
    L.append("static void m_dydx(double* d, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)t; (void)x; (void)p; (void)k;")
    ent = []
    for i, yi in enumerate(spec.y):
        for j, xj in enumerate(spec.x):
            if xj in yi.free_symbols:
                ent.append((j * ny + i, sp.diff(yi, xj)))
    _assign_block(L, "d", ent, pr, dense_len=nx * ny)
    L.append("}")
    L.append("static void m_dydp(double* d, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)t; (void)x; (void)p; (void)k;")
    ent = []
    for i, yi in enumerate(spec.y):
        for j, pj in enumerate(spec.p):
            if pj in yi.free_symbols:
                ent.append((j * ny + i, sp.diff(yi, pj)))
    _assign_block(L, "d", ent, pr, dense_len=np_ * ny)
    L.append("}")
    L.append("static void m_sigmay(double* s, const double* p, const double* k) {")
    L.append("    (void)p; (void)k;")
    _assign_block(L, "s", list(enumerate(spec.sigma_y)), pr, dense_len=ny)
    L.append("}")
    L.append("")
    L.append("static const oracle_model model = {")
    L.append(f'    "{spec.name}", {nx}, {np_}, {nk}, {ny},')
    L.append("    m_x0, m_dx0dp, m_xdot, m_jac, m_dxdotdp, m_y, m_dydx, m_dydp, m_sigmay};")
    L.append("const oracle_model* oracle_get_model(void) { return &model; }")
    return "\n".join(L) + "\n"


def spec_digest(spec: ModelSpec) -> str:
    """Stable hash of the symbolic model (used to key build outputs)."""
    h = hashlib.sha256()
    h.update(spec.name.encode())
    for part in (spec.x0, spec.w, sorted(spec.stoich.items()), spec.y, spec.sigma_y):
        h.update(repr([str(e) for e in part] if not isinstance(part, list) or not part
                      or not isinstance(part[0], tuple) else part).encode())
    return h.hexdigest()[:16]
