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

from .model_spec import RATE_X, ModelSpec, expand_heavisides


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
    spec = expand_heavisides(spec)
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
    L.append("static void m_dsigmaydp(double* d, const double* p, const double* k) {")
    L.append("    (void)p; (void)k;")
    ent = [(j * ny + i, sp.diff(si, pj)) for i, si in enumerate(spec.sigma_y) for j, pj in enumerate(spec.p)
           if pj in si.free_symbols]
    _assign_block(L, "d", ent, pr, dense_len=np_ * ny)
    L.append("}")
    codes = spec.noise_codes()
    L.append(f"static const int m_noise[{max(ny, 1)}] = {{{', '.join(map(str, codes or [0]))}}};")
    # events with explicit trigger times: times, their parameter derivatives,
    # boluses and the bolus derivatives
    spec.check_events()
    ne = spec.ne
    L.append("static void m_event_times(double* te, const double* p, const double* k) {")
    L.append("    (void)te; (void)p; (void)k;")
    if ne:  # zero-fill first: a trigger time of 0 is written by the fill
        _assign_block(L, "te", [(ie, sp.sympify(ev.time)) for ie, ev in enumerate(spec.events)
                                if ev.time is not None], pr, dense_len=ne)
    L.append("}")
    L.append("static void m_devent_times_dp(double* d, const double* p, const double* k) {")
    L.append("    (void)p; (void)k;")
    ent = [(j * ne + ie, sp.diff(sp.sympify(ev.time), pj)) for ie, ev in enumerate(spec.events)
           if ev.time is not None for j, pj in enumerate(spec.p)]
    _assign_block(L, "d", ent, pr, dense_len=np_ * ne)
    L.append("}")
    L.append("static void m_deltax(double* dx, int ie, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)t; (void)x; (void)p; (void)k;")
    L.append(f"    memset(dx, 0, sizeof(double) * {max(nx, 1)});")
    L.append("    switch (ie) {")
    for ie, ev in enumerate(spec.events):
        L.append(f"    case {ie}:")
        for i, d in sorted(ev.bolus.items()):
            if sp.sympify(d) != 0:
                L.append(f"        dx[{i}] = {pr(d)};")
        L.append("        break;")
    L.append("    default: break;")
    L.append("    }")
    L.append("}")
    L.append("static void m_ddeltaxdx(double* d, int ie) {")
    L.append(f"    memset(d, 0, sizeof(double) * {max(nx * nx, 1)});")
    L.append("    switch (ie) {")
    for ie, ev in enumerate(spec.events):
        L.append(f"    case {ie}:")
        for i, dv in sorted(ev.bolus.items()):
            for j, xj in enumerate(spec.x):
                c = sp.diff(sp.sympify(dv), xj)
                if c != 0:
                    L.append(f"        d[{j * nx + i}] = {pr(c)};")
        L.append("        break;")
    L.append("    default: break;")
    L.append("    }")
    L.append("}")
    L.append("static void m_ddeltaxdp(double* d, int ie, const double* p, const double* k) {")
    L.append("    (void)p; (void)k;")
    L.append(f"    memset(d, 0, sizeof(double) * {max(np_ * nx, 1)});")
    L.append("    switch (ie) {")
    for ie, ev in enumerate(spec.events):
        L.append(f"    case {ie}:")
        for i, dv in sorted(ev.bolus.items()):
            for j, pj in enumerate(spec.p):
                c = sp.diff(sp.sympify(dv), pj)
                if c != 0:
                    L.append(f"        d[{j * nx + i}] = {pr(c)};")
        L.append("        break;")
    L.append("    default: break;")
    L.append("    }")
    L.append("}")
    inits = [1 if ev.initial_value else 0 for ev in spec.events] or [1]
    L.append(f"static const int m_event_init[{len(inits)}] = {{{', '.join(map(str, inits))}}};")
    dirs = [ev.direction for ev in spec.events] or [1]
    L.append(f"static const int m_event_dir[{len(dirs)}] = {{{', '.join(map(str, dirs))}}};")
    # trigger functions (root finding): values and derivatives
    roots = spec.root_events()
    nr = len(roots)
    from .model_spec import TIME
    prt = _c_printer(spec)
    L.append(f"static const int m_root_event[{max(nr, 1)}] = {{{', '.join(map(str, roots or [0]))}}};")
    L.append("static void m_root(double* g, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)g; (void)t; (void)x; (void)p; (void)k;")
    for ir, ie in enumerate(roots):
        L.append(f"    g[{ir}] = {prt(sp.sympify(spec.events[ie].trigger))};")
    L.append("}")
    L.append("static void m_drootdx(double* d, int ir, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)t; (void)x; (void)p; (void)k;")
    L.append(f"    memset(d, 0, sizeof(double) * {max(nx, 1)});")
    L.append("    switch (ir) {")
    for ir, ie in enumerate(roots):
        L.append(f"    case {ir}:")
        trg = sp.sympify(spec.events[ie].trigger)
        for j, xj in enumerate(spec.x):
            dv = sp.diff(trg, xj)
            if dv != 0:
                L.append(f"        d[{j}] = {prt(dv)};")
        L.append("        break;")
    L += ["    default: break;", "    }", "}"]
    L.append("static void m_drootdp(double* d, int ir, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)t; (void)x; (void)p; (void)k;")
    L.append(f"    memset(d, 0, sizeof(double) * {max(np_, 1)});")
    L.append("    switch (ir) {")
    for ir, ie in enumerate(roots):
        L.append(f"    case {ir}:")
        trg = sp.sympify(spec.events[ie].trigger)
        for j, pj in enumerate(spec.p):
            dv = sp.diff(trg, pj)
            if dv != 0:
                L.append(f"        d[{j}] = {prt(dv)};")
        L.append("        break;")
    L += ["    default: break;", "    }", "}"]
    L.append("static double m_drootdt(int ir, double t, const double* x, const double* p, const double* k) {")
    L.append("    (void)t; (void)x; (void)p; (void)k;")
    L.append("    switch (ir) {")
    for ir, ie in enumerate(roots):
        dv = sp.diff(sp.sympify(spec.events[ie].trigger), TIME)
        L.append(f"    case {ir}: return {prt(dv)};")
    L += ["    default: break;", "    }", "    return 0.0;", "}"]
    L.append("")
    L.append("static const oracle_model model = {")
    L.append(f'    "{spec.name}", {nx}, {np_}, {nk}, {ny},')
    L.append("    m_x0, m_dx0dp, m_xdot, m_jac, m_dxdotdp, m_y, m_dydx, m_dydp, m_sigmay, m_dsigmaydp,")
    L.append(f"    m_noise, {ne}, m_event_times, m_devent_times_dp, m_deltax, m_ddeltaxdx, m_ddeltaxdp, m_event_init,")
    hev = spec.heaviside_events or [0]
    L.insert(len(L) - 5, f"static const int m_h_event[{len(hev)}] = {{{', '.join(map(str, hev))}}};")
    L.append(f"    {nr}, m_root_event, m_root, m_drootdx, m_drootdp, m_drootdt, {len(spec.heaviside_events)}, m_h_event,")
    L.append("    m_event_dir};")
    L.append("const oracle_model* oracle_get_model(void) { return &model; }")
    return "\n".join(L) + "\n"


def spec_digest(spec: ModelSpec) -> str:
    """Stable hash of the symbolic model (used to key build outputs)."""
    h = hashlib.sha256()
    h.update(spec.name.encode())
    for part in (spec.x0, spec.w, sorted(spec.stoich.items()), spec.y, spec.sigma_y):
        h.update(repr([str(e) for e in part] if not isinstance(part, list) or not part
                      or not isinstance(part[0], tuple) else part).encode())
    if spec.noise_distributions:
        h.update(repr(spec.noise_codes()).encode())
    for ev in spec.events:
        h.update(repr((str(ev.time), sorted((i, str(d)) for i, d in ev.bolus.items()), ev.initial_value,
                       str(ev.trigger))).encode())
    return h.hexdigest()[:16]


def _cuda_printer(spec: ModelSpec):
    pr = _c_printer(spec)
    return pr


def _fmt_list(vals, fmt="{}"):
    vals = list(vals)
    if not vals:
        return "{0}"
    out, line = [], []
    for v in vals:
        line.append(fmt.format(v))
        if len(line) == 16:
            out.append(", ".join(line))
            line = []
    if line:
        out.append(", ".join(line))
    return "{\n    " + ",\n    ".join(out) + "}"


def compact_jacobian(spec: ModelSpec):
    """The Jacobian on its structural pattern, row-major.

    Returns ``(entries, row_ptr, pos_a, pos_b)``: ``entries[p] = (i, j)`` in
    row-major order with row i at ``row_ptr[i]..row_ptr[i+1]``, and for every
    stoichiometry entry e (row i, flux r, in the order of the engine's
    stoichiometry rows) the positions of d w_r / d x_a and d w_r / d x_b in
    row i (-1: none; for a == b the whole derivative goes to ``pos_a``)."""
    mono, _ = spec.flux_forms()
    rows = [[] for _ in range(spec.nx)]
    for (i, r), sv in sorted(spec.stoich.items()):
        rows[i].append(r)
    struct = set()
    for i in range(spec.nx):
        for r in rows[i]:
            for a in (mono[r].a, mono[r].b):
                if a >= 0:
                    struct.add((i, a))
    entries = sorted(struct)
    pos = {e: p for p, e in enumerate(entries)}
    row_ptr = [0] * (spec.nx + 1)
    for (i, _a) in entries:
        row_ptr[i + 1] += 1
    for i in range(spec.nx):
        row_ptr[i + 1] += row_ptr[i]
    pos_a, pos_b = [], []
    for i in range(spec.nx):
        for r in rows[i]:
            a, b = mono[r].a, mono[r].b
            pos_a.append(pos[(i, a)] if a >= 0 else -1)
            pos_b.append(pos[(i, b)] if (b >= 0 and b != a) else -1)
    return entries, row_ptr, pos_a, pos_b


def sparse_lu_plan(spec: ModelSpec):
    """Static ordering and fill of the iteration matrix M = I - gamma*J.

    The structural pattern of J plus the diagonal is ordered by greedy
    minimum degree on its symmetrised graph (the role AMD plays for KLU,
    the reference's default linear solver), then eliminated symbolically.
    Returns ``(order, rows, cols, dense_flops, sparse_flops)``: ``order[i]``
    is the original index of permuted index i; ``rows[k]`` the permuted rows
    i > k of column k of L and ``cols[k]`` the permuted columns j > k of row
    k of U, fill included.  Pivots are taken on the diagonal in this order
    (no row exchanges at run time); a zero or non-finite pivot makes the
    factorisation report a singular matrix, which the integrator handles like
    any failed linear setup (smaller step, fresh Jacobian)."""
    n = spec.nx
    mono, _ = spec.flux_forms()
    P = np.eye(n, dtype=bool)
    for (i, r), _ in spec.stoich.items():
        for a in (mono[r].a, mono[r].b):
            if a >= 0:
                P[i, a] = True
    A = P | P.T
    elim = np.zeros(n, dtype=bool)
    order = []
    for _ in range(n):
        deg = np.where(elim, 1 << 30, A[:, ~elim].sum(axis=1))
        k = int(np.argmin(deg))
        order.append(k)
        elim[k] = True
        nb = np.where(A[k] & ~elim)[0]
        A[np.ix_(nb, nb)] = True
    Q = P[np.ix_(order, order)].copy()
    flops = 0
    rows, cols = [], []
    for k in range(n):
        r = np.where(Q[k + 1:, k])[0] + k + 1
        c = np.where(Q[k, k + 1:])[0] + k + 1
        Q[np.ix_(r, c)] = True
        flops += len(r) * len(c)
        rows.append([int(x) for x in r])
        cols.append([int(x) for x in c])
    return order, rows, cols, n ** 3 // 3, flops


def packed_lu_tables(n, rows, cols, jent, iorder, transposed=False):
    """Compressed storage of the factors for one elimination plan.

    The permuted matrix with its fill is stored row by row (CSR, columns
    ascending): row i holds (i, k) for the pivots k < i whose L column names
    row i, the diagonal, then its U row.  ``rows``/``cols`` are the plan's L
    columns and U rows (the forward plan for I - gamma*J; for the backward
    problem's I + gamma*J^T the forward plan's lists trade places).
    Returns ``rptr, col, diag`` (CSR), ``lpos[e]``: position of the e-th L
    entry in the order of the ``rows`` lists, ``span[e]``: entries of that
    row after it up to the last column of the pivot's U row (the stretch the
    pivot's update sweeps), and ``jpos[p]``: position of compact Jacobian
    entry p (transposed when ``transposed``)."""
    pat = [[] for _ in range(n)]
    for k in range(n):
        for i in rows[k]:
            pat[i].append(k)
    for i in range(n):
        pat[i] = sorted(pat[i]) + [i] + sorted(cols[i])
    rptr, col, pos = [0], [], {}
    for i in range(n):
        for j in pat[i]:
            pos[(i, j)] = len(col)
            col.append(j)
        rptr.append(len(col))
    diag = [pos[(i, i)] for i in range(n)]
    lpos, span = [], []
    for k in range(n):
        last = max(cols[k]) if cols[k] else k
        for i in rows[k]:
            pl = pos[(i, k)]
            lpos.append(pl)
            span.append(pos[(i, last)] - pl if cols[k] else 0)
    jpos = []
    for (i, a) in jent:
        r, c = iorder[i], iorder[a]
        jpos.append(pos[(c, r)] if transposed else pos[(r, c)])
    return rptr, col, diag, lpos, span, jpos


def _switch_x(name, arg, cases, pr, ret_default="0.0"):
    """Like ``_switch`` for expressions of the states as well."""
    lines = [f"    __device__ static double {name}(int {arg}, const double* x, const double* p, const double* k) {{",
             "        (void)x; (void)p; (void)k;", f"        switch ({arg}) {{"]
    for i, e in cases:
        if e == 0:
            continue
        lines.append(f"        case {i}: return {pr(e)};")
    lines += ["        default: break;", "        }", f"        return {ret_default};", "    }"]
    return lines


def _switch(name, arg, cases, pr, ret_default="0.0"):
    lines = [f"    __device__ static double {name}(int {arg}, const double* p, const double* k) {{",
             "        (void)p; (void)k;", f"        switch ({arg}) {{"]
    for i, e in enumerate(cases):
        if e == 0:
            continue
        lines.append(f"        case {i}: return {pr(e)};")
    lines += ["        default: break;", "        }", f"        return {ret_default};", "    }"]
    return lines


def _rate_law_printer():
    """C printer for rate laws: states ``xa``/``xb``, coefficients ``C[k]``."""
    repl = {RATE_X[0]: sp.Symbol("xa"), RATE_X[1]: sp.Symbol("xb")}

    def pr(expr):
        e = sp.sympify(expr)
        e = e.xreplace({**repl, **{c: sp.Symbol(f"C[{c.name[1:]}]") for c in e.free_symbols
                                   if c.name.startswith("C")}})
        return sp.ccode(sp.N(e, 17) if e.has(sp.Rational) and not e.is_Integer else e)

    return pr


def _rate_law_functions(laws):
    """Device functions evaluating the general rate laws (rate law t of
    ``laws`` is case t + 1; case 0 is the mass-action monomial): the flux
    value, its partial derivatives with respect to its two states, and its
    partial derivative with respect to one of its coefficients."""
    pr = _rate_law_printer()
    head = ["        const int a = W_A[r], b = W_B[r];",
            "        const double xa = a >= 0 ? y[a] : 0.0, xb = b >= 0 ? y[b] : 0.0;",
            "        const double* C = c + COFF[r];",
            "        (void)xa; (void)xb;"]
    L = ["    // general rate laws: case t evaluates rate law t for flux r at the states y",
         "    // with the per-instance coefficients c (all of them; flux r's start at COFF[r])",
         "    __device__ static double flux_value(int r, const double* y, const double* c) {", *head,
         "        switch (TPL[r]) {"]
    for t, law in enumerate(laws, 1):
        L.append(f"        case {t}: return {pr(law)};")
    L += ["        default: break;", "        }",
          "        double v = C[0];", "        if (a >= 0) v *= xa;", "        if (b >= 0) v *= xb;", "        return v;",
          "    }",
          "    __device__ static void flux_partials(int r, const double* y, const double* c, double& da, double& db) {",
          *head, "        switch (TPL[r]) {"]
    for t, law in enumerate(laws, 1):
        subs, (da, db) = sp.cse([sp.diff(law, RATE_X[0]), sp.diff(law, RATE_X[1])], symbols=sp.numbered_symbols("u"))
        L.append(f"        case {t}: {{")
        for sym, ex in subs:
            L.append(f"            const double {sym} = {pr(ex)};")
        L += [f"            da = {pr(da)};", f"            db = {pr(db)};", "            return;", "        }"]
    L += ["        default: break;", "        }",
          "        da = a < 0 ? 0.0 : (b < 0 ? C[0] : (a == b ? 2.0 * C[0] * xa : C[0] * xb));",
          "        db = (b >= 0 && b != a) ? C[0] * xa : 0.0;", "    }",
          "    // d w_r / d C_k for coefficient ci = COFF[r] + k",
          "    __device__ static double flux_dwdc(int ci, const double* y, const double* c) {",
          "        const int r = CF[ci], kk = ci - COFF[r];", *head, "        (void)kk;",
          "        switch (TPL[r]) {"]
    for t, law in enumerate(laws, 1):
        cs_ = sorted((c for c in law.free_symbols if c.name.startswith("C")), key=lambda c: int(c.name[1:]))
        L.append(f"        case {t}:")
        L.append("            switch (kk) {")
        for c in cs_:
            L.append(f"            case {c.name[1:]}: return {pr(sp.diff(law, c))};")
        L += ["            default: return 0.0;", "            }"]
    L += ["        default: break;", "        }",
          "        double v = 1.0;", "        if (a >= 0) v *= xa;", "        if (b >= 0) v *= xb;", "        return v;",
          "    }"]
    return L


def _event_functions(spec: ModelSpec, pr):
    """Device functions of the events: the trigger functions with their
    state, parameter and time derivatives (root finding), the trigger time of
    an explicit event and its parameter derivatives, the bolus of state i (an
    expression of x, p, k), the bolus's constant state coefficients applied
    to a vector, and its parameter derivatives."""
    spec.check_events()
    ne, nx, np_ = spec.ne, spec.nx, spec.np
    from .model_spec import TIME
    roots = spec.root_events()
    nr = len(roots)
    prt = _c_printer(spec)
    hev = list(getattr(spec, "heaviside_events", []) or [])
    L = [f"    static constexpr int NE = {ne};",
         "    // Heaviside indicators of the right-hand side: indicator j is fixed",
         "    // parameter NK + j, the Heaviside of the trigger of event heaviside_event(j)",
         f"    static constexpr int NH = {len(hev)};",
         "    __device__ static int heaviside_event(int j) {",
         "        switch (j) {",
         *[f"        case {j}: return {ie};" for j, ie in enumerate(hev)],
         "        default: return 0;",
         "        }",
         "    }",
         "    // events with a trigger function (root finding): root ir belongs to",
         "    // event root_event(ir); event_root(ie) is -1 for an explicit trigger time",
         f"    static constexpr int NR = {nr};",
         "    __device__ static int root_event(int ir) {",
         "        switch (ir) {"]
    for ir, ie in enumerate(roots):
        L.append(f"        case {ir}: return {ie};")
    L += ["        default: return -1;", "        }", "    }",
          "    __device__ static int event_root(int ie) {", "        switch (ie) {"]
    for ir, ie in enumerate(roots):
        L.append(f"        case {ie}: return {ir};")
    L += ["        default: return -1;", "        }", "    }",
          "    __device__ static double root(int ir, double t, const double* x, const double* p, const double* k) {",
          "        (void)t; (void)x; (void)p; (void)k;", "        switch (ir) {"]
    for ir, ie in enumerate(roots):
        L.append(f"        case {ir}: return {prt(sp.sympify(spec.events[ie].trigger))};")
    L += ["        default: break;", "        }", "        return 0.0;", "    }",
          "    // sum_j d g_ir / d x_j v[j * st]",
          "    __device__ static double root_dx_dot(int ir, double t, const double* x, const double* p, const double* k,",
          "                                         const double* v, int st) {",
          "        (void)t; (void)x; (void)p; (void)k; (void)v; (void)st;", "        double acc = 0.0;",
          "        switch (ir) {"]
    for ir, ie in enumerate(roots):
        trg = sp.sympify(spec.events[ie].trigger)
        L.append(f"        case {ir}:")
        for j, xj in enumerate(spec.x):
            dv = sp.diff(trg, xj)
            if dv != 0:
                L.append(f"            acc += ({prt(dv)}) * v[{j} * st];")
        L.append("            break;")
    L += ["        default: break;", "        }", "        return acc;", "    }",
          "    __device__ static double root_dp(int ir, int j, double t, const double* x, const double* p,",
          "                                     const double* k) {",
          "        (void)t; (void)x; (void)p; (void)k;", "        switch (ir * NP + j) {"]
    for ir, ie in enumerate(roots):
        trg = sp.sympify(spec.events[ie].trigger)
        for j, pj in enumerate(spec.p):
            dv = sp.diff(trg, pj)
            if dv != 0:
                L.append(f"        case {ir * np_ + j}: return {prt(dv)};")
    L += ["        default: break;", "        }", "        return 0.0;", "    }",
          "    __device__ static double root_dt(int ir, double t, const double* x, const double* p, const double* k) {",
          "        (void)t; (void)x; (void)p; (void)k;", "        switch (ir) {"]
    for ir, ie in enumerate(roots):
        dv = sp.diff(sp.sympify(spec.events[ie].trigger), TIME)
        if dv != 0:
            L.append(f"        case {ir}: return {prt(dv)};")
    L += ["        default: break;", "        }", "        return 0.0;", "    }"]
    L += ["    // the sign of an explicit trigger's time derivative: the trigger is",
          "    // direction * (t - te)",
          "    __device__ static int event_direction(int ie) {",
          "        switch (ie) {",
          *[f"        case {ie}: return -1;" for ie, ev in enumerate(spec.events) if ev.direction < 0],
          "        default: return 1;",
          "        }",
          "    }"]
    L += [
         "    // the trigger's value before t0 (false: an event at or before t0 fires at t0)",
         "    __device__ static bool event_initial_value(int ie) {",
         "        switch (ie) {"]
    for ie, ev in enumerate(spec.events):
        if not ev.initial_value:
            L.append(f"        case {ie}: return false;")
    L += ["        default: return true;", "        }", "    }"]
    L += _switch("event_time", "ie", [sp.sympify(ev.time) if ev.time is not None else sp.Integer(0)
                                      for ev in spec.events], pr)
    dte = [sp.diff(sp.sympify(ev.time), pj) if ev.time is not None else sp.Integer(0)
           for ev in spec.events for pj in spec.p]
    L += _switch("devent_time_dp_entry", "c", dte, pr)
    L += ["    __device__ __forceinline__ static double devent_time_dp(int ie, int j, const double* p, const double* k) {",
          "        return devent_time_dp_entry(ie * NP + j, p, k);", "    }"]
    bol = [(ie * nx + i, sp.sympify(d)) for ie, ev in enumerate(spec.events) for i, d in ev.bolus.items()]
    L += _switch_x("deltax_entry", "c", bol, pr)
    L += ["    __device__ __forceinline__ static double deltax(int ie, int i, const double* x, const double* p,",
          "                                                   const double* k) {",
          "        return deltax_entry(ie * NX + i, x, p, k);", "    }"]
    # sum_j d deltax_i / d x_j v_j (the coefficients are constants)
    v = [sp.Symbol(f"v[{j} * st]") for j in range(nx)]
    lin = []
    for ie, ev in enumerate(spec.events):
        for i, d in ev.bolus.items():
            e = sum((sp.diff(sp.sympify(d), xj) * v[j] for j, xj in enumerate(spec.x)), sp.Integer(0))
            lin.append((ie * nx + i, e))
    L += ["    __device__ static double ddeltaxdx_times(int ie, int i, const double* v, int st) {",
          "        (void)v; (void)st;", "        switch (ie * NX + i) {"]
    for c, e in lin:
        if e != 0:
            L.append(f"        case {c}: return {sp.ccode(sp.N(e, 17) if e.has(sp.Rational) else e)};")
    L += ["        default: break;", "        }", "        return 0.0;", "    }"]
    dp = [(ie * nx * np_ + i * np_ + j, sp.diff(sp.sympify(d), pj)) for ie, ev in enumerate(spec.events)
          for i, d in ev.bolus.items() for j, pj in enumerate(spec.p)]
    dp = [(c, e) for c, e in dp if e != 0]
    L += _switch_x("ddeltaxdp_entry", "c", dp, pr)
    L += ["    __device__ __forceinline__ static double ddeltaxdp(int ie, int i, int j, const double* x, const double* p,",
          "                                                      const double* k) {",
          "        return ddeltaxdp_entry((ie * NX + i) * NP + j, x, p, k);", "    }"]
    return L


def emit_engine_cuda(spec: ModelSpec) -> str:
    """CUDA translation unit defining the engine model type and its C ABI."""
    spec = expand_heavisides(spec)
    mono, laws = spec.flux_forms()
    general = bool(laws)
    # per-instance coefficients: flux r owns COFF[r]..COFF[r+1] (one each for
    # the monomials); CF maps a coefficient back to its flux
    coeffs, coff, cf = [], [0], []
    for r, f in enumerate(mono):
        coeffs += f.coeffs
        cf += [r] * len(f.coeffs)
        coff.append(len(coeffs))
    nc = len(coeffs)
    for e in spec.sigma_y:
        if e.free_symbols & set(spec.x):
            raise ValueError("noise scales must not depend on the states")
    # observation model: y = h(x, p, k) with the pattern and values of dh/dx
    # (a numeric table when every entry is a constant), dh/dp and dsigma/dp
    obs_ent = [(iy, j, sp.diff(yi, xj)) for iy, yi in enumerate(spec.y) for j, xj in enumerate(spec.x)
               if xj in yi.free_symbols]
    obs_ent = [(iy, j, d) for iy, j, d in obs_ent if d != 0]
    obs_numeric = all(not d.free_symbols for _, _, d in obs_ent)
    dydp = [(iy * spec.np + j, sp.diff(yi, pj)) for iy, yi in enumerate(spec.y) for j, pj in enumerate(spec.p)
            if pj in yi.free_symbols]
    dydp = [(c, d) for c, d in dydp if d != 0]
    dsig = [(iy * spec.np + j, sp.diff(si, pj)) for iy, si in enumerate(spec.sigma_y) for j, pj in enumerate(spec.p)
            if pj in si.free_symbols]
    dsig = [(c, d) for c, d in dsig if d != 0]
    noise = spec.noise_codes()
    pr = _cuda_printer(spec)
    nx, nw, np_, nk, ny = spec.nx, spec.nw, spec.np, spec.nk, spec.ny
    # stoichiometry in CSR by species
    rows = [[] for _ in range(nx)]
    for (i, r), s in sorted(spec.stoich.items()):
        rows[i].append((r, float(s)))
    s_ptr, s_r, s_v = [0], [], []
    for i in range(nx):
        for r, s in rows[i]:
            s_r.append(r)
            s_v.append(s)
        s_ptr.append(len(s_r))
    # packed tables for register caching: (flux | coef << 16), ((a+1) | (b+1) << 16)
    s_pk = []
    for r, v in zip(s_r, s_v):
        if v != int(v) or abs(int(v)) > 32767 or r > 65535:
            raise ValueError("GPU engine requires small integer stoichiometric coefficients")
        s_pk.append((r & 0xFFFF) | ((int(v) & 0xFFFF) << 16))
    s_pk = [x - (1 << 32) if x >= (1 << 31) else x for x in s_pk]
    w_ab = [(m.a + 1) | ((m.b + 1) << 16) for m in mono]
    # stoichiometry by flux (CSC): species | coef << 16
    cols = [[] for _ in range(nw)]
    for (i, r), s in sorted(spec.stoich.items(), key=lambda kv: (kv[0][1], kv[0][0])):
        cols[r].append((i, int(s)))
    sc_ptr, sc_pk = [0], []
    for r in range(nw):
        for i, s in cols[r]:
            sc_pk.append((i & 0xFFFF) | ((s & 0xFFFF) << 16))
        sc_ptr.append(len(sc_pk))
    sc_pk = [x - (1 << 32) if x >= (1 << 31) else x for x in sc_pk]
    rmax = max((s_ptr[i + 1] - s_ptr[i] for i in range(nx)), default=0)
    # reactant incidence by species (CSR) for the adjoint right-hand side
    # -J^T xB: species j lists (flux r, slot) with slot 0 if j is the first
    # reactant of r and 1 if it is a distinct second reactant
    ri = [[] for _ in range(nx)]
    for r, m in enumerate(mono):
        if m.a >= 0:
            ri[m.a].append(2 * r)
        if m.b >= 0 and m.b != m.a:
            ri[m.b].append(2 * r + 1)
    ri_ptr, ri_pk = [0], []
    for j in range(nx):
        ri_pk += ri[j]
        ri_ptr.append(len(ri_pk))
    # Jacobian structure
    jstruct = set()
    for i in range(nx):
        for r, _ in rows[i]:
            for sidx in (mono[r].a, mono[r].b):
                if sidx >= 0:
                    jstruct.add((i, sidx))
    # coefficient derivatives dC_ci/dp_j, grouped by parameter (CSC): for
    # parameter j the entries d in DP_PTR[j]..DP_PTR[j+1] name coefficient
    # DP_R[d] (for a model of monomials, coefficient r is flux r's); the value
    # is dcoeff(d, p, k), evaluated once per instance
    dp_entries = [[] for _ in range(np_)]
    for ci, ce in enumerate(coeffs):
        for j, pj in enumerate(spec.p):
            if pj in ce.free_symbols:
                dp_entries[j].append((ci, sp.diff(ce, pj)))
    dp_ptr, dp_r, dp_expr = [0], [], []
    for j in range(np_):
        for r, ex in dp_entries[j]:
            dp_r.append(r)
            dp_expr.append(ex)
        dp_ptr.append(len(dp_r))
    # initial-state derivatives dx0_i/dp_j (nonzero entries only)
    dx0 = [(i, j, sp.diff(e, pj)) for i, e in enumerate(spec.x0) for j, pj in enumerate(spec.p)
           if pj in e.free_symbols]
    # observables: CSR pattern of dh/dx (values numeric when constant)
    h_ptr, h_j, h_v, h_expr = [0], [], [], []
    for iy in range(ny):
        for (jy, j, d) in obs_ent:
            if jy == iy:
                h_j.append(j)
                h_v.append(float(d) if obs_numeric else 0.0)
                h_expr.append(d)
        h_ptr.append(len(h_j))
    jent, jr_ptr, jpa, jpb = compact_jacobian(spec)
    j_rc = [(i & 0xFFFF) | ((a & 0xFFFF) << 16) for (i, a) in jent]
    # sparse LU of the iteration matrix when the ordered fill saves most of
    # the dense work (models with more states than a warp has lanes)
    order, lrows, ucols, dflops, sflops = sparse_lu_plan(spec)
    sparse_lu = nx > 32 and sflops < 0.5 * dflops
    iorder = [0] * nx
    for pi, oi in enumerate(order):
        iorder[oi] = pi
    lu_rptr, lu_ridx, lu_cptr, lu_cidx = [0], [], [0], []
    for k in range(nx):
        lu_ridx += lrows[k]
        lu_rptr.append(len(lu_ridx))
        lu_cidx += ucols[k]
        lu_cptr.append(len(lu_cidx))
    # factors in compressed rows when dense N x N storage would crowd the
    # shared memory out (more than 48 KB in FP32)
    if spec.lu_storage not in ("auto", "dense", "packed"):
        raise ValueError(f"lu_storage must be auto, dense or packed, not {spec.lu_storage!r}")
    packed_lu = sparse_lu and (spec.lu_storage == "packed" or
                               (spec.lu_storage == "auto" and nx * nx * 4 > 48 * 1024))
    pk = packed_lu_tables(nx, lrows, ucols, jent, iorder) if packed_lu else ([0], [0], [0], [0], [0], [0])
    pkt = (packed_lu_tables(nx, ucols, lrows, jent, iorder, transposed=True) if packed_lu
           else ([0], [0], [0], [0], [0], [0]))
    nnz_pk = len(pk[1]) if packed_lu else 1
    assert nnz_pk < 32768, "packed factor positions are stored as int16"
    pk_lines = []
    # column indices and stretch lengths in one byte where they fit (the
    # factorisation and the sweeps read them from the L1 cache)
    col_t = "uint8_t" if nx <= 256 else "int16_t"
    for tag, (rp, cl, dg, lp, spn, jp) in (("PK", pk), ("PKT", pkt)):
        span_t = "uint8_t" if max(spn) <= 255 else "int16_t"
        pk_lines += [
            f"static __device__ const int32_t {tag}_RPTR[{len(rp)}] = {_fmt_list(rp)};",
            f"static __device__ const {col_t} {tag}_COL[{len(cl)}] = {_fmt_list(cl)};",
            f"static __device__ const int16_t {tag}_DIAG[{len(dg)}] = {_fmt_list(dg)};",
            f"static __device__ const int16_t {tag}_LPOS[{len(lp)}] = {_fmt_list(lp)};",
            f"static __device__ const {span_t} {tag}_SPAN[{len(spn)}] = {_fmt_list(spn)};",
            f"static __device__ const int16_t {tag}_JPOS[{len(jp)}] = {_fmt_list(jp)};"]
    ns = f"amici_model_{spec.name}"
    L = [
        f"// Generated by amici_gb300.codegen.emit_engine_cuda — model {spec.name}; do not edit.",
        "#pragma once",
        '#include "amici_gb300/csrc/abi.cuh"',
        "",
        f"namespace {ns} {{",
        f"static __device__ const int16_t W_A[{max(nw, 1)}] = {_fmt_list([m.a for m in mono])};",
        f"static __device__ const int16_t W_B[{max(nw, 1)}] = {_fmt_list([m.b for m in mono])};",
        f"static __device__ const int32_t S_PTR[{nx + 1}] = {_fmt_list(s_ptr)};",
        f"static __device__ const int16_t S_R[{max(len(s_r), 1)}] = {_fmt_list(s_r)};",
        f"static __device__ const double S_V[{max(len(s_v), 1)}] = {_fmt_list(s_v, '{!r}')};",
        f"static __device__ const int32_t S_PK[{max(len(s_r), 1)}] = {_fmt_list(s_pk)};",
        f"static __device__ const int32_t W_AB[{max(nw, 1)}] = {_fmt_list(w_ab)};",
        f"static __device__ const int32_t SC_PTR[{nw + 1}] = {_fmt_list(sc_ptr)};",
        f"static __device__ const int32_t SC_PK[{max(len(sc_pk), 1)}] = {_fmt_list(sc_pk)};",
        f"static __device__ const int32_t DP_PTR[{np_ + 1}] = {_fmt_list(dp_ptr)};",
        f"static __device__ const int32_t DP_R[{max(len(dp_r), 1)}] = {_fmt_list(dp_r)};",
        f"static __device__ const int32_t H_PTR[{ny + 1}] = {_fmt_list(h_ptr)};",
        f"static __device__ const int32_t RI_PTR[{nx + 1}] = {_fmt_list(ri_ptr)};",
        f"static __device__ const int16_t LU_ORDER[{nx}] = {_fmt_list(order)};",
        f"static __device__ const int16_t LU_IORDER[{nx}] = {_fmt_list(iorder)};",
        f"static __device__ const int32_t J_RC[{max(len(j_rc), 1)}] = {_fmt_list(j_rc)};",
        f"static __device__ const int32_t J_RPTR[{nx + 1}] = {_fmt_list(jr_ptr)};",
        f"static __device__ const int32_t J_PA[{max(len(jpa), 1)}] = {_fmt_list(jpa)};",
        f"static __device__ const int32_t J_PB[{max(len(jpb), 1)}] = {_fmt_list(jpb)};",
        f"static __device__ const int32_t LU_RPTR[{nx + 1}] = {_fmt_list(lu_rptr)};",
        f"static __device__ const int16_t LU_RIDX[{max(len(lu_ridx), 1)}] = {_fmt_list(lu_ridx)};",
        f"static __device__ const int32_t LU_CPTR[{nx + 1}] = {_fmt_list(lu_cptr)};",
        f"static __device__ const int16_t LU_CIDX[{max(len(lu_cidx), 1)}] = {_fmt_list(lu_cidx)};",
        f"static __device__ const int32_t RI_PK[{max(len(ri_pk), 1)}] = {_fmt_list(ri_pk)};",
        f"static __device__ const int16_t H_J[{max(len(h_j), 1)}] = {_fmt_list(h_j)};",
        f"static __device__ const double H_V[{max(len(h_v), 1)}] = {_fmt_list(h_v, '{!r}')};",
        f"static __device__ const int8_t NOISE[{max(ny, 1)}] = {_fmt_list(noise)};",
        *([f"static __device__ const int32_t COFF[{nw + 1}] = {_fmt_list(coff)};",
           f"static __device__ const int32_t CF[{max(nc, 1)}] = {_fmt_list(cf)};",
           f"static __device__ const int8_t TPL[{max(nw, 1)}] = {_fmt_list([f.template for f in mono])};"]
          if general else []),
        *pk_lines,
        "",
        "struct Model {",
        f"    static constexpr int NX = {nx}, NW = {nw}, NP = {np_}, NK = {nk}, NY = {ny};",
        f"    static constexpr int NNZ_J = {len(jstruct)}, RMAX = {max(rmax, 1)}, ND = {len(dp_r)};",
        "    // per-instance coefficients (NC; one per flux for a model of monomials)",
        "    // and whether some flux follows a general rate law",
        f"    static constexpr int NC = {nc};",
        f"    static constexpr bool GENERAL = {'true' if general else 'false'};",
        f'    static constexpr const char* NAME = "{spec.name}";',
        f"    // sparse LU: {sflops} update FMAs in the static order vs {dflops} dense",
        f"    static constexpr bool SPARSE_LU = {'true' if sparse_lu else 'false'};",
        "    // factors in compressed rows (PK_*: forward plan, PKT_*: transposed plan);",
        "    // LU_STORE = entries of the factor storage",
        f"    static constexpr bool PACKED_LU = {'true' if packed_lu else 'false'};",
        f"    static constexpr int LU_STORE = {nnz_pk if packed_lu else nx * nx};",
        "    template <bool TR> __device__ __forceinline__ static int pk_rptr(int i) { return TR ? PKT_RPTR[i] : PK_RPTR[i]; }",
        "    template <bool TR> __device__ __forceinline__ static int pk_col(int p) { return TR ? PKT_COL[p] : PK_COL[p]; }",
        "    template <bool TR> __device__ __forceinline__ static int pk_diag(int i) { return TR ? PKT_DIAG[i] : PK_DIAG[i]; }",
        "    template <bool TR> __device__ __forceinline__ static int pk_lpos(int e) { return TR ? PKT_LPOS[e] : PK_LPOS[e]; }",
        "    template <bool TR> __device__ __forceinline__ static int pk_span(int e) { return TR ? PKT_SPAN[e] : PK_SPAN[e]; }",
        "    template <bool TR> __device__ __forceinline__ static int pk_jpos(int p) { return TR ? PKT_JPOS[p] : PK_JPOS[p]; }",
        "    __device__ __forceinline__ static int lu_order(int i) { return LU_ORDER[i]; }",
        "    __device__ __forceinline__ static int lu_iorder(int i) { return LU_IORDER[i]; }",
        "    // compact Jacobian: entry p at (row, col) = J_RC[p]; row i holds J_RPTR[i]..J_RPTR[i+1]",
        "    __device__ __forceinline__ static int j_rc(int p) { return J_RC[p]; }",
        "    __device__ __forceinline__ static int j_rbegin(int i) { return J_RPTR[i]; }",
        "    __device__ __forceinline__ static int j_rend(int i) { return J_RPTR[i + 1]; }",
        "    // row i of J = S * dw/dx into the compact positions (zeroed first)",
        "    template <class T>",
        "    __device__ static void jac_row_sparse(int i, const double* c, const double* y, T* Jc) {",
        "        for (int p = J_RPTR[i]; p < J_RPTR[i + 1]; p++) Jc[p] = T(0);",
        "        for (int e = S_PTR[i]; e < S_PTR[i + 1]; e++) {",
        *(["            const int r = S_R[e], a = W_A[r], b = W_B[r];",
           "            if (a < 0) continue;",
           "            double da, db;",
           "            flux_partials(r, y, c, da, db);",
           "            Jc[J_PA[e]] += T(S_V[e] * da);",
           "            if (b >= 0 && b != a) Jc[J_PB[e]] += T(S_V[e] * db);"] if general else
          ["            const int r = S_R[e], a = W_A[r], b = W_B[r];",
           "            const double sc = S_V[e] * c[r];",
           "            if (a < 0) continue;",
           "            if (b < 0) Jc[J_PA[e]] += T(sc);",
           "            else if (a == b) Jc[J_PA[e]] += T(2.0 * sc * y[a]);",
           "            else {",
           "                Jc[J_PA[e]] += T(sc * y[b]);",
           "                Jc[J_PB[e]] += T(sc * y[a]);",
           "            }"]),
        "        }",
        "    }",
        "    __device__ __forceinline__ static int lu_rbegin(int k) { return LU_RPTR[k]; }",
        "    __device__ __forceinline__ static int lu_rend(int k) { return LU_RPTR[k + 1]; }",
        "    __device__ __forceinline__ static int lu_row(int e) { return LU_RIDX[e]; }",
        "    __device__ __forceinline__ static int lu_cbegin(int k) { return LU_CPTR[k]; }",
        "    __device__ __forceinline__ static int lu_cend(int k) { return LU_CPTR[k + 1]; }",
        "    __device__ __forceinline__ static int lu_col(int e) { return LU_CIDX[e]; }",
    ]
    L += _switch("flux_coeff", "ci", coeffs, pr)
    if general:
        L += _rate_law_functions(laws)
    L += [f"    __device__ __forceinline__ static int coef_flux(int ci) {{ return {'CF[ci]' if general else 'ci'}; }}"]
    L += _switch("x0", "i", spec.x0, pr)
    L += _switch("sigma", "iy", spec.sigma_y, pr, ret_default="1.0")
    L += _switch_x("observable", "iy", list(enumerate(spec.y)), pr)
    if not obs_numeric:
        L += _switch_x("obs_dydx", "e", list(enumerate(h_expr)), pr)
    L += _switch_x("obs_dydp_entry", "c", dydp, pr)
    dsig_map = dict(dsig)
    L += _switch("dsigma_dp_entry", "c", [dsig_map.get(c, 0) for c in range(ny * np_)] if dsig else [], pr)
    L += [f"    static constexpr bool HAS_DYDP = {'true' if dydp else 'false'}, "
          f"HAS_DSIGMA = {'true' if dsig else 'false'};",
          "    __device__ __forceinline__ static double obs_dydp(int iy, int j, const double* x, const double* p,",
          "                                                     const double* k) {",
          "        return obs_dydp_entry(iy * NP + j, x, p, k);",
          "    }",
          "    __device__ __forceinline__ static double dsigma_dp(int iy, int j, const double* p, const double* k) {",
          "        return dsigma_dp_entry(iy * NP + j, p, k);",
          "    }",
          "    __device__ __forceinline__ static int noise(int iy) { return NOISE[iy]; }"]
    L += _switch("dcoeff", "d", dp_expr, pr)
    # dx0/dp as a switch over (i * NP + j)
    dx0_lines = ["    __device__ static double dx0dp(int i, int j, const double* p, const double* k) {",
                 "        (void)p; (void)k;", "        switch (i * NP + j) {"]
    for i, j, ex in dx0:
        if ex != 0:
            dx0_lines.append(f"        case {i * np_ + j}: return {pr(ex)};")
    dx0_lines += ["        default: break;", "        }", "        return 0.0;", "    }"]
    L += dx0_lines
    L += _event_functions(spec, pr)
    L += [
        "    // packed tables (see codegen): stoichiometry rows and flux reactants",
        "    __device__ __forceinline__ static int row_begin(int i) { return S_PTR[i]; }",
        "    __device__ __forceinline__ static int row_end(int i) { return S_PTR[i + 1]; }",
        "    __device__ __forceinline__ static int row_packed(int e) { return S_PK[e]; }",
        "    __device__ __forceinline__ static int flux_ab(int r) { return W_AB[r]; }",
        "    __device__ __forceinline__ static int col_begin(int r) { return SC_PTR[r]; }",
        "    __device__ __forceinline__ static int col_end(int r) { return SC_PTR[r + 1]; }",
        "    __device__ __forceinline__ static int col_packed(int e) { return SC_PK[e]; }",
        "    __device__ __forceinline__ static int dp_begin(int j) { return DP_PTR[j]; }",
        "    __device__ __forceinline__ static int dp_end(int j) { return DP_PTR[j + 1]; }",
        "    __device__ __forceinline__ static int dp_coef(int d) { return DP_R[d]; }",
        "    // the tables the adjoint right-hand sides walk, staged in shared memory",
        f"    static constexpr int TB_SC_PTR = 0, TB_SC_PK = {nw + 1}, TB_RI_PTR = {nw + 1 + len(sc_pk)},",
        f"        TB_RI_PK = {nw + 1 + len(sc_pk) + nx + 1}, TB_W_AB = {nw + 1 + len(sc_pk) + nx + 1 + len(ri_pk)},",
        f"        TB_DP_PTR = {nw + 1 + len(sc_pk) + nx + 1 + len(ri_pk) + nw},",
        f"        TB_DP_R = {nw + 1 + len(sc_pk) + nx + 1 + len(ri_pk) + nw + np_ + 1},",
        f"        TB_TOTAL = {nw + 1 + len(sc_pk) + nx + 1 + len(ri_pk) + nw + np_ + 1 + len(dp_r)};",
        "    __device__ static void copy_tables(int* T, int tid, int nth) {",
        f"        for (int i = tid; i < {nw + 1}; i += nth) T[TB_SC_PTR + i] = SC_PTR[i];",
        f"        for (int i = tid; i < {len(sc_pk)}; i += nth) T[TB_SC_PK + i] = SC_PK[i];",
        f"        for (int i = tid; i < {nx + 1}; i += nth) T[TB_RI_PTR + i] = RI_PTR[i];",
        f"        for (int i = tid; i < {len(ri_pk)}; i += nth) T[TB_RI_PK + i] = RI_PK[i];",
        f"        for (int i = tid; i < {nw}; i += nth) T[TB_W_AB + i] = W_AB[i];",
        f"        for (int i = tid; i < {np_ + 1}; i += nth) T[TB_DP_PTR + i] = DP_PTR[i];",
        f"        for (int i = tid; i < {len(dp_r)}; i += nth) T[TB_DP_R + i] = DP_R[i];",
        "    }",
        "    __device__ __forceinline__ static int ri_begin(int j) { return RI_PTR[j]; }",
        "    __device__ __forceinline__ static int ri_end(int j) { return RI_PTR[j + 1]; }",
        "    __device__ __forceinline__ static int ri_packed(int e) { return RI_PK[e]; }",
        "    __device__ __forceinline__ static int obs_begin(int iy) { return H_PTR[iy]; }",
        "    __device__ __forceinline__ static int obs_end(int iy) { return H_PTR[iy + 1]; }",
        "    __device__ __forceinline__ static int obs_state(int e) { return H_J[e]; }",
        *(["    __device__ __forceinline__ static double obs_dydx(int e, const double* x, const double* p,",
            "                                                     const double* k) {",
            "        (void)x; (void)p; (void)k;",
            "        return H_V[e];",
            "    }"] if obs_numeric else []),
        "    __device__ __forceinline__ static double flux_monomial(int r, const double* y) {",
        "        const int a = W_A[r], b = W_B[r];",
        "        double v = a >= 0 ? y[a] : 1.0;",
        "        if (b >= 0) v *= y[b];",
        "        return v;",
        "    }",
        "    __device__ __forceinline__ static double stoich_row_dot(int i, const double* w) {",
        "        double s = 0.0;",
        "        for (int e = S_PTR[i]; e < S_PTR[i + 1]; e++) s += S_V[e] * w[S_R[e]];",
        "        return s;",
        "    }",
        "    // row i of J = S * dw/dx, accumulated into column-major J (ld = NX)",
        "    template <class T>",
        "    __device__ static void jac_row(int i, const double* c, const double* y, T* J) {",
        "        for (int e = S_PTR[i]; e < S_PTR[i + 1]; e++) {",
        *(["            const int r = S_R[e], a = W_A[r], b = W_B[r];",
           "            if (a < 0) continue;",
           "            double da, db;",
           "            flux_partials(r, y, c, da, db);",
           "            J[a * NX + i] += T(S_V[e] * da);",
           "            if (b >= 0 && b != a) J[b * NX + i] += T(S_V[e] * db);"] if general else
          ["            const int r = S_R[e], a = W_A[r], b = W_B[r];",
           "            const double sc = S_V[e] * c[r];",
           "            if (a < 0) continue;",
           "            if (b < 0) {",
           "                J[a * NX + i] += T(sc);",
           "            } else if (a == b) {",
           "                J[a * NX + i] += T(2.0 * sc * y[a]);",
           "            } else {",
           "                J[a * NX + i] += T(sc * y[b]);",
           "                J[b * NX + i] += T(sc * y[a]);",
           "            }"]),
        "        }",
        "    }",
        "};",
        f"}}  // namespace {ns}",
        f"using GeneratedModel = {ns}::Model;",
    ]
    return "\n".join(L) + "\n"


LANE_CHOICES = (1, 2, 4, 8, 16, 32)
MAX_SLOTS = 4  # register slots per lane (elements per lane) of the compiled variants


def lane_choices(spec: ModelSpec) -> tuple[int, ...]:
    """Lanes-per-instance values compiled for a model: those that keep every
    lane at <= MAX_SLOTS state elements, and always 32 (one warp per instance)."""
    return tuple(G for G in LANE_CHOICES if G == 32 or -(-spec.nx // G) <= MAX_SLOTS)


def emit_engine_units(spec: ModelSpec) -> dict[str, str]:
    """All translation units of one model library: ``model.cuh`` (tables and
    model type), one kernel unit per lanes-per-instance choice and one for the
    sensitivity kernels (compiled in parallel), and ``abi.cu`` (the exported C
    functions)."""
    lanes = lane_choices(spec)
    mask = sum(1 << G.bit_length() - 1 for G in lanes)
    fsa, asa, preeq = "fsa" in spec.families, "asa" in spec.families, "preeq" in spec.families
    posteq = "posteq" in spec.families
    flags = (f"    static constexpr int LANE_MASK = {mask};\n"
             f"    static constexpr bool HAS_FSA = {'true' if fsa else 'false'}, HAS_ASA = {'true' if asa else 'false'};\n"
             f"    static constexpr bool HAS_PREEQ = {'true' if preeq else 'false'};\n"
             f"    static constexpr bool HAS_POSTEQ = {'true' if posteq else 'false'};\n")
    model_text = emit_engine_cuda(spec)
    if fsa and "PACKED_LU = true" in model_text:
        raise ValueError(f"model {spec.name}: forward sensitivities need the dense factor storage "
                         "(lu_storage='dense', or leave 'fsa' out of families)")
    units = {"model.cuh": model_text.replace(
        "    static constexpr int NX =", flags + "    static constexpr int NX =", 1)}
    variants = {f"fwd_g{G}.cu": [(G, "float", "float", "false")] for G in lanes}
    # FP64 LU and the all-FP64 variant: one warp per instance
    variants["fwd_g32.cu"] += [(32, "double", "float", "false"), (32, "double", "double", "false")]
    # forward sensitivities (one instance per warp)
    if fsa:
        variants["fwd_sens32.cu"] = [(32, "float", "float", "true")]
        variants["fwd_sens64.cu"] = [(32, "double", "double", "true")]
    # pre-equilibration (simulation to steady state; one warp per instance)
    if preeq:
        variants["preeq.cu"] = [(32, lu, ctl, "false", "true") for lu, ctl in
                                (("float", "float"), ("double", "float"), ("double", "double"))]
        if fsa:
            variants["preeq_sens.cu"] = [(32, "float", "float", "true", "true"),
                                         (32, "double", "double", "true", "true")]
    # post-equilibration (outputs at t = inf; one warp per instance)
    if posteq:
        variants["posteq.cu"] = [(32, lu, ctl, "false", "false", "true") for lu, ctl in
                                 (("float", "float"), ("double", "float"), ("double", "double"))]
        if fsa:
            variants["posteq_sens.cu"] = [(32, "float", "float", "true", "false", "true"),
                                          (32, "double", "double", "true", "false", "true")]
    all_variants = []
    # adjoint sensitivities (one instance per warp), FP32 and FP64 iteration matrix
    for lu in ("float", "double") if asa else ():
        for ck, tag in (("true", "ck"), ("false", "es")):
            units[f"adj_{lu}_{tag}.cu"] = "\n".join([
                f"// Generated: adjoint kernel ({lu} iteration matrix, "
                f"{'check points' if tag == 'ck' else 'every step stored'}).", '#include "model.cuh"',
                f"template int agb::launch_adjoint_v<GeneratedModel, {lu}, {lu}, {ck}>(",
                "    const agb::Batch&, const agb::Opts&, cudaStream_t);", ""])
    for name, vs in variants.items():
        body = [f"// Generated: forward kernels ({name}).", '#include "model.cuh"']
        for v in vs:
            targs = ", ".join(map(str, v))
            body.append(f"template int agb::launch_forward<GeneratedModel, {targs}>(")
            body.append("    const agb::Batch&, const agb::Opts&, cudaStream_t);")
            all_variants.append(targs)
        units[name] = "\n".join(body + [""])
    lines = ["// Generated: exported C ABI.", '#include "model.cuh"',
             '#include "amici_gb300/csrc/noalloc.cuh"']
    for targs in all_variants:
        lines.append(f"extern template int agb::launch_forward<GeneratedModel, {targs}>(")
        lines.append("    const agb::Batch&, const agb::Opts&, cudaStream_t);")
    for lu in ("float", "double") if asa else ():
        for ck in ("true", "false"):
            lines.append(f"extern template int agb::launch_adjoint_v<GeneratedModel, {lu}, {lu}, {ck}>(")
            lines.append("    const agb::Batch&, const agb::Opts&, cudaStream_t);")
    lines += ["AMICI_GB300_DEFINE_ABI(GeneratedModel)", "AMICI_GB300_DEFINE_NOALLOC_ABI(GeneratedModel)", ""]
    units["abi.cu"] = "\n".join(lines)
    return units
