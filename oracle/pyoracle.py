"""Python front-end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Builds ``oracle/bdf_oracle.c`` together with the model's generated C (from
``amici_gb300.codegen.emit_oracle_c``) into a shared library under
``oracle/_build/`` and runs it through ctypes.  Only the tests, the smoke
check and the CPU-baseline leg of the benchmark import this module.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)


class OracleOptions(ctypes.Structure):
    _fields_ = [("rtol", ctypes.c_double), ("atol", ctypes.c_double),
                ("rtol_fsa", ctypes.c_double), ("atol_fsa", ctypes.c_double),
                ("maxsteps", ctypes.c_int64), ("sensi", ctypes.c_int32),
                ("max_nonlin_iters", ctypes.c_int32), ("max_conv_fails", ctypes.c_int32),
                ("lu_f32", ctypes.c_int32), ("max_step_size", ctypes.c_double),
                ("stldet", ctypes.c_int32), ("rtol_b", ctypes.c_double), ("atol_b", ctypes.c_double),
                ("rtol_quad", ctypes.c_double), ("atol_quad", ctypes.c_double),
                ("maxsteps_b", ctypes.c_int64)]


class OracleBatchExt(ctypes.Structure):
    _fields_ = [("k_preeq", _dp), ("x0", _dp), ("sx0", _dp), ("x_ss", _dp), ("sx_ss", _dp),
                ("preeq_status", _ip), ("preeq_numsteps", _ip), ("preeq_t", _dp), ("preeq_wrms", _dp),
                ("posteq_status", _ip), ("posteq_numsteps", _ip), ("posteq_t", _dp), ("posteq_wrms", _dp)]


def _ptr(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


def _ext(spec, n, npl, k_preeq, x0, sx0, out, posteq=False):
    """The batch extras (pre-equilibration, initial-state overrides,
    post-equilibration outputs) and their outputs, added to ``out``; None
    when none is given."""
    if k_preeq is None and x0 is None and sx0 is None and not posteq:
        return None
    keep = []

    def arr(a, shape):
        a = np.ascontiguousarray(np.broadcast_to(a, shape), dtype=np.float64)
        keep.append(a)
        return a
    e = OracleBatchExt()
    if k_preeq is not None:
        e.k_preeq = _ptr(arr(k_preeq, (n, spec.nk)) if spec.nk else arr(np.zeros((n, 1)), (n, 1)))
        out.update(x_ss=np.full((n, spec.nx), np.nan), sx_ss=np.full((n, npl, spec.nx), np.nan),
                   preeq_status=np.zeros(n, np.int32), preeq_numsteps=np.zeros(n, np.int32),
                   preeq_t=np.full(n, np.nan), preeq_wrms=np.full(n, np.nan))
        e.x_ss, e.sx_ss = _ptr(out["x_ss"]), _ptr(out["sx_ss"])
        e.preeq_status, e.preeq_numsteps = _ptr(out["preeq_status"], _ip), _ptr(out["preeq_numsteps"], _ip)
        e.preeq_t, e.preeq_wrms = _ptr(out["preeq_t"]), _ptr(out["preeq_wrms"])
    if posteq:
        out.update(posteq_status=np.zeros(n, np.int32), posteq_numsteps=np.zeros(n, np.int32),
                   posteq_t=np.full(n, np.nan), posteq_wrms=np.full(n, np.nan))
        e.posteq_status, e.posteq_numsteps = _ptr(out["posteq_status"], _ip), _ptr(out["posteq_numsteps"], _ip)
        e.posteq_t, e.posteq_wrms = _ptr(out["posteq_t"]), _ptr(out["posteq_wrms"])
    if x0 is not None:
        e.x0 = _ptr(arr(x0, (n, spec.nx)))
    if sx0 is not None:
        e.sx0 = _ptr(arr(sx0, (n, npl, spec.nx)))
    e._keep = keep
    return e


REF_ROOT = Path(os.environ.get("AMICI_GB300_REFERENCE", "/root/reference"))
REF_DIR = HERE / "_ref"


def reference_available() -> bool:
    """True if the reference CVODES can be (or was) built here."""
    return (REF_DIR / "libcvodes_ref.a").exists() or (REF_ROOT / "ThirdParty" / "sundials").is_dir()


def build_reference_lib() -> Path:
    lib = REF_DIR / "libcvodes_ref.a"
    if not lib.exists():
        subprocess.run(["make", "-s", "-j8", "-f", str(HERE / "Makefile.ref"), f"REF={REF_ROOT}"],
                       check=True)
    return lib


def build_oracle(spec, *, ref=False, force=False) -> Path:
    """Compile the oracle for ``spec`` (``ref=True``: the glue over the
    reference's own CVODES); returns the shared-library path."""
    from amici_gb300.codegen import emit_oracle_c, spec_digest

    out_dir = REF_DIR if ref else BUILD
    out_dir.mkdir(exist_ok=True)
    # the key covers the oracle sources and the generated model code
    c_text = emit_oracle_c(spec)
    src_hash = hashlib.sha256(b"".join(f.read_bytes() for f in sorted(HERE.glob("*.[ch]"))) +
                              c_text.encode()).hexdigest()[:8]
    tag = f"{spec.name}_{spec_digest(spec)}_{src_hash}"
    so = out_dir / (f"ref_{tag}.so" if ref else f"oracle_{tag}.so")
    if so.exists() and not force:
        return so
    src = out_dir / f"model_{tag}.c"
    src.write_text(c_text)
    tmp = so.with_suffix(f".so.tmp{os.getpid()}")
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11",
           "-D_DEFAULT_SOURCE", f"-I{HERE}", str(HERE / "amici_glue.c"), str(src)]
    if ref:
        lib = build_reference_lib()
        sun = REF_ROOT / "ThirdParty" / "sundials"
        cmd += [f"-I{sun / 'include' / 'sundials' / 'amici_matlab'}", f"-I{sun / 'include'}",
                f"-I{sun / 'src' / 'cvodes'}", f"-I{sun / 'src' / 'sundials'}",
                str(HERE / "ref_cvodes_driver.c"), str(lib)]
    else:
        cmd += [str(HERE / "bdf_oracle.c")]
    cmd += ["-lm", "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, so)
    return so


class Oracle:
    """ctypes binding of one compiled oracle library."""

    def __init__(self, spec, *, ref=False):
        self.spec = spec
        self.lib = ctypes.CDLL(str(build_oracle(spec, ref=ref)))
        f = self.lib.oracle_run_simulations_ext
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.POINTER(OracleOptions), ctypes.c_int, _dp, _ip, _dp,
                      ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _ip, _dp, _dp, _dp, _dp, _dp, _dp,
                      _dp, _ip, _ip, ctypes.POINTER(OracleBatchExt), ctypes.c_int]
        self.lib.oracle_get_model.restype = ctypes.c_void_p
        g = self.lib.oracle_run_simulations_asa_ext
        g.restype = ctypes.c_int
        g.argtypes = [ctypes.c_void_p, ctypes.POINTER(OracleOptions), ctypes.c_int, _dp, _ip, _dp,
                      ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _ip, _dp, _dp, _dp, _dp, _dp, _ip,
                      _ip, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(OracleBatchExt), ctypes.c_int]

    def run(self, p, pscale, k, ts, my=None, sigma=None, *, rtol=1e-8, atol=1e-16,
            sensi=0, plist=None, maxsteps=10000, lu_f32=False, nthreads=1,
            rtol_fsa=float("nan"), atol_fsa=float("nan"), stldet=True, k_preeq=None, x0=None, sx0=None):
        """Simulate a batch; arrays are [N, ...] numpy arrays.  Returns a dict
        with ReturnData-shaped outputs (x, y, sigmay, llh, sx, sy, sllh,
        numsteps, status).  ``stldet`` is CVODES' stability-limit detection,
        on by default as in the reference Solver (solver.h:2037).
        ``k_preeq`` [N, nk]: pre-equilibrate to steady state with these fixed
        parameters first (adds x_ss, sx_ss, preeq_status, preeq_numsteps,
        preeq_t, preeq_wrms); ``x0`` [N, nx] / ``sx0`` [N, nplist, nx]
        (w.r.t. the scaled parameters): ExpData initial-state overrides.
        Output times ``inf`` (after the finite ones) are post-equilibration
        outputs (adds posteq_status, posteq_numsteps, posteq_t,
        posteq_wrms)."""
        s = self.spec
        p = np.ascontiguousarray(np.atleast_2d(p), dtype=np.float64)
        n = p.shape[0]
        ts = np.ascontiguousarray(np.broadcast_to(ts, (n, np.shape(ts)[-1])), dtype=np.float64)
        nt = ts.shape[1]
        k = np.ascontiguousarray(np.broadcast_to(k, (n, s.nk)) if s.nk else np.zeros((n, 0)),
                                 dtype=np.float64)
        pscale = np.ascontiguousarray(pscale, dtype=np.int32)
        if plist is None:
            plist = np.arange(s.np, dtype=np.int32)
        plist = np.ascontiguousarray(plist, dtype=np.int32)
        nplist = len(plist) if sensi else 0
        if my is not None:
            my = np.ascontiguousarray(np.broadcast_to(my, (n, nt, s.ny)), dtype=np.float64)
        if sigma is not None:
            sigma = np.ascontiguousarray(np.broadcast_to(sigma, (n, nt, s.ny)), dtype=np.float64)
        out = dict(
            x=np.empty((n, nt, s.nx)), y=np.empty((n, nt, s.ny)), sigmay=np.empty((n, nt, s.ny)),
            llh=np.empty(n), sx=np.empty((n, nt, max(nplist, 0), s.nx)),
            sy=np.empty((n, nt, max(nplist, 0), s.ny)), sllh=np.empty((n, max(nplist, 0))),
            numsteps=np.empty((n, nt), np.int32), status=np.empty(n, np.int32))
        o = OracleOptions(rtol, atol, rtol_fsa, atol_fsa, maxsteps, 1 if sensi else 0, 3, 10,
                          1 if lu_f32 else 0, float("inf"), 1 if stldet else 0,
                          float("nan"), float("nan"), float("nan"), float("nan"), 0)
        posteq = bool(np.isinf(ts).any())
        if posteq and s.ne:
            raise NotImplementedError("post-equilibration of a model with events is not built")
        ext = _ext(s, n, nplist, k_preeq, x0, sx0, out, posteq)
        self.lib.oracle_run_simulations_ext(
            self.lib.oracle_get_model(), ctypes.byref(o), n, _ptr(p), _ptr(pscale, _ip), _ptr(k),
            nt, _ptr(ts), _ptr(my), _ptr(sigma), nplist, _ptr(plist, _ip), _ptr(out["x"]),
            _ptr(out["y"]), _ptr(out["sigmay"]), _ptr(out["llh"]), _ptr(out["sx"]),
            _ptr(out["sy"]), _ptr(out["sllh"]), _ptr(out["numsteps"], _ip),
            _ptr(out["status"], _ip), None if ext is None else ctypes.byref(ext), nthreads)
        if not sensi:
            out["sx"] = out["sy"] = out["sllh"] = None
        return out

    def run_asa(self, p, pscale, k, ts, my, sigma=None, *, rtol=1e-8, atol=1e-16, plist=None,
                maxsteps=10000, nthreads=1, rtol_b=float("nan"), atol_b=float("nan"),
                rtol_quad=1e-8, atol_quad=1e-12, maxsteps_b=0, stldet=True, k_preeq=None, x0=None,
                sx0=None):
        """Adjoint sensitivities (AMICI's backward problem with quadratures);
        returns a dict with x, y, sigmay, llh, sllh, numsteps, status and
        nst_b (backward steps).  The quadrature tolerances default to the
        reference Solver's (solver.h:2075-2078); NaN inherits rtol/atol.
        ``k_preeq``, ``x0``, ``sx0``: as in ``run`` (the pre-equilibration
        runs with forward sensitivities, whose sx_ss enter the gradient)."""
        s = self.spec
        p = np.ascontiguousarray(np.atleast_2d(p), dtype=np.float64)
        n = p.shape[0]
        ts = np.ascontiguousarray(np.broadcast_to(ts, (n, np.shape(ts)[-1])), dtype=np.float64)
        nt = ts.shape[1]
        k = np.ascontiguousarray(np.broadcast_to(k, (n, s.nk)) if s.nk else np.zeros((n, 0)),
                                 dtype=np.float64)
        pscale = np.ascontiguousarray(pscale, dtype=np.int32)
        plist = np.ascontiguousarray(np.arange(s.np) if plist is None else plist, dtype=np.int32)
        npl = len(plist)
        my = np.ascontiguousarray(np.broadcast_to(my, (n, nt, s.ny)), dtype=np.float64)
        if sigma is not None:
            sigma = np.ascontiguousarray(np.broadcast_to(sigma, (n, nt, s.ny)), dtype=np.float64)
        out = dict(x=np.empty((n, nt, s.nx)), y=np.empty((n, nt, s.ny)),
                   sigmay=np.empty((n, nt, s.ny)), llh=np.empty(n), sllh=np.empty((n, npl)),
                   numsteps=np.empty((n, nt), np.int32), status=np.empty(n, np.int32),
                   nst_b=np.zeros(n, np.int64))
        o = OracleOptions(rtol, atol, float("nan"), float("nan"), maxsteps, 2, 3, 10, 0,
                          float("inf"), 1 if stldet else 0, rtol_b, atol_b, rtol_quad, atol_quad,
                          maxsteps_b)
        if np.isinf(ts).any():
            raise NotImplementedError("adjoint sensitivities with post-equilibration are not built")
        ext = _ext(s, n, npl, k_preeq, x0, sx0, out)
        self.lib.oracle_run_simulations_asa_ext(
            self.lib.oracle_get_model(), ctypes.byref(o), n, _ptr(p), _ptr(pscale, _ip), _ptr(k),
            nt, _ptr(ts), _ptr(my), _ptr(sigma), npl, _ptr(plist, _ip), _ptr(out["x"]),
            _ptr(out["y"]), _ptr(out["sigmay"]), _ptr(out["llh"]), _ptr(out["sllh"]),
            _ptr(out["numsteps"], _ip), _ptr(out["status"], _ip),
            out["nst_b"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            None if ext is None else ctypes.byref(ext), nthreads)
        return out
