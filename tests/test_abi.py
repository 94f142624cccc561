"""The C-ABI library: builds for sm_103a, loads, exports every declared symbol,
and its structs match the ctypes mirror (no GPU needed)."""
import re
import subprocess
from pathlib import Path

import pytest

from amici_gb300 import _native
from amici_gb300.build import build_model_library
from amici_gb300.networks import robertson_model

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "amici_gb300.h"


def _declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(amici_gb300_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    so = build_model_library(robertson_model())
    nm = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True,
                        check=True).stdout
    exported = set(re.findall(r"\bT (amici_gb300_\w+)", nm))
    declared = _declared()
    assert declared, "no declarations parsed"
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    assert set(_native.EXPORTED) <= exported


def test_library_loads_and_reports_dims():
    lib = _native.ModelLibrary(build_model_library(robertson_model()))
    assert lib.name == "robertson"
    d = lib.dims
    assert (d.nx, d.np, d.nk, d.ny, d.nw) == (3, 3, 0, 3, 3)
    o = lib.default_options()
    assert o.rtol == 1e-8 and o.atol == 1e-16 and o.maxsteps == 10000
    assert o.max_nonlin_iters == 3 and o.max_conv_fails == 10
    assert o.stldet == 1  # stability-limit detection on, as in the reference Solver


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(f'''#include <stdio.h>
#include <stddef.h>
#include "{HEADER}"
int main(void) {{
  printf("%zu %zu %zu\\n", sizeof(amici_gb300_solver_options), sizeof(amici_gb300_batch),
         sizeof(amici_gb300_model_dims));
  printf("%zu %zu %zu %zu\\n", offsetof(amici_gb300_batch, p), offsetof(amici_gb300_batch, status),
         offsetof(amici_gb300_solver_options, checkpoint_steps), offsetof(amici_gb300_solver_options, stldet));
  printf("%zu %zu %zu\\n", offsetof(amici_gb300_batch, posteq), offsetof(amici_gb300_batch, posteq_status),
         offsetof(amici_gb300_batch, posteq_wrms));
  return 0;
}}''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    import ctypes
    exp = [ctypes.sizeof(_native.SolverOptions), ctypes.sizeof(_native.Batch), ctypes.sizeof(_native.ModelDims),
           _native.Batch.p.offset, _native.Batch.status.offset, _native.SolverOptions.checkpoint_steps.offset,
           _native.SolverOptions.stldet.offset, _native.Batch.posteq.offset, _native.Batch.posteq_status.offset,
           _native.Batch.posteq_wrms.offset]
    assert list(map(int, out)) == exp
