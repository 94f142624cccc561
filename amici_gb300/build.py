"""Compile a generated model into its engine library ``libamici_gb300_<model>.so``.

Each model library is built in-tree under ``amici_gb300/_build/<model>_<hash>/``
from the code generator's translation units, compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into one shared
object that exports the C ABI of ``include/amici_gb300.h``.  The hash covers
the generated sources and the engine headers, so a library is rebuilt exactly
when either changes.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

from .codegen import emit_engine_units
from .model_spec import ModelSpec

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
BUILD_ROOT = PKG / "_build"
ENGINE_SOURCES = sorted((PKG / "csrc").glob("*.cuh")) + [REPO / "include" / "amici_gb300.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{REPO}"]

_locks: dict[str, threading.Lock] = {}
_locks_guard = threading.Lock()


def _lock_for(key: Path) -> threading.Lock:
    with _locks_guard:
        return _locks.setdefault(str(key), threading.Lock())


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build model libraries")
    return exe


def _digest(units: dict[str, str]) -> str:
    h = hashlib.sha256()
    for name in sorted(units):
        h.update(name.encode())
        h.update(units[name].encode())
    for f in ENGINE_SOURCES:
        h.update(f.read_bytes())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()[:16]


def library_path(spec: ModelSpec) -> Path:
    units = emit_engine_units(spec)
    return BUILD_ROOT / f"{spec.name}_{_digest(units)}" / f"libamici_gb300_{spec.name}.so"


def build_model_library(spec: ModelSpec, *, jobs: int | None = None, verbose: bool = False) -> Path:
    """Generate, compile and link the engine library for ``spec``; returns its path."""
    units = emit_engine_units(spec)
    out_dir = BUILD_ROOT / f"{spec.name}_{_digest(units)}"
    so = out_dir / f"libamici_gb300_{spec.name}.so"
    with _lock_for(so):
        if so.exists():
            return so
        out_dir.mkdir(parents=True, exist_ok=True)
        for name, text in units.items():
            (out_dir / name).write_text(text)
        sources = sorted(n for n in units if n.endswith(".cu"))
        exe = nvcc()

        def compile_one(name):
            obj = out_dir / (name[:-3] + ".o")
            cmd = [exe, *ARCH, *NVCC_FLAGS, "-c", str(out_dir / name), "-o", str(obj)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr[-4000:]}")
            if verbose and r.stderr.strip():
                print(r.stderr)
            return obj

        jobs = jobs or max(1, min(len(sources), (os.cpu_count() or 2) // 2))
        with ThreadPoolExecutor(jobs) as ex:
            objs = list(ex.map(compile_one, sources))
        tmp = so.with_suffix(f".so.tmp{os.getpid()}")
        cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, so)
        return so


def build_probe_library() -> Path:
    """The FP64 throughput probe used for the benchmark's roofline denominator."""
    src = PKG / "csrc" / "probe.cu"
    h = hashlib.sha256(src.read_bytes() + " ".join(ARCH).encode()).hexdigest()[:16]
    out = BUILD_ROOT / f"probe_{h}" / "libamici_gb300_probe.so"
    with _lock_for(out):
        if out.exists():
            return out
        out.parent.mkdir(parents=True, exist_ok=True)
        tmp = out.with_suffix(f".so.tmp{os.getpid()}")
        cmd = [nvcc(), *ARCH, "-O3", "-Xcompiler", "-fPIC", "-shared", str(src), "-o", str(tmp)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for probe.cu:\n{r.stderr[-4000:]}")
        os.replace(tmp, out)
        return out
