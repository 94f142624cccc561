"""ctypes binding of one model's engine library (``include/amici_gb300.h``)."""
from __future__ import annotations

import ctypes
import math
from pathlib import Path

import numpy as np

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)

ABI_VERSION = 3


class ModelDims(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("np", ctypes.c_int32), ("nk", ctypes.c_int32),
                ("ny", ctypes.c_int32), ("nw", ctypes.c_int32), ("nnz_jac", ctypes.c_int32)]


class SolverOptions(ctypes.Structure):
    _fields_ = [("rtol", ctypes.c_double), ("atol", ctypes.c_double),
                ("rtol_fsa", ctypes.c_double), ("atol_fsa", ctypes.c_double),
                ("rtol_b", ctypes.c_double), ("atol_b", ctypes.c_double),
                ("rtol_quad", ctypes.c_double), ("atol_quad", ctypes.c_double),
                ("maxsteps", ctypes.c_int64), ("max_step_size", ctypes.c_double),
                ("sensi_order", ctypes.c_int32), ("sensi_meth", ctypes.c_int32),
                ("max_nonlin_iters", ctypes.c_int32), ("max_conv_fails", ctypes.c_int32),
                ("lu_precision", ctypes.c_int32), ("lanes_per_instance", ctypes.c_int32),
                ("checkpoint_steps", ctypes.c_int32), ("control_precision", ctypes.c_int32),
                ("launch_mode", ctypes.c_int32), ("instances_per_sm", ctypes.c_int32),
                ("stldet", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Batch(ctypes.Structure):
    _fields_ = [("n_instances", ctypes.c_int32), ("nt", ctypes.c_int32),
                ("nplist", ctypes.c_int32), ("posteq", ctypes.c_int32),
                ("p", ctypes.c_void_p), ("pscale", ctypes.c_void_p), ("k", ctypes.c_void_p),
                ("ts", ctypes.c_void_p), ("my", ctypes.c_void_p), ("sigma_y", ctypes.c_void_p),
                ("plist", ctypes.c_void_p), ("x", ctypes.c_void_p), ("y", ctypes.c_void_p),
                ("sigmay", ctypes.c_void_p), ("llh", ctypes.c_void_p), ("sx", ctypes.c_void_p),
                ("sy", ctypes.c_void_p), ("sllh", ctypes.c_void_p), ("numsteps", ctypes.c_void_p),
                ("status", ctypes.c_void_p), ("diag", ctypes.c_void_p),
                ("k_preeq", ctypes.c_void_p), ("x0", ctypes.c_void_p), ("sx0", ctypes.c_void_p),
                ("x_ss", ctypes.c_void_p), ("sx_ss", ctypes.c_void_p), ("preeq_status", ctypes.c_void_p),
                ("preeq_numsteps", ctypes.c_void_p), ("preeq_t", ctypes.c_void_p),
                ("preeq_wrms", ctypes.c_void_p), ("posteq_status", ctypes.c_void_p),
                ("posteq_numsteps", ctypes.c_void_p), ("posteq_t", ctypes.c_void_p),
                ("posteq_wrms", ctypes.c_void_p)]


EXPORTED = ("amici_gb300_abi_version", "amici_gb300_model_name", "amici_gb300_model_dims_get",
            "amici_gb300_default_options", "amici_gb300_run_simulations_device",
            "amici_gb300_run_simulations_host", "amici_gb300_last_error",
            "amici_gb300_run_simulations_device_noalloc")


class EngineError(RuntimeError):
    pass


class ModelLibrary:
    """A loaded ``libamici_gb300_<model>.so``."""

    def __init__(self, path: str | Path):
        self.path = Path(path)
        self.lib = ctypes.CDLL(str(self.path))
        L = self.lib
        L.amici_gb300_abi_version.restype = ctypes.c_int32
        L.amici_gb300_model_name.restype = ctypes.c_char_p
        L.amici_gb300_model_dims_get.argtypes = [ctypes.POINTER(ModelDims)]
        L.amici_gb300_model_dims_get.restype = ctypes.c_int32
        L.amici_gb300_default_options.argtypes = [ctypes.POINTER(SolverOptions)]
        L.amici_gb300_default_options.restype = None
        for fn in ("amici_gb300_run_simulations_device", "amici_gb300_run_simulations_host",
                   "amici_gb300_run_simulations_device_noalloc"):
            f = getattr(L, fn)
            f.argtypes = [ctypes.POINTER(SolverOptions), ctypes.POINTER(Batch), ctypes.c_void_p]
            f.restype = ctypes.c_int32
        L.amici_gb300_last_error.restype = ctypes.c_char_p
        if L.amici_gb300_abi_version() != ABI_VERSION:
            raise EngineError(f"{self.path}: ABI version mismatch")
        d = ModelDims()
        L.amici_gb300_model_dims_get(ctypes.byref(d))
        self.dims = d
        self.name = L.amici_gb300_model_name().decode()

    def default_options(self) -> SolverOptions:
        o = SolverOptions()
        self.lib.amici_gb300_default_options(ctypes.byref(o))
        return o

    def check(self, rc: int, what: str):
        if rc != 0:
            msg = self.lib.amici_gb300_last_error().decode()
            raise EngineError(f"{what} failed (code {rc}): {msg}")

    def run_host(self, opts: SolverOptions, batch: Batch, stream: int = 0):
        self.check(self.lib.amici_gb300_run_simulations_host(ctypes.byref(opts), ctypes.byref(batch),
                                                             ctypes.c_void_p(stream)),
                   "amici_gb300_run_simulations_host")

    def run_device(self, opts: SolverOptions, batch: Batch, stream: int = 0):
        self.check(self.lib.amici_gb300_run_simulations_device(ctypes.byref(opts), ctypes.byref(batch),
                                                               ctypes.c_void_p(stream)),
                   "amici_gb300_run_simulations_device")


    def run_device_noalloc(self, opts: SolverOptions, batch: Batch, stream: int = 0):
        """The allocation-free device entry point (see include/amici_gb300.h)."""
        self.check(self.lib.amici_gb300_run_simulations_device_noalloc(
            ctypes.byref(opts), ctypes.byref(batch), ctypes.c_void_p(stream)),
            "amici_gb300_run_simulations_device_noalloc")


def nan_or(v):
    return float("nan") if v is None else float(v)


def addr(a) -> int | None:
    """Address of a numpy array or torch tensor (None stays None)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()
