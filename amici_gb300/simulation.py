"""AMICI-compatible simulation API on the GB300 engine.

Mirrors the reference's Python surface for the simulation path
(``python/sdist/amici/sim/sundials/_swig_wrappers.py:46-133``):
``run_simulation(model, solver, edata=None)``,
``run_simulations(model, solver, edata_list, failfast=True, num_threads=1)``
(alias ``runAmiciSimulations``), ``Model``/``Solver``/``ExpData`` with the
reference's snake_case setters, and ``ReturnDataView`` with the fields
``x, y, sigmay, llh, sx, sy, sllh, numsteps, status`` in the shapes of
``python/sdist/amici/sim/sundials/_numpy.py:414-440``.

All instances of a ``run_simulations`` call that share a time grid length are
integrated by one batched kernel launch; there is no CPU integration path:
without a usable GPU the calls raise.
"""
from __future__ import annotations

import enum
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native
from .build import build_model_library
from .model_spec import ModelSpec


class SensitivityOrder(enum.IntEnum):
    none = 0
    first = 1


class SensitivityMethod(enum.IntEnum):
    none = 0
    forward = 1
    adjoint = 2


class ParameterScaling(enum.IntEnum):
    none = 0
    ln = 1
    log10 = 2


# AMICI status codes (include/amici/defines.h:66-104)
AMICI_SUCCESS = 0
AMICI_TOO_MUCH_WORK = -1
AMICI_TOO_MUCH_ACC = -2
AMICI_ERR_FAILURE = -3
AMICI_CONV_FAILURE = -4
AMICI_ILL_INPUT = -22
AMICI_ERROR = -99
AMICI_NOT_RUN = -1001

_STATUS_NAMES = {0: "AMICI_SUCCESS", -1: "AMICI_TOO_MUCH_WORK", -2: "AMICI_TOO_MUCH_ACC",
                 -3: "AMICI_ERR_FAILURE", -4: "AMICI_CONV_FAILURE", -22: "AMICI_ILL_INPUT",
                 -99: "AMICI_ERROR", -1001: "AMICI_NOT_RUN"}


def simulation_status_to_str(status: int) -> str:
    """``amici::simulation_status_to_str`` (src/amici.cpp:30-63)."""
    return _STATUS_NAMES.get(int(status), f"AMICI_UNKNOWN({int(status)})")


def _require_gpu():
    try:
        import torch
    except ImportError as e:  # pragma: no cover
        raise RuntimeError("amici_gb300 needs PyTorch with CUDA for device management") from e
    if not torch.cuda.is_available():
        raise RuntimeError("amici_gb300: no CUDA device available; the engine has no CPU path")
    return torch


class Model:
    """A compiled model (``amici.Model`` counterpart).

    Holds the symbolic spec, the engine library and the model-level settings
    that ExpData may override: parameters, parameter scales, fixed parameters
    and timepoints.
    """

    def __init__(self, spec: ModelSpec, library=None):
        self.spec = spec
        self._lib = library
        self._p = np.array(spec.p_nominal, dtype=np.float64)  # unscaled values
        self._pscale = np.zeros(spec.np, dtype=np.int32)
        self._k = np.array(spec.k_nominal, dtype=np.float64)
        self._ts = np.zeros(0)
        self._plist = np.arange(spec.np, dtype=np.int32)

    # -- library ---------------------------------------------------------------
    @property
    def library(self) -> _native.ModelLibrary:
        if self._lib is None:
            self._lib = _native.ModelLibrary(build_model_library(self.spec))
        return self._lib

    # -- dimensions (amici::ModelDimensions) -----------------------------------
    @property
    def nx_rdata(self):
        return self.spec.nx

    nx_solver = nx_rdata

    @property
    def ny(self):
        return self.spec.ny

    def np(self):
        return self.spec.np

    def nk(self):
        return self.spec.nk

    def get_name(self):
        return self.spec.name

    def get_parameter_ids(self):
        return list(self.spec.parameter_ids)

    def get_state_ids(self):
        return list(self.spec.state_ids)

    def get_observable_ids(self):
        return list(self.spec.observable_ids)

    def get_fixed_parameter_ids(self):
        return list(self.spec.fixed_parameter_ids)

    # -- parameters (model.h set_parameters / set_parameter_scale) --------------
    def set_parameter_scale(self, scale):
        if np.ndim(scale) == 0:
            self._pscale[:] = int(scale)
        else:
            self._pscale = np.asarray(scale, dtype=np.int32).copy()

    def get_parameter_scale(self):
        return self._pscale.copy()

    def set_parameters(self, p_scaled):
        """Set parameters in their current scale."""
        p_scaled = np.asarray(p_scaled, dtype=np.float64)
        self._p = _unscale(p_scaled, self._pscale)

    def get_parameters(self):
        return _scale(self._p, self._pscale)

    def set_unscaled_parameters(self, p):
        self._p = np.asarray(p, dtype=np.float64).copy()

    def get_unscaled_parameters(self):
        return self._p.copy()

    def set_fixed_parameters(self, k):
        self._k = np.asarray(k, dtype=np.float64).copy()

    def get_fixed_parameters(self):
        return self._k.copy()

    def set_timepoints(self, ts):
        self._ts = np.asarray(ts, dtype=np.float64).copy()

    def get_timepoints(self):
        return self._ts.copy()

    def set_parameter_list(self, plist):
        self._plist = np.asarray(plist, dtype=np.int32).copy()

    def get_parameter_list(self):
        return self._plist.copy()

    def create_solver(self) -> "Solver":
        return Solver()


def _unscale(p, scale):
    p = np.asarray(p, dtype=np.float64)
    scale = np.broadcast_to(np.asarray(scale), p.shape)
    return np.where(scale == 1, np.exp(p), np.where(scale == 2, 10.0 ** p, p))


def _scale(p, scale):
    p = np.asarray(p, dtype=np.float64)
    scale = np.broadcast_to(np.asarray(scale), p.shape)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(scale == 1, np.log(p), np.where(scale == 2, np.log10(p), p))


class Solver:
    """Solver options (``amici::Solver`` setters, defaults of include/amici/solver.h)."""

    def __init__(self):
        self.rtol = 1e-8
        self.atol = 1e-16
        self.rtol_fsa = None
        self.atol_fsa = None
        self.rtol_b = None
        self.atol_b = None
        self.rtol_quad = 1e-8
        self.atol_quad = 1e-12
        self.maxsteps = 10000
        self.max_step_size = math.inf
        self.sensi = SensitivityOrder.none
        self.sensi_meth = SensitivityMethod.forward
        self.max_nonlin_iters = 3
        self.max_conv_fails = 10
        self.lu_precision = 32
        self.lanes_per_instance = 0
        self.checkpoint_steps = 50
        self.control_precision = 32
        self.launch_mode = 0
        self.instances_per_sm = 0
        self.stldet = True

    # reference setters/getters
    def set_relative_tolerance(self, v): self.rtol = float(v)
    def get_relative_tolerance(self): return self.rtol
    def set_absolute_tolerance(self, v): self.atol = float(v)
    def get_absolute_tolerance(self): return self.atol
    def set_relative_tolerance_fsa(self, v): self.rtol_fsa = float(v)
    def get_relative_tolerance_fsa(self): return self.rtol if self.rtol_fsa is None else self.rtol_fsa
    def set_absolute_tolerance_fsa(self, v): self.atol_fsa = float(v)
    def get_absolute_tolerance_fsa(self): return self.atol if self.atol_fsa is None else self.atol_fsa
    def set_relative_tolerance_b(self, v): self.rtol_b = float(v)
    def set_absolute_tolerance_b(self, v): self.atol_b = float(v)
    def set_relative_tolerance_quadratures(self, v): self.rtol_quad = float(v)
    def set_absolute_tolerance_quadratures(self, v): self.atol_quad = float(v)
    def set_max_steps(self, v): self.maxsteps = int(v)
    def get_max_steps(self): return self.maxsteps
    def set_max_step_size(self, v): self.max_step_size = float(v)
    def set_sensitivity_order(self, v): self.sensi = SensitivityOrder(int(v))
    def get_sensitivity_order(self): return self.sensi
    def set_sensitivity_method(self, v): self.sensi_meth = SensitivityMethod(int(v))
    def get_sensitivity_method(self): return self.sensi_meth
    def set_max_nonlin_iters(self, v): self.max_nonlin_iters = int(v)
    def set_max_conv_fails(self, v): self.max_conv_fails = int(v)
    def set_stability_limit_flag(self, v): self.stldet = bool(v)
    def get_stability_limit_flag(self): return self.stldet
    # GB300-specific knobs
    def set_lu_precision(self, bits): self.lu_precision = int(bits)
    def set_lanes_per_instance(self, g): self.lanes_per_instance = int(g)
    def set_checkpoint_steps(self, k): self.checkpoint_steps = int(k)
    def set_control_precision(self, bits): self.control_precision = int(bits)
    def set_launch_mode(self, mode): self.launch_mode = int(mode)
    # at most this many resident instances per SM (0: automatic); the on-chip
    # memory they leave serves as L1 cache
    def set_instances_per_sm(self, v): self.instances_per_sm = int(v)
    def get_instances_per_sm(self): return self.instances_per_sm

    def to_options(self) -> _native.SolverOptions:
        o = _native.SolverOptions()
        o.rtol, o.atol = self.rtol, self.atol
        o.rtol_fsa, o.atol_fsa = _native.nan_or(self.rtol_fsa), _native.nan_or(self.atol_fsa)
        o.rtol_b, o.atol_b = _native.nan_or(self.rtol_b), _native.nan_or(self.atol_b)
        o.rtol_quad, o.atol_quad = self.rtol_quad, self.atol_quad
        o.maxsteps = self.maxsteps
        o.max_step_size = self.max_step_size
        o.sensi_order = int(self.sensi)
        o.sensi_meth = int(self.sensi_meth)
        o.max_nonlin_iters = self.max_nonlin_iters
        o.max_conv_fails = self.max_conv_fails
        o.lu_precision = self.lu_precision
        o.lanes_per_instance = self.lanes_per_instance
        o.checkpoint_steps = self.checkpoint_steps
        o.control_precision = self.control_precision
        o.launch_mode = self.launch_mode
        o.instances_per_sm = self.instances_per_sm
        o.stldet = 1 if self.stldet else 0
        return o


@dataclass(slots=True)
class ExpData:
    """Per-condition data (``amici::ExpData``, include/amici/edata.h).

    ``fixed_parameters_pre_equilibration``: bring the instance to steady
    state at these fixed parameters before the simulation (the reference's
    default steady-state computation, simulation only); ``x0`` [nx] and
    ``sx0`` [nplist * nx, parameter-major, w.r.t. the scaled parameters]
    replace the model's initial states and their sensitivities
    (simulation_parameters.h:174,183).  Output times ``inf`` after the
    finite ones ask for post-equilibration (the model needs "posteq" among
    its families; forward simulation and forward sensitivities).  Pre-simulation
    (``fixed_parameters_presimulation``, ``t_presim``) and the
    reinitialisation of fixed-parameter-dependent initial states
    (``reinitialize_fixed_parameter_initial_states``) are not part of this
    engine: setting them makes the simulation call raise instead of ignoring
    them, and any other unknown attribute is refused on assignment."""

    ts: np.ndarray
    measurements: np.ndarray | None = None   # [nt, ny], NaN = missing
    noise_scales: np.ndarray | None = None   # [nt, ny], NaN = model value
    fixed_parameters: np.ndarray | None = None
    parameters: np.ndarray | None = None     # scaled by pscale (overrides the model's)
    pscale: np.ndarray | None = None
    plist: np.ndarray | None = None
    id: str = ""
    fixed_parameters_pre_equilibration: np.ndarray | None = None
    fixed_parameters_presimulation: np.ndarray | None = None
    t_presim: float = 0.0
    x0: np.ndarray | None = None
    sx0: np.ndarray | None = None
    reinitialize_fixed_parameter_initial_states: bool = False

    @classmethod
    def from_model(cls, model: Model, **kw):
        return cls(ts=model.get_timepoints(), **kw)

    def set_timepoints(self, ts): self.ts = np.asarray(ts, dtype=np.float64)
    def get_timepoints(self): return self.ts
    def set_measurements(self, m): self.measurements = np.asarray(m, dtype=np.float64)
    def get_measurements(self): return self.measurements
    def set_noise_scales(self, s): self.noise_scales = np.asarray(s, dtype=np.float64)
    def get_noise_scales(self): return self.noise_scales


@dataclass
class ReturnDataView:
    """Simulation results of one instance (``amici::ReturnData`` fields)."""

    ts: np.ndarray
    x: np.ndarray
    y: np.ndarray
    sigmay: np.ndarray
    llh: float
    numsteps: np.ndarray
    status: int
    sx: np.ndarray | None = None
    sy: np.ndarray | None = None
    sllh: np.ndarray | None = None
    messages: list = field(default_factory=list)
    # wall time (ms) of the batched call that produced this result; the
    # instances of a batch run concurrently, so it is not a per-instance time
    cpu_time: float = 0.0
    # solver counters over the whole run (the reference reports them per
    # output): steps, rhs_evals, newton_iters, linear_setups,
    # error_test_fails, conv_fails, jac_evals, backward_steps
    diagnostics: dict = field(default_factory=dict)
    # pre-equilibration (None without one): steady state [nx], its
    # sensitivities [nplist, nx] w.r.t. the scaled parameters, the status of
    # the simulation to steady state (1 success, -2 step budget exhausted or
    # too much work, -5 time overflow, -1 other failure; the reference's
    # preeq_status[1]), its steps, time and residual norm
    x_ss: np.ndarray | None = None
    sx_ss: np.ndarray | None = None
    preeq_status: int | None = None
    preeq_numsteps: int | None = None
    preeq_t: float | None = None
    preeq_wrms: float | None = None
    # post-equilibration (None without outputs at t = inf): status of the
    # simulation to steady state (the reference's posteq_status[1]), its
    # steps, time and residual norm
    posteq_status: int | None = None
    posteq_numsteps: int | None = None
    posteq_t: float | None = None
    posteq_wrms: float | None = None

    def __getitem__(self, key):
        return getattr(self, key)


DIAGNOSTIC_NAMES = ("steps", "rhs_evals", "newton_iters", "linear_setups", "error_test_fails", "conv_fails",
                    "jac_evals", "backward_steps")


def _check_supported(e: ExpData):
    v = e.fixed_parameters_presimulation
    if v is not None and np.size(v) > 0:
        raise NotImplementedError("ExpData.fixed_parameters_presimulation: pre-simulation is not part of this engine")
    if e.t_presim:
        raise NotImplementedError("ExpData.t_presim: pre-simulation is not part of this engine")
    ts = np.asarray(e.ts, dtype=np.float64)
    fin = ts[np.isfinite(ts)]
    if np.isinf(ts).any() and (np.isneginf(ts).any() or not np.isinf(ts[len(fin):]).all()):
        raise ValueError("ExpData.ts: outputs at t = inf (post-equilibration) must follow the finite ones")
    if e.reinitialize_fixed_parameter_initial_states:
        raise NotImplementedError("ExpData.reinitialize_fixed_parameter_initial_states: reinitialising initial "
                                  "states after pre-equilibration is not part of this engine")


def _given(v):
    return v is not None and np.size(v) > 0


def _stack_inputs(model: Model, edata_list):
    for e in edata_list:
        _check_supported(e)
    nt = len(edata_list[0].ts)
    n = len(edata_list)
    np_, nk, ny = model.spec.np, model.spec.nk, model.spec.ny
    p = np.empty((n, np_))
    k = np.empty((n, nk))
    ts = np.empty((n, nt))
    have_my = any(e.measurements is not None for e in edata_list)
    have_sg = any(e.noise_scales is not None for e in edata_list)
    my = np.full((n, nt, ny), np.nan) if have_my else None
    sg = np.full((n, nt, ny), np.nan) if have_sg else None
    # an ExpData's parameter scale overrides the model's; the model's
    # parameters are then taken on that scale (edata.h pscale)
    e0 = edata_list[0]
    pscale = model.get_parameter_scale() if e0.pscale is None else np.asarray(e0.pscale, dtype=np.int32)
    plist = e0.plist
    for i, e in enumerate(edata_list):
        ps = model.get_parameter_scale() if e.pscale is None else np.asarray(e.pscale, dtype=np.int32)
        if not np.array_equal(ps, pscale):
            raise ValueError("all ExpData of one batch must share the parameter scale")
        if (e.plist is None) != (plist is None) or (plist is not None and not np.array_equal(e.plist, plist)):
            raise ValueError("all ExpData of one batch must share the parameter list")
        p[i] = _scale(model.get_unscaled_parameters(), pscale) if e.parameters is None else e.parameters
        k[i] = model.get_fixed_parameters() if e.fixed_parameters is None else e.fixed_parameters
        ts[i] = e.ts
        if have_my and e.measurements is not None:
            my[i] = np.asarray(e.measurements).reshape(nt, ny)
        if have_sg and e.noise_scales is not None:
            sg[i] = np.asarray(e.noise_scales).reshape(nt, ny)
    plist = None if plist is None else np.asarray(plist, dtype=np.int32)
    # pre-equilibration and initial-state overrides: given for all or none of a batch
    extra = {"k_preeq": None, "x0": None, "sx0": None}
    npl = len(plist) if plist is not None else len(model.get_parameter_list())
    for name, shape in (("k_preeq", (nk,)), ("x0", (model.spec.nx,)), ("sx0", (npl, model.spec.nx))):
        attr = "fixed_parameters_pre_equilibration" if name == "k_preeq" else name
        vals = [getattr(e, attr) for e in edata_list]
        given = [_given(v) for v in vals]
        if any(given) and not all(given):
            raise ValueError(f"all ExpData of one batch must give ExpData.{attr}, or none")
        if all(given):
            extra[name] = np.stack([np.asarray(v, dtype=np.float64).reshape(shape) for v in vals])
        elif name == "k_preeq" and nk == 0 and any(v is not None for v in vals):
            extra[name] = np.zeros((n, 0))  # a pre-equilibration of a model without fixed parameters
    return p, pscale, k, ts, my, sg, plist, extra


def simulate_batch(model: Model, solver: Solver, p, k, ts, my=None, sigma=None, *, pscale=None,
                   plist=None, stream: int = 0, k_preeq=None, x0=None, sx0=None):
    """Integrate a batch given as host arrays ([N, ...], row-major); returns a
    dict of ReturnData-shaped arrays.  Goes through the host-buffer C entry
    point (copies in, one kernel launch, copies out).  With the solver's
    sensitivity order first and method forward, also sx [N, nt, nplist, nx],
    sy [N, nt, nplist, ny] and sllh [N, nplist] for the parameters ``plist``
    (default: the model's parameter list); with method adjoint, sllh from
    the backward problem (``diag[:, 7]`` counts its steps).  ``k_preeq``
    [N, nk]: pre-equilibrate every instance at these fixed parameters first
    (adds x_ss, sx_ss, preeq_status, preeq_numsteps, preeq_t, preeq_wrms);
    ``x0`` [N, nx] / ``sx0`` [N, nplist, nx] (scaled parameters): given
    initial states and sensitivities.  Output times ``inf`` after the finite
    ones are post-equilibration outputs (adds posteq_status,
    posteq_numsteps, posteq_t, posteq_wrms; the model needs "posteq" in its
    families)."""
    _require_gpu()
    spec = model.spec
    lib = model.library
    p = np.ascontiguousarray(np.atleast_2d(p), dtype=np.float64)
    n = p.shape[0]
    ts = np.ascontiguousarray(np.broadcast_to(ts, (n, np.shape(ts)[-1])), dtype=np.float64)
    nt = ts.shape[1]
    k = np.ascontiguousarray(np.broadcast_to(k, (n, spec.nk)) if spec.nk else np.zeros((n, 0)))
    pscale = np.ascontiguousarray(model.get_parameter_scale() if pscale is None else pscale,
                                  dtype=np.int32)
    if my is not None:
        my = np.ascontiguousarray(np.broadcast_to(my, (n, nt, spec.ny)), dtype=np.float64)
    if sigma is not None:
        sigma = np.ascontiguousarray(np.broadcast_to(sigma, (n, nt, spec.ny)), dtype=np.float64)
    fsa = int(solver.sensi) > 0 and solver.sensi_meth == SensitivityMethod.forward
    asa = int(solver.sensi) > 0 and solver.sensi_meth == SensitivityMethod.adjoint
    sensi = fsa or asa
    if sensi:
        plist = np.ascontiguousarray(model.get_parameter_list() if plist is None else plist,
                                     dtype=np.int32)
    npl = len(plist) if sensi else 0
    out = dict(x=np.empty((n, nt, spec.nx)), y=np.empty((n, nt, spec.ny)),
               sigmay=np.empty((n, nt, spec.ny)), llh=np.empty(n),
               numsteps=np.empty((n, nt), np.int32), status=np.empty(n, np.int32),
               diag=np.empty((n, 8), np.int32))
    if fsa:
        out["sx"] = np.empty((n, nt, npl, spec.nx))
        out["sy"] = np.empty((n, nt, npl, spec.ny))
    if sensi:
        out["sllh"] = np.empty((n, npl))
    b = _native.Batch()
    b.n_instances, b.nt, b.nplist = n, nt, npl
    A = _native.addr
    b.p, b.pscale, b.k, b.ts = A(p), A(pscale), A(k), A(ts)
    b.my, b.sigma_y, b.plist = A(my), A(sigma), A(plist) if sensi else None
    b.x, b.y, b.sigmay, b.llh = A(out["x"]), A(out["y"]), A(out["sigmay"]), A(out["llh"])
    b.sx, b.sy = (A(out["sx"]), A(out["sy"])) if fsa else (None, None)
    b.sllh = A(out["sllh"]) if sensi else None
    b.numsteps, b.status, b.diag = A(out["numsteps"]), A(out["status"]), A(out["diag"])
    keep = []
    if k_preeq is not None:
        k_preeq = np.ascontiguousarray(np.broadcast_to(k_preeq, (n, spec.nk)), dtype=np.float64)
        out.update(x_ss=np.empty((n, spec.nx)), preeq_status=np.empty(n, np.int32),
                   preeq_numsteps=np.empty(n, np.int32), preeq_t=np.empty(n), preeq_wrms=np.empty(n))
        out["sx_ss"] = np.empty((n, npl, spec.nx)) if sensi else None
        b.k_preeq = A(k_preeq) if spec.nk else A(np.zeros(1))
        keep.append(k_preeq)
        b.x_ss, b.sx_ss = A(out["x_ss"]), A(out["sx_ss"]) if sensi else None
        b.preeq_status, b.preeq_numsteps = A(out["preeq_status"]), A(out["preeq_numsteps"])
        b.preeq_t, b.preeq_wrms = A(out["preeq_t"]), A(out["preeq_wrms"])
    if np.isinf(ts).any():
        out.update(posteq_status=np.empty(n, np.int32), posteq_numsteps=np.empty(n, np.int32),
                   posteq_t=np.empty(n), posteq_wrms=np.empty(n))
        b.posteq = 1
        b.posteq_status, b.posteq_numsteps = A(out["posteq_status"]), A(out["posteq_numsteps"])
        b.posteq_t, b.posteq_wrms = A(out["posteq_t"]), A(out["posteq_wrms"])
    if x0 is not None:
        x0 = np.ascontiguousarray(np.broadcast_to(x0, (n, spec.nx)), dtype=np.float64)
        keep.append(x0)
        b.x0 = A(x0)
    if sx0 is not None and sensi:
        sx0 = np.ascontiguousarray(np.broadcast_to(sx0, (n, npl, spec.nx)), dtype=np.float64)
        keep.append(sx0)
        b.sx0 = A(sx0)
    lib.run_host(solver.to_options(), b, stream)
    if not fsa:
        out["sx"] = out["sy"] = None
    if not sensi:
        out["sllh"] = None
    return out


def _not_run(model: Model, solver: Solver, ts, npl: int | None) -> ReturnDataView:
    """The empty ReturnData the reference returns for an instance that
    ``failfast`` skipped (``ReturnData(solver, model)``, src/rdata.cpp:104-200):
    status AMICI_NOT_RUN, llh and sllh NaN, every other array zero."""
    spec = model.spec
    nt = len(ts)
    fsa = int(solver.sensi) > 0 and solver.sensi_meth == SensitivityMethod.forward
    return ReturnDataView(
        ts=np.asarray(ts, dtype=np.float64), x=np.zeros((nt, spec.nx)), y=np.zeros((nt, spec.ny)),
        sigmay=np.zeros((nt, spec.ny)), llh=float("nan"), numsteps=np.zeros(nt, np.int32),
        status=AMICI_NOT_RUN, sx=np.zeros((nt, npl, spec.nx)) if fsa else None,
        sy=np.zeros((nt, npl, spec.ny)) if fsa else None,
        sllh=np.full(npl, np.nan) if npl is not None else None,
        messages=["skipped: an earlier simulation of this call failed (failfast)"],
        diagnostics=dict.fromkeys(DIAGNOSTIC_NAMES, 0))


def run_simulations(model: Model, solver: Solver, edata_list, failfast: bool = True,
                    num_threads: int = 1):
    """Simulate every ExpData (``amici::run_simulations``, src/amici.cpp:220-264).

    All instances run concurrently on the GPU (``num_threads`` is accepted
    for signature compatibility).  ``failfast``: as in the reference with one
    thread, every ExpData after the first failed one (status < 0, in list
    order) gets the empty result of a skipped instance, status AMICI_NOT_RUN
    (src/amici.cpp:245-260).  Returns one ReturnDataView per ExpData.
    """
    edata_list = list(edata_list)
    if not edata_list:
        return []
    # one batch per output grid length, parameter list, parameter scale and
    # use of pre-equilibration and initial-state overrides
    groups: dict[tuple, list[int]] = {}
    for i, e in enumerate(edata_list):
        key = (len(e.ts), None if e.plist is None else tuple(int(v) for v in e.plist),
               None if e.pscale is None else tuple(int(v) for v in e.pscale),
               e.fixed_parameters_pre_equilibration is not None, _given(e.x0), _given(e.sx0))
        groups.setdefault(key, []).append(i)
    results = [None] * len(edata_list)
    for idx in groups.values():
        sub = [edata_list[i] for i in idx]
        p, pscale, k, ts, my, sg, plist, extra = _stack_inputs(model, sub)
        t0 = time.perf_counter()
        out = simulate_batch(model, solver, p, k, ts, my, sg, pscale=pscale, plist=plist, **extra)
        wall_ms = (time.perf_counter() - t0) * 1e3
        pre = extra["k_preeq"] is not None
        post = "posteq_status" in out
        for j, i in enumerate(idx):
            results[i] = ReturnDataView(
                ts=ts[j], x=out["x"][j], y=out["y"][j], sigmay=out["sigmay"][j],
                llh=float(out["llh"][j]), numsteps=out["numsteps"][j], status=int(out["status"][j]),
                sx=None if out["sx"] is None else out["sx"][j],
                sy=None if out["sy"] is None else out["sy"][j],
                sllh=None if out["sllh"] is None else out["sllh"][j], cpu_time=wall_ms,
                diagnostics=dict(zip(DIAGNOSTIC_NAMES, (int(v) for v in out["diag"][j]))),
                x_ss=out["x_ss"][j] if pre else None,
                sx_ss=out["sx_ss"][j] if pre and out.get("sx_ss") is not None else None,
                preeq_status=int(out["preeq_status"][j]) if pre else None,
                preeq_numsteps=int(out["preeq_numsteps"][j]) if pre else None,
                preeq_t=float(out["preeq_t"][j]) if pre else None,
                preeq_wrms=float(out["preeq_wrms"][j]) if pre else None,
                posteq_status=int(out["posteq_status"][j]) if post else None,
                posteq_numsteps=int(out["posteq_numsteps"][j]) if post else None,
                posteq_t=float(out["posteq_t"][j]) if post else None,
                posteq_wrms=float(out["posteq_wrms"][j]) if post else None)
    if failfast:
        failed = [i for i, r in enumerate(results) if r.status < 0]
        if failed:
            for i in range(failed[0] + 1, len(results)):
                r = results[i]
                npl = None if r.sllh is None else len(r.sllh)
                results[i] = _not_run(model, solver, r.ts, npl)
    return results


def run_simulation(model: Model, solver: Solver, edata: ExpData | None = None) -> ReturnDataView:
    """``amici::run_simulation`` (src/amici.cpp:65-218) for one condition."""
    if edata is None:
        edata = ExpData(ts=model.get_timepoints())
    return run_simulations(model, solver, [edata])[0]


runAmiciSimulations = run_simulations
runAmiciSimulation = run_simulation
