"""amici_gb300 — GB300-native batched stiff-ODE simulation engine.

A drop-in for AMICI's simulation path (``run_simulations(model, solver,
edata_list)`` with ReturnData fields x, y, sigmay, llh, sx, sy, sllh) whose
integration runs entirely in hand-written sm_103a CUDA kernels.
"""
from . import _native
from .autograd import LogLikelihood, log_likelihood_and_gradient
from .de_import import model_spec_from_de_model
from .model_spec import Event, ModelSpec, mass_action_model
from .objective import ConditionMapping, Objective
from .simulation import (AMICI_SUCCESS, ExpData, Model, ParameterScaling, ReturnDataView,
                         SensitivityMethod, SensitivityOrder, Solver, runAmiciSimulation,
                         runAmiciSimulations, run_simulation, run_simulations, simulate_batch,
                         simulation_status_to_str)

__all__ = [
    "Event", "ModelSpec", "mass_action_model", "Model", "Solver", "ExpData", "ReturnDataView",
    "SensitivityMethod", "SensitivityOrder", "ParameterScaling", "run_simulation",
    "run_simulations", "runAmiciSimulation", "runAmiciSimulations", "simulate_batch",
    "simulation_status_to_str", "AMICI_SUCCESS", "LogLikelihood", "log_likelihood_and_gradient",
    "ConditionMapping", "Objective", "model_spec_from_de_model",
]
