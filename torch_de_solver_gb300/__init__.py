"""GB300-native training hot path for TEDEouS-style physics-informed neural networks.

Drop-in names: Domain, Conditions, Equation (tedeous.data), Model (tedeous.model), Optimizer
(tedeous.optimizers.optimizer), Callback, Cache (tedeous.callbacks), parameter_registr
(tedeous.models), solver_device. The per-step loss, residual, boundary
terms and parameter gradient run in hand-written sm_103a CUDA kernels (libtdg.so, include/tdg.h).
"""
from .data import Conditions, Domain, Equation
from .device import check_device, device_type, solver_device
from .callbacks import Cache, CachePreprocessing, Callback, CallbackList
from .optimizer import FusedAdam, LBFGS64, Optimizer
from .solution import DevicePlan, Solution
from .model import BatchedModel, Model, parameter_registr

__all__ = ['Domain', 'Conditions', 'Equation', 'Model', 'BatchedModel', 'Optimizer', 'FusedAdam', 'LBFGS64', 'Solution',
           'DevicePlan', 'Callback', 'CallbackList', 'Cache', 'CachePreprocessing',
           'parameter_registr',
           'solver_device', 'check_device', 'device_type']
