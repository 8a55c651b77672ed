"""GB300-native DYNAMITE hot path: 2D-interpolation renormalisation, memory-kernel
convolutions, EOM right-hand side with r(t), adaptive RK stages and sparsify,
as hand-written sm_103a CUDA kernels behind the C ABI of include/dyn.h."""
from . import checkpoint, grid
from ._lib import DynError, lib
from .batch import Batch, Quench, mixed_length_quenches
from .grid import Grid
from .simulation import METHODS, Model, Simulation, State, StepResult, serk2_method

__all__ = ["Batch", "Grid", "Model", "Quench", "Simulation", "State", "StepResult", "DynError", "METHODS",
           "checkpoint", "mixed_length_quenches", "grid", "lib", "serk2_method"]
