"""GB300-native (sm_103a) per-step particle update of the self-propelled
particle simulator hamidallaei/SPP, behind the C ABI of include/spp.h."""
from . import abi, autotune, configs
from .abi import SppError, SppParams, SppObservables, new_params
from .system import Batch, Box, Snapshot, System

__all__ = ["abi", "autotune", "configs", "Batch", "Box", "Snapshot", "System", "SppError", "SppParams",
           "SppObservables", "new_params"]
