"""binary2d — GB300 implementation of binary2d's finite-volume RK step.

Host mirror of the reference's configuration types and of scheme::advance
over the C ABI of include/b2d.h (libb2d.so).
"""
from .config import (ORBITAL_PERIOD, DiskModel, Euler, Isothermal, Mesh, Physics, num_fields, to_c)
from .scheme import (ITEMS, PRECISIONS, B2DException, HydroError, Run, Runtime, initial_state, pin, set_device, unpin)
from . import presets

__all__ = [
    "ORBITAL_PERIOD", "DiskModel", "Euler", "Isothermal", "Mesh", "Physics", "num_fields", "to_c",
    "ITEMS", "PRECISIONS", "B2DException", "HydroError", "Run", "Runtime", "initial_state", "pin", "set_device", "unpin",
    "presets",
]
