"""GB300-native D3Q19 cascaded-LBM + immersed-boundary time step.

The package is loaded by path (its directory name is not a Python identifier):

    import importlib, sys
    sys.path.insert(0, "<repo root>")
    clbm = importlib.import_module("clbm_ibm-moving-airfoil_gb300")

Drop-in modules for the reference driver (``clbm_moving``, ``airfoil_moving`` and a
``taichi`` import shim) live in ``compat/``; put that directory first on PYTHONPATH.
"""

from . import analysis, closure, config, driver
from ._lib import CLBMError, DivergedError, EXPORTED, lib, lib_path
from .build import build
from .config import (SimConfig, fish_case, force_coefficients, full_case,
                     highre_airplane_case, reference_airplane_case, small_case, wing_case)
from .solver import IBM, Ensemble, PinnedBuffer, Simulation, Solver

__all__ = [
    "CLBMError", "DivergedError", "EXPORTED", "Ensemble", "IBM", "PinnedBuffer", "SimConfig", "Simulation",
    "Solver", "analysis", "build", "closure", "config", "driver", "fish_case", "force_coefficients", "full_case",
    "highre_airplane_case", "lib", "lib_path", "reference_airplane_case", "small_case",
    "wing_case",
]
