"""Locate and import the GB300 package for the drop-in modules in this directory."""

import importlib
import os
import sys

_ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if _ROOT not in sys.path:
    sys.path.append(_ROOT)

pkg = importlib.import_module("clbm_ibm-moving-airfoil_gb300")

# Most recently created drop-in solver; DroneMovingIBM binds to it when it is created
# after CLBMSolver (main_moving.py:104-105), or to the solver whose velocity fields are
# passed to its first compute_force call.
latest_solver = None
