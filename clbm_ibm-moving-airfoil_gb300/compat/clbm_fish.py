"""Drop-in ``clbm_fish`` module (fish/clbm_fish.py): the ``clbm_moving`` drop-in's
CLBMSolver reading ``config_fish`` (fish/clbm_fish.py:12-13 imports the same names from it
as clbm_moving.py does from config_moving)."""

import _variant

_impl = _variant.load("clbm_moving", "config_fish", "_clbm_fish_impl")
CLBMSolver = _impl.CLBMSolver
