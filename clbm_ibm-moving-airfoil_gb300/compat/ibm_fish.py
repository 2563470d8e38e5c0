"""Drop-in ``ibm_fish`` module (fish/ibm_fish.py): the ``airfoil_moving`` drop-in's IBM
reading ``config_fish``, under the fish variant's class name FishIBM (fish/ibm_fish.py:41;
the same compute_force API as DroneMovingIBM)."""

import _variant

_impl = _variant.load("airfoil_moving", "config_fish", "_ibm_fish_impl")
FishIBM = _impl.DroneMovingIBM
N = _impl.N
