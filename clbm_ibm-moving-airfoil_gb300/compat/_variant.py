"""Load a drop-in module under another configuration module.

The reference's fish variant repeats clbm_moving.py and airfoil_moving.py as
fish/clbm_fish.py and fish/ibm_fish.py with only the configuration import changed
(``config_fish`` instead of ``config_moving``). The drop-in forms of those files are the
drop-in ``clbm_moving`` / ``airfoil_moving`` modules executed once more with the variant's
configuration module standing in for ``config_moving`` -- the aliasing main_highRe.py:26-27
uses for its own variant.
"""

import importlib
import importlib.util
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))


def load(base, config_name, module_name):
    """Execute drop-in module `base` (file name without .py) as `module_name`, with the
    module `config_name` imported under the name ``config_moving`` while it loads."""
    cfg = importlib.import_module(config_name)
    saved = sys.modules.get("config_moving")
    sys.modules["config_moving"] = cfg
    try:
        spec = importlib.util.spec_from_file_location(module_name, os.path.join(_HERE, base + ".py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
    finally:
        if saved is None:
            sys.modules.pop("config_moving", None)
        else:
            sys.modules["config_moving"] = saved
    return mod
