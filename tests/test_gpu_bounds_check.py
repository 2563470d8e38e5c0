"""The bounds-checked build (-DCLBM_CHECK): the same library with an index test before every
population, force-field, macro-field and stencil access of the stream-collide, band and IBM
bodies (an access outside its array is skipped and reported instead of faulting). The
checked build runs the cases of the parity tests -- every storage form and kernel variant,
the wing across the periodic y seam, a force box at the outlet column of an odd lattice,
caller-supplied dense forces, the ensemble in both step forms -- and reports no access
outside an array; its self test shows that a report reaches the host."""

import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = r'''
import ctypes, importlib, os, sys
from dataclasses import replace
import numpy as np
sys.path.insert(0, ".")
pkg = importlib.import_module("clbm_ibm-moving-airfoil_gb300")
on = ctypes.c_int32()
assert pkg.lib().clbm_bounds_checked(ctypes.byref(on)) == 0 and on.value == 1, "not the checked build"
s = pkg.Solver(40, 8, 4, 1.5)
rc = pkg.lib().clbm_selftest_bounds(s.handle)
assert rc == 4 and b"as intended" in pkg.lib().clbm_last_error(), rc
s.step()
s.synchronize()
s.close()
for storage in ("f32", "f16", "bf16"):
    for variant in (("cell", "staged") if storage == "f32" else ("cell", "pair", "staged")):
        os.environ["CLBM_KERNEL"] = variant
        for cfg in (pkg.small_case(storage=storage), replace(pkg.small_case(storage=storage), y0=2.0),
                    replace(pkg.wing_case(61, 40, 6, 16, storage=storage, name="outlet"),
                            x0=61.0 - 0.75 * 16.0 - 1.0)):
            for graph in (True, False):
                sim = pkg.Simulation(cfg)
                sim.run(12, graph=graph)
                sim.solver.synchronize()
                sim.close()
    os.environ.pop("CLBM_KERNEL")
    f = pkg.Solver(37, 9, 5, 1.4, storage=storage)
    F = [np.full((37, 9, 5), 1e-4, np.float32) for _ in range(3)]
    for _ in range(3):
        f.step_host_force(*F)
    f.synchronize()
    f.close()
    cases = [pkg.config.ensemble_case(k, storage=storage, lattices=((47, 20, 4), (64, 20, 6), (41, 16, 3)))
             for k in range(4)]
    for form in ("launches", "persistent"):
        if form == "persistent":
            os.environ["CLBM_ENS_STEP"] = "persistent"
        ens = pkg.Ensemble(cases)
        os.environ.pop("CLBM_ENS_STEP", None)
        ens.run(10)
        ens.synchronize()
        ens.close()
print("clean")
'''


def test_bounds_checked_build_runs_clean(built_pkg):
    built_pkg.build(check=True)
    env = dict(os.environ, CLBM_CHECK_BUILD="1")
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "clean" in r.stdout
