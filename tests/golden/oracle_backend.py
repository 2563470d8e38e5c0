"""Oracle-backed stand-in for the GB300 package, as the drop-in modules use it (test
infrastructure only).

The drop-in modules under ``compat/`` (``clbm_moving``, ``airfoil_moving``, ``taichi``)
reach the GPU library through ``_clbm_gb300_pkg.pkg``: ``Solver``, ``IBM`` and ``lib``. On
a machine without a GPU, ``install()`` puts this module in that place, so that the
reference's own driver (main_moving.py) can be run unmodified through the drop-in modules
here: every call they make is answered by the CPU oracle (oracle/clbm_oracle.c, the
reference's arithmetic) and recorded in ``TRACE``. The recorded calls are what a GPU test
replays through the same drop-in modules with the real library.

Recorded events: ("compute_force", xc, yc, theta, vx, vy, omega), ("step",),
("step_host_force",), ("read_macro", name) -- the package-level calls behind
``ibm.compute_force(lbm.ux, lbm.uy, ...)``, ``lbm.step(fx, fy, fz)`` and
``lbm.<name>.to_numpy()``.
"""

import sys
import types

import numpy as np

from oracle.oracle import Oracle

TRACE = []


class Solver:
    def __init__(self, nx, ny, nz, s_v, s_e=1.0, ux_in=0.05, uy_in=0.0, storage="f32",
                 device=0):
        if storage != "f32":
            raise ValueError("the oracle stand-in computes float32 only")
        self.shape = (nx, ny, nz)
        self._args = (nx, ny, nz, s_v, s_e, ux_in, uy_in)
        self._o = Oracle(*self._args, [], [], [])
        self._fresh = True      # still the initial state (macro fields exactly rho = 1, u_in)

    def _attach(self, X0, Y0, Z0):
        """The oracle holds the lattice and the markers together: re-create it with the
        markers, carrying the current populations over (an imported state recomputes the
        macroscopic fields, so the initial state is not carried but re-created)."""
        f = None if self._fresh else self._o.f()
        self._o.close()
        self._o = Oracle(*self._args, X0, Y0, Z0)
        if f is not None:
            self._o.set_f(f)
        return self._o

    def step(self, ibm=None):
        TRACE.append(("step",))
        self._fresh = False
        self._o.lbm_step()

    def step_host_force(self, fx, fy, fz=None):
        TRACE.append(("step_host_force",))
        self._fresh = False
        fz = np.zeros(self.shape, np.float32) if fz is None else fz
        self._o.set_forces(fx, fy, fz)
        self._o.lbm_step()

    def read_macro(self, which=("rho", "ux", "uy", "uz")):
        vals = dict(zip(("rho", "ux", "uy", "uz"), self._o.macro()))
        for k in which:
            TRACE.append(("read_macro", k))
        return {k: np.asarray(vals[k], np.float32) for k in which}

    def read_populations(self):
        return self._o.f()

    def write_populations(self, f):
        self._fresh = False
        self._o.set_f(f)

    def close(self):
        self._o.close()


class IBM:
    def __init__(self, solver, X0, Y0, Z0):
        self._solver = solver
        self._o = solver._attach(X0, Y0, Z0)

    def compute_force(self, xc, yc, theta, vx, vy, omega):
        TRACE.append(("compute_force", xc, yc, theta, vx, vy, omega))
        self._o.compute_force(xc, yc, theta, vx, vy, omega)

    def read_forces(self):
        return tuple(np.asarray(a, np.float32) for a in self._o.forces())

    def read_markers(self):
        return self._o.markers()

    def force_history(self, count=None):
        return self._o.body_force()[None, :]

    def close(self):
        pass


def lib():
    return None


def install():
    """Make the drop-in modules' package handle this stand-in; returns the module object
    that replaced ``_clbm_gb300_pkg``."""
    stand_in = types.ModuleType("_clbm_gb300_pkg")
    stand_in.pkg = sys.modules[__name__]
    stand_in.latest_solver = None
    sys.modules["_clbm_gb300_pkg"] = stand_in
    TRACE.clear()
    return stand_in
