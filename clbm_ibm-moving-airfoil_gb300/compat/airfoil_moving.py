"""Drop-in ``airfoil_moving`` module: the reference's DroneMovingIBM API
(airfoil_moving.py:44-255) backed by the GB300 library.

Reads the marker arrays from ``config_moving`` as the reference does
(airfoil_moving.py:17-19) and exposes:
  DroneMovingIBM()                          marker template upload (:64-95)
  .compute_force(ux, uy, xc, yc, theta, vx, vy, omega) -> (fx, fy, fz)   (:230-255)
  .fx .fy .fz                               clipped Eulerian force, .to_numpy() (Nx, Ny, Nz)
  .X_marker .Y_marker .Z_marker .VX_body .VY_body .U_k .V_k .FX_k .FY_k   .to_numpy() (N,)
  .body_force()                             lift/drag support (not in the reference):
                                            force on the body from the last call, in double
``ux``/``uy`` must be the velocity fields of a drop-in CLBMSolver; the interpolation reads
that solver's current state.
"""

import numpy as np

from config_moving import (Nx, Ny, Nz, N_MARKERS_2D, N_MARKERS,  # noqa: F401
                           X_marker_np, Y_marker_np, Z_marker_np)

import _clbm_gb300_pkg as _g  # noqa: E402  (this directory is on sys.path)

N = N_MARKERS

_MARKER_NAMES = ("X", "Y", "Z", "VX", "VY", "Uk", "Vk", "FXk", "FYk")


class _ForceField:
    def __init__(self, owner, comp):
        self._ibm_owner = owner
        self._comp = comp
        self.shape = (Nx, Ny, Nz)

    def to_numpy(self):
        if self._ibm_owner._ibm is None:
            return np.zeros(self.shape, np.float32)
        return self._ibm_owner._ibm.read_forces()[self._comp]


class _MarkerField:
    def __init__(self, owner, name):
        self._owner = owner
        self._name = name
        self.shape = (N,)

    def to_numpy(self):
        if self._owner._ibm is None:
            if self._name in ("X", "Y", "Z"):
                return {"X": X_marker_np, "Y": Y_marker_np, "Z": Z_marker_np}[self._name].copy()
            return np.zeros(N, np.float32)
        return self._owner._ibm.read_markers()[self._name]


class DroneMovingIBM:
    """Direct-forcing IBM for the marker set of config_moving (GB300 implementation)."""

    def __init__(self):
        self.N = N
        self.X0 = np.asarray(X_marker_np, np.float32)
        self.Y0 = np.asarray(Y_marker_np, np.float32)
        self.Z0 = np.asarray(Z_marker_np, np.float32)
        self._ibm = None
        self._solver_owner = None
        self.fx = _ForceField(self, 0)
        self.fy = _ForceField(self, 1)
        self.fz = _ForceField(self, 2)
        (self.X_marker, self.Y_marker, self.Z_marker, self.VX_body, self.VY_body, self.U_k,
         self.V_k, self.FX_k, self.FY_k) = (_MarkerField(self, n) for n in _MARKER_NAMES)
        if _g.latest_solver is not None:
            self._bind(_g.latest_solver)

    def _bind(self, solver_owner):
        if self._solver_owner is solver_owner:
            return
        if self._ibm is not None:
            self._ibm.close()
        self._ibm = _g.pkg.IBM(solver_owner._solver, self.X0, self.Y0, self.Z0)
        self._solver_owner = solver_owner

    def _bound_to(self, solver_owner):
        return self._solver_owner is solver_owner

    def compute_force(self, ux, uy, xc, yc, theta, vx, vy, omega):
        owner = getattr(ux, "_owner", None)
        if owner is None or getattr(uy, "_owner", None) is not owner:
            raise TypeError("compute_force expects the ux/uy fields of a drop-in CLBMSolver")
        self._bind(owner)
        self._ibm.compute_force(float(xc), float(yc), float(theta), float(vx), float(vy),
                                float(omega))
        return self.fx, self.fy, self.fz

    def body_force(self):
        """Force on the body from the last compute_force: (Fx, Fy) = -(sum of the clipped
        Eulerian force), in double."""
        h = self._ibm.force_history(1)[0]
        return -h[0], -h[1]
