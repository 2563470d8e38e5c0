"""Drop-in ``clbm_moving`` module: the reference's CLBMSolver API (clbm_moving.py:41-343)
backed by the GB300 library.

Reads the same names from ``config_moving`` as the reference (clbm_moving.py:15-16) and
exposes:
  CLBMSolver()                 allocate and initialise to feq(rho = 1, u_in) (:54-91)
  .rho .ux .uy .uz             fields with .to_numpy() -> float32 (Nx, Ny, Nz) (:59-63)
  .f                           populations, .to_numpy() / .from_numpy() (Nx, Ny, Nz, 19)
  .M_inv                       19 x 19 inverse raw-moment matrix, .to_numpy()
  .step(fx, fy, fz)            one time step (:326-343)
The fused GPU step keeps the post-collision state, so field reads materialise the
post-stream macroscopic values on demand; the values are those _macro_post produces.

Storage form: float32 by default; set CLBM_STORAGE=f16 or bf16 for the shifted 16-bit
population forms.
"""

import math
import os

import numpy as np

from config_moving import (Nx, Ny, Nz, cs2, s_v, s_e, s_q, s_pi,  # noqa: F401
                           U_inf, AoA0_deg, M_raw_inv_np)

import _clbm_gb300_pkg as _g  # noqa: E402  (this directory is on sys.path)

_AoA_rad = math.radians(AoA0_deg)
_UX_IN = float(U_inf * math.cos(_AoA_rad))
_UY_IN = float(-U_inf * math.sin(_AoA_rad))


class _MacroField:
    """One of rho/ux/uy/uz of a solver."""

    def __init__(self, owner, name):
        self._owner = owner
        self._name = name
        self.shape = (Nx, Ny, Nz)
        self.dtype = np.float32

    def to_numpy(self):
        return self._owner._solver.read_macro((self._name,))[self._name]


class _PopulationField:
    def __init__(self, owner):
        self._owner = owner
        self.shape = (Nx, Ny, Nz, 19)

    def to_numpy(self):
        return self._owner._solver.read_populations()

    def from_numpy(self, a):
        self._owner._solver.write_populations(a)


class _ConstField:
    def __init__(self, a):
        self._a = np.asarray(a, np.float32)
        self.shape = self._a.shape

    def to_numpy(self):
        return self._a.copy()


class CLBMSolver:
    """CLBM D3Q19 fluid solver on an Nx x Ny x Nz lattice (GB300 implementation)."""

    def __init__(self):
        storage = os.environ.get("CLBM_STORAGE", "f32")
        self._solver = _g.pkg.Solver(Nx, Ny, Nz, s_v, s_e, _UX_IN, _UY_IN, storage=storage)
        self.rho = _MacroField(self, "rho")
        self.ux = _MacroField(self, "ux")
        self.uy = _MacroField(self, "uy")
        self.uz = _MacroField(self, "uz")
        self.f = _PopulationField(self)
        self.M_inv = _ConstField(M_raw_inv_np)
        _g.latest_solver = self

    def step(self, fx, fy, fz):
        """Advance one LBM step with body-force density (fx, fy, fz)."""
        ibm = getattr(fx, "_ibm_owner", None)
        if (ibm is not None and getattr(fy, "_ibm_owner", None) is ibm
                and getattr(fz, "_ibm_owner", None) is ibm and ibm._bound_to(self)):
            self._solver.step(ibm._ibm)
            return
        arrs = [a.to_numpy() if hasattr(a, "to_numpy") else np.asarray(a) for a in (fx, fy, fz)]
        self._solver.step_host_force(*arrs)
