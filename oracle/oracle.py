"""ctypes wrapper for the CPU oracle (test infrastructure, see clbm_oracle.c).

``Oracle`` mirrors the reference objects: ``compute_force`` is
``DroneMovingIBM.compute_force`` (airfoil_moving.py:230-255) and ``lbm_step`` is
``CLBMSolver.step`` (clbm_moving.py:326-343); arrays come back in the reference layout,
(Nx, Ny, Nz) and (Nx, Ny, Nz, 19), z fastest.
"""

import ctypes
import os

import numpy as np

from . import build as _build

_LIBS = {}


def load(real="f32"):
    if real not in _LIBS:
        path = _build.lib_path(real)
        if not os.path.exists(path):
            _build.build()
        lib = ctypes.CDLL(path)
        vp, d, i, ll = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_longlong
        P = ctypes.c_void_p
        lib.oracle_create.restype = vp
        lib.oracle_create.argtypes = [i, i, i, d, d, d, d, i, P, P, P]
        lib.oracle_destroy.argtypes = [vp]
        lib.oracle_compute_force.argtypes = [vp] + [d] * 6
        lib.oracle_lbm_step.argtypes = [vp]
        lib.oracle_motion_state.argtypes = [ll] + [d] * 7 + [P]
        lib.oracle_body_force.argtypes = [vp, P]
        lib.oracle_run.argtypes = [vp, ll, i] + [d] * 7 + [P]
        for name in ("oracle_get_f", "oracle_set_f", "oracle_minv", "oracle_get_markers"):
            getattr(lib, name).argtypes = [vp, P]
        lib.oracle_get_macro.argtypes = [vp, P, P, P, P]
        lib.oracle_get_forces.argtypes = [vp, P, P, P]
        lib.oracle_set_forces.argtypes = [vp, P, P, P]
        lib.oracle_set_threads.argtypes = [i]
        lib.oracle_max_threads.restype = i
        lib.oracle_real_size.restype = i
        lib.oracle_set_closure.argtypes = [vp, P]
        lib.oracle_closure_nparams.restype = i
        lib.oracle_closure_features.argtypes = [P, i, P]
        lib.oracle_closure_samples.argtypes = [P, P, i, i, i, P, i, P]
        lib.oracle_closure_filter.argtypes = [P, i, i, i, P]
        lib.oracle_closure_forward.argtypes = [P, P, i, i, P]
        lib.oracle_closure_loss_grad.argtypes = [P, P, i, d, i, P, P]
        _LIBS[real] = lib
    return _LIBS[real]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def motion_state(step, m):
    """_motion_state(step) (main_moving.py:62-74) for a motion dict with keys
    x0, y0, a_heave, a_pitch, phi_pitch, aoa0, omega."""
    out = np.zeros(6, np.float64)
    load().oracle_motion_state(int(step), m["x0"], m["y0"], m["a_heave"], m["a_pitch"],
                               m["phi_pitch"], m["aoa0"], m["omega"], _ptr(out))
    return out


class Oracle:
    def __init__(self, nx, ny, nz, s_v, s_e, ux_in, uy_in, X0, Y0, Z0, real="f32",
                 threads=None):
        self.lib = load(real)
        self.dtype = np.float32 if real == "f32" else np.float64
        self.shape = (nx, ny, nz)
        self.X0 = np.ascontiguousarray(X0, np.float32)
        self.Y0 = np.ascontiguousarray(Y0, np.float32)
        self.Z0 = np.ascontiguousarray(Z0, np.float32)
        self.n = len(self.X0)
        if threads:
            self.lib.oracle_set_threads(int(threads))
        self.h = self.lib.oracle_create(nx, ny, nz, s_v, s_e, ux_in, uy_in, self.n,
                                        _ptr(self.X0), _ptr(self.Y0), _ptr(self.Z0))
        if not self.h:
            raise ValueError("oracle_create rejected the configuration")

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def compute_force(self, xc, yc, theta, vx, vy, omega):
        self.lib.oracle_compute_force(self.h, xc, yc, theta, vx, vy, omega)

    def set_closure(self, params):
        """Learned closure in later collisions (parameter array), None: off."""
        if params is None:
            self.lib.oracle_set_closure(self.h, None)
        else:
            self._closure = np.ascontiguousarray(params, np.float32)
            self.lib.oracle_set_closure(self.h, _ptr(self._closure))

    def lbm_step(self):
        self.lib.oracle_lbm_step(self.h)

    def run(self, step0, nsteps, m, record=True):
        hist = np.zeros((nsteps, 4), np.float64) if record else None
        self.lib.oracle_run(self.h, int(step0), int(nsteps), m["x0"], m["y0"], m["a_heave"],
                            m["a_pitch"], m["phi_pitch"], m["aoa0"], m["omega"],
                            _ptr(hist) if record else None)
        return hist

    def body_force(self):
        out = np.zeros(4, np.float64)
        self.lib.oracle_body_force(self.h, _ptr(out))
        return out

    def f(self):
        out = np.empty(self.shape + (19,), self.dtype)
        self.lib.oracle_get_f(self.h, _ptr(out))
        return out

    def set_f(self, f):
        f = np.ascontiguousarray(f, self.dtype)
        assert f.shape == self.shape + (19,)
        self.lib.oracle_set_f(self.h, _ptr(f))

    def macro(self):
        outs = [np.empty(self.shape, self.dtype) for _ in range(4)]
        self.lib.oracle_get_macro(self.h, *[_ptr(a) for a in outs])
        return outs

    def forces(self):
        outs = [np.empty(self.shape, self.dtype) for _ in range(3)]
        self.lib.oracle_get_forces(self.h, *[_ptr(a) for a in outs])
        return outs

    def set_forces(self, fx, fy, fz):
        ins = [np.ascontiguousarray(a, self.dtype) for a in (fx, fy, fz)]
        self.lib.oracle_set_forces(self.h, *[_ptr(a) for a in ins])

    def markers(self):
        out = np.empty((9, max(self.n, 1)), self.dtype)
        self.lib.oracle_get_markers(self.h, _ptr(out))
        names = ("X", "Y", "Z", "VX", "VY", "Uk", "Vk", "FXk", "FYk")
        return {k: out[t, :self.n] for t, k in enumerate(names)}

    def minv(self):
        out = np.empty((19, 19), self.dtype)
        self.lib.oracle_minv(self.h, _ptr(out))
        return out


# ---------------------------------------------------------------- learned closure
def closure_features(f):
    """Features (non-equilibrium central moments / rho, M_raw order) of populations
    f [..., 19], computed directly as sums of f (e - u)^p (e - v)^q (e - w)^r."""
    f = np.ascontiguousarray(np.asarray(f, np.float64).reshape(-1, 19))
    x = np.empty((f.shape[0], 19), np.float64)
    load("f64").oracle_closure_features(_ptr(f), int(f.shape[0]), _ptr(x))
    return x


def closure_filter(f_fine):
    """Box filter of fine post-stream populations (nx, ny, nz, 19) onto the coarse lattice:
    (nx/2, ny/2, nz/2, 28) with the mean populations, velocity and velocity products."""
    f = np.ascontiguousarray(f_fine, np.float64)
    nx, ny, nz, _ = f.shape
    out = np.empty((nx // 2, ny // 2, nz // 2, 28), np.float64)
    load("f64").oracle_closure_filter(_ptr(f), nx, ny, nz, _ptr(out))
    return out


def closure_samples(f0, f1, cells):
    """Samples [n, 38] of coarse cells from two filtered states (nx, ny, nz, 28)."""
    f0 = np.ascontiguousarray(f0, np.float64)
    f1 = np.ascontiguousarray(f1, np.float64)
    nx, ny, nz, _ = f0.shape
    c = np.ascontiguousarray(cells, np.int64)
    out = np.empty((c.size, 38), np.float64)
    load("f64").oracle_closure_samples(_ptr(f0), _ptr(f1), nx, ny, nz, _ptr(c), int(c.size),
                                       _ptr(out))
    return out


def closure_forward(params, x, round_bf16=True):
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float64)
    s = np.empty(x.shape[0], np.float64)
    load("f64").oracle_closure_forward(_ptr(p), _ptr(x), int(x.shape[0]), int(round_bf16), _ptr(s))
    return s


def closure_loss_grad(params, samples, wscale, round_bf16=True, grad=True):
    """Loss sum over the samples and the gradient of the mean loss (trainable block)."""
    p = np.ascontiguousarray(params, np.float32)
    sm = np.ascontiguousarray(samples, np.float64)
    loss = np.zeros(1, np.float64)
    g = np.zeros(2145, np.float64) if grad else None
    load("f64").oracle_closure_loss_grad(_ptr(p), _ptr(sm), int(sm.shape[0]), float(wscale),
                                         int(round_bf16), _ptr(loss), _ptr(g) if grad else None)
    return (loss[0], g) if grad else loss[0]
