"""Host-side objects over the C ABI: ``Solver`` (the CLBMSolver of clbm_moving.py) and
``IBM`` (the DroneMovingIBM of airfoil_moving.py), plus ``Simulation``, the driver loop
of main_moving.py:116-122 with on-device motion and CUDA-graph replay.

All arrays returned to Python are NumPy copies in the reference layout: (Nx, Ny, Nz) with
z fastest, and (Nx, Ny, Nz, 19) for populations.
"""

import ctypes
import weakref

import numpy as np

from . import _lib
from ._lib import check, lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class PinnedBuffer:
    """Page-locked host memory viewed as a NumPy array."""

    def __init__(self, shape, dtype=np.float32):
        self.shape = tuple(shape)
        self.dtype = np.dtype(dtype)
        nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        self._p = ctypes.c_void_p()
        check(lib().clbm_host_alloc(max(nbytes, 1), ctypes.byref(self._p)))
        buf = (ctypes.c_char * max(nbytes, 1)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(np.prod(self.shape))).reshape(self.shape)

    def close(self):
        if self._p is not None and self._p.value:
            lib().clbm_host_free(self._p)
        self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """D3Q19 cascaded LBM on one GPU (CLBMSolver, clbm_moving.py:41-343)."""

    def __init__(self, nx, ny, nz, s_v, s_e=1.0, ux_in=0.05, uy_in=0.0, storage="f32",
                 device=0):
        if storage not in _lib.STORAGE:
            raise ValueError(f"storage must be one of {sorted(_lib.STORAGE)}")
        self.shape = (int(nx), int(ny), int(nz))
        self.storage = storage
        cfg = _lib.Config(nx=nx, ny=ny, nz=nz, s_v=s_v, s_e=s_e, ux_in=ux_in, uy_in=uy_in,
                          storage=_lib.STORAGE[storage], device=int(device))
        self._h = ctypes.c_void_p()
        check(lib().clbm_create(ctypes.byref(cfg), ctypes.byref(self._h)))
        self._pinned = None
        self._ibms = weakref.WeakSet()

    @classmethod
    def from_config(cls, cfg, device=0):
        return cls(cfg.nx, cfg.ny, cfg.nz, cfg.s_v, cfg.s_e, cfg.ux_in, cfg.uy_in, cfg.storage,
                   device=device)

    @property
    def handle(self):
        return self._h

    def close(self):
        for ibm in list(getattr(self, "_ibms", ())):
            ibm.close()
        if self._h is not None and self._h.value:
            lib().clbm_destroy(self._h)
        self._h = None
        if self._pinned is not None:
            self._pinned.close()
            self._pinned = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- stepping -----------------------------------------------------------------
    def step(self, ibm=None):
        """One fused stream + collide step with the forces of ibm's last compute_force."""
        check(lib().clbm_step(self._h, ibm._h if ibm is not None else None))

    def step_dense_force(self, fx_ptr, fy_ptr, fz_ptr=None):
        """One step with caller-owned device force fields (reference layout, float32)."""
        check(lib().clbm_step_dense_force(self._h, fx_ptr, fy_ptr, fz_ptr))

    def step_host_force(self, fx, fy, fz=None):
        """One step with force fields given as host arrays (Nx, Ny, Nz), used unclipped."""
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (fx, fy, fz)]
        for a in arrs:
            if a is not None and a.shape != self.shape:
                raise ValueError(f"force fields must have shape {self.shape}")
        check(lib().clbm_step_host_force(self._h, *[_ptr(a) for a in arrs]))

    def run(self, ibm, motion, nsteps, graph=True):
        m = _lib.Motion(**{k: motion[k] for k in ("x0", "y0", "a_heave", "a_pitch",
                                                    "phi_pitch", "aoa0")}, w=motion["omega"])
        check(lib().clbm_run(self._h, ibm._h if ibm is not None else None, ctypes.byref(m),
                             int(nsteps), 1 if graph else 0))

    def synchronize(self):
        """Wait for the solver's work; raises DivergedError when the device divergence
        monitor fired (a collision met a density below the floor or not finite)."""
        check(lib().clbm_synchronize(self._h))

    def set_rho_floor(self, rho_floor):
        """Density floor of the device divergence monitor (default 0.3, the threshold of
        main_moving.py:143); a negative floor keeps only the non-finite test."""
        check(lib().clbm_set_rho_floor(self._h, float(rho_floor)))

    def selftest_wait_timeout(self, spin_limit=4096):
        """Make one staged launch's bounded wait run out on purpose; returns the error the
        library reports (a CLBMError with code CLBM_ERR_STATE is the expected outcome)."""
        rc = lib().clbm_selftest_wait_timeout(self._h, int(spin_limit))
        try:
            check(rc)
        except _lib.CLBMError as e:
            return e
        return None

    def stream_handle(self):
        """cudaStream_t of the solver as an integer (for torch.cuda.ExternalStream)."""
        p = ctypes.c_void_p()
        check(lib().clbm_stream(self._h, ctypes.byref(p)))
        return p.value or 0

    # --- fields -------------------------------------------------------------------
    def _pinned_fields(self):
        if self._pinned is None:
            self._pinned = PinnedBuffer((4,) + self.shape)
        return self._pinned.array

    def read_macro(self, which=("rho", "ux", "uy", "uz")):
        """rho, ux, uy, uz of the current state (_macro_post) as float32 arrays."""
        buf = self._pinned_fields()
        names = ("rho", "ux", "uy", "uz")
        ptrs = [_ptr(buf[i]) if n in which else None for i, n in enumerate(names)]
        check(lib().clbm_read_macro(self._h, *ptrs))
        return {n: buf[i].copy() for i, n in enumerate(names) if n in which}

    def read_vorticity(self, z=None):
        """z-vorticity d(ux)/dy - d(uy)/dx of plane z (default mid-span), (Nx, Ny) float32,
        with NumPy gradient edge rules as the reference's renderers use."""
        z = self.shape[2] // 2 if z is None else int(z)
        out = np.empty(self.shape[:2], np.float32)
        check(lib().clbm_read_vorticity_slice(self._h, z, _ptr(out)))
        return out

    def read_populations(self):
        out = np.empty(self.shape + (19,), np.float32)
        check(lib().clbm_read_populations(self._h, _ptr(out)))
        return out

    def write_populations(self, f):
        f = np.ascontiguousarray(f, np.float32)
        if f.shape != self.shape + (19,):
            raise ValueError(f"populations must have shape {self.shape + (19,)}")
        check(lib().clbm_write_populations(self._h, _ptr(f)))

    def check(self, rho_floor=0.3):
        """Divergence statistics; raises DivergedError like main_moving.py:143-145 breaks."""
        rmin, rmax, umax = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        bad = ctypes.c_int64()
        rc = lib().clbm_check(self._h, rho_floor, ctypes.byref(rmin), ctypes.byref(rmax),
                              ctypes.byref(umax), ctypes.byref(bad))
        stats = dict(rho_min=rmin.value, rho_max=rmax.value, u_max=umax.value,
                     nonfinite=bad.value)
        try:
            check(rc)
        except _lib.CLBMError as e:
            e.stats = stats
            raise
        return stats

    # --- profiling ----------------------------------------------------------------
    def profile(self, on):
        check(lib().clbm_profile_enable(self._h, 1 if on else 0))

    def profile_read(self):
        ms, n, tot = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
        check(lib().clbm_profile_read(self._h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(tot)))
        bms, bn, xms, xn = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_int64()
        check(lib().clbm_profile_read_split(self._h, ctypes.byref(bms), ctypes.byref(bn),
                                            ctypes.byref(xms), ctypes.byref(xn)))
        return dict(fused_ms=ms.value, fused_launches=n.value, total_launches=tot.value,
                    bulk_ms=bms.value, bulk_launches=bn.value, box_ms=xms.value,
                    box_launches=xn.value)

    def device_bytes(self):
        b = ctypes.c_int64()
        check(lib().clbm_device_bytes(self._h, ctypes.byref(b)))
        return b.value

    def set_closure(self, params):
        """Use the learned closure (a parameter array of closure.Layout, or a
        closure.ClosureNet) for the bulk pass of later steps; None restores the plain
        cascaded collision."""
        if params is None:
            check(lib().clbm_closure_set(self._h, None))
            return
        p = np.ascontiguousarray(getattr(params, "params", params), np.float32)
        check(lib().clbm_closure_set(self._h, _ptr(p)))

    VARIANTS = ("cell", "pair", "staged")

    def save_state(self):
        """The solver's state as stored on the device (population buffer in its storage
        form, then the macro fields) and its flags, for a checkpoint."""
        n = ctypes.c_int64()
        check(lib().clbm_state_bytes(self._h, ctypes.byref(n)))
        buf = np.empty(n.value, np.uint8)
        flags = ctypes.c_int32()
        check(lib().clbm_save_state(self._h, _ptr(buf), n.value, ctypes.byref(flags)))
        return buf, flags.value

    def load_state(self, buf, flags):
        """Put back a state that save_state returned (same lattice and storage form)."""
        buf = np.ascontiguousarray(buf, np.uint8)
        check(lib().clbm_load_state(self._h, _ptr(buf), buf.size, int(flags)))

    def kernel_variant(self):
        """Full-grid kernel chosen at creation and the autotune time per launch of each
        variant in microseconds (absent: not timed)."""
        v = ctypes.c_int32()
        ms = (ctypes.c_float * len(self.VARIANTS))()
        check(lib().clbm_kernel_variant(self._h, ctypes.byref(v), ms))
        return dict(variant=self.VARIANTS[v.value],
                    us_per_launch={n: round(ms[i] * 1e3, 2) for i, n in enumerate(self.VARIANTS)
                                   if ms[i] > 0})


class IBM:
    """Direct-forcing immersed boundary bound to one Solver (DroneMovingIBM,
    airfoil_moving.py:44-255)."""

    def __init__(self, solver, X0, Y0, Z0):
        self.solver = solver
        self.X0 = np.ascontiguousarray(X0, np.float32)
        self.Y0 = np.ascontiguousarray(Y0, np.float32)
        self.Z0 = np.ascontiguousarray(Z0, np.float32)
        self.n = len(self.X0)
        if not (len(self.Y0) == self.n == len(self.Z0)):
            raise ValueError("X0, Y0, Z0 must have equal length")
        self._h = ctypes.c_void_p()
        check(lib().ibm_create(solver.handle, _ptr(self.X0), _ptr(self.Y0), _ptr(self.Z0),
                               self.n, ctypes.byref(self._h)))
        solver._ibms.add(self)

    def close(self):
        if self._h is not None and self._h.value:
            lib().ibm_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def compute_force(self, xc, yc, theta, vx, vy, omega):
        check(lib().ibm_compute_force(self._h, xc, yc, theta, vx, vy, omega))

    def compute_force_motion(self, motion):
        m = _lib.Motion(**{k: motion[k] for k in ("x0", "y0", "a_heave", "a_pitch",
                                                    "phi_pitch", "aoa0")}, w=motion["omega"])
        check(lib().ibm_compute_force_motion(self._h, ctypes.byref(m)))

    def read_forces(self):
        shape = self.solver.shape
        fx, fy, fz = (np.empty(shape, np.float32) for _ in range(3))
        check(lib().ibm_read_forces(self._h, _ptr(fx), _ptr(fy), _ptr(fz)))
        return fx, fy, fz

    def read_markers(self):
        out = np.empty((9, max(self.n, 1)), np.float32)
        check(lib().ibm_read_markers(self._h, _ptr(out)))
        names = ("X", "Y", "Z", "VX", "VY", "Uk", "Vk", "FXk", "FYk")
        return {k: out[i, :self.n].copy() for i, k in enumerate(names)}

    def force_history(self, count=None):
        n = self.step_count() if count is None else int(count)
        n = min(n, 1 << 16)
        out = np.empty((n, 4), np.float64)
        check(lib().ibm_read_force_history(self._h, n, _ptr(out)))
        return out

    def step_count(self):
        v = ctypes.c_int64()
        check(lib().ibm_step_count(self._h, ctypes.byref(v)))
        return v.value

    def load_state(self, calls, history):
        """Resume at `calls` completed compute_force calls with the given history entries
        (the last len(history) of them); the force fields are written again by the next
        compute_force."""
        h = np.ascontiguousarray(history, np.float64).reshape(-1, 4)
        check(lib().ibm_load_state(self._h, int(calls), _ptr(h), h.shape[0]))


class Simulation:
    """A SimConfig run on the GPU: solver + IBM + the driver loop."""

    def __init__(self, cfg, device=0):
        self.cfg = cfg
        self.solver = Solver.from_config(cfg, device=device)
        self.ibm = IBM(self.solver, cfg.X0, cfg.Y0, cfg.Z0) if cfg.n_markers > 0 else None

    def run(self, nsteps, graph=True):
        self.solver.run(self.ibm, self.cfg.motion(), nsteps, graph=graph)

    def step_host_motion(self, step):
        """One step of main_moving.py's loop with the motion evaluated on the host."""
        if self.ibm is not None:
            self.ibm.compute_force(*self.cfg.motion_state(step))
        self.solver.step(self.ibm)

    def coefficients(self, count=None):
        from .config import force_coefficients
        return force_coefficients(self.ibm.force_history(count), self.cfg)

    def save_checkpoint(self, path):
        """Write the run's state to `path` (.npz): the solver's stored populations and macro
        fields, the IBM call counter (the motion law's step) and the lift/drag history.
        load_checkpoint on a Simulation of the same case continues bit for bit."""
        state, flags = self.solver.save_state()
        calls = self.ibm.step_count() if self.ibm is not None else 0
        hist = self.ibm.force_history(min(calls, 1 << 16)) if self.ibm is not None else np.zeros((0, 4))
        np.savez(path, format=np.int32(1), lattice=np.array([self.cfg.nx, self.cfg.ny, self.cfg.nz]),
                 storage=np.array(self.cfg.storage), markers=np.int64(self.cfg.n_markers),
                 state=state, flags=np.int32(flags), calls=np.int64(calls), history=hist)

    def load_checkpoint(self, path):
        """Resume from a file save_checkpoint wrote for the same case."""
        with np.load(path) as z:
            if int(z["format"]) != 1:
                raise ValueError(f"{path}: unknown checkpoint format {int(z['format'])}")
            if (tuple(int(v) for v in z["lattice"]) != (self.cfg.nx, self.cfg.ny, self.cfg.nz)
                    or str(z["storage"]) != self.cfg.storage
                    or int(z["markers"]) != self.cfg.n_markers):
                raise ValueError(f"{path}: a checkpoint of another case")
            self.solver.load_state(z["state"], int(z["flags"]))
            if self.ibm is not None:
                self.ibm.load_state(int(z["calls"]), z["history"])

    def close(self):
        if self.ibm is not None:
            self.ibm.close()
        self.solver.close()


class Ensemble:
    """Many independent cases stepped together by batched launches (one Simulation per
    member; members stay readable individually through `sims`)."""

    def __init__(self, cfgs, device=0):
        self.sims = [Simulation(c, device=device) for c in cfgs]
        n = len(self.sims)
        if n == 0:
            raise ValueError("an ensemble needs at least one case")
        solvers = (ctypes.c_void_p * n)(*[s.solver.handle.value for s in self.sims])
        ibms = (ctypes.c_void_p * n)(*[(s.ibm._h.value if s.ibm is not None else None)
                                       for s in self.sims])
        motions = (_lib.Motion * n)()
        for i, s in enumerate(self.sims):
            m = s.cfg.motion()
            motions[i] = _lib.Motion(x0=m["x0"], y0=m["y0"], a_heave=m["a_heave"],
                                     a_pitch=m["a_pitch"], phi_pitch=m["phi_pitch"],
                                     aoa0=m["aoa0"], w=m["omega"])
        self._h = ctypes.c_void_p()
        check(lib().clbm_ensemble_create(solvers, ibms, motions, n, ctypes.byref(self._h)))

    @property
    def cells(self):
        return sum(s.cfg.cells for s in self.sims)

    def run(self, nsteps, graph=True):
        check(lib().clbm_ensemble_run(self._h, int(nsteps), 1 if graph else 0))

    def stream_handle(self):
        p = ctypes.c_void_p()
        check(lib().clbm_ensemble_stream(self._h, ctypes.byref(p)))
        return p.value or 0

    def tuning(self):
        """Bulk-pass schedule chosen at creation and the time of one bulk pass of all
        members with it, alone (bulk_us)."""
        w, b, t, ms = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64(), ctypes.c_float()
        r = ctypes.c_int32()
        check(lib().clbm_ensemble_tuning(self._h, ctypes.byref(w), ctypes.byref(b), ctypes.byref(t),
                                         ctypes.byref(ms), ctypes.byref(r)))
        return dict(tile_width=w.value, blocks=b.value, tiles=t.value, bulk_us=round(ms.value * 1e3, 2),
                    rows_per_block=r.value)

    @staticmethod
    def selftest_grid_barrier(blocks=2):
        """Make the persistent step's grid barrier wait for a block that does not exist, so
        every bounded wait runs out on purpose; returns the error the library reports (a
        CLBMError with code CLBM_ERR_STATE is the expected outcome)."""
        rc = lib().clbm_selftest_grid_barrier(int(blocks))
        try:
            check(rc)
        except _lib.CLBMError as e:
            return e
        return None

    def schedule(self):
        """Step form chosen at creation: persistent (one cooperative launch per step,
        CLBM_ENS_STEP=persistent) with its grid, or the seven launches (blocks 0)."""
        p, b = ctypes.c_int32(), ctypes.c_int32()
        check(lib().clbm_ensemble_schedule(self._h, ctypes.byref(p), ctypes.byref(b)))
        return dict(persistent=bool(p.value), blocks=b.value)

    def phase_times(self):
        """Phase clock of the last persistent step in microseconds: markers, offsets,
        band prepare, spreading, and force sums + box pass + the rest of the bulk pass (as
        seen by block 0)."""
        us = (ctypes.c_double * 5)()
        check(lib().clbm_ensemble_phase_times(self._h, us))
        return dict(zip(("markers", "offsets", "band_prepare", "spreading", "sums_box_rest"),
                        (round(v, 2) for v in us)))

    def synchronize(self):
        for s in self.sims:
            s.solver.synchronize()

    def close(self):
        if self._h is not None and self._h.value:
            lib().clbm_ensemble_destroy(self._h)
        self._h = None
        for s in self.sims:
            s.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
