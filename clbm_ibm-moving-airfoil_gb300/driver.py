"""The driver loop of main_moving.py:87-203 on the GPU, with the same output.

Every `vis_interval` steps: divergence statistics on the device (rho min/max, max |u|,
non-finite count; main_moving.py:130-145), the status line, and ``frame_%06d.npz`` with
float32 ``ux, uy, uz, rho`` of shape (Nx, Ny, Nz) (main_moving.py:147-155). At the end:
``meta.npz`` with ``xc, yc, theta, step, X_template, Y_template, X_htail_tmpl,
Y_htail_tmpl, grid_meta`` (main_moving.py:173-200, the 24-entry ``grid_meta`` in the same
order). In addition (not in the reference): ``forces.npz`` with the per-step force sums
and lift/drag coefficients.

The GPU steps in chunks of `vis_interval` (graph-replayed or direct); compressing a frame
runs on writer threads while the next chunk is already stepping.
"""

import concurrent.futures
import math
import os
import time

import numpy as np

from ._lib import DivergedError
from .config import force_coefficients
from .solver import Simulation

#: grid_meta entries in main_moving.py:185-198 order
GRID_META_KEYS = ("Nx", "Ny", "Nz", "U_inf", "Re", "x0", "y0", "z0", "fuse_ax", "fuse_ay",
                  "b_half", "z_wing_start", "z_wing_end", "IZ", "IX", "vis_interval", "fuse_az",
                  "x_tail_arm", "c_htail", "b_half_htail", "z_htail_start", "z_htail_end",
                  "c_vtail", "h_vtail")

FRAME_KEYS = ("ux", "uy", "uz", "rho")
META_KEYS = ("xc", "yc", "theta", "step", "X_template", "Y_template", "X_htail_tmpl",
             "Y_htail_tmpl", "grid_meta")


def grid_meta(cfg, vis_interval, geometry=None):
    """The 24 grid_meta values; `geometry` supplies the airplane dimensions (fuse_ax, b_half,
    ...) where the case has them, the rest are 0."""
    g = dict(geometry or {})
    z0 = float(cfg.nz) / 2.0
    vals = dict(Nx=cfg.nx, Ny=cfg.ny, Nz=cfg.nz, U_inf=cfg.u_inf, Re=cfg.re, x0=cfg.x0,
                y0=cfg.y0, z0=z0, IZ=float(int(round(z0))), IX=float(int(round(cfg.x0))),
                vis_interval=vis_interval)
    vals.update(g)
    return np.array([float(vals.get(k, 0.0)) for k in GRID_META_KEYS], dtype=np.float64)


def _save_frame(path, fields):
    np.savez_compressed(path, **{k: fields[k].astype(np.float32) for k in FRAME_KEYS})


def run(cfg, n_steps, vis_interval, data_dir, graph=True, geometry=None, templates=None,
        writers=2, log=print, rho_floor=0.3):
    """Run `n_steps` steps of `cfg` writing frames/meta into `data_dir`.
    Returns dict(steps, frames, diverged, seconds, forces)."""
    os.makedirs(data_dir, exist_ok=True)
    sim = Simulation(cfg)
    pool = concurrent.futures.ThreadPoolExecutor(max_workers=max(1, writers))
    pending = []
    snap = {"xc": [], "yc": [], "theta": [], "step": []}
    sums = []
    frame_idx = 0
    diverged = False
    step = 0
    t0 = last = time.perf_counter()
    try:
        while step < n_steps:
            k = min(vis_interval - (step % vis_interval), n_steps - step)
            tripped = False
            try:
                sim.run(k, graph=graph)
            except DivergedError:
                # the collisions' divergence monitor stopped the run (main_moving.py:143-145
                # stops at its next vis step); the check below reports it
                tripped = True
            if sim.ibm is not None:
                sums.append(sim.ibm.force_history(k))
            step += k
            if step % vis_interval and not tripped:
                continue
            xc, yc, theta = cfg.motion_state(step)[:3]
            try:
                st = sim.solver.check(rho_floor)
                bad = False
            except Exception as exc:  # DivergedError: statistics still reported
                st = getattr(exc, "stats", None) or {"rho_min": float("nan"),
                                                     "rho_max": float("nan"),
                                                     "u_max": float("nan")}
                bad = True
            bad = bad or tripped
            now = time.perf_counter()
            rate = vis_interval / (now - last)
            last = now
            log(f"  step {step:6d}  |  u_max={st['u_max']:.5f}  "
                f"rho=[{st['rho_min']:.4f},{st['rho_max']:.4f}]  "
                f"yc={yc:.2f}  theta={math.degrees(theta):.2f} deg"
                f"  |  {rate:.0f} steps/s")
            if bad:
                log(f"\n*** Diverged at step {step}!  rho_min={st['rho_min']:.4f} ***")
                diverged = True
                break
            frame_idx += 1
            fields = sim.solver.read_macro()
            path = os.path.join(data_dir, f"frame_{frame_idx:06d}.npz")
            pending.append(pool.submit(_save_frame, path, fields))
            snap["xc"].append(xc)
            snap["yc"].append(yc)
            snap["theta"].append(theta)
            snap["step"].append(step)
        for p in pending:
            p.result()
    finally:
        pool.shutdown(wait=True)
    elapsed = time.perf_counter() - t0
    forces = None
    if sums:
        s = np.concatenate(sums, axis=0)
        c = force_coefficients(s, cfg)
        forces = dict(sums=s, **c)
        np.savez_compressed(os.path.join(data_dir, "forces.npz"), **forces)
    if frame_idx:
        tmpl = dict(templates if templates is not None else (cfg.templates or {}))
        geometry = geometry if geometry is not None else cfg.geometry
        X2 = tmpl.get("X_template", cfg.X0[:0] if cfg.X0 is not None else np.zeros(0, np.float32))
        np.savez_compressed(
            os.path.join(data_dir, "meta.npz"),
            xc=np.array(snap["xc"], dtype=np.float32),
            yc=np.array(snap["yc"], dtype=np.float32),
            theta=np.array(snap["theta"], dtype=np.float32),
            step=np.array(snap["step"], dtype=np.int32),
            X_template=np.asarray(X2, np.float32),
            Y_template=np.asarray(tmpl.get("Y_template", X2), np.float32),
            X_htail_tmpl=np.asarray(tmpl.get("X_htail_tmpl", np.zeros(0)), np.float32),
            Y_htail_tmpl=np.asarray(tmpl.get("Y_htail_tmpl", np.zeros(0)), np.float32),
            grid_meta=grid_meta(cfg, vis_interval, geometry),
        )
    sim.close()
    return dict(steps=step, frames=frame_idx, diverged=diverged, seconds=elapsed, forces=forces)
