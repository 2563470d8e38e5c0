"""Generate golden vectors by running the reference solver's own kernels on tiny lattices.

Run in a container that has the reference checkout (read-only is fine):

    python tests/golden/make_golden.py /root/reference

The reference's ``clbm_moving.py``, ``airfoil_moving.py`` and ``main_moving.py`` are
imported unmodified. ``taichi`` is replaced by ``taichi_emulator`` (serial float32
evaluation of the kernels) and ``config_moving`` by a small in-memory configuration
module, selected through ``sys.modules`` aliasing exactly as the reference's own
``main_highRe.py`` selects ``config_highRe``. Geometry helpers (``_naca0012_2d``,
``_ellipsoid_markers``) and ``M_raw_inv_np`` come from the reference's
``config_moving.py`` itself.

Each case drives the same loop as ``main_moving.main`` (main_moving.py:116-122):
``_motion_state(step)`` -> ``ibm.compute_force(lbm.ux, lbm.uy, ...)`` -> ``lbm.step``.
Outputs are ``golden_<case>.npz`` next to this script. Only this generator reads the
reference; the tests read the ``.npz`` files.
"""

import importlib.util
import math
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


# Case definitions. Lattices are tiny so the serial emulator finishes in seconds.
CASES = {
    # Reference-flavoured: inflow rotated by AoA0, mid-chord pivot, an ellipsoid body
    # with fractional z markers in addition to the extruded NACA sections.
    "A": dict(Nx=24, Ny=16, Nz=4, U_inf=0.05, Re=10.0, chord=8.0, s_e=1.0,
              AoA0_deg=8.0, theta0_deg=8.0, x0=9.0, y0=8.0, A_heave=1.5,
              A_pitch_deg=5.0, k_reduced=0.5, ds=0.7, ellipsoid=(3.0, 1.0, 1.0),
              n_steps=30, record=(1, 2, 5, 10, 20, 30), f_record=(1, 30)),
    # Edges: unrotated inflow with a separate mean pitch angle, markers straddling the
    # y-periodic seam and stencils clamped at x = 0, s_e != 1 (trace relaxation path).
    "B": dict(Nx=16, Ny=10, Nz=3, U_inf=0.05, Re=12.0, chord=6.0, s_e=1.3,
              AoA0_deg=0.0, theta0_deg=8.0, x0=4.0, y0=0.7, A_heave=1.0,
              A_pitch_deg=10.0, k_reduced=0.5, ds=0.7, ellipsoid=None,
              n_steps=20, record=(1, 2, 10, 20), f_record=(1, 20)),
}


def make_config_module(refcfg, p):
    """Build an in-memory ``config_moving`` with the names the reference modules import."""
    m = types.ModuleType("config_moving")
    Nx, Ny, Nz = p["Nx"], p["Ny"], p["Nz"]
    c = p["chord"]
    m.Nx, m.Ny, m.Nz = Nx, Ny, Nz
    m.U_inf = p["U_inf"]
    m.Re = p["Re"]
    m.cs2 = 1.0 / 3.0
    m.nu = m.U_inf * c / m.Re
    m.tau = 0.5 + m.nu / m.cs2
    m.s_v = 1.0 / m.tau
    m.s_e = p["s_e"]
    m.s_q = 1.0
    m.s_pi = 1.0
    m.M_raw_inv_np = refcfg.M_raw_inv_np
    m.AoA0_deg = p["AoA0_deg"]

    X2, Y2 = refcfg._naca0012_2d(c, p["ds"])
    layers = np.arange(0, Nz, 1.0, dtype=np.float32)
    X = [np.tile(X2, len(layers))]
    Y = [np.tile(Y2, len(layers))]
    Z = [np.repeat(layers, len(X2))]
    if p["ellipsoid"] is not None:
        ex, ey, ez = refcfg._ellipsoid_markers(*p["ellipsoid"], p["ds"])
        X.append(ex)
        Y.append(ey)
        Z.append((ez + Nz / 2.0).astype(np.float32))
    m.X_marker_np = np.concatenate(X).astype(np.float32)
    m.Y_marker_np = np.concatenate(Y).astype(np.float32)
    m.Z_marker_np = np.concatenate(Z).astype(np.float32)
    m.N_MARKERS_2D = len(X2)
    m.N_MARKERS = len(m.X_marker_np)
    m.X_template, m.Y_template = X2, Y2
    m.X_htail_tmpl, m.Y_htail_tmpl = X2, Y2

    m.x0, m.y0, m.z0 = p["x0"], p["y0"], Nz / 2.0
    m.k_reduced = p["k_reduced"]
    m.f_motion = m.k_reduced * m.U_inf / (np.pi * c)
    m.A_heave = p["A_heave"]
    m.A_pitch = np.radians(p["A_pitch_deg"])
    m.phi_pitch = np.pi / 2.0
    m.AoA0_rad = np.radians(p["theta0_deg"])
    # names main_moving.py imports for its banner/metadata only
    for name in ("fuse_ax", "fuse_ay", "fuse_az", "b_half", "z_wing_start", "z_wing_end",
                 "x_tail_arm", "c_htail", "b_half_htail", "z_htail_start", "z_htail_end",
                 "c_vtail", "h_vtail"):
        setattr(m, name, 0.0)
    m.N_steps = p["n_steps"]
    m.vis_interval = 1
    m.DATA_DIR = "unused"
    return m


def run_case(ref_dir, name, p):
    import taichi_emulator
    sys.modules["taichi"] = taichi_emulator
    refcfg = _load("_reference_config_moving", os.path.join(ref_dir, "config_moving.py"))
    cfg = make_config_module(refcfg, p)
    sys.modules["config_moving"] = cfg
    for mod in ("clbm_moving", "airfoil_moving", "main_moving"):
        sys.modules.pop(mod, None)
    clbm = _load("clbm_moving", os.path.join(ref_dir, "clbm_moving.py"))
    ibmmod = _load("airfoil_moving", os.path.join(ref_dir, "airfoil_moving.py"))
    main = _load("main_moving", os.path.join(ref_dir, "main_moving.py"))

    lbm = clbm.CLBMSolver()
    ibm = ibmmod.DroneMovingIBM()
    out = {
        "Nx": cfg.Nx, "Ny": cfg.Ny, "Nz": cfg.Nz, "U_inf": cfg.U_inf, "Re": cfg.Re,
        "chord": p["chord"], "s_v": cfg.s_v, "s_e": cfg.s_e, "AoA0_deg": cfg.AoA0_deg,
        "AoA0_rad": cfg.AoA0_rad, "x0": cfg.x0, "y0": cfg.y0, "A_heave": cfg.A_heave,
        "A_pitch": cfg.A_pitch, "phi_pitch": cfg.phi_pitch, "f_motion": cfg.f_motion,
        "X0": cfg.X_marker_np, "Y0": cfg.Y_marker_np, "Z0": cfg.Z_marker_np,
        "M_raw_inv": cfg.M_raw_inv_np,
        "f_init": lbm.f.to_numpy(), "n_steps": p["n_steps"],
        "record": np.array(p["record"], dtype=np.int32),
        "f_record": np.array(p["f_record"], dtype=np.int32),
    }
    motion = []
    for step in range(1, p["n_steps"] + 1):
        ms = main._motion_state(step)
        motion.append(ms)
        fx, fy, fz = ibm.compute_force(lbm.ux, lbm.uy, *ms)
        if step in p["record"]:
            out[f"s{step}_X"] = ibm.X_marker.to_numpy()
            out[f"s{step}_Y"] = ibm.Y_marker.to_numpy()
            out[f"s{step}_Z"] = ibm.Z_marker.to_numpy()
            out[f"s{step}_VX"] = ibm.VX_body.to_numpy()
            out[f"s{step}_VY"] = ibm.VY_body.to_numpy()
            out[f"s{step}_Uk"] = ibm.U_k.to_numpy()
            out[f"s{step}_Vk"] = ibm.V_k.to_numpy()
            out[f"s{step}_FXk"] = ibm.FX_k.to_numpy()
            out[f"s{step}_FYk"] = ibm.FY_k.to_numpy()
            out[f"s{step}_fx"] = fx.to_numpy()
            out[f"s{step}_fy"] = fy.to_numpy()
            out[f"s{step}_fz"] = fz.to_numpy()
        lbm.step(fx, fy, fz)
        if step in p["record"]:
            out[f"s{step}_rho"] = lbm.rho.to_numpy()
            out[f"s{step}_ux"] = lbm.ux.to_numpy()
            out[f"s{step}_uy"] = lbm.uy.to_numpy()
            out[f"s{step}_uz"] = lbm.uz.to_numpy()
        if step in p["f_record"]:
            out[f"s{step}_f"] = lbm.f.to_numpy()
        print(f"  case {name} step {step}", flush=True)
    out["motion"] = np.array(motion, dtype=np.float64)
    return out


def _sha(*arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make_geometry(ref_dir):
    """Marker geometry and M_raw^-1 of the reference's own config module (the airplane of
    config_moving.py:196-307 and the section builders it uses)."""
    cfg = _load("_reference_config_moving", os.path.join(ref_dir, "config_moving.py"))
    out = {
        "airplane_n": cfg.N_MARKERS,
        "airplane_sha": _sha(cfg.X_marker_np, cfg.Y_marker_np, cfg.Z_marker_np),
        "airplane_sample": np.stack([cfg.X_marker_np[::97], cfg.Y_marker_np[::97],
                                     cfg.Z_marker_np[::97]]),
        "M_raw_inv": cfg.M_raw_inv_np,
        "interior_80_07_sha": _sha(*cfg._naca0012_interior(80, 0.7)),
        "ellipsoid_sha": _sha(*cfg._ellipsoid_markers(75.0, 10.0, 10.0, 0.7)),
        "wing_layers": cfg.Nz_layers, "wing_2d": cfg.N_MARKERS_2D,
    }
    for chord, ds in ((32, 1.0), (80, 1.0), (160, 1.0), (80, 0.7), (8, 0.7)):
        X, Y = cfg._naca0012_2d(chord, ds)
        out[f"naca_{chord}_{str(ds).replace('.', '')}"] = np.stack([X, Y])
    hre = _load("_reference_config_highRe", os.path.join(ref_dir, "config_highRe.py"))
    out["highre_n"] = hre.N_MARKERS
    out["highre_sha"] = _sha(hre.X_marker_np, hre.Y_marker_np, hre.Z_marker_np)
    fish = _load("_reference_config_fish", os.path.join(ref_dir, "fish", "config_fish.py"))
    out["fish_n"] = fish.N_MARKERS
    out["fish_sha"] = _sha(fish.X_marker_np, fish.Y_marker_np, fish.Z_marker_np)
    return out


def main(argv):
    ref_dir = argv[1] if len(argv) > 1 else "/root/reference"
    sys.dont_write_bytecode = True
    sys.path.insert(0, HERE)
    names = argv[2:] or sorted(CASES) + ["geometry"]
    if "geometry" in names:
        names = [n for n in names if n != "geometry"]
        path = os.path.join(HERE, "golden_geometry.npz")
        np.savez_compressed(path, **make_geometry(ref_dir))
        print(f"wrote {path} ({os.path.getsize(path)} bytes)")
    for name in names:
        out = run_case(ref_dir, name, CASES[name])
        path = os.path.join(HERE, f"golden_{name}.npz")
        np.savez_compressed(path, **out)
        print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    main(sys.argv)
