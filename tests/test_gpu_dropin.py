"""The drop-in modules on the GPU, driven by the reference's own drivers, and the
reference's configuration variants stepped on the GPU.

tests/test_dropin.py runs main_moving.py and main_highRe.py unmodified through the drop-in
modules (``compat/``) on the CPU and pins the calls they make (the committed trace in
tests/golden/dropin_<driver>.npz): per step ``ibm.compute_force(lbm.ux, lbm.uy, xc, yc,
theta, vx, vy, omega)`` with the arguments of ``_motion_state(step)``, then
``lbm.step(fx, fy, fz)``, and on every vis step ``lbm.rho/ux/uy/uz.to_numpy()``
(main_moving.py:116-128). Here the same calls go through the same drop-in modules backed by
the CUDA library, and the fields they return are compared with the frames the reference's
own solver wrote (the fixture's frames). The driver's ``ti.init`` (main_moving.py:28-37)
goes through the drop-in ``taichi``: the GPU arch initialises, the CPU fallback raises.
"""

import importlib
import os
import sys
import types

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, rel_l2

pytestmark = pytest.mark.gpu

COMPAT = os.path.join(ROOT, "clbm_ibm-moving-airfoil_gb300", "compat")
FIELDS = ("rho", "ux", "uy", "uz")


@pytest.fixture()
def dropin_env():
    saved = dict(sys.modules)
    path = list(sys.path)
    for name in ("taichi", "clbm_moving", "airfoil_moving", "config_moving", "config_highRe",
                 "_clbm_gb300_pkg", "clbm_fish", "ibm_fish", "config_fish", "_variant"):
        sys.modules.pop(name, None)
    sys.path.insert(0, COMPAT)
    yield
    for name in list(sys.modules):
        if name not in saved:
            del sys.modules[name]
    sys.modules.update(saved)
    sys.path[:] = path


def _config_module(fix, name):
    m = types.ModuleType(name)
    for key in fix.files:
        if key.startswith("cfg_"):
            v = fix[key]
            setattr(m, key[4:], v.item() if v.ndim == 0 else v)
    return m


@pytest.mark.parametrize("driver", ["main_moving", "main_highRe"])
def test_reference_driver_calls_through_dropin_modules(built_pkg, dropin_env, driver):
    fix = np.load(os.path.join(GOLDEN, f"dropin_{driver}.npz"))
    cfg = _config_module(fix, "config_moving")
    if driver == "main_highRe":
        sys.modules["config_highRe"] = cfg      # main_highRe.py:26-27
    sys.modules["config_moving"] = cfg
    ti = importlib.import_module("taichi")
    assert ti.__file__.startswith(COMPAT)
    ti.init(arch=ti.gpu, default_fp=ti.f32, default_ip=ti.i32, fast_math=True)
    with pytest.raises(RuntimeError):
        ti.init(arch=ti.cpu, default_fp=ti.f32, default_ip=ti.i32, cpu_max_num_threads=8)
    clbm_moving = importlib.import_module("clbm_moving")
    airfoil_moving = importlib.import_module("airfoil_moving")
    assert clbm_moving.__file__.startswith(COMPAT) and airfoil_moving.__file__.startswith(COMPAT)

    lbm = clbm_moving.CLBMSolver()
    ibm = airfoil_moving.DroneMovingIBM()
    frames, cur = [], {}
    fx = fy = fz = None
    for kind, args, field in zip(fix["trace_kind"], fix["trace_args"], fix["trace_field"]):
        if kind == 0:
            fx, fy, fz = ibm.compute_force(lbm.ux, lbm.uy, *[float(a) for a in args])
        elif kind == 1:
            lbm.step(fx, fy, fz)
        else:
            name = FIELDS[int(field)]
            a = getattr(lbm, name).to_numpy()
            assert a.shape == (int(cfg.Nx), int(cfg.Ny), int(cfg.Nz)) and a.dtype == np.float32
            cur[name] = a
            if len(cur) == 4:
                frames.append(cur)
                cur = {}
    assert len(frames) == int(fix["n_frames"])
    for k, fr in enumerate(frames, start=1):
        want = {n: fix[f"frame{k}_{n}"] for n in FIELDS}
        e_rho = rel_l2(fr["rho"], want["rho"])
        e_u = rel_l2(np.stack([fr["ux"], fr["uy"], fr["uz"]]),
                     np.stack([want["ux"], want["uy"], want["uz"]]))
        assert e_rho < 1e-5 and e_u < 1e-5, (driver, k, e_rho, e_u)
        assert rel_l2(fr["ux"], want["ux"]) < 1e-5 and rel_l2(fr["uy"], want["uy"]) < 1e-5
    # the lift/drag support of the drop-in IBM reads the last step's force sums
    Fx, Fy = ibm.body_force()
    assert np.isfinite(Fx) and np.isfinite(Fy) and (Fx != 0.0 or Fy != 0.0)
    lbm._solver.close()


def _variant_against_oracle(pkg, oracle_mod, cfg, steps):
    sim = pkg.Simulation(cfg)
    ref = oracle_mod.Oracle(cfg.nx, cfg.ny, cfg.nz, cfg.s_v, cfg.s_e, cfg.ux_in, cfg.uy_in,
                            cfg.X0, cfg.Y0, cfg.Z0)
    for step in range(1, steps + 1):
        sim.step_host_motion(step)
        ref.compute_force(*cfg.motion_state(step))
        ref.lbm_step()
    got = sim.solver.read_macro()
    mk = sim.ibm.read_markers()
    sim.close()
    rho, ux, uy, uz = ref.macro()
    want_mk = ref.markers()
    ref.close()
    e = {"rho": rel_l2(got["rho"], rho), "ux": rel_l2(got["ux"], ux), "uy": rel_l2(got["uy"], uy),
         "FXk": rel_l2(mk["FXk"], want_mk["FXk"]), "FYk": rel_l2(mk["FYk"], want_mk["FYk"])}
    print(cfg.name, {k: f"{v:.2e}" for k, v in e.items()})
    assert e["rho"] < 1e-5 and e["ux"] < 1e-5 and e["uy"] < 1e-5
    assert e["FXk"] < 1e-4 and e["FYk"] < 1e-4


def test_fish_variant_against_oracle(built_pkg, oracle_mod):
    """The swimmer of fish/config_fish.py (800x250x25, 4:1 ellipse, Re 300, k = 0.8)
    stepped on the GPU through the same API, against the oracle."""
    _variant_against_oracle(built_pkg, oracle_mod, built_pkg.fish_case(), 20)


def test_highre_airplane_variant_against_oracle(built_pkg, oracle_mod):
    """The high-Re airplane of config_highRe.py (800x260x220, chord 120, Re 1000, 8 degree
    inflow, the reference's own marker set) stepped on the GPU, against the oracle."""
    _variant_against_oracle(built_pkg, oracle_mod, built_pkg.highre_airplane_case(), 3)


def small_fish_config(pkg, m_raw_inv):
    """An in-memory ``config_fish`` (the names fish/clbm_fish.py and fish/ibm_fish.py import)
    for a reduced swimmer: 120x48x6, 4:1 ellipse of chord 24, Re 300, heave 0.25c, pitch
    15 deg, k = 0.8 (the motion law of fish/config_fish.py); and the same case as a
    SimConfig for the oracle."""
    X2, Y2 = pkg.config.ellipse_section(24.0, 6.0, 0.7)
    X, Y, Z = pkg.config.extrude_layers(X2, Y2, 6)
    ref = pkg.config.SimConfig(nx=120, ny=48, nz=6, chord=24.0, u_inf=0.05, re=300.0, x0=48.0,
                               y0=24.0, a_heave=6.0, a_pitch=float(np.radians(15.0)),
                               phi_pitch=float(np.pi / 2.0), aoa0=0.0, k_reduced=0.8,
                               span=6.0, name="fish-120x48x6", X0=X, Y0=Y, Z0=Z)
    m = types.ModuleType("config_fish")
    m.Nx, m.Ny, m.Nz = ref.nx, ref.ny, ref.nz
    m.cs2, m.s_v, m.s_e, m.s_q, m.s_pi = 1.0 / 3.0, ref.s_v, 1.0, 1.0, 1.0
    m.U_inf, m.AoA0_deg, m.M_raw_inv_np = 0.05, 0.0, m_raw_inv
    m.N_MARKERS_2D, m.N_MARKERS = len(X2), len(X)
    m.X_marker_np, m.Y_marker_np, m.Z_marker_np = X, Y, Z
    return m, ref


def test_fish_dropin_modules_against_oracle(built_pkg, oracle_mod, dropin_env):
    """fish/main_fish.py's solver and IBM modules (``from clbm_fish import CLBMSolver``,
    ``from ibm_fish import FishIBM``, main_fish.py:51-52) through the drop-in modules, called
    as that driver calls them, against the oracle of the same case."""
    fix = np.load(os.path.join(GOLDEN, "dropin_main_moving.npz"))
    cfg_mod, ref = small_fish_config(built_pkg, fix["cfg_M_raw_inv_np"])
    sys.modules["config_fish"] = cfg_mod
    clbm_fish = importlib.import_module("clbm_fish")
    ibm_fish = importlib.import_module("ibm_fish")
    assert clbm_fish.__file__.startswith(COMPAT) and ibm_fish.__file__.startswith(COMPAT)
    assert "config_moving" not in sys.modules   # the alias is only held while loading
    lbm = clbm_fish.CLBMSolver()
    ibm = ibm_fish.FishIBM()
    o = oracle_mod.Oracle(ref.nx, ref.ny, ref.nz, ref.s_v, ref.s_e, ref.ux_in, ref.uy_in,
                          ref.X0, ref.Y0, ref.Z0)
    for step in range(1, 21):
        ms = ref.motion_state(step)
        fx, fy, fz = ibm.compute_force(lbm.ux, lbm.uy, *ms)
        lbm.step(fx, fy, fz)
        o.compute_force(*ms)
        o.lbm_step()
    rho, ux, uy, uz = o.macro()
    o.close()
    got = {n: getattr(lbm, n).to_numpy() for n in FIELDS}
    assert rel_l2(got["rho"], rho) < 1e-5
    assert rel_l2(np.stack([got["ux"], got["uy"], got["uz"]]), np.stack([ux, uy, uz])) < 1e-5
    assert ibm.X_marker.to_numpy().shape == (cfg_mod.N_MARKERS,)
    lbm._solver.close()


def test_dropin_modules_under_a_generated_configuration(built_pkg, dropin_env):
    """config.to_config_module makes any case of this package a ``config_moving``: the
    drop-in CLBMSolver / DroneMovingIBM loaded under the module generated for a small wing,
    called as main_moving.py calls them (compute_force with the host motion law, then step),
    give the bits of Simulation.step_host_motion on the same case."""
    cfg = built_pkg.wing_case(96, 40, 6, 16, name="wing-96x40x6")
    sys.modules["config_moving"] = built_pkg.config.to_config_module(cfg)
    clbm_moving = importlib.import_module("clbm_moving")
    airfoil_moving = importlib.import_module("airfoil_moving")
    assert clbm_moving.__file__.startswith(COMPAT)
    lbm = clbm_moving.CLBMSolver()
    ibm = airfoil_moving.DroneMovingIBM()
    sim = built_pkg.Simulation(cfg)
    for step in range(1, 16):
        fx, fy, fz = ibm.compute_force(lbm.ux, lbm.uy, *cfg.motion_state(step))
        lbm.step(fx, fy, fz)
        sim.step_host_motion(step)
    got = {k: getattr(lbm, k).to_numpy() for k in FIELDS}
    want = sim.solver.read_macro()
    for k in FIELDS:
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    np.testing.assert_array_equal(lbm.f.to_numpy(), sim.solver.read_populations())
    sim.close()
