"""The drop-in modules under the reference's own drivers, on the CPU.

main_moving.py and main_highRe.py (which selects its configuration by aliasing it as
``config_moving`` in ``sys.modules``, main_highRe.py:26-27) are imported from the reference
checkout unmodified and their ``main()`` runs with this project's ``taichi``,
``clbm_moving`` and ``airfoil_moving`` modules (``compat/``). Without a GPU, the drop-in
modules' package calls are answered by the CPU oracle (tests/golden/oracle_backend.py).
The frames and meta.npz the drivers write must equal, bit for bit, those the same drivers
write with the reference's own solver modules (run on the Taichi emulator), and the calls
the drop-in modules make must equal the committed trace that tests/test_gpu_dropin.py
replays on the GPU. These tests need the reference checkout and are skipped without it.
"""

import importlib.util
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

REF_DIR = os.environ.get("CLBM_REFERENCE_DIR", "/root/reference")
COMPAT = os.path.join(ROOT, "clbm_ibm-moving-airfoil_gb300", "compat")
DRIVERS = ("main_moving", "main_highRe")

needs_reference = pytest.mark.skipif(not os.path.exists(os.path.join(REF_DIR, "main_moving.py")),
                                     reason="reference checkout not present")


def _make_dropin():
    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)
    import make_dropin
    return make_dropin


@pytest.fixture(autouse=True)
def _restore_modules():
    saved = dict(sys.modules)
    path = list(sys.path)
    yield
    for name in list(sys.modules):
        if name not in saved:
            del sys.modules[name]
    sys.modules.update(saved)
    sys.path[:] = path


@needs_reference
@pytest.mark.parametrize("driver", DRIVERS)
def test_reference_driver_runs_unmodified_through_dropin_modules(driver):
    md = _make_dropin()
    fix = np.load(os.path.join(GOLDEN, f"dropin_{driver}.npz"))
    got, trace, config = md.run_dropin(REF_DIR, driver)
    # the driver's own outputs: every frame and every meta.npz entry, bit for bit
    assert int(got["n_frames"]) == int(fix["n_frames"]) >= 3
    for key in fix.files:
        if key.startswith(("frame", "meta_")):
            assert np.array_equal(got[key], fix[key]), key
    assert sorted(got["meta_keys"]) == ["X_htail_tmpl", "X_template", "Y_htail_tmpl",
                                        "Y_template", "grid_meta", "step", "theta", "xc", "yc"]
    # the calls the drop-in modules made: the trace the GPU test replays
    kind, args, field = md.encode_trace(trace)
    assert np.array_equal(kind, fix["trace_kind"])
    assert np.array_equal(args, fix["trace_args"])
    assert np.array_equal(field, fix["trace_field"])
    for k, v in config.items():
        assert np.array_equal(v, fix[k]), k


@needs_reference
def test_fixture_frames_are_the_reference_solver_output():
    """The committed frames are what main_moving.py writes with the reference's own
    clbm_moving / airfoil_moving kernels (Taichi emulator)."""
    md = _make_dropin()
    fix = np.load(os.path.join(GOLDEN, "dropin_main_moving.npz"))
    ref = md.run_reference(REF_DIR, "main_moving")
    for key, v in ref.items():
        assert np.array_equal(np.asarray(v), fix[key]), key


def test_taichi_shim_has_no_cpu_backend():
    spec = importlib.util.spec_from_file_location("_compat_taichi_probe",
                                                  os.path.join(COMPAT, "taichi", "__init__.py"))
    ti = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ti)
    # main_moving.py:34-37 falls back to ti.init(arch=ti.cpu): here that is an error
    with pytest.raises(RuntimeError):
        ti.init(arch=ti.cpu, default_fp=ti.f32, default_ip=ti.i32, cpu_max_num_threads=8)


def test_trace_fixtures_are_consistent():
    """Per fixture: one compute_force and one step per time step, four field reads per
    written frame, and the motion arguments of main_moving.py:_motion_state."""
    for driver in DRIVERS:
        fix = np.load(os.path.join(GOLDEN, f"dropin_{driver}.npz"))
        kind = fix["trace_kind"]
        n = int(fix["n_steps"])
        assert (kind == 0).sum() == n and (kind == 1).sum() == n
        assert (kind == 2).sum() == 4 * int(fix["n_frames"])
        assert int(fix["n_frames"]) == n // int(fix["vis_interval"])
        steps = fix["meta_step"]
        assert np.array_equal(steps, np.arange(1, len(steps) + 1) * int(fix["vis_interval"]))


def test_fish_dropin_modules_load_under_their_configuration(tmp_path, monkeypatch):
    """fish/main_fish.py imports ``clbm_fish.CLBMSolver`` and ``ibm_fish.FishIBM``, which read
    ``config_fish``: the drop-in modules load the clbm_moving / airfoil_moving drop-ins with
    that module standing in for ``config_moving`` and remove the alias afterwards."""
    import types
    import numpy as np
    cfg = types.ModuleType("config_fish")
    X = np.arange(12, dtype=np.float32)
    cfg.Nx, cfg.Ny, cfg.Nz, cfg.cs2, cfg.s_v, cfg.s_e, cfg.s_q, cfg.s_pi = 32, 16, 2, 1 / 3, 1.5, 1.0, 1.0, 1.0
    cfg.U_inf, cfg.AoA0_deg, cfg.M_raw_inv_np = 0.05, 0.0, np.eye(19)
    cfg.N_MARKERS_2D, cfg.N_MARKERS = 6, 12
    cfg.X_marker_np, cfg.Y_marker_np, cfg.Z_marker_np = X, X, X
    saved = dict(sys.modules)
    try:
        for name in ("clbm_fish", "ibm_fish", "config_fish", "config_moving", "_variant",
                     "_clbm_gb300_pkg"):
            sys.modules.pop(name, None)
        monkeypatch.syspath_prepend(COMPAT)
        sys.modules["config_fish"] = cfg
        import clbm_fish
        import ibm_fish
        assert clbm_fish.__file__.startswith(COMPAT) and ibm_fish.__file__.startswith(COMPAT)
        assert isinstance(clbm_fish.CLBMSolver, type) and isinstance(ibm_fish.FishIBM, type)
        assert ibm_fish.N == 12
        assert "config_moving" not in sys.modules
    finally:
        for name in list(sys.modules):
            if name not in saved:
                del sys.modules[name]
        sys.modules.update(saved)
