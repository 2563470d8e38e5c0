"""Output path (frames and meta.npz as main_moving.py writes them) and the reference's
configuration variants (high-Re airplane, fish) through the same API."""

import hashlib
import os

import numpy as np
import pytest

from conftest import load_golden, rel_l2


def _sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_variant_geometries_bit_identical(pkg):
    g = load_golden("geometry")
    hre = pkg.highre_airplane_case()
    assert hre.n_markers == int(g["highre_n"]) and _sha(hre.X0, hre.Y0, hre.Z0) == str(g["highre_sha"])
    fish = pkg.fish_case()
    assert fish.n_markers == int(g["fish_n"]) and _sha(fish.X0, fish.Y0, fish.Z0) == str(g["fish_sha"])


def test_grid_meta_order_matches_reference_driver(pkg):
    cfg = pkg.reference_airplane_case()
    gm = pkg.driver.grid_meta(cfg, 200, cfg.geometry)
    # main_moving.py:185-198 order
    want = [600, 200, 160, 0.05, 200, 160.0, 100.0, 80.0, 75.0, 10.0, 60, 20.0, 140.0, 80.0,
            160.0, 200, 10.0, 80.0, 36.0, 32.0, 48.0, 112.0, 36.0, 28.0]
    np.testing.assert_allclose(gm, want)
    assert gm.dtype == np.float64 and len(gm) == 24


@pytest.mark.gpu
def test_vorticity_slice_matches_numpy_gradient(built_pkg):
    """Device z-vorticity against render_2d.py's formula applied to the exported fields."""
    pkg = built_pkg
    cfg = pkg.wing_case(64, 32, 6, 10.0, re=30.0)
    sim = pkg.Simulation(cfg)
    sim.run(25)
    m = sim.solver.read_macro()
    for z in (0, 3, 5):
        want = (np.gradient(m["ux"][:, :, z], 1.0, axis=1)
                - np.gradient(m["uy"][:, :, z], 1.0, axis=0))
        got = sim.solver.read_vorticity(z)
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-7)
    k, p = pkg.analysis.wake_vorticity_spectrum(sim.solver.read_vorticity(), cfg.chord, 30)
    assert k[0] == 0 and np.all(np.isfinite(p))
    sim.close()


@pytest.mark.gpu
def test_driver_frames_and_meta_match_oracle(built_pkg, oracle_mod, tmp_path):
    pkg = built_pkg
    cfg = pkg.wing_case(48, 24, 4, 8.0, re=20.0)
    lines = []
    res = pkg.driver.run(cfg, 30, 10, str(tmp_path), graph=True, log=lines.append)
    assert res["frames"] == 3 and not res["diverged"] and len(lines) == 3
    ref = oracle_mod.Oracle(cfg.nx, cfg.ny, cfg.nz, cfg.s_v, cfg.s_e, cfg.ux_in, cfg.uy_in,
                            cfg.X0, cfg.Y0, cfg.Z0)
    hist = []
    for k in range(1, 4):
        hist.append(ref.run(10 * (k - 1), 10, cfg.motion()))
        fr = np.load(os.path.join(tmp_path, f"frame_{k:06d}.npz"))
        assert sorted(fr.files) == sorted(pkg.driver.FRAME_KEYS)
        want = dict(zip(("rho", "ux", "uy", "uz"), ref.macro()))
        for key in ("rho", "ux", "uy"):
            assert fr[key].dtype == np.float32 and fr[key].shape == (48, 24, 4)
            assert rel_l2(fr[key], want[key]) < 1e-5, (k, key)
    meta = np.load(os.path.join(tmp_path, "meta.npz"))
    assert sorted(meta.files) == sorted(pkg.driver.META_KEYS)
    np.testing.assert_array_equal(meta["step"], [10, 20, 30])
    assert meta["grid_meta"].shape == (24,)
    forces = np.load(os.path.join(tmp_path, "forces.npz"))
    assert forces["sums"].shape == (30, 4)
    assert rel_l2(forces["sums"], np.concatenate(hist)) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [True, False])
def test_runs_that_diverge_are_reported_not_raised(built_pkg, tmp_path, graph):
    """A case that diverges within a few hundred steps (64x32x4, Re 1e5, U = 0.2: s_v
    within 2e-4 of 2; the float32 oracle's density leaves [0.3, inf) by step 150): the
    collisions' divergence monitor stops the steps, and the output driver and the study
    drivers report the divergence with the step it was found at, as main_moving.py:143-145
    does, instead of raising."""
    from importlib import import_module
    pkg = built_pkg
    cfg = pkg.wing_case(64, 32, 4, 8, re=1e5, u_inf=0.2, name="diverging")
    out = pkg.driver.run(cfg, 2000, 100, str(tmp_path), graph=graph, log=lambda m: None)
    assert out["diverged"] and out["steps"] < 2000
    study = import_module(pkg.__name__ + ".closure_study")
    sim = pkg.Simulation(cfg)
    wall, done, bad = study._run(sim, 2000, 200)
    sim.close()
    assert bad is not None and done < 2000 and "rho_min" in bad
