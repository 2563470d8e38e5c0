"""Marker geometry and case configuration against the reference's config module
(golden_geometry.npz is generated from config_moving.py itself)."""

import hashlib
import math

import numpy as np

from conftest import load_golden


def _sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_airplane_markers_bit_identical(pkg):
    g = load_golden("geometry")
    X, Y, Z = pkg.config.airplane_markers()
    assert len(X) == int(g["airplane_n"]) == 74201
    assert _sha(X, Y, Z) == str(g["airplane_sha"])
    np.testing.assert_array_equal(np.stack([X[::97], Y[::97], Z[::97]]), g["airplane_sample"])


def test_sections_and_fills_bit_identical(pkg):
    g = load_golden("geometry")
    for key in g.files:
        if key.startswith("naca_"):
            chord, ds = key.split("_")[1:]
            ds = float(ds[0] + "." + ds[1:])
            X, Y = pkg.config.naca0012_section(int(chord), ds)
            np.testing.assert_array_equal(np.stack([X, Y]), g[key])
    assert _sha(*pkg.config.naca0012_interior(80, 0.7)) == str(g["interior_80_07_sha"])
    assert _sha(*pkg.config.ellipsoid_markers(75.0, 10.0, 10.0, 0.7)) == str(g["ellipsoid_sha"])


def test_benchmark_cases(pkg):
    c0, c1 = pkg.small_case(), pkg.full_case()
    assert (c0.nx, c0.ny, c0.nz, c0.n_markers) == (200, 80, 16, 102 * 16)
    assert (c1.nx, c1.ny, c1.nz, c1.n_markers) == (600, 200, 50, 252 * 50)
    assert math.isclose(c1.nu, 0.05 * 80 / 200)
    assert math.isclose(c1.s_v, 1.0 / (0.5 + 3 * c1.nu))
    # omega = 2 k U / c
    assert math.isclose(c1.omega_motion, 2 * 0.5 * 0.05 / 80)
    # pivot at quarter chord: the leading edge sits c/4 ahead of the pivot
    assert math.isclose(float(c1.X0.min()), -20.0, abs_tol=1e-4)
    assert math.isclose(float(c1.X0.max()), 60.0, abs_tol=1e-4)
    # theta(t) = 8 deg + 10 deg sin(w t + 90 deg), h = 0.25 c sin(w t)
    xc, yc, th, vx, vy, om = c1.motion_state(0)
    assert math.isclose(th, math.radians(18.0)) and math.isclose(yc, 100.0)
    assert (c1.ux_in, c1.uy_in) == (0.05, 0.0)


def test_reference_case_matches_config_module(pkg):
    c = pkg.reference_airplane_case()
    assert c.n_markers == 74201 and (c.nx, c.ny, c.nz) == (600, 200, 160)
    assert math.isclose(c.ux_in, 0.05 * math.cos(math.radians(8)))
    assert math.isclose(c.uy_in, -0.05 * math.sin(math.radians(8)))


def test_force_coefficients(pkg):
    cfg = pkg.full_case()
    q = 0.5 * 0.05 ** 2 * 80 * 50
    sums = np.array([[-2.0 * q, -3.0 * q, -2.0 * q, -3.0 * q]])
    c = pkg.force_coefficients(sums, cfg)
    np.testing.assert_allclose([c["cd"][0], c["cl"][0]], [2.0, 3.0])
    np.testing.assert_allclose([c["cd_m"][0], c["cl_m"][0]], [2.0, 3.0])
