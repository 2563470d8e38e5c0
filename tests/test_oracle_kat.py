"""Known-answer tests of the oracle's physics, including the reference quirks the GPU path
reproduces (inlet momentum 4/3 rho u_in, Peskin weights of wrapped stencil nodes,
net Guo momentum (3 - s_v)/2 F)."""

import numpy as np

from conftest import rel_l2


def _feq(ux, uy, uz=0.0):
    ex = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0], np.float64)
    ey = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1], np.float64)
    ez = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1], np.float64)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    eu = ex * ux + ey * uy + ez * uz
    u2 = ux * ux + uy * uy + uz * uz
    return w * (1 + 3 * eu + 4.5 * eu * eu - 1.5 * u2), ex, ey, ez


def test_minv_entries_are_exact_dyadic(oracle_mod):
    o = oracle_mod.Oracle(4, 3, 3, 1.5, 1.0, 0.0, 0.0, [], [], [])
    m = o.minv().astype(np.float64)
    assert set(np.unique(m * 4).tolist()) <= {-4.0, -2.0, -1.0, 0.0, 1.0, 2.0, 4.0}
    assert int((m != 0).sum()) == 91


def test_rest_state_is_fixed_point(oracle_mod):
    o = oracle_mod.Oracle(8, 5, 4, 1.4, 1.0, 0.0, 0.0, [], [], [])
    f0 = o.f().copy()
    for _ in range(5):
        o.lbm_step()
    assert np.max(np.abs(o.f() - f0)) < 2e-7


def test_inlet_injects_four_thirds_momentum(oracle_mod):
    # Zou-He with the reference's coefficients (clbm_moving.py:288-294) gives
    # sum_q e_x f_q = 4/3 rho_in u_in at x = 0.
    o = oracle_mod.Oracle(8, 4, 3, 1.2, 1.0, 0.04, 0.01, [], [], [], real="f64")
    o.lbm_step()
    f = o.f()[0]
    _, ex, ey, ez = _feq(0, 0)
    rho_known = f[..., [0, 3, 4, 5, 6, 15, 16, 17, 18]].sum(-1)
    rho_out = f[..., [2, 8, 10, 12, 14]].sum(-1)
    rho_in = (rho_known + 2 * rho_out) / (1 - 0.04)
    mx = (f * ex).sum(-1)
    np.testing.assert_allclose(mx, 4.0 / 3.0 * rho_in * 0.04, rtol=1e-12)


def test_guo_net_momentum(oracle_mod):
    # one step from rest under a uniform force F: interior momentum per cell is
    # m + F/2 + (1 - s_v/2) F = (3 - s_v)/2 F   (clbm_moving.py:113-115, :200-202, :240-249)
    nx, ny, nz, s_v = 10, 4, 4, 1.3
    o = oracle_mod.Oracle(nx, ny, nz, s_v, 1.0, 0.0, 0.0, [], [], [], real="f64")
    F = (1e-4, -2e-4, 5e-5)
    o.set_forces(*[np.full((nx, ny, nz), v) for v in F])
    o.lbm_step()
    f = o.f()[2:nx - 2]
    _, ex, ey, ez = _feq(0, 0)
    for e, Fc in zip((ex, ey, ez), F):
        np.testing.assert_allclose((f * e).sum(-1), (3.0 - s_v) / 2.0 * Fc, rtol=1e-9)


def _markers_at(zs, y=6.3, x=10.4):
    X = np.array([0.0] * len(zs), np.float32)
    Y = np.array([0.0] * len(zs), np.float32)
    return X, Y, np.array(zs, np.float32), (x, y)


def test_peskin_partition_of_unity_and_seam_weights(oracle_mod):
    # uniform velocity u_in: interpolated U_k = u_in * sum(phi); sum(phi) = 1 away from the
    # periodic seam and 3/4 on the first and last z layers, where the reference evaluates
    # the weight at the wrapped node index (airfoil_moving.py:161-165).
    nz = 6
    X, Y, Z, (xc, yc) = _markers_at([0.0, 1.0, 2.5, 3.0, 5.0])
    o = oracle_mod.Oracle(24, 14, nz, 1.2, 1.0, 0.05, 0.0, X, Y, Z, real="f64")
    o.compute_force(xc, yc, 0.0, 0.0, 0.0, 0.0)
    uk = o.markers()["Uk"]
    np.testing.assert_allclose(uk / 0.05, [0.75, 1.0, 1.0, 1.0, 0.75], rtol=1e-12)


def test_spreading_conserves_force_before_clip(oracle_mod):
    X, Y, Z, (xc, yc) = _markers_at([1.0, 2.0, 2.25, 3.0])
    o = oracle_mod.Oracle(24, 14, 6, 1.2, 1.0, 0.01, 0.0, X, Y, Z, real="f64")
    o.compute_force(xc, yc, 0.0, 0.0, 0.0, 0.0)
    s = o.body_force()
    np.testing.assert_allclose(s[0], s[2], rtol=1e-12)
    np.testing.assert_allclose(s[2], -0.01 * 4, rtol=1e-12)


def test_f32_and_f64_oracles_agree_on_short_run(oracle_mod, pkg):
    cfg = pkg.wing_case(48, 24, 4, 8.0, re=20.0)
    runs = {}
    for real in ("f32", "f64"):
        o = oracle_mod.Oracle(cfg.nx, cfg.ny, cfg.nz, cfg.s_v, cfg.s_e, cfg.ux_in, cfg.uy_in,
                              cfg.X0, cfg.Y0, cfg.Z0, real=real)
        hist = o.run(0, 20, cfg.motion())
        runs[real] = (o.macro(), hist)
    (r32, u32, v32, w32), (r64, u64, v64, w64) = runs["f32"][0], runs["f64"][0]
    for a, b in ((r32, r64), (u32, u64), (v32, v64)):
        assert rel_l2(a, b) < 1e-5
    assert np.max(np.abs(w32 - w64)) < 1e-6   # uz is round-off around zero
    assert rel_l2(runs["f32"][1], runs["f64"][1]) < 1e-4
