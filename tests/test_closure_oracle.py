"""CPU checks of the learned-closure oracle (oracle/closure_oracle.c): analytic gradient
against finite differences, the plain limit s_h = 1, the direct central-moment features
against an independent NumPy form, and the parameter layout against the library's."""

import numpy as np
import pytest

from conftest import rel_l2

EX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
EY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
EZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
PQR = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1), (2, 0, 0),
       (0, 2, 0), (0, 0, 2), (2, 1, 0), (1, 2, 0), (2, 0, 1), (0, 2, 1), (1, 0, 2), (0, 1, 2),
       (2, 2, 0), (2, 0, 2), (0, 2, 2)]


def feq(rho, u):
    eu = EX * u[0] + EY * u[1] + EZ * u[2]
    return rho * W * (1 + 3 * eu + 4.5 * eu ** 2 - 1.5 * (u @ u))


def random_params(rng, span=0.6, mode=0, nu=0.005):
    p = np.zeros(2188, np.float32)
    p[0:19] = rng.standard_normal(19) * 1e-4
    p[19:38] = np.exp(rng.uniform(5, 9, 19))
    p[40:1064].reshape(32, 32)[:, :19] = rng.standard_normal((32, 19)) * 0.3
    p[1064:1096] = rng.standard_normal(32) * 0.1
    p[1096:2120] = rng.standard_normal(1024) * 0.2
    p[2120:2152] = rng.standard_normal(32) * 0.1
    p[2152:2184] = rng.standard_normal(32) * 0.3
    p[2184] = 0.05
    p[2185] = span
    p[2186] = mode
    p[2187] = nu
    return p


def random_samples(rng, n):
    """Features of perturbed equilibria with synthetic targets whose ideal closure depends
    on one feature z: nine higher-order targets t = (1 - s*) p (s* = 1 + tanh(z) / 2), then
    tau = -2 nu_t* S over five deviatoric components with a random strain rate S and
    nu_t* = nu (2^(1.5 max(tanh(z), 0)) - 1), nu = 0.005."""
    f = np.array([feq(1 + 0.01 * rng.standard_normal(), 0.05 * rng.standard_normal(3)) *
                  (1 + 2e-3 * rng.standard_normal(19)) for _ in range(n)])
    from oracle import oracle
    x = oracle.closure_features(f)
    z4 = x[:, 4] / x[:, 4].std()
    z5 = x[:, 5] / x[:, 5].std()
    s_star = 1.0 + 0.5 * np.tanh(z4)
    t = (1.0 - s_star)[:, None] * x[:, 10:19] + 1e-8 * rng.standard_normal((n, 9))
    S = 1e-3 * rng.standard_normal((n, 5))
    nut = 0.005 * (2.0 ** (1.5 * np.maximum(np.tanh(z5), 0.0)) - 1.0)
    tau = -2.0 * nut[:, None] * S + 1e-9 * rng.standard_normal((n, 5))
    return np.concatenate([x, t, tau, S], axis=1)


def test_features_match_numpy(oracle_mod):
    rng = np.random.default_rng(3)
    f = np.array([feq(1 + 0.02 * rng.standard_normal(), 0.08 * rng.standard_normal(3)) *
                  (1 + 0.01 * rng.standard_normal(19)) for _ in range(20)])
    x = oracle_mod.closure_features(f)
    for c in range(20):
        r = f[c].sum()
        u = np.array([EX @ f[c], EY @ f[c], EZ @ f[c]]) / r
        want = np.array([np.sum(f[c] * (EX - u[0]) ** p * (EY - u[1]) ** q * (EZ - u[2]) ** s)
                         for p, q, s in PQR])
        want[0] -= r
        want[7:10] -= r / 3
        want[16:19] -= r / 9
        np.testing.assert_allclose(x[c], want / r, rtol=1e-9, atol=1e-14)
    # equilibrium at rest: first four features vanish, second/fourth-order equal zero
    x0 = oracle_mod.closure_features(feq(1.0, np.zeros(3))[None])
    np.testing.assert_allclose(x0[0], 0.0, atol=1e-15)


def loss_scale(sm, mode):
    p = sm[:, 28:33] if mode == 1 else sm[:, 10:19]
    return 1.0 / np.mean(np.sum(p ** 2, axis=1))


@pytest.mark.parametrize("mode", [0, 1])
def test_gradient_matches_finite_differences(oracle_mod, mode):
    rng = np.random.default_rng(5)
    p = random_params(rng, mode=mode, span=0.6 if mode == 0 else 1.5)
    sm = random_samples(rng, 64)
    wscale = loss_scale(sm, mode)
    loss, g = oracle_mod.closure_loss_grad(p, sm, wscale, round_bf16=False)
    assert np.isfinite(loss) and np.linalg.norm(g) > 0
    # central differences in double through the float32 parameter array: perturb by
    # steps the float32 grid represents exactly and divide by the realised step
    idx = list(rng.choice(np.arange(0, 1024), 6)) + [1024 + 3, 1056 + 77, 2080 + 5, 2112 + 9, 2144]
    for j in idx:
        k = 40 + j
        base = float(p[k])
        h = max(abs(base), 1e-2) * 2e-3
        pp, pm = p.copy(), p.copy()
        pp[k] = np.float32(base + h)
        pm[k] = np.float32(base - h)
        lp = oracle_mod.closure_loss_grad(pp, sm, wscale, round_bf16=False, grad=False)
        lm = oracle_mod.closure_loss_grad(pm, sm, wscale, round_bf16=False, grad=False)
        fd = (lp - lm) / (float(pp[k]) - float(pm[k])) / len(sm)
        if (j < 1024) and (j % 32) >= 19:
            continue
        assert abs(fd - g[j]) <= 2e-4 * max(abs(g[j]), 1e-3 * np.abs(g).max()), (j, fd, g[j])


@pytest.mark.parametrize("mode", [0, 1])
def test_plain_limit(oracle_mod, mode):
    """W3 = b3 = 0 gives the plain rates (s_h = 1; s_eff = s_v): the loss is that of the
    plain method and the oracle solver with the closure equals the plain one bit for bit."""
    rng = np.random.default_rng(7)
    s_v = 1.6
    nu = (1.0 / s_v - 0.5) / 3.0
    p = random_params(rng, mode=mode, nu=nu)
    p[2152:2185] = 0.0
    sm = random_samples(rng, 32)
    s = oracle_mod.closure_forward(p, sm[:, :19])
    np.testing.assert_allclose(s, 1.0 if mode == 0 else 1.0 / (0.5 + 3.0 * float(np.float32(nu))), rtol=1e-12)
    loss = oracle_mod.closure_loss_grad(p, sm, 1.0, grad=False)
    want = np.sum(sm[:, 19:28] ** 2) if mode == 0 else np.sum(sm[:, 28:33] ** 2)
    assert loss == pytest.approx(want, rel=1e-12)
    shape = (12, 6, 4)
    f0 = np.broadcast_to(feq(1.0, np.array([0.04, 0.0, 0.0])), shape + (19,)).copy()
    f0 *= 1 + 1e-3 * rng.standard_normal(f0.shape)
    out = []
    for closure in (None, p):
        o = oracle_mod.Oracle(*shape, s_v, 1.0, 0.04, 0.0, [], [], [], real="f64")
        o.set_f(f0)
        o.set_closure(closure)
        for _ in range(3):
            o.lbm_step()
        out.append(o.f())
        o.close()
    if mode == 0:
        np.testing.assert_array_equal(out[0], out[1])
    else:   # s_v through the viscosity and back: equal to rounding
        np.testing.assert_allclose(out[1], out[0], rtol=0, atol=1e-14)


@pytest.mark.parametrize("mode", [0, 1])
def test_closure_changes_the_collision(oracle_mod, mode):
    """With rates other than the plain ones the populations differ from the plain run by
    an amount of the order of the moments the closure acts on."""
    rng = np.random.default_rng(8)
    p = random_params(rng, span=0.9 if mode == 0 else 1.5, mode=mode, nu=(1 / 1.6 - 0.5) / 3)
    shape = (12, 6, 4)
    f0 = np.broadcast_to(feq(1.0, np.array([0.04, 0.0, 0.0])), shape + (19,)).copy()
    f0 *= 1 + 1e-3 * rng.standard_normal(f0.shape)
    out = []
    for closure in (None, p):
        o = oracle_mod.Oracle(*shape, 1.6, 1.0, 0.04, 0.0, [], [], [], real="f64")
        o.set_f(f0)
        o.set_closure(closure)
        o.lbm_step()
        out.append(o.f())
        o.close()
    d = rel_l2(out[1] - W, out[0] - W)
    assert 1e-4 < d < 1.0, d


def test_layout_matches_library(built_pkg, oracle_mod):
    L = built_pkg.closure.Layout()
    assert (L.mu, L.sinv, L.W1, L.b1, L.W2, L.b2, L.W3, L.b3, L.span, L.mode, L.nu, L.total) == \
        (0, 19, 40, 1064, 1096, 2120, 2152, 2184, 2185, 2186, 2187, 2188)
    assert L.n_trainable == 2145 and L.n_targets == 9 and L.n_sgs == 10
    assert L.sample_floats == 38 and L.n_stats == 40
    from oracle import oracle
    assert oracle.load("f64").oracle_closure_nparams() == L.total


def test_filter_matches_numpy(oracle_mod):
    rng = np.random.default_rng(9)
    ff = np.broadcast_to(feq(1.0, np.array([0.04, 0.01, 0.0])), (8, 6, 4, 19)).copy()
    ff *= 1 + 1e-2 * rng.standard_normal(ff.shape)
    out = oracle_mod.closure_filter(ff)
    blk = ff.reshape(4, 2, 3, 2, 2, 2, 19)
    np.testing.assert_allclose(out[..., :19], blk.mean(axis=(1, 3, 5)), rtol=1e-13)
    r = ff.sum(-1)
    u = np.stack([ff @ EX, ff @ EY, ff @ EZ], -1) / r[..., None]
    ub = u.reshape(4, 2, 3, 2, 2, 2, 3).mean(axis=(1, 3, 5))
    np.testing.assert_allclose(out[..., 19:22], ub, rtol=1e-12)
    prod = np.stack([u[..., 0] ** 2, u[..., 1] ** 2, u[..., 2] ** 2, u[..., 0] * u[..., 1],
                     u[..., 0] * u[..., 2], u[..., 1] * u[..., 2]], -1)
    np.testing.assert_allclose(out[..., 22:28], prod.reshape(4, 2, 3, 2, 2, 2, 6).mean(axis=(1, 3, 5)),
                               rtol=1e-10, atol=1e-18)
