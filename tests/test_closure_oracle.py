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


def random_params(rng, span=0.6):
    p = np.zeros(2186, np.float32)
    p[0:19] = rng.standard_normal(19) * 1e-4
    p[19:38] = np.exp(rng.uniform(5, 9, 19))
    p[40:1064].reshape(32, 32)[:, :19] = rng.standard_normal((32, 19)) * 0.3
    p[1064:1096] = rng.standard_normal(32) * 0.1
    p[1096:2120] = rng.standard_normal(1024) * 0.2
    p[2120:2152] = rng.standard_normal(32) * 0.1
    p[2152:2184] = rng.standard_normal(32) * 0.3
    p[2184] = 0.05
    p[2185] = span
    return p


def random_samples(rng, n):
    """Features of perturbed equilibria and synthetic targets t = (1 - s*) p + noise."""
    f = np.array([feq(1 + 0.01 * rng.standard_normal(), 0.05 * rng.standard_normal(3)) *
                  (1 + 2e-3 * rng.standard_normal(19)) for _ in range(n)])
    from oracle import oracle
    x = oracle.closure_features(f)
    s_star = 1.0 + 0.5 * np.tanh(200.0 * x[:, 4])
    t = (1.0 - s_star)[:, None] * x[:, 10:19] + 1e-6 * rng.standard_normal((n, 9))
    return np.concatenate([x, t], axis=1)


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


def test_gradient_matches_finite_differences(oracle_mod):
    rng = np.random.default_rng(5)
    p = random_params(rng)
    sm = random_samples(rng, 64)
    wscale = 1.0 / np.mean(np.sum(sm[:, 10:19] ** 2, axis=1))
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


def test_plain_limit(oracle_mod):
    """W3 = b3 = 0 gives s_h = 1: the loss equals sum t^2 and the oracle solver with the
    closure equals the plain one bit for bit."""
    rng = np.random.default_rng(7)
    p = random_params(rng)
    p[2152:2185] = 0.0
    sm = random_samples(rng, 32)
    s = oracle_mod.closure_forward(p, sm[:, :19])
    np.testing.assert_array_equal(s, 1.0)
    loss = oracle_mod.closure_loss_grad(p, sm, 1.0, grad=False)
    assert loss == pytest.approx(np.sum(sm[:, 19:] ** 2), rel=1e-12)
    shape = (12, 6, 4)
    f0 = np.broadcast_to(feq(1.0, np.array([0.04, 0.0, 0.0])), shape + (19,)).copy()
    f0 *= 1 + 1e-3 * rng.standard_normal(f0.shape)
    out = []
    for closure in (None, p):
        o = oracle_mod.Oracle(*shape, 1.6, 1.0, 0.04, 0.0, [], [], [], real="f64")
        o.set_f(f0)
        o.set_closure(closure)
        for _ in range(3):
            o.lbm_step()
        out.append(o.f())
        o.close()
    np.testing.assert_array_equal(out[0], out[1])


def test_closure_changes_the_collision(oracle_mod):
    """With s_h != 1 the third/fourth-order moments survive the collision: the populations
    differ from the plain run by an amount of the order of those moments."""
    rng = np.random.default_rng(8)
    p = random_params(rng, span=0.9)
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
    assert (L.mu, L.sinv, L.W1, L.b1, L.W2, L.b2, L.W3, L.b3, L.span, L.total) == \
        (0, 19, 40, 1064, 1096, 2120, 2152, 2184, 2185, 2186)
    assert L.n_trainable == 2145 and L.n_targets == 9 and L.sample_floats == 28
    from oracle import oracle
    assert oracle.load("f64").oracle_closure_nparams() == L.total
