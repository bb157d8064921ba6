"""The CPU restatement of the MLP surrogate: analytic gradient against finite
differences (float64, no BF16 rounding), conservation of the closure, and the
untrained network reducing to the Roe f-wave solver."""
import numpy as np

import surrogate as S


def edges(n, seed):
    rng = np.random.default_rng(seed)
    hL = rng.uniform(0.5, 20.0, n)
    hR = hL * rng.uniform(0.5, 1.5, n)
    huL = hL * rng.normal(0, 2.0, n)
    huR = hR * rng.normal(0, 2.0, n)
    bL = rng.normal(-5, 1.0, n)
    bR = bL + rng.normal(0, 0.3, n)
    return [a.astype(np.float32) for a in (hL, hR, huL, huR, bL, bR)]


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = S.init_params(3)
    P = S.unpack(p)
    P["W4"] = rng.normal(0, 0.2, P["W4"].shape)
    P["b4"] = rng.normal(0, 0.1, 4)
    p = S.pack(P, np.float64)
    e = edges(64, 2)
    t = [rng.normal(0, 1.0, 64) for _ in range(4)]
    loss, g = S.loss_and_grad(p, e, t, rounding=False)
    idx = rng.choice(S.N_PARAMS, 40, replace=False)
    for i in idx:
        h = 1e-6 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        num = (S.loss_and_grad(pp, e, t, rounding=False)[0] - S.loss_and_grad(pm, e, t, rounding=False)[0]) / (2 * h)
        assert abs(num - g[i]) <= 1e-5 * max(abs(num), 1e-2 * np.abs(g).max()), (i, num, g[i])


def test_closure_conserves_the_flux_difference():
    p = S.init_params(5)
    e = edges(200, 4)
    x, aux = S.features(*e)
    o, _ = S.forward(p, x)
    o = o + np.random.default_rng(0).normal(0, 0.3, o.shape).astype(np.float32)
    W = S.waves(o.astype(np.float64), aux)
    # the two waves sum to the flux difference: h updates to dF1, hu updates to dF2
    assert np.allclose(W["U"][:, 0] + W["U"][:, 1], aux["dF1"], rtol=1e-9, atol=1e-6)
    assert np.allclose(W["U"][:, 2] + W["U"][:, 3], aux["dF2"], rtol=1e-8, atol=1e-4)


def test_untrained_network_is_the_roe_fwave_solver():
    p = S.init_params(7)  # last layer zero
    e = edges(100, 6)
    x, aux = S.features(*e)
    o, _ = S.forward(p, x)
    assert np.all(o == 0)
    W = S.waves(o.astype(np.float64), aux)
    assert np.allclose(W["s1"], aux["s10"]) and np.allclose(W["s2"], aux["s20"])
