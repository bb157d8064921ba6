"""MLP surrogate on the tensor cores against its CPU restatement
(oracle/surrogate.py): the GEMM readings the kernels use, forward outputs,
loss and gradient, the solve with its augmented-solver fallback, and Adam
training that must bring the surrogate closer to the augmented Riemann solver
than the f-wave solver it starts from.

Tolerances: the network runs BF16 operands with FP32 accumulation on both
sides, but the device's SiLU uses the hardware tanh (relative error about
2^-11) and accumulates in another order, so a BF16 rounding of an activation
can land one unit apart; outputs agree to about 1e-2 relative, gradients to a
cosine above 0.999 and, element by element, to 1e-3 of each parameter
block's largest entry (measured: about 1e-5)."""
import numpy as np
import pytest

import surrogate as S

pytestmark = pytest.mark.gpu


def bf16(x):
    return S.bf16(x)


def wet_edges(n, seed, spread=0.3):
    rng = np.random.default_rng(seed)
    hL = rng.uniform(0.5, 30.0, n)
    hR = hL * np.exp(rng.normal(0, spread, n))
    huL = hL * rng.normal(0, 2.0, n)
    huR = hR * rng.normal(0, 2.0, n)
    bL = rng.normal(-20, 5.0, n)
    bR = bL + rng.normal(0, 0.5, n)
    return np.stack([hL, hR, huL, huR, bL, bR]).astype(np.float32)


def random_params(seed, scale=0.3):
    rng = np.random.default_rng(seed)
    p = S.init_params(seed)
    P = S.unpack(p)
    P["W4"] = rng.normal(0, scale, P["W4"].shape).astype(np.float32)
    P["b4"] = rng.normal(0, 0.05, 4).astype(np.float32)
    for b in ("b1", "b2", "b3"):
        P[b] = rng.normal(0, 0.1, P[b].shape).astype(np.float32)
    return S.pack(P)


# ---------------------------------------------------------------------------
# the tensor-core operand readings
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("n,k", [(16, 16), (64, 16), (64, 64), (128, 32), (16, 64)])
def test_tc_gemm_kmajor(swe, n, k):
    rng = np.random.default_rng(n * 100 + k)
    a = rng.normal(size=(128, k)).astype(np.float32)
    b = rng.normal(size=(n, k)).astype(np.float32)
    d = swe.tc_gemm_check(a, b, mode=0)
    ref = bf16(a).astype(np.float64) @ bf16(b).astype(np.float64).T
    assert np.allclose(d, ref, rtol=1e-5, atol=1e-4), np.abs(d - ref).max()


@pytest.mark.parametrize("w1,w2", [(64, 64), (64, 16), (16, 64), (16, 16), (32, 48)])
def test_tc_gemm_weight_gradient_reading(swe, w1, w2):
    """D = X^T Y with K over the 128 stored rows: how dW = dZ^T A is formed"""
    rng = np.random.default_rng(w1 * 7 + w2)
    x = rng.normal(size=(128, w1)).astype(np.float32)
    y = rng.normal(size=(128, w2)).astype(np.float32)
    d = swe.tc_gemm_check(x, y, mode=1)[:w1]
    ref = bf16(x).astype(np.float64).T @ bf16(y).astype(np.float64)
    assert np.allclose(d, ref, rtol=1e-5, atol=1e-3), np.abs(d - ref).max()


@pytest.mark.parametrize("w1,w2", [(64, 64), (16, 64), (64, 16), (32, 32)])
def test_tc_gemm_data_gradient_reading(swe, w1, w2):
    """D = X Y with Y stored as [K rows x N]: how dA = dZ W is formed"""
    rng = np.random.default_rng(w1 * 11 + w2)
    x = rng.normal(size=(128, w1)).astype(np.float32)
    y = rng.normal(size=(w1, w2)).astype(np.float32)
    d = swe.tc_gemm_check(x, y, mode=2)
    ref = bf16(x).astype(np.float64) @ bf16(y).astype(np.float64)
    assert np.allclose(d, ref, rtol=1e-5, atol=1e-3), np.abs(d - ref).max()


# ---------------------------------------------------------------------------
# network
# ---------------------------------------------------------------------------
def test_params_round_trip_and_initial_state(swe):
    m = swe.Surrogate(seed=5)
    p = m.params
    P = S.unpack(p)
    assert np.all(P["W4"] == 0) and np.all(P["b4"] == 0) and np.all(P["b1"] == 0)
    lim = np.sqrt(6.0 / (64 + 6))
    # U(-lim, lim) has standard deviation lim / sqrt(3)
    assert np.abs(P["W1"]).max() <= lim and P["W1"].std() > 0.4 * lim
    q = random_params(3)
    m.params = q
    assert np.array_equal(m.params, q)
    m.close()


@pytest.mark.parametrize("n", [1, 127, 128, 5000])
def test_forward_matches_oracle(swe, n):
    e = wet_edges(n, 10 + n)
    p = random_params(4)
    m = swe.Surrogate()
    m.params = p
    out = m.forward(e).T
    m.close()
    x, _ = S.features(*e)
    ref, _ = S.forward(p, x)
    scale = np.sqrt(np.mean(ref ** 2, axis=0))
    err = np.abs(out - ref) / scale
    assert np.median(err) < 2e-3, np.median(err)
    assert err.max() < 3e-2, err.max()


def test_loss_and_gradient_match_oracle(swe):
    n = 3000
    e = wet_edges(n, 21)
    rng = np.random.default_rng(22)
    p = random_params(6, scale=0.1)
    x, aux = S.features(*e)
    o, _ = S.forward(p, x)
    W = S.waves(o.astype(np.float64), aux)
    t = (W["U"] * (1 + 0.2 * rng.normal(size=W["U"].shape))).T.astype(np.float32)
    loss_ref, g_ref = S.loss_and_grad(p, e, t)
    m = swe.Surrogate()
    m.params = p
    loss, g = m.loss_grad(e, t)
    m.close()
    assert abs(loss - loss_ref) <= 1e-2 * abs(loss_ref), (loss, loss_ref)
    cos = float(g @ g_ref / (np.linalg.norm(g) * np.linalg.norm(g_ref)))
    rel = float(np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref))
    assert cos > 0.999 and rel < 0.05, (cos, rel)
    # every block of the flat vector (weights and biases of each layer)
    off = 0
    for name, shape in S.SIZES:
        k = int(np.prod(shape))
        a, b = g[off:off + k], g_ref[off:off + k]
        assert np.linalg.norm(a - b) <= 0.05 * np.linalg.norm(b) + 1e-12, name
        # element by element too: one wrong row or column of a block (a bias
        # gradient read from the wrong accumulator column, say) stands out
        # against the block's largest entry
        err = np.abs(a - b).max() / (np.abs(b).max() + 1e-30)
        print("%s: max elementwise deviation %.3e of the block's largest entry" % (name, err))
        assert err <= 1e-3, (name, err)  # measured about 1e-5
        off += k


def test_loss_gradient_of_masked_edges_is_zero(swe):
    """dry or shallow edges carry no gradient"""
    e = wet_edges(256, 30)
    e[0, ::2] = 0.05  # left side shallower than 0.1 m
    t = np.zeros((4, 256), np.float32)
    m = swe.Surrogate()
    m.params = random_params(7)
    _, g_all = m.loss_grad(e, t)
    _, g_wet = m.loss_grad(e[:, 1::2], t[:, 1::2])
    m.close()
    # the mean over 256 edges of which 128 contribute equals half the mean over the 128
    assert np.allclose(g_all, 0.5 * g_wet, rtol=2e-2, atol=1e-6 * np.abs(g_wet).max())


@pytest.fixture(scope="module")
def trained(swe, oracle_mod):
    """a surrogate trained with Adam on augmented-solver targets of 2^16 edges"""
    e = wet_edges(1 << 16, 60, spread=0.5)
    t = np.stack(oracle_mod.solve_edges(2, *e)[:4]).astype(np.float32)
    m = swe.Surrogate(seed=2)
    loss0, _ = m.loss_grad(e, t)
    losses = m.train(e, t, epochs=30, batch=4096, lr=2e-3, seed=3)
    loss1, _ = m.loss_grad(e, t)
    p = m.params
    m.close()
    return dict(params=p, loss0=loss0, loss1=loss1, losses=losses)


def test_solve_falls_back_to_the_augmented_solver(swe, oracle_mod, trained):
    n = 4096
    e = wet_edges(n, 40)
    e[0, :512] = 0.0        # dry left side
    e[1, 512:1024] = 0.05   # shallow right side
    out = {}
    for name, p in (("untrained", None), ("trained", trained["params"])):
        m = swe.Surrogate(seed=1)
        if p is not None:
            m.params = p
        else:
            assert np.all(m.forward(e) == 0.0)  # zero last layer: Roe speeds, zero predicted strengths
        out[name] = m.solve(e)
        m.close()
    aug = oracle_mod.solve_edges(2, *e)
    for name, (upd, spd, used) in out.items():
        assert not used[:1024].any(), name
        # every edge the gate rejects is the augmented solver's, bit for bit
        for k in range(4):
            assert np.array_equal(upd[k, ~used].view(np.uint32), aug[k][~used].view(np.uint32)), name
        assert np.array_equal(spd[~used].view(np.uint32), aug[4][~used].view(np.uint32)), name
        # closure: the h updates of the two cells sum to the flux difference
        dF1 = e[3] - e[2]
        assert np.allclose((upd[0] + upd[1])[used], dF1[used], rtol=1e-5, atol=1e-4 * np.abs(dF1).max())
    # predicted strengths of zero are inconsistent with the closure: the untrained gate rejects
    assert out["untrained"][2].mean() < 0.05


def test_solve_matches_oracle_gate(swe, trained):
    n = 20000
    e = wet_edges(n, 50, spread=0.5)
    p = trained["params"]
    m = swe.Surrogate()
    m.params = p
    upd, spd, used = m.solve(e)
    m.close()
    x, aux = S.features(*e)
    o, _ = S.forward(p, x)
    W = S.waves(o.astype(np.float64), aux)
    gate = S.gate(aux, W)
    agree = (gate == used).mean()
    assert agree > 0.99 and used.mean() > 0.2, (agree, used.mean())
    both = gate & used
    for k in range(4):
        scale = np.abs(W["U"][both, k]).max()
        assert np.abs(upd[k][both] - W["U"][both, k]).max() <= 2e-2 * scale
    s_ref = np.maximum(np.abs(W["s1"]), np.abs(W["s2"]))
    assert np.allclose(spd[both], s_ref[both], rtol=2e-2)


def test_training_beats_the_f_wave_solver(swe, oracle_mod, trained):
    """The loss falls; on held-out edges where the trained surrogate's gate
    accepts, it is closer to the augmented solver than the f-wave solver
    (the untrained surrogate) is."""
    losses = trained["losses"]
    assert np.all(np.isfinite(losses)) and np.isfinite(trained["params"]).all()
    assert losses[-1] < losses[0] and trained["loss1"] < 0.7 * trained["loss0"], trained
    hold = wet_edges(8192, 61, spread=0.5)
    aug = np.stack(oracle_mod.solve_edges(2, *hold)[:4])
    fw = np.stack(oracle_mod.solve_edges(1, *hold)[:4])
    m = swe.Surrogate()
    m.params = trained["params"]
    upd, _, used = m.solve(hold)
    m.close()
    assert used.mean() > 0.2, used.mean()
    err_sur = np.abs(upd[:, used] - aug[:, used]).sum()
    err_fw = np.abs(fw[:, used] - aug[:, used]).sum()
    assert err_sur < err_fw, (err_sur, err_fw, used.mean())
