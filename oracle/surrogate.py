"""ORACLE -- test infrastructure only: CPU restatement of the MLP surrogate
solver (the GPU implementation is swe-ppm_gb300/csrc/swe_mlp.cu).  Used by
tests/ to check the tensor-core forward and backward passes.

The surrogate replaces the augmented Riemann solver (George 2008) on wet edges
(both sides >= 0.1 m; the reference's hybrid solver switches there,
src/blocks/SWE_DimensionalSplittingMpi.cpp:403-410 call sites).  It is an
f-wave solver whose two wave speeds are the Roe speeds plus learned
corrections; the strengths follow from the speeds by the f-wave closure, so
the waves sum exactly to the flux difference and mass is conserved by
construction.  The network also predicts the two strengths; their distance to
the closure's is the consistency gate that sends an edge back to the
augmented solver.

Network: 6 inputs -> 64 -> 64 -> 64 -> 4, SiLU, weights and the activations
fed to each GEMM rounded to BF16, FP32 accumulation.  Flat parameter layout:
W1[64][6], b1[64], W2[64][64], b2[64], W3[64][64], b3[64], W4[4][64], b4[4].
"""
import numpy as np

G = np.float32(9.81)
HALF_G = np.float32(0.5 * 9.81)
N_IN, N_H, N_OUT = 6, 64, 4
SIZES = [("W1", (N_H, N_IN)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)), ("W3", (N_H, N_H)),
         ("b3", (N_H,)), ("W4", (N_OUT, N_H)), ("b4", (N_OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)
LAMBDA = 0.1          # weight of the strength-consistency term
GATE_TAU = 0.25       # gate: |strengths - closure| <= tau (|closure|) + 1e-3 h c
MIN_SPREAD = 0.5      # gate: s2 - s1 >= 0.5 c
TRAIN_SPREAD = 0.1    # training: edges with s2 - s1 < 0.1 c carry no gradient
WET = 0.1             # both sides at least this deep, else the augmented solver
FEATURE_CLIP = 8.0


def unpack(p, dtype=np.float32):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], dtype=dtype).reshape(shape)
        o += n
    return out


def pack(d, dtype=np.float32):
    return np.concatenate([np.asarray(d[name], dtype=dtype).ravel() for name, _ in SIZES])


def bf16(x):
    """round-to-nearest-even to BF16, kept in float32"""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u + np.uint32(0x7FFF) + ((u >> np.uint32(16)) & np.uint32(1))) & np.uint32(0xFFFF0000)).astype(np.uint32)
    return r.view(np.float32)


def features(hL, hR, huL, huR, bL, bR):
    """inputs of the network and the edge quantities the surrogate needs (float32)"""
    f = lambda a: np.asarray(a, dtype=np.float32)
    hL, hR, huL, huR, bL, bR = map(f, (hL, hR, huL, huR, bL, bR))
    hm = np.float32(0.5) * (hL + hR)
    c = np.sqrt(G * hm)
    rhm, rc = np.float32(1) / hm, np.float32(1) / c
    uL, uR = huL / hL, huR / hR
    x = np.stack([(hL - hm) * rhm, (hR - hm) * rhm, uL * rc, uR * rc, (bR - bL) * rhm,
                  ((hL + bL) - (hR + bR)) * rhm], axis=1)
    x = np.clip(x, -FEATURE_CLIP, FEATURE_CLIP).astype(np.float32)
    sqL, sqR = np.sqrt(hL), np.sqrt(hR)
    uRoe = (uL * sqL + uR * sqR) / (sqL + sqR)
    dF1 = huR - huL
    dF2 = (huR * uR + HALF_G * hR * hR) - (huL * uL + HALF_G * hL * hL) + HALF_G * (hL + hR) * (bR - bL)
    aux = dict(hm=hm, c=c, s10=uRoe - c, s20=uRoe + c, dF1=dF1, dF2=dF2, hmin=np.minimum(hL, hR))
    return x, aux


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x, rounding=True):
    """network outputs and the intermediates (pre-activations z, BF16 GEMM
    inputs a); rounding=False keeps everything in float64 (derivative checks)"""
    P = unpack(p, np.float32 if rounding else np.float64)
    if not rounding:
        r = lambda a: np.asarray(a, dtype=np.float64)
        a0 = r(x)
        z1 = a0 @ r(P["W1"]).T + P["b1"]
        a1 = silu(z1)
        z2 = a1 @ r(P["W2"]).T + P["b2"]
        a2 = silu(z2)
        z3 = a2 @ r(P["W3"]).T + P["b3"]
        a3 = silu(z3)
        o = a3 @ r(P["W4"]).T + P["b4"]
        return o, dict(a0=a0, z1=z1, a1=a1, z2=z2, a2=a2, z3=z3, a3=a3)
    a0 = bf16(x)
    z1 = (a0.astype(np.float64) @ bf16(P["W1"]).astype(np.float64).T + P["b1"]).astype(np.float32)
    a1 = bf16(silu(z1.astype(np.float64)).astype(np.float32))
    z2 = (a1.astype(np.float64) @ bf16(P["W2"]).astype(np.float64).T + P["b2"]).astype(np.float32)
    a2 = bf16(silu(z2.astype(np.float64)).astype(np.float32))
    z3 = (a2.astype(np.float64) @ bf16(P["W3"]).astype(np.float64).T + P["b3"]).astype(np.float32)
    a3 = bf16(silu(z3.astype(np.float64)).astype(np.float32))
    o = (a3.astype(np.float64) @ bf16(P["W4"]).astype(np.float64).T + P["b4"]).astype(np.float32)
    return o, dict(a0=a0, z1=z1, a1=a1, z2=z2, a2=a2, z3=z3, a3=a3)


def left_share(s):
    return np.where(s < -1e-7, 1.0, np.where(s > 1e-7, 0.0, 0.5))


def waves(o, aux):
    """speeds, closure strengths and net updates of the surrogate (float64)"""
    c, hm = aux["c"].astype(np.float64), aux["hm"].astype(np.float64)
    s1 = aux["s10"] + c * o[:, 0]
    s2 = aux["s20"] + c * o[:, 1]
    D = s2 - s1
    dF1, dF2 = aux["dF1"].astype(np.float64), aux["dF2"].astype(np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        b1 = (s2 * dF1 - dF2) / D
        b2 = (dF2 - s1 * dF1) / D
    bh1, bh2 = o[:, 2] * hm * c, o[:, 3] * hm * c
    w1, w2 = left_share(s1), left_share(s2)
    U = np.stack([w1 * b1 + w2 * b2, (1 - w1) * b1 + (1 - w2) * b2,
                  w1 * b1 * s1 + w2 * b2 * s2, (1 - w1) * b1 * s1 + (1 - w2) * b2 * s2], axis=1)
    return dict(s1=s1, s2=s2, D=D, b1=b1, b2=b2, bh1=bh1, bh2=bh2, w1=w1, w2=w2, U=U)


def gate(aux, W):
    """True where the surrogate is used (else the augmented solver)"""
    c, hm = aux["c"].astype(np.float64), aux["hm"].astype(np.float64)
    ok = (aux["hmin"] >= WET) & (W["D"] >= MIN_SPREAD * c)
    err = np.abs(W["bh1"] - W["b1"]) + np.abs(W["bh2"] - W["b2"])
    ok &= err <= GATE_TAU * (np.abs(W["b1"]) + np.abs(W["b2"])) + 1e-3 * hm * c
    return ok & np.all(np.isfinite(W["U"]), axis=1)


def loss_and_grad(p, edges, targets, rounding=True):
    """mean loss over the edges and its gradient (flat), as the GPU computes
    it: net-update error scaled by h c (h updates) and h c^2 (hu updates), plus
    LAMBDA times the strength inconsistency; BF16 operands in the backward GEMMs
    (the bias gradients are sums of the BF16-rounded dZ, as the tensor cores
    form them); edges with a side shallower than WET carry no gradient"""
    P = unpack(p, np.float32 if rounding else np.float64)
    x, aux = features(*edges)
    o, I = forward(p, x, rounding)
    W = waves(o.astype(np.float64), aux)
    n = x.shape[0]
    c, hm = aux["c"].astype(np.float64), aux["hm"].astype(np.float64)
    ish, ishu = 1.0 / (hm * c) ** 2, 1.0 / (hm * c * c) ** 2
    T = np.stack([np.asarray(t, dtype=np.float64) for t in targets], axis=1)
    mask = (aux["hmin"] >= WET) & (W["D"] >= TRAIN_SPREAD * c) & np.all(np.isfinite(W["U"]), axis=1)
    e = np.where(mask[:, None], W["U"] - T, 0.0)
    db1 = np.where(mask, W["bh1"] - W["b1"], 0.0)
    db2 = np.where(mask, W["bh2"] - W["b2"], 0.0)
    L = (e[:, 0] ** 2 + e[:, 1] ** 2) * ish + (e[:, 2] ** 2 + e[:, 3] ** 2) * ishu + LAMBDA * (db1 ** 2 + db2 ** 2) * ish
    loss = L.sum() / n
    gU = np.stack([2 * e[:, 0] * ish, 2 * e[:, 1] * ish, 2 * e[:, 2] * ishu, 2 * e[:, 3] * ishu], axis=1) / n
    gl1, gl2 = 2 * LAMBDA * db1 * ish / n, 2 * LAMBDA * db2 * ish / n
    w1, w2, s1, s2, b1, b2, D = W["w1"], W["w2"], W["s1"], W["s2"], W["b1"], W["b2"], W["D"]
    with np.errstate(divide="ignore", invalid="ignore"):
        gb1 = gU[:, 0] * w1 + gU[:, 1] * (1 - w1) + gU[:, 2] * w1 * s1 + gU[:, 3] * (1 - w1) * s1 - gl1
        gb2 = gU[:, 0] * w2 + gU[:, 1] * (1 - w2) + gU[:, 2] * w2 * s2 + gU[:, 3] * (1 - w2) * s2 - gl2
        gs1 = gU[:, 2] * w1 * b1 + gU[:, 3] * (1 - w1) * b1 + (gb1 - gb2) * b1 / D
        gs2 = gU[:, 2] * w2 * b2 + gU[:, 3] * (1 - w2) * b2 + (gb1 - gb2) * b2 / D
    dO = np.stack([gs1 * c, gs2 * c, gl1 * hm * c, gl2 * hm * c], axis=1)
    dO = np.where(mask[:, None], dO, 0.0)
    if rounding:
        dO = dO.astype(np.float32)
    # backward through the layers: BF16 operands in the GEMMs, FP32 elsewhere
    f64 = lambda a: np.asarray(a, dtype=np.float64)
    if not rounding:
        bf = lambda a: np.asarray(a, dtype=np.float64)
        f32 = lambda a: a
    else:
        bf = bf16
        f32 = lambda a: a.astype(np.float32)
    g = {}
    dz4 = dO
    g["b4"] = f64(bf(dz4)).sum(0)
    g["W4"] = f64(bf(dz4)).T @ f64(I["a3"])
    dz3 = f32(f64(bf(dz4)) @ f64(bf(P["W4"]))) * f32(dsilu(f64(I["z3"])))
    g["b3"] = f64(bf(dz3)).sum(0)
    g["W3"] = f64(bf(dz3)).T @ f64(I["a2"])
    dz2 = f32(f64(bf(dz3)) @ f64(bf(P["W3"]))) * f32(dsilu(f64(I["z2"])))
    g["b2"] = f64(bf(dz2)).sum(0)
    g["W2"] = f64(bf(dz2)).T @ f64(I["a1"])
    dz1 = f32(f64(bf(dz2)) @ f64(bf(P["W2"]))) * f32(dsilu(f64(I["z1"])))
    g["b1"] = f64(bf(dz1)).sum(0)
    g["W1"] = f64(bf(dz1)).T @ f64(I["a0"])
    return float(loss), pack(g, np.float32 if rounding else np.float64)


def init_params(seed):
    """Glorot-uniform weights, zero biases (the last layer starts at zero: the
    untrained surrogate is the Roe f-wave solver)"""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SIZES:
        if name.startswith("b"):
            d[name] = np.zeros(shape, np.float32)
        else:
            lim = np.sqrt(6.0 / (shape[0] + shape[1]))
            d[name] = rng.uniform(-lim, lim, shape).astype(np.float32)
    d["W4"][:] = 0.0
    return pack(d)
