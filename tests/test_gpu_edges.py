"""GPU per-edge solvers (swe_gpu_solve_edges on device arrays) against the
oracle: bit-exact on the golden edge states and on 2^20 seeded states."""
import numpy as np
import pytest

from conftest import load_golden
from helpers import assert_bitwise

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SOLVERS = {"hlle": 4, "fwave": 1, "augrie": 2, "hybrid": 3}


def gpu_edges(swe, solver, ins):
    dev = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda() for a in ins]
    n = dev[0].numel()
    outs = [torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(5)]
    swe.solve_edges_device(solver, [t.data_ptr() for t in dev], [t.data_ptr() for t in outs], n)
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in outs]


def seeded_edges(n, seed):
    rng = np.random.default_rng(seed)
    hL = rng.uniform(0, 30, n).astype(np.float32)
    hR = rng.uniform(0, 30, n).astype(np.float32)
    hL[rng.random(n) < 0.1] = 0.0
    hR[rng.random(n) < 0.1] = np.float32(0.005)
    huL = (rng.normal(0, 3, n) * hL).astype(np.float32)
    huR = (rng.normal(0, 3, n) * hR).astype(np.float32)
    bL = rng.normal(-10, 10, n).astype(np.float32)
    bR = np.where(rng.random(n) < 0.5, bL, bL + rng.normal(0, 3, n)).astype(np.float32)
    return hL, hR, huL, huR, bL, bR


@pytest.mark.parametrize("name", ["hlle", "fwave", "augrie"])
def test_golden_edges(swe, name):
    g = load_golden("edges_" + name)
    outs = gpu_edges(swe, SOLVERS[name], [g[k] for k in ("hL", "hR", "huL", "huR", "bL", "bR")])
    for o, k in zip(outs, ("hUpdL", "hUpdR", "huUpdL", "huUpdR", "speed")):
        assert_bitwise(o, g[k], k)


@pytest.mark.parametrize("name", ["hlle", "fwave", "augrie", "hybrid"])
def test_seeded_edges(swe, oracle_mod, name):
    ins = seeded_edges(1 << 20, 7 + SOLVERS[name])
    outs = gpu_edges(swe, SOLVERS[name], ins)
    ref = oracle_mod.solve_edges(SOLVERS[name], *ins)
    for o, r, k in zip(outs, ref, ("hUpdL", "hUpdR", "huUpdL", "huUpdR", "speed")):
        assert_bitwise(o, r, k)


def signed_zero_edges():
    """every combination of dry, near-dry and wet depths with momenta and
    bathymetry of both zero signs, tiny and moderate values: lakes at rest,
    walls (a reflected zero momentum is -0) and supersonic states"""
    hs = np.array([0.0, 0.005, 1.0, 10.0], np.float32)
    hus = np.array([0.0, -0.0, 1e-30, -1e-30, 3.0, -3.0, 40.0, -40.0], np.float32)
    bs = np.array([0.0, -0.0, 1.0], np.float32)
    g = np.meshgrid(hs, hs, hus, hus, bs, bs, indexing="ij")
    return [a.ravel().copy() for a in g]


@pytest.mark.parametrize("name", ["hlle", "fwave", "augrie", "hybrid"])
def test_signed_zero_edges(swe, oracle_mod, name):
    ins = signed_zero_edges()
    outs = gpu_edges(swe, SOLVERS[name], ins)
    ref = oracle_mod.solve_edges(SOLVERS[name], *ins)
    for o, r, k in zip(outs, ref, ("hUpdL", "hUpdR", "huUpdL", "huUpdR", "speed")):
        assert_bitwise(o, r, k)
