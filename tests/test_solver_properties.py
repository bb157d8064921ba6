"""Properties of the solver restatement that hold whatever the (absent)
original module did: flux-difference conservation, lake at rest, dry/dry,
mirror symmetry, FP32 vs FP64 agreement, and convergence to the exact 1D
dam-break solutions (Stoker wet bed, Ritter dry bed).  The solver parity
itself is unpinned (no golden data of the original solver exists)."""
import numpy as np
import pytest

SOLVERS = {"fwave": 1, "augrie": 2, "hybrid": 3, "hlle": 4}
G = 9.81


def wet_edges(n, seed, flat=False):
    rng = np.random.default_rng(seed)
    hL = rng.uniform(0.5, 30, n)
    hR = rng.uniform(0.5, 30, n)
    huL = rng.normal(0, 3, n) * hL
    huR = rng.normal(0, 3, n) * hR
    bL = np.zeros(n) if flat else rng.normal(-10, 3, n)
    bR = bL.copy() if flat else bL + rng.normal(0, 0.5, n)
    return hL, hR, huL, huR, bL, bR


@pytest.mark.parametrize("name", list(SOLVERS))
def test_mass_flux_conservation(oracle_mod, name):
    ins = wet_edges(20000, 1)
    hUL, hUR, _, _, _ = oracle_mod.solve_edges(SOLVERS[name], *ins, precision=64)
    np.testing.assert_allclose(hUL + hUR, ins[3] - ins[2], rtol=1e-10, atol=1e-8)


@pytest.mark.parametrize("name", ["fwave", "hlle"])
def test_momentum_flux_with_source(oracle_mod, name):
    """f-wave form: the momentum fluctuations sum to the flux jump plus source."""
    hL, hR, huL, huR, bL, bR = wet_edges(20000, 2)
    _, _, uL, uR, _ = oracle_mod.solve_edges(SOLVERS[name], hL, hR, huL, huR, bL, bR, precision=64)
    phi = lambda h, hu: hu * hu / h + 0.5 * G * h * h
    expect = phi(hR, huR) - phi(hL, huL) + 0.5 * G * (hL + hR) * (bR - bL)
    np.testing.assert_allclose(uL + uR, expect, rtol=1e-9, atol=1e-6)


@pytest.mark.parametrize("name", list(SOLVERS))
@pytest.mark.parametrize("precision,tol", [(64, 1e-9), (32, 2e-3)])
def test_lake_at_rest(oracle_mod, name, precision, tol):
    rng = np.random.default_rng(3)
    n = 5000
    bL = rng.uniform(-50, -1, n)
    bR = np.clip(bL + rng.normal(0, 2, n), -60, -0.5)
    eta = 0.0
    outs = oracle_mod.solve_edges(SOLVERS[name], eta - bL, eta - bR, np.zeros(n), np.zeros(n), bL, bR,
                                  precision=precision)
    for o in outs[:4]:
        assert np.abs(o).max() < tol


@pytest.mark.parametrize("name", list(SOLVERS))
def test_dry_dry_gives_nothing(oracle_mod, name):
    n = 100
    z = np.zeros(n)
    outs = oracle_mod.solve_edges(SOLVERS[name], z + 0.001, z, z, z, z, z + 1)
    for o in outs:
        assert np.all(o == 0)


@pytest.mark.parametrize("name", list(SOLVERS))
def test_mirror_symmetry(oracle_mod, name):
    """Reflecting the edge (left <-> right, momentum negated) swaps the fluctuations."""
    hL, hR, huL, huR, bL, bR = wet_edges(5000, 4)
    a = oracle_mod.solve_edges(SOLVERS[name], hL, hR, huL, huR, bL, bR, precision=64)
    b = oracle_mod.solve_edges(SOLVERS[name], hR, hL, -huR, -huL, bR, bL, precision=64)
    np.testing.assert_allclose(a[0], b[1], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(a[2], -b[3], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(a[4], b[4], rtol=1e-12)


@pytest.mark.parametrize("name", list(SOLVERS))
def test_fp32_close_to_fp64(oracle_mod, name):
    ins = wet_edges(20000, 5)
    a = oracle_mod.solve_edges(SOLVERS[name], *ins, precision=32)
    b = oracle_mod.solve_edges(SOLVERS[name], *ins, precision=64)
    for x, y in zip(a, b):
        scale = np.abs(y).max()
        assert np.abs(x - y).max() <= 1e-4 * scale + 1e-5


# --- exact 1D dam breaks ------------------------------------------------------
def stoker(x, t, hl, hr, x0):
    """Exact wet-bed dam break (rarefaction + shock)."""
    cl, cr = np.sqrt(G * hl), np.sqrt(G * hr)
    # middle state: solve 2 (cl - cm) = (hm - hr) sqrt(g/2 (1/hm + 1/hr))
    hm = 0.5 * (hl + hr)
    for _ in range(100):
        cm = np.sqrt(G * hm)
        f = 2 * (cl - cm) - (hm - hr) * np.sqrt(0.5 * G * (1 / hm + 1 / hr))
        df = -G / cm - np.sqrt(0.5 * G * (1 / hm + 1 / hr)) + (hm - hr) * 0.25 * G / hm ** 2 / np.sqrt(
            0.5 * G * (1 / hm + 1 / hr))
        hm -= f / df
    um = 2 * (cl - np.sqrt(G * hm))
    s = hm * um / (hm - hr)
    xi = (x - x0) / t
    h = np.where(xi < -cl, hl, np.where(xi < um - np.sqrt(G * hm), (2 * cl - xi) ** 2 / (9 * G),
                                         np.where(xi < s, hm, hr)))
    return h


def ritter(x, t, hl, x0):
    cl = np.sqrt(G * hl)
    xi = (x - x0) / t
    return np.where(xi < -cl, hl, np.where(xi < 2 * cl, (2 * cl - xi) ** 2 / (9 * G), 0.0))


def run_1d(oracle_mod, solver, nx, h0, length, t_end):
    dx = length / nx
    D = oracle_mod.Domain([nx], [1], dx, dx, outer=[0, 0, 1, 1], solver=solver, precision=64)
    h = np.zeros((nx + 2, 3))
    h[1:-1, 1] = h0
    h[0, :], h[-1, :] = h[1, 1], h[-2, 1]
    h[:, 0], h[:, 2] = h[:, 1], h[:, 1]
    z = np.zeros_like(h)
    D.set_state(h.ravel(), z.ravel(), z.ravel(), z.ravel(), dtype=np.float64)
    D.advance(t_end)
    out = D.get_state(np.float64)[0].reshape(nx + 2, 3)[1:-1, 1]
    return out, D.time


@pytest.mark.parametrize("name", ["fwave", "hlle", "augrie", "hybrid"])
def test_stoker_convergence(oracle_mod, name):
    errs = []
    for nx in (100, 400):
        x = (np.arange(nx) + 0.5) * (1000.0 / nx)
        h, t = run_1d(oracle_mod, SOLVERS[name], nx, np.where(x < 500, 10.0, 2.0), 1000.0, 20.0)
        errs.append(np.abs(h - stoker(x, t, 10.0, 2.0, 500.0)).mean())
    assert errs[1] < 0.5 * errs[0], errs
    assert errs[1] < 0.05, errs


@pytest.mark.parametrize("name", ["augrie", "hybrid"])
def test_ritter_dry_bed_convergence(oracle_mod, name):
    """Inundation of a dry bed needs the augmented solver (the f-wave and HLLE
    solvers treat a dry neighbour as a wall)."""
    errs = []
    for nx in (100, 400):
        x = (np.arange(nx) + 0.5) * (1000.0 / nx)
        h, t = run_1d(oracle_mod, SOLVERS[name], nx, np.where(x < 500, 5.0, 0.0), 1000.0, 15.0)
        errs.append(np.abs(h - ritter(x, t, 5.0, 500.0)).mean())
    assert errs[1] < 0.75 * errs[0], errs
    assert errs[1] < 0.05, errs
