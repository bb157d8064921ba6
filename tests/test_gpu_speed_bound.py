"""The bounded speed pass (default for f-wave / HLLE unsplit steps) against
the full speed pass and the oracle: every dt and every state array must be
bit-identical, whichever edges the bounds let the pass skip."""
import numpy as np
import pytest

from helpers import assert_bitwise

pytestmark = pytest.mark.gpu


def run(swe, geo, state, solver, nsteps, speed_pass, tile_cols=0, api="split"):
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver,
                   speed_pass=speed_pass, tile_cols=tile_cols)
    D.upload(*state)
    D.exchange_bathymetry()
    dts = []
    if api == "split":
        for _ in range(nsteps):
            D.set_ghost_layer()
            D.compute_fluxes()
            dts.append(D.max_timestep())
            D.update_unknowns()
    else:
        D.step(nsteps)
        D.sync()
    out = D.download()
    assert D.status() == 0
    D.close()
    return out, np.asarray(dts, np.float32)


CASES = [
    # scenario, nx, ny, blocks, params
    ("tsunami", 384, 320, 4, None),
    ("shoreline", 256, 256, 4, None),
    ("radial_dam_break", 200, 136, 6, None),
    ("half_domain_dry", 160, 96, 1, None),
]
SCEN = {"tsunami": 11, "shoreline": 12, "radial_dam_break": 0, "half_domain_dry": 3}


def setup(swe, name, nx, ny, nb):
    sid = SCEN[name]
    params = [nx, 7.0, 100000.0] if name == "tsunami" else ([5.0] if name == "shoreline" else None)
    geo, h, hu, hv, b = swe.init_domain(sid, nx, ny, nb, params)
    return geo, (h, hu, hv, b)


@pytest.mark.parametrize("solver", [4, 1])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_bounded_equals_full(swe, case, solver):
    name, nx, ny, nb, _ = case
    geo, st = setup(swe, name, nx, ny, nb)
    full, dts_full = run(swe, geo, st, solver, 40, speed_pass=1)
    bnd, dts_bnd = run(swe, geo, st, solver, 40, speed_pass=0)
    assert_bitwise(dts_bnd, dts_full, "dt")
    for a, b_, k in zip(bnd, full, "h hu hv b".split()):
        assert_bitwise(a, b_, k)


def test_bounded_matches_oracle_over_many_steps(swe, oracle_mod):
    geo, st = setup(swe, "tsunami", 256, 256, 4)
    (h, hu, hv, _), _ = run(swe, geo, st, 4, 25, speed_pass=0, api="step")
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=4)
    R.set_state(*st)
    R.bathymetry_ghosts()
    R.step(25)
    ref = R.get_state()
    assert_bitwise(h, ref[0], "h")
    assert_bitwise(hu, ref[1], "hu")
    assert_bitwise(hv, ref[2], "hv")


def test_upload_between_steps_invalidates_bounds(swe):
    """A state uploaded mid-run whose fastest edge sits where the old bounds
    were small must still give the exact dt."""
    geo, st = setup(swe, "tsunami", 256, 192, 4)
    outs = []
    for sp in (1, 0):
        D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=4,
                       speed_pass=sp)
        D.upload(*st)
        D.exchange_bathymetry()
        D.step(5)
        h, hu, hv, b = D.download()
        hu = hu.copy()
        hu[len(hu) // 3] += np.float32(5000.0)  # one fast cell far from the old maximum
        D.upload(h, hu, hv, None)
        dts = []
        for _ in range(6):
            D.compute_fluxes()
            dts.append(D.max_timestep())
            D.update_unknowns()
        outs.append((np.asarray(dts, np.float32), D.download()))
        assert D.status() == 0
        D.close()
    assert_bitwise(outs[1][0], outs[0][0], "dt after upload")
    for a, b_, k in zip(outs[1][1], outs[0][1], "h hu hv b".split()):
        assert_bitwise(a, b_, k)


def test_repeated_compute_fluxes_keeps_dt(swe):
    geo, st = setup(swe, "radial_dam_break", 128, 128, 4)
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=4)
    D.upload(*st)
    D.exchange_bathymetry()
    D.step(3)
    D.compute_fluxes()
    a = D.max_timestep()
    D.compute_fluxes()
    b = D.max_timestep()
    assert np.float32(a).tobytes() == np.float32(b).tobytes()
    D.close()


def test_random_states_with_narrow_segments(swe):
    """Random wet/dry states, segments of a few columns (many segment
    boundaries), bounded vs full."""
    rng = np.random.default_rng(3)
    cols, rows = [70, 45], [33, 90]
    ncell = sum((c + 2) * (r + 2) for c in cols for r in rows)
    h = rng.uniform(0.0, 3.0, ncell).astype(np.float32)
    h[rng.random(ncell) < 0.2] = 0.0
    hu = rng.normal(0, 2.0, ncell).astype(np.float32)
    hv = rng.normal(0, 2.0, ncell).astype(np.float32)
    b = rng.normal(-1.0, 0.3, ncell).astype(np.float32)
    geo = dict(nx_cols=cols, ny_rows=rows, dx=1.5, dy=2.0, boundary=[0, 1, 1, 0])
    for solver in (4, 1):
        full, d1 = run(swe, geo, (h, hu, hv, b), solver, 12, speed_pass=1, tile_cols=5)
        bnd, d0 = run(swe, geo, (h, hu, hv, b), solver, 12, speed_pass=0, tile_cols=5)
        assert_bitwise(d0, d1, "dt")
        for a, b_, k in zip(bnd, full, "h hu hv b".split()):
            assert_bitwise(a, b_, k)


def test_passive_ghosts_with_the_fastest_edges(swe):
    """Ghosts that the step never rewrites (PASSIVE / INFLOW sides) carry the
    fastest edges; the bounds must not let the pass skip them."""
    rng = np.random.default_rng(11)
    cols, rows = [96, 64], [80]
    shapes = [(c, r) for c in cols for r in rows]
    parts = []
    for nx, ny in shapes:
        h = rng.uniform(1.0, 2.0, (nx + 2, ny + 2)).astype(np.float32)
        hu = rng.normal(0, 0.5, (nx + 2, ny + 2)).astype(np.float32)
        hv = rng.normal(0, 0.5, (nx + 2, ny + 2)).astype(np.float32)
        hu[0, :] = 40.0   # left ghost column: fast inflow
        hv[:, -1] = -35.0  # top ghost row
        parts.append((h.ravel(), hu.ravel(), hv.ravel(), np.zeros_like(h).ravel()))
    st = tuple(np.concatenate([p[i] for p in parts]) for i in range(4))
    geo = dict(nx_cols=cols, ny_rows=rows, dx=1.0, dy=1.0, boundary=[5, 2, 0, 5])  # PASSIVE, INFLOW, OUTFLOW, PASSIVE
    full, d1 = run(swe, geo, st, 4, 15, speed_pass=1)
    bnd, d0 = run(swe, geo, st, 4, 15, speed_pass=0)
    assert_bitwise(d0, d1, "dt")
    for a, b_, k in zip(bnd, full, "h hu hv b".split()):
        assert_bitwise(a, b_, k)
