"""Where the reference sources exist (not on the GPU machine), rebuild the
reference's block code (oracle/_ref) and pin the oracle against it on fresh
seeded cases beyond the committed fixtures: other sizes, boundary types,
ragged decompositions and local time stepping."""
import numpy as np
import pytest

from helpers import assert_bitwise

oracle = pytest.importorskip("oracle")
pytestmark = pytest.mark.skipif(not oracle.reference_available(), reason="reference sources not present")

MACROS = {0: 4, 1: 1, 2: 2}  # WAVE_PROPAGATION_SOLVER -> oracle solver id


@pytest.mark.parametrize("macro", [0, 1, 2])
@pytest.mark.parametrize("nx,ny,bnd,scenario,params", [
    (17, 13, [1, 1, 1, 1], 3, []),
    (33, 8, [0, 1, 1, 0], 1, []),
    (24, 24, [0, 0, 0, 0], 12, [7, 50000.0]),
    (9, 31, [1, 0, 0, 1], 6, []),
])
def test_unsplit_random_cases(oracle_mod, macro, nx, ny, bnd, scenario, params):
    geo = oracle.ref_geometry(scenario, params, nx, ny)
    dx, dy = float(geo[0]), float(geo[1])
    h0, hu0, hv0, b0 = oracle.ref_init_block(scenario, params, nx, ny, dx, dy, float(geo[2]), float(geo[3]), bnd)
    rh, rhu, rhv, rdts = oracle.ref_run("unsplit", macro, nx, ny, dx, dy, bnd, h0, hu0, hv0, b0, 12)
    D = oracle.Domain([nx], [ny], dx, dy, outer=bnd, solver=MACROS[macro])
    D.set_state(h0, hu0, hv0, b0)
    dts = D.step(12)
    h, hu, hv, _ = D.get_state()
    assert_bitwise(dts.astype(np.float32), rdts, "dt")
    assert_bitwise(h, rh, "h")
    assert_bitwise(hu, rhu, "hu")
    assert_bitwise(hv, rhv, "hv")


def _overdecomp_init(scenario, params, nxt, nyt, nblocks, outer):
    geo = oracle.ref_geometry(scenario, params, nxt, nyt)
    dx, dy = float(geo[0]), float(geo[1])
    by = int(np.sqrt(nblocks))
    while nblocks % by:
        by -= 1
    bx = nblocks // by
    cols = [nxt // bx] * (bx - 1) + [nxt - (bx - 1) * (nxt // bx)]
    rows = [nyt // by] * (by - 1) + [nyt - (by - 1) * (nyt // by)]
    parts = [[], [], [], []]
    for k in range(bx * by):
        px, py = k // by, k % by
        ox = np.float32(geo[2]) + np.float32(np.float32(px) * np.float32(dx) * np.float32(nxt // bx))
        oy = np.float32(geo[3]) + np.float32(np.float32(py) * np.float32(dy) * np.float32(nyt // by))
        bnd = [4 if px > 0 else outer[0], 4 if px < bx - 1 else outer[1], 4 if py > 0 else outer[2],
               4 if py < by - 1 else outer[3]]
        arrs = oracle.ref_init_block(scenario, params, cols[px], rows[py], dx, dy, float(ox), float(oy), bnd)
        for i in range(4):
            parts[i].append(arrs[i])
    return cols, rows, dx, dy, [np.concatenate(p) for p in parts]


@pytest.mark.parametrize("macro", [0, 2])
@pytest.mark.parametrize("nxt,nyt,nblocks", [(23, 17, 6), (32, 32, 16), (20, 11, 3)])
def test_overdecomp_ragged(oracle_mod, macro, nxt, nyt, nblocks):
    outer = [0, 1, 1, 0]
    cols, rows, dx, dy, (H0, HU0, HV0, B0) = _overdecomp_init(1, [], nxt, nyt, nblocks, outer)
    rh, rhu, rhv, rb, rdts, _ = oracle.ref_run_overdecomp(macro, cols, rows, dx, dy, outer, H0, HU0, HV0, B0, 10)
    D = oracle.Domain(cols, rows, dx, dy, outer=outer, solver=MACROS[macro])
    D.set_state(H0, HU0, HV0, B0)
    D.bathymetry_ghosts()
    dts = D.step(10)
    h, hu, hv, b = D.get_state()
    assert_bitwise(dts.astype(np.float32), rdts, "dt")
    assert_bitwise(h, rh, "h")
    assert_bitwise(hu, rhu, "hu")
    assert_bitwise(hv, rhv, "hv")
    assert_bitwise(b, rb, "b")


@pytest.mark.parametrize("macro", [0, 2])
def test_local_timestepping_matches_reference(oracle_mod, macro):
    """Overdecomposed blocks with local time stepping (power-of-two substeps,
    time-interpolated ghost layers; src/blocks/SWE_Block.hh:311-562)."""
    outer = [0, 0, 0, 0]
    cols, rows, dx, dy, (H0, HU0, HV0, B0) = _overdecomp_init(12, [11, 50000.0], 32, 32, 4, outer)
    lts, duration, intervals = 2.0, 10.0, 3
    rh, rhu, rhv, rb, rdts, rsteps = oracle.ref_run_overdecomp(macro, cols, rows, dx, dy, outer, H0, HU0, HV0, B0,
                                                               intervals, lts_max_timestep=lts, duration=duration)
    D = oracle.Domain(cols, rows, dx, dy, outer=outer, solver=MACROS[macro], lts_max_timestep=lts, duration=duration)
    D.set_state(H0, HU0, HV0, B0)
    D.bathymetry_ghosts()
    steps = []
    for _ in range(intervals):
        it, st = D.lts_interval()
        assert it > 0
        steps.append(st)
    h, hu, hv, b = D.get_state()
    assert_bitwise(steps[-1], rsteps, "block step divisors")
    assert_bitwise(h, rh, "h")
    assert_bitwise(hu, rhu, "hu")
    assert_bitwise(hv, rhv, "hv")
