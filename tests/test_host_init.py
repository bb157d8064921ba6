"""The library's host-side set-up (scenario sampling, boundary conditions,
geometry, decomposition) against the reference's initScenario output
(golden vectors) and the drivers' formulas."""
import numpy as np
import pytest

from conftest import load_golden
from helpers import assert_bitwise

NAMES = ["radial_bathymetry_dam_break", "radial_dam_break", "sea_at_rest", "half_domain_dry", "splashing_cone",
         "dam_break_1000m"]


@pytest.mark.parametrize("name", NAMES)
def test_init_block_matches_reference(swe, name):
    g = load_golden("init_" + name)
    nx, ny = int(g["nx"]), int(g["ny"])
    geo = swe.scenario_geometry(int(g["scenario"]), nx, ny, list(g["params"]))
    assert_bitwise(np.asarray(geo, np.float32), g["geometry"], "geometry")
    h, hu, hv, b = swe.init_block(int(g["scenario"]), nx, ny, geo[0], geo[1], geo[2], geo[3], g["bnd"],
                                  list(g["params"]))
    for a, k in zip((h, hu, hv, b), ("h", "hu", "hv", "b")):
        assert_bitwise(a, g[k], k)


@pytest.mark.parametrize("nblocks,expect", [(1, (1, 1)), (2, (2, 1)), (6, (3, 2)), (16, (4, 4)), (64, (8, 8)),
                                            (7, (7, 1)), (12, (4, 3))])
def test_decomposition_matches_driver(swe, nblocks, expect):
    cols, rows, ox, oy = swe.decompose(2049, 1023, nblocks, 0.5, 0.25)
    assert (len(cols), len(rows)) == expect
    bx, by = expect
    assert sum(cols) == 2049 and sum(rows) == 1023
    assert all(c == 2049 // bx for c in cols[:-1]) and cols[-1] == 2049 - (bx - 1) * (2049 // bx)
    for i in range(bx):
        assert ox[i] == np.float32(np.float32(i) * np.float32(0.5) * np.float32(2049 // bx))


def test_scenario_boundaries(swe):
    assert swe.scenario_boundary(swe.SCENARIO_HALF_DOMAIN_DRY) == [1, 1, 1, 1]
    assert swe.scenario_boundary(swe.SCENARIO_TSUNAMI, [256]) == [0, 0, 0, 0]


def test_tsunami_scenario_is_seeded_and_blockwise_consistent(swe):
    """The seeded noise is a function of the global cell only: 4 blocks give the
    same interior as one block (bathymetry is what the step reads)."""
    p = [64, 99, 100000.0]
    geo1, h1, hu1, hv1, b1 = swe.init_domain(swe.SCENARIO_TSUNAMI, 64, 64, 1, p)
    geo4, h4, hu4, hv4, b4 = swe.init_domain(swe.SCENARIO_TSUNAMI, 64, 64, 4, p)
    from helpers import blocks_to_global
    g1 = blocks_to_global(b1, geo1["nx_cols"], geo1["ny_rows"])
    g4 = blocks_to_global(b4, geo4["nx_cols"], geo4["ny_rows"])
    assert np.abs(g1 - g4).max() < 1e-3  # block origins are rounded floats; the noise cell is the same
    _, _, _, _, b1b = swe.init_domain(swe.SCENARIO_TSUNAMI, 64, 64, 1, p)
    assert_bitwise(b1, b1b, "reproducible")
    _, _, _, _, b1c = swe.init_domain(swe.SCENARIO_TSUNAMI, 64, 64, 1, [64, 100, 100000.0])
    assert not np.array_equal(b1, b1c)
