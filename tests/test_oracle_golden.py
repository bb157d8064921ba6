"""The oracle (CPU restatement) against golden vectors written by the
reference's own compiled block code (tests/golden/make_golden.py): bit-exact."""
import numpy as np
import pytest

from conftest import load_golden
from helpers import assert_bitwise

SOLVERS = {"hlle": 4, "fwave": 1, "augrie": 2}


@pytest.mark.parametrize("name", ["hlle", "fwave", "augrie"])
def test_edges_match_reference(oracle_mod, name):
    g = load_golden("edges_" + name)
    outs = oracle_mod.solve_edges(SOLVERS[name], g["hL"], g["hR"], g["huL"], g["huR"], g["bL"], g["bR"])
    for o, key in zip(outs, ("hUpdL", "hUpdR", "huUpdL", "huUpdR", "speed")):
        assert_bitwise(o, g[key], key)


@pytest.mark.parametrize("case", ["unsplit", "shoreline"])
@pytest.mark.parametrize("name", ["hlle", "fwave", "augrie"])
def test_unsplit_block_matches_reference(oracle_mod, case, name):
    g = load_golden("%s_%s" % (case, name))
    nx, ny = int(g["nx"]), int(g["ny"])
    D = oracle_mod.Domain([nx], [ny], float(g["dx"]), float(g["dy"]), outer=g["bnd"], solver=SOLVERS[name])
    D.set_state(g["h0"], g["hu0"], g["hv0"], g["b0"])
    dts = D.step(len(g["dts"]))
    h, hu, hv, _ = D.get_state()
    assert_bitwise(dts.astype(np.float32), g["dts"], "dt")
    assert_bitwise(h, g["h"], "h")
    assert_bitwise(hu, g["hu"], "hu")
    assert_bitwise(hv, g["hv"], "hv")


def test_split_block_matches_reference(oracle_mod):
    g = load_golden("split_hybrid")
    nx, ny = int(g["nx"]), int(g["ny"])
    D = oracle_mod.Domain([nx], [ny], float(g["dx"]), float(g["dy"]), outer=g["bnd"], solver=oracle_mod.HYBRID,
                          semantics=oracle_mod.SPLIT, split_dt_mode=oracle_mod.SPLIT_DT_LAST_EDGE)
    D.set_state(g["h0"], g["hu0"], g["hv0"], g["b0"])
    dts = D.step(len(g["dts"]))
    h, hu, hv, _ = D.get_state()
    assert_bitwise(dts.astype(np.float32), g["dts"], "dt")
    assert_bitwise(h, g["h"], "h")
    assert_bitwise(hu, g["hu"], "hu")
    assert_bitwise(hv, g["hv"], "hv")


@pytest.mark.parametrize("name", ["hlle", "fwave", "augrie"])
def test_overdecomposed_blocks_match_reference(oracle_mod, name):
    g = load_golden("overdecomp_" + name)
    D = oracle_mod.Domain(g["nx_cols"], g["ny_rows"], float(g["dx"]), float(g["dy"]), outer=g["outer"],
                          solver=SOLVERS[name])
    D.set_state(g["h0"], g["hu0"], g["hv0"], g["b0"])
    D.bathymetry_ghosts()
    dts = D.step(len(g["dts"]))
    h, hu, hv, b = D.get_state()
    assert_bitwise(dts.astype(np.float32), g["dts"], "dt")
    assert_bitwise(h, g["h"], "h")
    assert_bitwise(hu, g["hu"], "hu")
    assert_bitwise(hv, g["hv"], "hv")
    assert_bitwise(b, g["b"], "b")
