"""Writes the golden vectors in tests/golden/ from the reference's OWN compiled
block code (oracle/_ref, built by oracle/ref/Makefile from the reference
sources plus the solver restatement, single-rank MPI stand-in).

Run here, where the reference sources exist:  python tests/golden/make_golden.py
The fixtures are small .npz files; the GPU machine never needs the reference.

Contents:
  init_<name>.npz     SWE_Block::initScenario output of one block (h, hu, hv, b)
  unsplit_<solver>.npz  SWE_DimensionalSplittingMpi: initial state, state and dt
                      after N steps (solver macro 0 HLLEFun, 1 FWave, 2 AugRie)
  split_hybrid.npz    serial SWE_DimensionalSplitting (Hybrid), one OpenMP thread
  overdecomp_<solver>.npz  2 x 3 SWE_DimensionalSplittingMPIOverdecomp blocks
  edges_<solver>.npz  per-edge solver outputs on seeded edge states
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

SEED = 20261203


def edge_states(n, rng):
    """Seeded edge states covering wet/wet, wet/dry, dry/dry and bathymetry steps."""
    hL = rng.uniform(0.0, 20.0, n).astype(np.float32)
    hR = rng.uniform(0.0, 20.0, n).astype(np.float32)
    dry = rng.random(n)
    hL[dry < 0.1] = rng.uniform(0, 0.02, int((dry < 0.1).sum())).astype(np.float32)
    hR[(dry > 0.9)] = rng.uniform(0, 0.02, int((dry > 0.9).sum())).astype(np.float32)
    huL = (rng.normal(0, 5, n) * hL).astype(np.float32)
    huR = (rng.normal(0, 5, n) * hR).astype(np.float32)
    bL = rng.normal(-5, 5, n).astype(np.float32)
    bR = (bL + rng.normal(0, 2, n)).astype(np.float32)
    flat = rng.random(n) < 0.3
    bR[flat] = bL[flat]
    return hL, hR, huL, huR, bL, bR


def main():
    rng = np.random.default_rng(SEED)
    out = {}
    # --- initScenario -----------------------------------------------------
    inits = {
        "radial_bathymetry_dam_break": (1, [], 48, 40, [O.OUTFLOW] * 4),
        "radial_dam_break": (0, [], 40, 40, [O.OUTFLOW] * 4),
        "sea_at_rest": (2, [], 32, 32, [O.OUTFLOW] * 4),
        "half_domain_dry": (3, [], 32, 24, [O.WALL] * 4),
        "splashing_cone": (6, [], 32, 32, [O.OUTFLOW] * 4),
        "dam_break_1000m": (10, [1000.0, 100.0, 15.0, 10.0, 0.0], 64, 64, [O.OUTFLOW] * 4),
    }
    for name, (sid, params, nx, ny, bnd) in inits.items():
        geo = O.ref_geometry(sid, params, nx, ny)
        h, hu, hv, b = O.ref_init_block(sid, params, nx, ny, float(geo[0]), float(geo[1]), float(geo[2]),
                                        float(geo[3]), bnd)
        np.savez_compressed(os.path.join(HERE, "init_%s.npz" % name), scenario=sid, params=np.asarray(params, float),
                            nx=nx, ny=ny, geometry=geo, bnd=np.asarray(bnd), h=h, hu=hu, hv=hv, b=b)
        out[name] = nx * ny

    # --- unsplit block, one rank -----------------------------------------
    nx, ny, steps = 48, 40, 25
    geo = O.ref_geometry(1, [], nx, ny)
    dx, dy = float(geo[0]), float(geo[1])
    bnd = [O.OUTFLOW, O.WALL, O.OUTFLOW, O.WALL]
    h0, hu0, hv0, b0 = O.ref_init_block(1, [], nx, ny, dx, dy, 0.0, 0.0, bnd)
    for macro, name in ((0, "hlle"), (1, "fwave"), (2, "augrie")):
        h, hu, hv, dts = O.ref_run("unsplit", macro, nx, ny, dx, dy, bnd, h0, hu0, hv0, b0, steps)
        np.savez_compressed(os.path.join(HERE, "unsplit_%s.npz" % name), nx=nx, ny=ny, dx=dx, dy=dy,
                            bnd=np.asarray(bnd), h0=h0, hu0=hu0, hv0=hv0, b0=b0, h=h, hu=hu, hv=hv, dts=dts)

    # --- a shoreline (wet/dry) block: exercises the dry clamp and AugRie --
    nx, ny, steps = 40, 24, 30
    p = [SEED, 50000.0]
    geo = O.ref_geometry(12, p, nx, ny)
    dx, dy = float(geo[0]), float(geo[1])
    bnd = [O.OUTFLOW] * 4
    h0, hu0, hv0, b0 = O.ref_init_block(12, p, nx, ny, dx, dy, 0.0, 0.0, bnd)
    for macro, name in ((0, "hlle"), (1, "fwave"), (2, "augrie")):
        h, hu, hv, dts = O.ref_run("unsplit", macro, nx, ny, dx, dy, bnd, h0, hu0, hv0, b0, steps)
        np.savez_compressed(os.path.join(HERE, "shoreline_%s.npz" % name), nx=nx, ny=ny, dx=dx, dy=dy,
                            bnd=np.asarray(bnd), h0=h0, hu0=hu0, hv0=hv0, b0=b0, h=h, hu=hu, hv=hv, dts=dts)

    # --- serial split block (Hybrid), one thread ---------------------------
    nx, ny, steps = 40, 40, 20
    p = [1000.0, 100.0, 15.0, 10.0, 0.0]
    geo = O.ref_geometry(10, p, nx, ny)
    dx, dy = float(geo[0]), float(geo[1])
    bnd = [O.OUTFLOW] * 4
    h0, hu0, hv0, b0 = O.ref_init_block(10, p, nx, ny, dx, dy, 0.0, 0.0, bnd)
    h, hu, hv, dts = O.ref_run("split", 0, nx, ny, dx, dy, bnd, h0, hu0, hv0, b0, steps)
    np.savez_compressed(os.path.join(HERE, "split_hybrid.npz"), nx=nx, ny=ny, dx=dx, dy=dy, bnd=np.asarray(bnd),
                        h0=h0, hu0=hu0, hv0=hv0, b0=b0, h=h, hu=hu, hv=hv, dts=dts)

    # --- overdecomposed 2 x 3 blocks on one rank ---------------------------
    nxt, nyt, nblocks, steps = 40, 30, 6, 15
    geo = O.ref_geometry(1, [], nxt, nyt)
    dx, dy = float(geo[0]), float(geo[1])
    outer = [O.OUTFLOW, O.WALL, O.OUTFLOW, O.WALL]
    by = int(np.sqrt(nblocks))
    while nblocks % by:
        by -= 1
    bx = nblocks // by
    cols = [nxt // bx] * (bx - 1) + [nxt - (bx - 1) * (nxt // bx)]
    rows = [nyt // by] * (by - 1) + [nyt - (by - 1) * (nyt // by)]
    parts = [[], [], [], []]
    for k in range(bx * by):
        px, py = k // by, k % by
        ox = np.float32(np.float32(px) * np.float32(dx) * np.float32(nxt // bx))
        oy = np.float32(np.float32(py) * np.float32(dy) * np.float32(nyt // by))
        bnd = [O.CONNECT_WITHIN_RANK if px > 0 else outer[0], O.CONNECT_WITHIN_RANK if px < bx - 1 else outer[1],
               O.CONNECT_WITHIN_RANK if py > 0 else outer[2], O.CONNECT_WITHIN_RANK if py < by - 1 else outer[3]]
        arrs = O.ref_init_block(1, [], cols[px], rows[py], dx, dy, float(ox), float(oy), bnd)
        for i in range(4):
            parts[i].append(arrs[i])
    H0, HU0, HV0, B0 = [np.concatenate(p) for p in parts]
    for macro, name in ((0, "hlle"), (1, "fwave"), (2, "augrie")):
        h, hu, hv, b, dts, _ = O.ref_run_overdecomp(macro, cols, rows, dx, dy, outer, H0, HU0, HV0, B0, steps)
        np.savez_compressed(os.path.join(HERE, "overdecomp_%s.npz" % name), nx_cols=np.asarray(cols),
                            ny_rows=np.asarray(rows), dx=dx, dy=dy, outer=np.asarray(outer), h0=H0, hu0=HU0, hv0=HV0,
                            b0=B0, h=h, hu=hu, hv=hv, b=b, dts=dts)

    # --- per-edge solver outputs -------------------------------------------
    ins = edge_states(4096, rng)
    for macro, name in ((0, "hlle"), (1, "fwave"), (2, "augrie")):
        outs = O.ref_solve_edges(macro, *ins)
        np.savez_compressed(os.path.join(HERE, "edges_%s.npz" % name), hL=ins[0], hR=ins[1], huL=ins[2],
                            huR=ins[3], bL=ins[4], bR=ins[5], hUpdL=outs[0], hUpdR=outs[1], huUpdL=outs[2],
                            huUpdR=outs[3], speed=outs[4])
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
