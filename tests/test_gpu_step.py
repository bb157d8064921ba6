"""GPU parity: the CUDA block step (through the C ABI) against the oracle on
the same inputs.  The kernels follow the oracle's operation order with
explicit FMAs and IEEE division/sqrt, so the bar is BIT-EXACT equality of
every state array and every dt (tolerance 0)."""
import numpy as np
import pytest

from conftest import load_golden
from helpers import assert_bitwise

pytestmark = pytest.mark.gpu

SOLVERS = {"hlle": 4, "fwave": 1, "augrie": 2, "hybrid": 3}


def gpu_run(swe, cols, rows, dx, dy, outer, solver, h0, hu0, hv0, b0, nsteps, semantics=0, mode=0, tile_rows=0,
            tile_cols=0, api="split"):
    D = swe.Domain(cols, rows, dx, dy, boundary=outer, solver=solver, semantics=semantics, split_dt_mode=mode,
                   tile_rows=tile_rows, tile_cols=tile_cols)
    D.upload(h0, hu0, hv0, b0)
    D.exchange_bathymetry()
    dts = []
    if api == "split":  # setGhostLayer / computeNumericalFluxes / getMaxTimestep / updateUnknowns
        for _ in range(nsteps):
            D.set_ghost_layer()
            D.compute_fluxes()
            dt = D.max_timestep()
            D.update_unknowns(dt)
            dts.append(dt)
    else:
        D.step(nsteps)
        D.sync()
    out = D.download()
    assert D.status() == 0
    D.close()
    return out, np.asarray(dts, np.float32)


def oracle_run(oracle, cols, rows, dx, dy, outer, solver, h0, hu0, hv0, b0, nsteps, semantics=0, mode=0,
               precision=32, parallel=False):
    D = oracle.Domain(cols, rows, dx, dy, outer=outer, solver=solver, semantics=semantics, split_dt_mode=mode,
                      precision=precision)
    D.set_state(h0, hu0, hv0, b0)
    D.bathymetry_ghosts()
    dts = D.step_parallel(nsteps)[0] if parallel else D.step(nsteps)
    return D.get_state(np.float32 if precision == 32 else np.float64), dts


def compare(gpu, ref, what):
    for a, b, k in zip(gpu, ref, ("h", "hu", "hv", "b")):
        assert_bitwise(a, b, "%s %s" % (what, k))


@pytest.mark.parametrize("name", ["hlle", "fwave", "augrie"])
@pytest.mark.parametrize("case", ["unsplit", "shoreline"])
def test_golden_unsplit(swe, oracle_mod, case, name):
    g = load_golden("%s_%s" % (case, name))
    (h, hu, hv, _), dts = gpu_run(swe, [int(g["nx"])], [int(g["ny"])], float(g["dx"]), float(g["dy"]), g["bnd"],
                                  SOLVERS[name], g["h0"], g["hu0"], g["hv0"], g["b0"], len(g["dts"]))
    assert_bitwise(dts, g["dts"], "dt")
    assert_bitwise(h, g["h"], "h")
    assert_bitwise(hu, g["hu"], "hu")
    assert_bitwise(hv, g["hv"], "hv")


def test_golden_split_hybrid(swe):
    g = load_golden("split_hybrid")
    (h, hu, hv, _), dts = gpu_run(swe, [int(g["nx"])], [int(g["ny"])], float(g["dx"]), float(g["dy"]), g["bnd"],
                                  SOLVERS["hybrid"], g["h0"], g["hu0"], g["hv0"], g["b0"], len(g["dts"]),
                                  semantics=1, mode=1)
    assert_bitwise(dts, g["dts"], "dt")
    assert_bitwise(h, g["h"], "h")
    assert_bitwise(hu, g["hu"], "hu")
    assert_bitwise(hv, g["hv"], "hv")


@pytest.mark.parametrize("name", ["hlle", "fwave", "augrie"])
def test_golden_overdecomposed(swe, name):
    g = load_golden("overdecomp_" + name)
    (h, hu, hv, b), dts = gpu_run(swe, list(g["nx_cols"]), list(g["ny_rows"]), float(g["dx"]), float(g["dy"]),
                                  g["outer"], SOLVERS[name], g["h0"], g["hu0"], g["hv0"], g["b0"], len(g["dts"]))
    assert_bitwise(dts, g["dts"], "dt")
    assert_bitwise(h, g["h"], "h")
    assert_bitwise(hu, g["hu"], "hu")
    assert_bitwise(hv, g["hv"], "hv")
    assert_bitwise(b, g["b"], "b")


CASES = [
    # scenario, params, nx, ny, nblocks, outer, tile_rows, tile_cols
    (1, [], 300, 517, 1, [0, 1, 1, 0], 256, 32),
    (3, [], 97, 65, 6, [1, 1, 1, 1], 64, 7),
    (12, [5, 50000.0], 160, 96, 4, [0, 0, 0, 0], 32, 128),
    (11, [128, 3, 100000.0], 128, 128, 16, [0, 0, 0, 0], 128, 16),
    (6, [], 33, 257, 2, [0, 1, 0, 1], 256, 1),
]


@pytest.mark.parametrize("solver", ["hlle", "fwave", "augrie", "hybrid"])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_random_domains_unsplit(swe, oracle_mod, solver, case):
    sid, params, nx, ny, nb, outer, tr, tc = CASES[case]
    geo, h0, hu0, hv0, b0 = swe.init_domain(sid, nx, ny, nb, params, boundary=outer)
    args = (geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer, SOLVERS[solver], h0, hu0, hv0, b0, 8)
    gpu, gdts = gpu_run(swe, *args, tile_rows=tr, tile_cols=tc, api="split" if case % 2 else "fused")
    ref, rdts = oracle_run(oracle_mod, *args)
    if case % 2:
        assert_bitwise(gdts, rdts.astype(np.float32), "dt")
    compare(gpu, ref, "case %d %s" % (case, solver))


@pytest.mark.parametrize("solver", ["hlle", "augrie"])
@pytest.mark.parametrize("case", [0, 1, 4])
def test_set_ghost_layer_after_update_equals_recomputed_ring(swe, solver, case):
    """setGhostLayer right after an update pass only marks the ring the pass
    pushed as current; the ring must equal the one the ghost kernel computes
    from scratch for the same interior (walls, outflow, intra-rank copies,
    corners), bit for bit."""
    sid, params, nx, ny, nb, outer, tr, tc = CASES[case]
    geo, h0, hu0, hv0, b0 = swe.init_domain(sid, nx, ny, nb, params, boundary=outer)

    def domain():
        D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=outer, solver=SOLVERS[solver])
        return D

    D = domain()
    D.upload(h0, hu0, hv0, b0)
    D.exchange_bathymetry()
    D.step(5)
    D.set_ghost_layer()
    pushed = D.download()
    assert D.status() == 0
    D.close()
    E = domain()
    E.upload(*pushed)  # an upload invalidates the ring: the ghost kernel recomputes it
    E.set_ghost_layer()
    fresh = E.download()
    E.close()
    for a, r, k in zip(pushed, fresh, "h hu hv b".split()):
        assert_bitwise(a, r, k)


@pytest.mark.parametrize("solver", ["hybrid", "hlle", "fwave", "augrie"])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("shape", [(64, 64, 256, 32), (77, 301, 64, 5)])
def test_split_semantics(swe, oracle_mod, solver, mode, shape):
    nx, ny, tr, tc = shape
    geo, h0, hu0, hv0, b0 = swe.init_domain(10, nx, ny, 1, [1000.0, 100.0, 15.0, 10.0, 0.0])
    args = (geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], geo["boundary"], SOLVERS[solver], h0, hu0, hv0,
            b0, 10)
    gpu, gdts = gpu_run(swe, *args, semantics=1, mode=mode, tile_rows=tr, tile_cols=tc)
    ref, rdts = oracle_run(oracle_mod, *args, semantics=1, mode=mode)
    assert_bitwise(gdts, rdts.astype(np.float32), "dt")
    compare(gpu, ref, "split %s mode %d" % (solver, mode))


@pytest.mark.parametrize("solver", ["hlle", "hybrid"])
def test_advance_matches_checkpoint_loop(swe, oracle_mod, solver):
    """swe_gpu_advance runs `while (t < t_end) { step; t += dt; }` on the device."""
    geo, h0, hu0, hv0, b0 = swe.init_domain(1, 96, 80, 4, [])
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"],
                   solver=SOLVERS[solver])
    D.upload(h0, hu0, hv0, b0)
    D.exchange_bathymetry()
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"],
                          solver=SOLVERS[solver])
    R.set_state(h0, hu0, hv0, b0)
    R.bathymetry_ghosts()
    # checkpoint instants accumulate in float like the drivers (src/examples/swe_mpi.cpp:132-139)
    delta = np.float32(np.float32(3.0) / np.float32(3))
    cp = np.float32(0)
    for i in range(3):
        cp = np.float32(cp + delta)
        n, t = D.advance(float(cp))
        rdts = R.advance(float(cp))
        assert n == len(rdts)
        assert np.float32(t) == np.float32(R.time)
        compare(D.download(), R.get_state(), "checkpoint %d" % i)
    D.close()


def test_multiblock_equals_single_block(swe):
    """4 x 4 blocks with on-device halo copies give the same bits as one block
    holding the whole grid (same interior and ghost values)."""
    from helpers import blocks_to_global
    geo1, h, hu, hv, b = swe.init_domain(11, 256, 256, 1, [256, 9, 100000.0])
    g = [blocks_to_global(a, geo1["nx_cols"], geo1["ny_rows"]) for a in (h, hu, hv, b)]
    cols, rows = [64] * 4, [64] * 4
    parts = [[], [], [], []]
    full = [np.pad(a, 1, mode="edge") for a in g]
    for k in range(16):
        px, py = k // 4, k % 4
        for i in range(4):
            parts[i].append(full[i][px * 64:px * 64 + 66, py * 64:py * 64 + 66].ravel())
    h4, hu4, hv4, b4 = [np.concatenate(p) for p in parts]
    single = [np.pad(a, 1, mode="edge").ravel() for a in g]
    (o1, _) = gpu_run(swe, [256], [256], geo1["dx"], geo1["dy"], [0] * 4, 4, *single, 20, api="fused")
    (o4, _) = gpu_run(swe, cols, rows, geo1["dx"], geo1["dy"], [0] * 4, 4, h4, hu4, hv4, b4, 20, api="fused")
    for i, k in enumerate(("h", "hu", "hv")):
        assert_bitwise(blocks_to_global(o4[i], cols, rows), blocks_to_global(o1[i], [256], [256]), k)


def test_nan_state_sets_status_flag(swe):
    """Failure detection without a fault: a NaN state is reported through the
    device status word and the C ABI's error code."""
    geo, h, hu, hv, b = swe.init_domain(10, 64, 64, 1, [1000.0, 100.0, 15.0, 10.0, 0.0])
    h = h.copy()
    h[(64 + 2) * 10 + 10] = np.nan
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], solver=4)
    D.upload(h, hu, hv, b)
    D.step(1)
    D.sync()
    assert D.status() & 2
    with pytest.raises(swe.SweGpuError):
        D.advance(1.0, max_steps=2)
    D.close()


def test_per_block_transfers_with_padded_rows(swe, oracle_mod):
    """swe_gpu_upload_block / swe_gpu_download_block with a column stride ld >
    ny+2 (caller-owned Float2D-like arrays) round-trip and step like the
    whole-domain path."""
    geo, h0, hu0, hv0, b0 = swe.init_domain(1, 70, 45, 6, [])
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=4)
    off = 0
    for k, (nx, ny) in enumerate(D.shapes):
        n = (nx + 2) * (ny + 2)
        ld = ny + 2 + 5
        padded = []
        for a in (h0, hu0, hv0, b0):
            p = np.full((nx + 2, ld), np.nan, dtype=np.float32)
            p[:, :ny + 2] = a[off:off + n].reshape(nx + 2, ny + 2)
            padded.append(p)
        import ctypes
        rc = swe.lib().swe_gpu_upload_block(D.handle, k, *[p.ctypes.data_as(ctypes.c_void_p) for p in padded], ld)
        assert rc == 0
        off += n
    D.exchange_bathymetry()
    D.step(5)
    D.sync()
    out = D.download()
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=4)
    R.set_state(h0, hu0, hv0, b0)
    R.bathymetry_ghosts()
    R.step(5)
    compare(out, R.get_state(), "per-block upload")
    blk = D.download_block(3)
    o0, o1 = D.offsets[3], D.offsets[4]
    for a, b_ in zip(blk, out):
        assert_bitwise(a, b_[o0:o1], "download_block")
    D.close()


@pytest.mark.parametrize("solver", ["hlle", "fwave", "hybrid"])
@pytest.mark.parametrize("semantics", [0, 1])
def test_signed_zero_momenta_through_the_sweep(swe, oracle_mod, solver, semantics):
    """Sea at rest over rough bathymetry with -0 and +0 momenta (and a wet
    patch over -0 bathymetry): the sweep hands out left-going parts of
    subsonic edges without the + 0 of the per-edge form (the sum they join
    starts at +0 or holds a right-going part), so the state, signed zeros
    included, must still equal the oracle's bit for bit after a few steps."""
    rng = np.random.default_rng(11 + semantics)
    nx, ny = (96, 80) if semantics == 0 else (64, 70)
    n = (nx + 2) * (ny + 2)
    b = rng.uniform(-8.0, -2.0, n).astype(np.float32)
    b[rng.random(n) < 0.1] = np.float32(-0.0)
    h = (np.float32(10.0) - b).astype(np.float32)
    hu = np.where(rng.random(n) < 0.5, np.float32(-0.0), np.float32(0.0)).astype(np.float32)
    hv = np.where(rng.random(n) < 0.5, np.float32(-0.0), np.float32(0.0)).astype(np.float32)
    outer = [1, 0, 1, 0]  # walls and outflow sides
    args = ([nx], [ny], 10.0, 10.0, outer, SOLVERS[solver], h, hu, hv, b, 5)
    gpu, _ = gpu_run(swe, *args, semantics=semantics, api="fused")
    ref, _ = oracle_run(oracle_mod, *args, semantics=semantics)
    compare(gpu, ref, "signed zeros %s semantics %d" % (solver, semantics))
