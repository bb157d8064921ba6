"""GPU parity of the fast-arithmetic step (SWE_ARITH_FAST): approximate
reciprocal / square root and fused multiply-adds, one launch per step that
also computes the next maxTimestep.  Results are not bit-identical to the
reference's float solver; the bar is a stated tolerance against the FP32
oracle (the CPU restatement of src/blocks/SWE_DimensionalSplittingMpi.cpp:383-518,
pinned bit for bit to the reference's compiled code by the other tests):

  * every dt within DT_RTOL of the oracle's dt of the same step;
  * after N steps, per field (h, hu, hv): max |fast - FP32 oracle| at most
    4 times the FP32 oracle's own max distance to the FP64 oracle (plus a few
    ulp of the field's scale), and the L1 distance to the FP64 oracle at
    most 1.5 times the FP32 oracle's (check_tolerance);
  * the fused maxTimestep of the next state equals the one a separate
    speed pass over the written state computes (DT_RTOL), including edges
    between work segments (pieces) and edges to boundary ghosts;
  * mass and the FP64 error are no worse than the bit-exact path's.
"""
import numpy as np
import pytest

from helpers import blocks_to_global, interior_mask

pytestmark = pytest.mark.gpu

FAST = 1
FWAVE, HLLE = 1, 4
OUTFLOW, WALL, INFLOW, CONNECT, CONNECT_WITHIN_RANK, PASSIVE = range(6)

DT_RTOL = 2e-5     # relative difference of a dt (a few ulp of the speeds, accumulated time)


def fast_domain(swe, geo, solver, **kw):
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver,
                   arithmetic=FAST, **kw)
    return D


def run_fast(swe, geo, state, solver, nsteps, api="step", **kw):
    D = fast_domain(swe, geo, solver, **kw)
    D.upload(*state)
    D.exchange_bathymetry()
    dts = []
    for _ in range(nsteps):
        # computeNumericalFluxes: the fast step computed this state's dt in
        # the previous launch (a speed pass runs only before the first step)
        if api == "split":
            D.set_ghost_layer()
        D.compute_fluxes()
        dts.append(D.max_timestep())
        if api == "split":
            D.update_unknowns()
        else:
            D.step(1)
    out = D.download()
    status = D.status()
    D.close()
    assert status == 0, status
    return out, np.asarray(dts, np.float64)


def run_oracle(oracle_mod, geo, state, solver, nsteps, precision=32, parallel=False):
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=solver,
                          precision=precision)
    R.set_state(*state)
    R.bathymetry_ghosts()
    dts = R.step_parallel(nsteps)[0] if parallel else R.step(nsteps)
    return R.get_state(np.float32 if precision == 32 else np.float64), np.asarray(dts, np.float64)


def check_tolerance(geo, out, ref, ref64, what):
    """FP32 round-off: the fast step's distance to the FP32 oracle is bounded
    by the FP32 oracle's own distance to the FP64 oracle (the reference's
    float solver is itself only that close to the scheme's exact values):
    per field, max |fast - ref32| <= 4 max |ref32 - ref64| + a few ulp of the
    field's scale, and the L1 distance of the fast step to FP64 is at most
    1.5 times the FP32 oracle's."""
    m = interior_mask(geo["nx_cols"], geo["ny_rows"])
    for i, name in enumerate(("h", "hu", "hv")):
        a = np.asarray(out[i], np.float64)[m]
        r = np.asarray(ref[i], np.float64)[m]
        r64 = np.asarray(ref64[i], np.float64)[m]
        scale = max(np.abs(r64).max(), 1e-3)
        d_fast = np.abs(a - r).max()
        d_ref = np.abs(r - r64).max()
        l1_fast = np.abs(a - r64).sum()
        l1_ref = np.abs(r - r64).sum()
        print("%s %s: max|fast-ref32| %.3e, max|ref32-ref64| %.3e, L1 to FP64: fast %.3e ref32 %.3e (scale %.3e)" % (
            what, name, d_fast, d_ref, l1_fast, l1_ref, scale))
        assert d_fast <= 4.0 * d_ref + 8 * 2.0 ** -23 * scale, (what, name, d_fast, d_ref)
        assert l1_fast <= 1.5 * l1_ref + 8 * 2.0 ** -23 * scale * a.size, (what, name, l1_fast, l1_ref)
    np.testing.assert_array_equal(out[3], ref[3])  # bathymetry untouched


def check_dts(dts, rdts, what):
    rel = np.abs(dts - rdts) / np.abs(rdts)
    print("%s: max relative dt difference %.3e" % (what, rel.max()))
    assert rel.max() <= DT_RTOL, (what, rel.max())


CASES = {
    # scenario, nx, ny, blocks, params, boundary (None = the scenario's)
    "dam_break_2x2": ("SCENARIO_DAM_BREAK", 96, 80, 4, [1000.0, 100.0, 15.0, 10.0, 0.0], None),
    "shoreline_4": ("SCENARIO_SHORELINE", 160, 96, 4, [5, 50000.0], None),
    "dam_break_walls": ("SCENARIO_DAM_BREAK", 130, 70, 6, [1000.0, 120.0, 14.0, 6.0, 0.0], [WALL, OUTFLOW, WALL, PASSIVE]),
    "tsunami_1": ("SCENARIO_TSUNAMI", 256, 256, 1, [256, 3, 100000.0], None),
}


@pytest.mark.parametrize("solver", [HLLE, FWAVE])
@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("api", ["step", "split"])
def test_fast_matches_oracle(swe, oracle_mod, case, solver, api):
    scen, nx, ny, nb, params, bnd = CASES[case]
    geo, *state = swe.init_domain(getattr(swe, scen), nx, ny, nb, params, boundary=bnd)
    nsteps = 30
    out, dts = run_fast(swe, geo, state, solver, nsteps, api=api, tile_rows=64 if nb > 1 else 0)
    ref, rdts = run_oracle(oracle_mod, geo, state, solver, nsteps)
    ref64, _ = run_oracle(oracle_mod, geo, state, solver, nsteps, precision=64)
    check_dts(dts, rdts, case)
    check_tolerance(geo, out, ref, ref64, "%s solver %d" % (case, solver))


@pytest.mark.parametrize("solver", [HLLE, FWAVE])
def test_fast_step_sequences_agree(swe, solver):
    """step(), the reference's call sequence and advance() (captured graphs)
    launch the same kernel: identical results bit for bit."""
    geo, *state = swe.init_domain(swe.SCENARIO_DAM_BREAK, 96, 80, 4, [1000.0, 100.0, 15.0, 10.0, 0.0])
    outs = []
    for mode in ("step", "split", "advance"):
        D = fast_domain(swe, geo, solver)
        D.upload(*state)
        D.exchange_bathymetry()
        if mode == "step":
            D.step(40)
        elif mode == "split":
            for _ in range(40):
                D.set_ghost_layer()
                D.compute_fluxes()
                D.update_unknowns()
        else:
            n, _ = D.advance(1e30, max_steps=40)
            assert n == 40
        outs.append((D.download(), D.time()))
        D.close()
    for o, t in outs[1:]:
        assert t == outs[0][1]
        for a, b in zip(o, outs[0][0]):
            np.testing.assert_array_equal(a, b)


def spike_state(geo, cells, u):
    """h = 2 m at rest, b = 0, and velocity u (x or y) in the listed cells
    (block, x, y, dir) of the concatenated block arrays"""
    shapes = [(geo["nx_cols"][k // len(geo["ny_rows"])], geo["ny_rows"][k % len(geo["ny_rows"])])
              for k in range(len(geo["nx_cols"]) * len(geo["ny_rows"]))]
    offs = np.cumsum([0] + [(nx + 2) * (ny + 2) for nx, ny in shapes])
    n = int(offs[-1])
    h = np.full(n, 2.0, np.float32)
    hu = np.zeros(n, np.float32)
    hv = np.zeros(n, np.float32)
    b = np.zeros(n, np.float32)
    for blk, x, y, d in cells:
        ny = shapes[blk][1]
        i = offs[blk] + x * (ny + 2) + y
        (hv if d else hu)[i] = 2.0 * u
    return h, hu, hv, b


def fused_vs_speed_pass(swe, geo, state, solver, **kw):
    """dt the fast step fused into its launch, against a speed pass over the
    state it wrote (bit-exact arithmetic)"""
    D = fast_domain(swe, geo, solver, **kw)
    D.upload(*state)
    D.exchange_bathymetry()
    D.step(1)
    dt_fused = D.max_timestep()
    new = D.download()
    D.close()
    E = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver,
                   speed_pass=1)
    E.upload(*new)
    E.exchange_bathymetry()
    E.set_ghost_layer()
    E.compute_fluxes()
    dt_exact = E.max_timestep()
    E.close()
    return dt_fused, dt_exact


@pytest.mark.parametrize("solver", [HLLE, FWAVE])
def test_fused_dt_covers_pieces(swe, solver):
    """A fast jet across each piece (edges between two work segments) makes
    that piece's edge the fastest of the next state; the fused dt must match
    the speed pass over the written state."""
    geo = dict(dx=10.0, dy=10.0, nx_cols=[70, 58], ny_rows=[100, 60], boundary=[OUTFLOW] * 4)
    D = fast_domain(swe, geo, solver, tile_rows=64, tile_cols=16)
    pieces = D.fast_pieces()
    D.close()
    assert len(pieces) > 20
    for blk, d, x0, y0, ln in pieces:
        if d == 0:  # x-edge (x0-1 | x0) in row y0 + len/2: both cells fast
            y = y0 + ln // 2
            cells = [(blk, x0 - 1, y, 0), (blk, x0, y, 0)]
        else:
            x = x0 + ln // 2
            cells = [(blk, x, y0 - 1, 1), (blk, x, y0, 1)]
        # a ghost cell (x0-1 = 0 or y0-1 = 0) is rewritten by the ghost layer:
        # put the jet into the neighbour block's rim cell instead
        fixed = []
        for c in cells:
            b, x, y, dd = c
            if x == 0:
                nb = b - len(geo["ny_rows"])
                fixed.append((nb, geo["nx_cols"][nb // len(geo["ny_rows"])], y, dd))
            elif y == 0:
                nb = b - 1
                fixed.append((nb, x, geo["ny_rows"][nb % len(geo["ny_rows"])], dd))
            else:
                fixed.append(c)
        state = spike_state(geo, fixed, 40.0)
        f, e = fused_vs_speed_pass(swe, geo, state, solver, tile_rows=64, tile_cols=16)
        assert abs(f / e - 1.0) <= DT_RTOL, ((blk, d, x0, y0, ln), f, e)


@pytest.mark.parametrize("solver", [HLLE, FWAVE])
@pytest.mark.parametrize("bnd", [OUTFLOW, WALL, INFLOW, PASSIVE])
def test_fused_dt_boundary_ghosts(swe, solver, bnd):
    """Jets into every side of the domain: the edge to the ghost is the
    fastest; outflow copies, walls mirror, the other types keep the ghost."""
    geo = dict(dx=10.0, dy=10.0, nx_cols=[50, 40], ny_rows=[70], boundary=[bnd] * 4)
    for cells, u in (([(0, 1, 30, 0)], -40.0), ([(1, 40, 30, 0)], 40.0), ([(0, 20, 1, 1)], -40.0),
                     ([(1, 20, 70, 1)], 40.0)):
        state = spike_state(geo, cells, u)
        f, e = fused_vs_speed_pass(swe, geo, state, solver, tile_rows=64)
        assert abs(f / e - 1.0) <= DT_RTOL, (cells, f, e)


def test_fused_dt_random_states(swe):
    """Random wet/dry states (dry cells, shallow cells, fast cells) over
    several blocks: fused dt = speed pass dt."""
    rng = np.random.default_rng(7)
    geo = dict(dx=5.0, dy=7.0, nx_cols=[64, 33, 40], ny_rows=[90, 45], boundary=[WALL, OUTFLOW, OUTFLOW, WALL])
    shapes = [(geo["nx_cols"][k // 2], geo["ny_rows"][k % 2]) for k in range(6)]
    n = sum((nx + 2) * (ny + 2) for nx, ny in shapes)
    for trial in range(8):
        h = rng.uniform(0.0, 3.0, n).astype(np.float32)
        h[rng.random(n) < 0.1] = 0.0
        hu = (h * rng.normal(0, 2.0, n)).astype(np.float32)
        hv = (h * rng.normal(0, 2.0, n)).astype(np.float32)
        b = rng.uniform(-1.0, 0.5, n).astype(np.float32)
        for solver in (HLLE, FWAVE):
            f, e = fused_vs_speed_pass(swe, geo, (h, hu, hv, b), solver, tile_rows=64, tile_cols=12)
            assert abs(f / e - 1.0) <= DT_RTOL, (trial, solver, f, e)


def test_fast_ensemble_matches_oracle(swe, oracle_mod):
    """An ensemble in fast arithmetic: every instance within tolerance of its
    own oracle run (own dt)."""
    inst, states = swe.dam_break_ensemble(6, seed=11, sizes=(64, 96, 128, 160))
    E = swe.Ensemble(inst, solver=HLLE, arithmetic=FAST)
    E.upload(*[np.concatenate([st[i] for st in states]) for i in range(4)])
    E.exchange_bathymetry()
    E.step(25)
    out = E.download()
    E.close()
    off = 0
    for (nx, ny, dx, dy, bnd), st in zip(inst, states):
        n = (nx + 2) * (ny + 2)
        geo = dict(dx=dx, dy=dy, nx_cols=[nx], ny_rows=[ny], boundary=list(bnd))
        ref, _ = run_oracle(oracle_mod, geo, st, HLLE, 25)
        ref64, _ = run_oracle(oracle_mod, geo, st, HLLE, 25, precision=64)
        check_tolerance(geo, [a[off:off + n] for a in out], ref, ref64, "instance %dx%d" % (nx, ny))
        off += n


def test_fast_fullsize_tolerance_mass_fp64(swe, oracle_mod):
    """2048^2 as 4 x 4 blocks of 512^2 (the benchmark's configuration), 100
    fast steps against the oracle (FP32, all host cores): dt and state within
    tolerance; mass drift in FP64 no larger than the bit-exact path's plus
    FP32 round-off; relative L1 h error against the FP64 oracle at 512^2 no
    worse than the bit-exact path's bound."""
    N = 2048
    geo, *state = swe.init_domain(swe.SCENARIO_TSUNAMI, N, N, 16, [N, 20261203, 100000.0])
    out, dts = run_fast(swe, geo, state, HLLE, 100)
    ref, rdts = run_oracle(oracle_mod, geo, state, HLLE, 100, parallel=True)
    check_dts(dts, rdts, "2048^2")
    # FP64 reference at this size: the oracle on all host cores
    ref64, _ = run_oracle(oracle_mod, geo, state, HLLE, 100, precision=64, parallel=True)
    check_tolerance(geo, out, ref, ref64, "2048^2 after 100 steps")
    m = interior_mask(geo["nx_cols"], geo["ny_rows"])
    m0 = np.sum(state[0][m].astype(np.float64))
    drift_fast = abs(np.sum(out[0][m].astype(np.float64)) - m0) / m0
    drift_ref = abs(np.sum(ref[0][m].astype(np.float64)) - m0) / m0
    print("mass drift: fast %.3e, oracle %.3e" % (drift_fast, drift_ref))
    assert drift_fast <= drift_ref + 1e-6


def test_fast_error_against_fp64_oracle(swe, oracle_mod):
    geo, *state = swe.init_domain(swe.SCENARIO_TSUNAMI, 512, 512, 4, [512, 5, 100000.0])
    out, _ = run_fast(swe, geo, state, HLLE, 50)
    ref64, _ = run_oracle(oracle_mod, geo, state, HLLE, 50, precision=64)
    ref32, _ = run_oracle(oracle_mod, geo, state, HLLE, 50)
    m = interior_mask(geo["nx_cols"], geo["ny_rows"])
    rel_fast = np.abs(out[0][m] - ref64[0][m]).sum() / np.abs(ref64[0][m]).sum()
    rel_ref = np.abs(ref32[0][m] - ref64[0][m]).sum() / np.abs(ref64[0][m]).sum()
    print("relative L1 h error vs FP64 after 50 steps: fast %.3e, FP32 oracle %.3e" % (rel_fast, rel_ref))
    assert rel_fast < 1e-5


def test_fast_rejects_unsupported(swe):
    geo = dict(dx=1.0, dy=1.0, nx_cols=[16], ny_rows=[16], boundary=[OUTFLOW] * 4)
    for kw in (dict(solver=2), dict(solver=3), dict(solver=4, semantics=1), dict(solver=4, lts_max_timestep=1.0)):
        with pytest.raises(swe.SweGpuError):
            swe.Domain(geo["nx_cols"], geo["ny_rows"], 1.0, 1.0, arithmetic=FAST, **kw)
    for variant in (1, 2, 3):  # one thread mapping: a non-zero kernel_variant is refused
        with pytest.raises(swe.SweGpuError):
            swe.Domain(geo["nx_cols"], geo["ny_rows"], 1.0, 1.0, solver=4, kernel_variant=variant)
