"""Local time stepping on the device against the oracle's restatement of the
reference's local time stepping (itself pinned to the reference's compiled
overdecomposed driver): per interval, every block's power-of-two step count
and, after several intervals, every state array must be bit-identical."""
import numpy as np
import pytest

from helpers import assert_bitwise

pytestmark = pytest.mark.gpu

SOLVERS = {"hlle": 4, "fwave": 1, "augrie": 2, "hybrid": 3}


def run_pair(swe, oracle_mod, solver, nx, ny, nblocks, tsync, duration, intervals, speed_pass=0, seed=11):
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_SHORELINE, nx, ny, nblocks, [seed, 50000.0])
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=solver,
                          lts_max_timestep=tsync, duration=duration)
    R.set_state(h, hu, hv, b)
    R.bathymetry_ghosts()
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver,
                   speed_pass=speed_pass, lts_max_timestep=tsync, duration=duration)
    D.upload(h, hu, hv, b)
    D.exchange_bathymetry()
    t = 0.0
    for i in range(intervals):
        it, rsteps = R.lts_interval()
        assert it > 0, "oracle interval did not finish"
        n, t = D.lts_advance(t + 0.5 * tsync)
        assert n == 1
        _, nint, _, steps = D.lts_state()
        assert nint == i + 1
        assert_bitwise(steps, rsteps.astype(np.int32), "block step counts, interval %d" % i)
    out = D.download()
    assert D.status() == 0
    D.close()
    return out, R.get_state()


@pytest.mark.parametrize("name", ["hlle", "fwave", "augrie", "hybrid"])
def test_lts_matches_oracle(swe, oracle_mod, name):
    (h, hu, hv, _), ref = run_pair(swe, oracle_mod, SOLVERS[name], 128, 96, 16, 1.0, 40.0, 4)
    assert_bitwise(h, ref[0], "h")
    assert_bitwise(hu, ref[1], "hu")
    assert_bitwise(hv, ref[2], "hv")


def test_lts_full_speed_pass_and_uneven_blocks(swe, oracle_mod):
    (h, hu, hv, _), ref = run_pair(swe, oracle_mod, 4, 150, 70, 6, 1.0, 40.0, 3, speed_pass=1)
    assert_bitwise(h, ref[0], "h")
    assert_bitwise(hu, ref[1], "hu")
    assert_bitwise(hv, ref[2], "hv")


@pytest.mark.parametrize("name", ["hlle", "fwave"])
def test_lts_blocks_above_the_check_speed_size(swe, oracle_mod, name):
    """f-wave / HLLE blocks of 144^2 cells, above the 128^2 up to which the
    check kernel runs an interval start's speed pass itself: these take the
    separate speed launch (the smaller blocks of the other tests the check)."""
    (h, hu, hv, _), ref = run_pair(swe, oracle_mod, SOLVERS[name], 288, 288, 4, 1.0, 40.0, 2)
    assert_bitwise(h, ref[0], "h")
    assert_bitwise(hu, ref[1], "hu")
    assert_bitwise(hv, ref[2], "hv")


def test_lts_three_levels_and_half_second_intervals(swe, oracle_mod):
    """Blocks at 8, 4 and 2 steps per interval over the shoreline ramp, and
    an interval of 0.5 (the reference rounds with the absolute dt; its rounding
    assumes an interval of 1 and is reproduced as is)."""
    (h, hu, hv, _), ref = run_pair(swe, oracle_mod, 4, 512, 64, 16, 1.0, 40.0, 2)
    assert_bitwise(h, ref[0], "h")
    assert_bitwise(hu, ref[1], "hu")
    assert_bitwise(hv, ref[2], "hv")
    (h, hu, hv, _), ref = run_pair(swe, oracle_mod, 4, 96, 96, 9, 0.5, 40.0, 3)
    assert_bitwise(h, ref[0], "h")
    assert_bitwise(hu, ref[1], "hu")
    assert_bitwise(hv, ref[2], "hv")


def test_lts_last_interval_reaches_duration(swe, oracle_mod):
    """Intervals up to the duration: the last-timestep notice and DONE ghost
    layers (src/blocks/SWE_Block.hh:375-436)."""
    (h, hu, hv, _), ref = run_pair(swe, oracle_mod, 4, 64, 64, 4, 1.0, 3.0, 4)
    assert_bitwise(h, ref[0], "h")
    assert_bitwise(hu, ref[1], "hu")
    assert_bitwise(hv, ref[2], "hv")


@pytest.mark.parametrize("solver", [4, 2], ids=["hlle_one_cta_check", "augrie_two_cta_check"])
def test_lts_iteration_budget_resumes_bitwise(swe, oracle_mod, solver):
    """swe_gpu_lts_advance with a budget of 2 inner iterations per call: each
    call stops at the budget (graph replays queued past it do nothing) and
    carries the ghost ring into the current buffer; the next call resumes.
    Every interval takes the oracle's number of inner iterations in
    ceil(iterations / 2) calls, and two intervals run that way give the
    oracle's step counts and state bit for bit.  HLLE on these small blocks
    checks with one CTA per block (which also runs the speed pass), the
    augmented solver with two."""
    budget = 2
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_SHORELINE, 128, 96, 16, [11, 50000.0])
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=solver,
                          lts_max_timestep=1.0, duration=40.0)
    R.set_state(h, hu, hv, b)
    R.bathymetry_ghosts()
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver,
                   lts_max_timestep=1.0, duration=40.0)
    D.upload(h, hu, hv, b)
    D.exchange_bathymetry()
    for i in range(2):
        it, rsteps = R.lts_interval()
        assert it > budget
        _, _, start, _ = D.lts_state()
        calls = 0
        while True:
            _, _, it0, _ = D.lts_state()
            D.lts_advance(i + 0.5, max_iterations=budget)
            _, nint, it1, steps = D.lts_state()
            calls += 1
            if nint == i + 1:
                assert 0 < it1 - it0 <= budget
                break
            assert it1 - it0 == budget and calls < 100
        assert it1 - start == it, "inner iterations of interval %d" % i
        assert calls == -(-it // budget)
        assert_bitwise(steps, rsteps.astype(np.int32), "block step counts, interval %d" % i)
    out = D.download()
    assert D.status() == 0
    D.close()
    ref = R.get_state()
    for a, r, name in zip(out, ref, "h hu hv".split()):
        assert_bitwise(a, r, name)


def test_lts_domain_refuses_global_steps(swe):
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_SHORELINE, 64, 64, 4, [11, 50000.0])
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=4,
                   lts_max_timestep=1.0, duration=10.0)
    with pytest.raises(swe.SweGpuError):
        D.step(1)
    D.close()
