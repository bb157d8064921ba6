"""Mass budget of the GPU step, accumulated in FP64 (the dry clamp of
src/blocks/SWE_DimensionalSplittingMpi.cpp:502-515 is the scheme's only mass
source: h < 0 is reset to 0).

  * Shoreline ramp (wet and dry cells, a moving shoreline) inside walls, so
    no mass leaves: the FP32 oracle's clamp never fires there, and the
    drift of every GPU path (bit-exact and fast arithmetic, HLLE and f-wave)
    minus that clamp mass stays at FP32 round-off (MASS_RTOL of the mass).
  * A diverging flow into near vacuum (f-wave), where the clamp does fire:
    the bit-exact GPU path matches the FP32 oracle's mass bit for bit, and
    the FP64 oracle's drift equals its clamp mass to round-off.  So the clamp
    bookkeeping the bench lines report is the only mass source of the scheme
    in exact arithmetic.  The FP32 arithmetic itself loses more than
    round-off there: as the two wave speeds of an edge approach each other,
    the wave strengths grow and their rounding no longer cancels.
"""
import numpy as np
import pytest

from helpers import interior_mask

pytestmark = pytest.mark.gpu

OUTFLOW, WALL = 0, 1
FWAVE, HLLE = 1, 4
EXACT, FAST = 0, 1
MASS_RTOL = 1e-6   # FP32 round-off of a few hundred steps, relative to the mass


def global_to_blocks(a, nx_cols, ny_rows):
    """(sum nx, sum ny) interior array -> concatenated block arrays with zero ghosts."""
    by = len(ny_rows)
    x0s = np.cumsum([0] + list(nx_cols))
    y0s = np.cumsum([0] + list(ny_rows))
    parts = []
    for k in range(len(nx_cols) * by):
        px, py = k // by, k % by
        blk = np.zeros((nx_cols[px] + 2, ny_rows[py] + 2), np.float32)
        blk[1:-1, 1:-1] = a[x0s[px]:x0s[px] + nx_cols[px], y0s[py]:y0s[py] + ny_rows[py]]
        parts.append(blk.ravel())
    return np.concatenate(parts)


def gpu_mass(swe, geo, state, solver, arithmetic, steps):
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver,
                   arithmetic=arithmetic)
    D.upload(*state)
    D.exchange_bathymetry()
    D.step(steps)
    h = D.download()[0]
    assert D.status() == 0
    D.close()
    return h


def oracle_run(oracle_mod, geo, state, solver, steps, precision):
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=solver,
                          precision=precision)
    R.set_state(*state)
    R.bathymetry_ghosts()
    R.step(steps)
    return R.get_state(np.float32 if precision == 32 else np.float64)[0], R.clamp_mass


@pytest.mark.parametrize("solver", [HLLE, FWAVE])
@pytest.mark.parametrize("arithmetic", [EXACT, FAST])
def test_shoreline_mass_budget(swe, oracle_mod, solver, arithmetic):
    geo, *state = swe.init_domain(swe.SCENARIO_SHORELINE, 256, 256, 4, [5, 50000.0], boundary=[WALL] * 4)
    m = interior_mask(geo["nx_cols"], geo["ny_rows"])
    assert (state[0][m] < 0.01).any() and (state[0][m] > 0.01).any()  # wet and dry cells
    steps = 300
    m0 = np.sum(state[0][m], dtype=np.float64)
    h = gpu_mass(swe, geo, state, solver, arithmetic, steps)
    _, clamp32 = oracle_run(oracle_mod, geo, state, solver, steps, 32)
    drift = np.sum(h[m], dtype=np.float64) - m0
    print("shoreline solver %d arithmetic %d: drift %.3e, clamp %.3e, (drift - clamp) / mass %.3e"
          % (solver, arithmetic, drift, clamp32, (drift - clamp32) / m0))
    assert abs(drift - clamp32) <= MASS_RTOL * m0


def test_near_vacuum_clamp_mass(swe, oracle_mod):
    geo, *_ = swe.init_domain(swe.SCENARIO_DAM_BREAK, 128, 128, 4, [1000.0, 150.0, 12.0, 5.0, 0.0],
                              boundary=[WALL] * 4)
    n = 128
    x = (np.arange(n) + 0.5) / n
    X = np.meshgrid(x, x, indexing="ij")[0]
    h2 = np.ones((n, n), np.float32)
    hu2 = (60.0 * np.sign(X - 0.5)).astype(np.float32)  # 1 m of water leaving the centre line at 60 m/s
    cols, rows = geo["nx_cols"], geo["ny_rows"]
    zero = global_to_blocks(np.zeros((n, n), np.float32), cols, rows)
    state = [global_to_blocks(h2, cols, rows), global_to_blocks(hu2, cols, rows), zero, zero.copy()]
    m = interior_mask(cols, rows)
    steps = 50
    m0 = np.sum(state[0][m], dtype=np.float64)
    h = gpu_mass(swe, geo, state, FWAVE, EXACT, steps)
    h32, clamp32 = oracle_run(oracle_mod, geo, state, FWAVE, steps, 32)
    h64, clamp64 = oracle_run(oracle_mod, geo, state, FWAVE, steps, 64)
    drift = np.sum(h[m], dtype=np.float64) - m0
    drift32 = np.sum(h32[m], dtype=np.float64) - m0
    drift64 = np.sum(h64[m], dtype=np.float64) - m0
    print("near vacuum: GPU drift %.6e, FP32 oracle drift %.6e clamp %.6e, FP64 drift %.6e clamp %.6e"
          % (drift, drift32, clamp32, drift64, clamp64))
    assert clamp32 > 1e-3 * m0 and clamp64 > 1e-3 * m0   # the clamp fires
    assert drift == drift32                                 # bit-identical states
    assert abs(drift64 - clamp64) <= 1e-10 * m0            # FP64: the clamp is the only source
