"""Full-size checks at the benchmark's configuration: 2048 x 2048 cells as
4 x 4 blocks of 512^2, synthetic tsunami, HLLE, unsplit step.
  * bit-exact against the oracle for a few steps (oracle on all host cores);
  * size-independent properties over a longer run: mass conservation in FP64
    (the bump stays away from the outflow boundary), x/y mirror symmetry of a
    symmetric set-up, and the relative L1 height error against the FP64 oracle."""
import numpy as np
import pytest

from helpers import assert_bitwise, blocks_to_global, interior_mask

pytestmark = pytest.mark.gpu

N, NB = 2048, 16
PARAMS = [2048, 20261203, 100000.0]


@pytest.fixture(scope="module")
def tsunami(swe):
    return swe.init_domain(swe.SCENARIO_TSUNAMI, N, N, NB, PARAMS)


def test_fullsize_bitexact_vs_oracle(swe, oracle_mod, tsunami):
    geo, h0, hu0, hv0, b0 = tsunami
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=4)
    D.upload(h0, hu0, hv0, b0)
    D.exchange_bathymetry()
    dts = []
    for _ in range(3):
        D.set_ghost_layer()
        D.compute_fluxes()
        dts.append(D.max_timestep())
        D.update_unknowns()
    out = D.download()
    D.close()
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=4)
    R.set_state(h0, hu0, hv0, b0)
    R.bathymetry_ghosts()
    rdts, _ = R.step_parallel(3)
    ref = R.get_state()
    assert_bitwise(np.asarray(dts, np.float32), rdts.astype(np.float32), "dt")
    for a, b, k in zip(out, ref, ("h", "hu", "hv", "b")):
        assert_bitwise(a, b, k)


def test_fullsize_mass_conservation(swe, tsunami):
    geo, h0, hu0, hv0, b0 = tsunami
    m = interior_mask(geo["nx_cols"], geo["ny_rows"])
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=4)
    D.upload(h0, hu0, hv0, b0)
    D.exchange_bathymetry()
    D.step(200)
    D.sync()
    h = D.download()[0]
    assert D.status() == 0
    D.close()
    m0 = np.sum(h0[m].astype(np.float64))
    m1 = np.sum(h[m].astype(np.float64))
    # FP32 round-off of 200 updates per cell, accumulated in FP64
    assert abs(m1 - m0) / m0 < 2e-6, (m0, m1)


def test_symmetric_setup_stays_symmetric(swe):
    """A radial dam break centred in the box, flat bottom: the x<->y mirror of
    the solution is the solution (unsplit step, HLLE, 2 x 2 blocks)."""
    geo, h0, hu0, hv0, b0 = swe.init_domain(swe.SCENARIO_DAM_BREAK, 512, 512, 4, [1000.0, 150.0, 12.0, 5.0, 0.0])
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=4)
    D.upload(h0, hu0, hv0, b0)
    D.exchange_bathymetry()
    D.step(60)
    D.sync()
    h, hu, hv, _ = [blocks_to_global(a, geo["nx_cols"], geo["ny_rows"]) for a in D.download()]
    D.close()
    assert np.allclose(h, h.T, rtol=0, atol=1e-4)
    assert np.allclose(hu, hv.T, rtol=0, atol=1e-4)


def test_error_against_fp64_oracle(swe, oracle_mod):
    """Relative L1 height error of the FP32 GPU step against the FP64 oracle of
    the same scheme (reported; bound 1e-5 after 50 steps at 512^2)."""
    geo, h0, hu0, hv0, b0 = swe.init_domain(swe.SCENARIO_TSUNAMI, 512, 512, 4, [512, 5, 100000.0])
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=4)
    D.upload(h0, hu0, hv0, b0)
    D.exchange_bathymetry()
    D.step(50)
    D.sync()
    h = D.download()[0]
    D.close()
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=4,
                          precision=64)
    R.set_state(h0, hu0, hv0, b0)
    R.bathymetry_ghosts()
    R.step(50)
    h64 = R.get_state(np.float64)[0]
    m = interior_mask(geo["nx_cols"], geo["ny_rows"])
    rel = np.abs(h[m] - h64[m]).sum() / np.abs(h64[m]).sum()
    print("relative L1 h error vs FP64 oracle after 50 steps: %.3e" % rel)
    assert rel < 1e-5
