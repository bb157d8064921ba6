"""getRoundTimestep on the device against the oracle at its sensitive points.

The reference picks a block's step size as 2^-ceil(log(dt)/log(2)) with the
float log of the time step (src/blocks/SWE_Block.hh:536-555).  Near a power
of two the ceiling depends on the last bit of that float logarithm, which the
device takes from CUDA's logf and the oracle (like the reference) from the
C library's.  This test puts time steps at powers of two times the interval
and up to 4 ulp either side of them, plus seeded random ones, and requires
the same step sizes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def sensitive_timesteps(tsync):
    out = []
    for k in range(0, 11):
        t0 = np.float32(tsync * 2.0 ** -k)
        up = dn = t0
        out.append(t0)
        for _ in range(4):
            up = np.nextafter(up, np.float32(np.inf))
            dn = np.nextafter(dn, np.float32(0))
            out += [up, dn]
    rng = np.random.default_rng(20261203)
    out += list(np.exp(rng.uniform(np.log(tsync / 2048), np.log(tsync * 2), 4000)).astype(np.float32))
    return np.asarray(out, np.float32)


@pytest.mark.parametrize("tsync", [1.0, 0.5, 3.0, 0.1])
def test_round_timestep_matches_oracle(swe, oracle_mod, tsync):
    t = sensitive_timesteps(tsync)
    dev = swe.lts_round_timesteps(t, tsync, 1024)
    ref = oracle_mod.lts_round_timesteps(t, tsync, 1024)
    bad = np.nonzero(dev != ref)[0]
    assert bad.size == 0, [(float(t[i]), int(dev[i]), int(ref[i])) for i in bad[:10]]
