"""GPU checkpoint path: device snapshots (big-endian (y, x) slabs) equal the
host writer's encoding, and the driver executable's checkpoint loop with
NetCDF output matches the oracle's checkpoint loop."""
import os
import subprocess

import numpy as np
import pytest

from helpers import assert_bitwise

pytestmark = pytest.mark.gpu
scipy_io = pytest.importorskip("scipy.io")


def test_snapshot_slabs_match_host_encoding(swe, tmp_path):
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_RADIAL_BATHYMETRY_DAM_BREAK, 96, 70, 4)
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=4)
    D.upload(h, hu, hv, b)
    D.exchange_bathymetry()
    D.step(7)
    D.sync()
    state = D.download()
    for k, (nx, ny) in enumerate(D.shapes):
        bufs = [np.zeros(nx * ny, dtype=">f4") for _ in range(3)]
        D.snapshot_slabs(k, [a.ctypes.data for a in bufs])
        D.snapshot_wait()
        o0, o1 = D.offsets[k], D.offsets[k + 1]
        for a, s in zip(bufs, state[:3]):
            expect = s[o0:o1].reshape(nx + 2, ny + 2)[1:-1, 1:-1].T.ravel()
            assert_bitwise(a.astype(np.float32), expect, "slab block %d" % k)
    D.close()


def test_driver_checkpoints_match_oracle(swe, oracle_mod, tmp_path):
    exe = os.path.join(os.path.dirname(swe.LIB_PATH), "swe_gb300")
    base = str(tmp_path / "run")
    nx, ny, nb, T, ncp = 64, 48, 4, 2.0, 2
    r = subprocess.run([exe, "-t", str(T), "-n", str(ncp), "-x", str(nx), "-y", str(ny), "-o", base, "-w", "1",
                        "--blocks", str(nb), "--solver", "hlle"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Write timestep" in r.stdout
    assert os.path.exists(base + ".log")
    # oracle: same set-up, same checkpoint loop
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_RADIAL_BATHYMETRY_DAM_BREAK, nx, ny, nb)
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=4)
    R.set_state(h, hu, hv, b)
    R.bathymetry_ghosts()
    cp = np.float32(0)
    delta = np.float32(np.float32(T) / np.float32(ncp))
    snaps = []
    for i in range(ncp):
        cp = np.float32(cp + delta)
        R.advance(float(cp))
        snaps.append((np.float32(R.time), R.get_state()))
    by = len(geo["ny_rows"])
    offs = np.cumsum([0] + [(geo["nx_cols"][k // by] + 2) * (geo["ny_rows"][k % by] + 2)
                            for k in range(len(geo["nx_cols"]) * by)])
    for k in range(len(geo["nx_cols"]) * by):
        f = scipy_io.netcdf_file("%s_%d.nc" % (base, k), "r", mmap=False)
        bnx, bny = geo["nx_cols"][k // by], geo["ny_rows"][k % by]
        times = f.variables["time"][:]
        assert len(times) == ncp + 1 and times[0] == 0.0
        for i, (t, st) in enumerate(snaps):
            assert times[i + 1] == t
            for name, a in zip(("ah", "hu", "hv"), st[:3]):
                expect = a[offs[k]:offs[k + 1]].reshape(bnx + 2, bny + 2)[1:-1, 1:-1].T
                assert_bitwise(f.variables[name][i + 1], expect, "block %d %s checkpoint %d" % (k, name, i))
        f.close()


def test_driver_local_timestepping_matches_oracle(swe, oracle_mod, tmp_path):
    """swe_gb300 -l 1: the checkpoint loop over synchronisation intervals,
    NetCDF output bit-identical to the oracle's local time stepping."""
    exe = os.path.join(os.path.dirname(swe.LIB_PATH), "swe_gb300")
    base = str(tmp_path / "lts")
    nx, ny, nb, T, ncp = 128, 96, 16, 3.0, 3
    r = subprocess.run([exe, "-t", str(T), "-n", str(ncp), "-x", str(nx), "-y", str(ny), "-o", base, "-w", "1",
                        "--blocks", str(nb), "--solver", "hlle", "-l", "1", "--scenario", "shoreline", "--seed", "11"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_SHORELINE, nx, ny, nb, [11, 50000.0])
    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=4,
                          lts_max_timestep=1.0, duration=T)
    R.set_state(h, hu, hv, b)
    R.bathymetry_ghosts()
    for _ in range(ncp):
        assert R.lts_interval()[0] > 0
    st = R.get_state()
    by = len(geo["ny_rows"])
    offs = np.cumsum([0] + [(geo["nx_cols"][k // by] + 2) * (geo["ny_rows"][k % by] + 2)
                            for k in range(len(geo["nx_cols"]) * by)])
    for k in range(len(geo["nx_cols"]) * by):
        f = scipy_io.netcdf_file("%s_%d.nc" % (base, k), "r", mmap=False)
        bnx, bny = geo["nx_cols"][k // by], geo["ny_rows"][k % by]
        assert len(f.variables["time"][:]) == ncp + 1
        for name, a in zip(("ah", "hu", "hv"), st[:3]):
            expect = a[offs[k]:offs[k + 1]].reshape(bnx + 2, bny + 2)[1:-1, 1:-1].T
            assert_bitwise(f.variables[name][ncp], expect, "block %d %s" % (k, name))
        f.close()
