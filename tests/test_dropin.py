"""The drop-in block class for the reference's own class hierarchy
(swe-ppm_gb300/host/SWE_DimensionalSplittingGpu.hh, shown in INTEGRATION.md)
compiled against the reference's headers (src/blocks/SWE_Block.hh,
src/tools/Float2DNative.hh, src/scenarios/SWE_simple_scenarios.hh) into a
program that runs the reference's per-step driver sequence
(src/examples/swe_mpi.cpp:307-316), linked with libswe_gb300.

CPU: the program compiles and links (no GPU call).  GPU: it runs, and its
dts, final state and the reference's host computeMaxTimestep estimate on the
mirrored state (src/blocks/SWE_Block.hh:693-717) are compared with the
oracle bit for bit (exact arithmetic)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_headers():
    import oracle
    src = os.path.join(oracle.REFERENCE_SRC, "src")
    return src if os.path.isdir(os.path.join(src, "blocks")) else None


def build_driver(swe, out):
    src = reference_headers()
    if src is None:
        pytest.skip("no reference tree (stage it with oracle/ref/stage.sh)")
    libdir = os.path.dirname(swe.LIB_PATH)
    cmd = ["g++", "-O2", "-std=c++14", "-w", "-I" + src, "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "swe-ppm_gb300", "host"), os.path.join(ROOT, "tests", "dropin", "drive.cpp"),
           "-L" + libdir, "-lswe_gb300", "-Wl,-rpath," + libdir, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return out


def test_dropin_class_compiles_against_reference_headers(swe, oracle_mod, tmp_path):
    exe = build_driver(swe, str(tmp_path / "drive"))
    assert os.path.getsize(exe) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("solver", [4, 1, 2])
def test_dropin_driver_matches_oracle(swe, oracle_mod, tmp_path, solver):
    exe = build_driver(swe, str(tmp_path / "drive"))
    nx, ny, steps = 120, 90, 12
    out = str(tmp_path / "state.bin")
    r = subprocess.run([exe, out, str(nx), str(ny), str(steps), str(solver)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    n = (nx + 2) * (ny + 2)
    raw = np.fromfile(out, dtype=np.float32)
    h0, hu0, hv0, b0 = (raw[i * n:(i + 1) * n] for i in range(4))
    dts = raw[4 * n:4 * n + steps]
    est = raw[4 * n + steps]
    fin = [raw[4 * n + steps + 1 + i * n:4 * n + steps + 1 + (i + 1) * n] for i in range(3)]
    # the same block from the same initial state, outflow sides, the oracle
    dx = np.float32(1000.0) / nx
    dy = np.float32(1000.0) / ny
    R = oracle_mod.Domain([nx], [ny], float(dx), float(dy), outer=[0, 0, 0, 0], solver=solver)
    R.set_state(h0, hu0, hv0, b0)
    R.bathymetry_ghosts()
    rdts = R.step(steps).astype(np.float32)
    ref = R.get_state()
    np.testing.assert_array_equal(dts.view(np.uint32), rdts.view(np.uint32))
    for a, b_, k in zip(fin, ref, ("h", "hu", "hv")):
        a2 = a.reshape(nx + 2, ny + 2)[1:-1, 1:-1]
        b2 = b_.reshape(nx + 2, ny + 2)[1:-1, 1:-1]
        np.testing.assert_array_equal(a2.view(np.uint32), b2.view(np.uint32), err_msg=k)
    # computeMaxTimestep of the reference on the mirrored final state (dry
    # tolerance 0.1, CFL 0.4), restated in float
    h = ref[0].reshape(nx + 2, ny + 2)[1:-1, 1:-1]
    hu = ref[1].reshape(nx + 2, ny + 2)[1:-1, 1:-1]
    hv = ref[2].reshape(nx + 2, ny + 2)[1:-1, 1:-1]
    wet = h > np.float32(0.1)
    mom = np.maximum(np.abs(hu), np.abs(hv))[wet]
    speed = (mom / h[wet]).astype(np.float32) + np.sqrt(np.float32(9.81) * h[wet]).astype(np.float32)
    expect = np.float32(np.float32(min(dx, dy)) / np.float32(speed.max())) * np.float32(0.4)
    assert est == expect, (est, expect)
