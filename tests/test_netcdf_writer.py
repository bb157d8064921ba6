"""NetCDF snapshot files: the reference writer's variables and layout
(src/writer/NetCdfWriter.cpp:84-234), readable by a NetCDF reader (scipy)."""
import numpy as np
import pytest

scipy_io = pytest.importorskip("scipy.io")


def test_writer_layout_and_values(swe, tmp_path):
    nx, ny = 7, 5
    rng = np.random.default_rng(1)
    b = rng.normal(size=(nx + 2) * (ny + 2)).astype(np.float32)
    path = str(tmp_path / "blk.nc")
    W = swe.NetCdfWriter(path, nx, ny, 2.5, 4.0, 10.0, 20.0, b)
    states = []
    for k, t in enumerate((0.0, 1.25, 2.5)):
        s = [rng.normal(size=(nx + 2) * (ny + 2)).astype(np.float32) for _ in range(3)]
        W.write(t, *s)
        states.append((t, s))
    W.close()
    f = scipy_io.netcdf_file(path, "r", mmap=False)
    assert f.dimensions["x"] == nx and f.dimensions["y"] == ny and f.dimensions["time"] is None
    for v in ("time", "x", "y", "ah", "hu", "hv", "b"):
        assert v in f.variables
    assert f.variables["ah"].dimensions == ("time", "y", "x")
    assert f.variables["b"].dimensions == ("y", "x")
    assert f.variables["time"].units == b"seconds since simulation start"
    assert f.Conventions == b"CF-1.5"
    # cell centres accumulated in float: origin + dx/2, then += dx
    xs = [np.float32(10.0) + np.float32(0.5) * np.float32(2.5)]
    for _ in range(nx - 1):
        xs.append(np.float32(xs[-1] + np.float32(2.5)))
    np.testing.assert_array_equal(f.variables["x"][:], np.asarray(xs, np.float32))
    inner = lambda a: a.reshape(nx + 2, ny + 2)[1:-1, 1:-1].T  # (y, x)
    np.testing.assert_array_equal(f.variables["b"][:], inner(b))
    np.testing.assert_array_equal(f.variables["time"][:], np.asarray([0.0, 1.25, 2.5], np.float32))
    for k, (t, s) in enumerate(states):
        for name, a in zip(("ah", "hu", "hv"), s):
            np.testing.assert_array_equal(f.variables[name][k], inner(a))
    f.close()


def test_writer_file_cut_short_keeps_completed_steps(swe, tmp_path):
    """numrecs is rewritten after each step: a reader sees every finished step."""
    nx, ny = 4, 3
    b = np.zeros((nx + 2) * (ny + 2), np.float32)
    path = str(tmp_path / "cut.nc")
    W = swe.NetCdfWriter(path, nx, ny, 1.0, 1.0, 0.0, 0.0, b)
    z = np.ones_like(b)
    W.write(0.5, z, z, z)
    f = scipy_io.netcdf_file(path, "r", mmap=False)  # writer still open
    assert f.variables["ah"].shape == (1, ny, nx)
    f.close()
    W.close()
