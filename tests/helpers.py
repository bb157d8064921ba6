"""Shared helpers of the test-suite (block-array bookkeeping)."""
import numpy as np


def block_shapes(nx_cols, ny_rows):
    by = len(ny_rows)
    return [(int(nx_cols[k // by]), int(ny_rows[k % by])) for k in range(len(nx_cols) * len(ny_rows))]


def interior_mask(nx_cols, ny_rows):
    """Boolean mask selecting interior cells of the concatenated block arrays."""
    parts = []
    for nx, ny in block_shapes(nx_cols, ny_rows):
        m = np.zeros((nx + 2, ny + 2), dtype=bool)
        m[1:-1, 1:-1] = True
        parts.append(m.ravel())
    return np.concatenate(parts)


def blocks_to_global(arr, nx_cols, ny_rows):
    """Concatenated block arrays -> (sum nx, sum ny) interior array indexed [x, y]."""
    bx, by = len(nx_cols), len(ny_rows)
    out = np.zeros((sum(nx_cols), sum(ny_rows)), dtype=arr.dtype)
    off = 0
    x0s = np.cumsum([0] + list(nx_cols))
    y0s = np.cumsum([0] + list(ny_rows))
    for k in range(bx * by):
        px, py = k // by, k % by
        nx, ny = nx_cols[px], ny_rows[py]
        a = arr[off:off + (nx + 2) * (ny + 2)].reshape(nx + 2, ny + 2)
        out[x0s[px]:x0s[px] + nx, y0s[py]:y0s[py] + ny] = a[1:-1, 1:-1]
        off += (nx + 2) * (ny + 2)
    return out


def assert_bitwise(a, b, what=""):
    """Equal bit patterns (so +0 and -0 differ); NaNs match any NaN, whose
    payload the IEEE operations leave to the implementation."""
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, what
    if a.dtype == b.dtype and a.dtype in (np.float32, np.float64):
        ui = np.uint32 if a.dtype == np.float32 else np.uint64
        same = (a.view(ui) == b.view(ui)) | (np.isnan(a) & np.isnan(b))
    else:
        same = (a == b) | (np.isnan(a) & np.isnan(b))
    if not same.all():
        idx = np.argwhere(~same)[:5]
        raise AssertionError("%s: %d of %d values differ, first %s: %s vs %s" % (
            what, int((~same).sum()), a.size, idx.ravel().tolist(), a[~same][:5], b[~same][:5]))
