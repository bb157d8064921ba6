"""Asynchronous whole-domain transfers: a pipeline of upload / step /
download with a different input every step and a separate output array per
step must give, step for step, exactly the synchronous path's results (the
second staging slot and the copy stream must not let one step's download see
another step's state)."""
import numpy as np
import pytest

from helpers import assert_bitwise

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def pinned(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).pin_memory().numpy()


@pytest.mark.parametrize("solver", [4, 2])
def test_pipelined_transfers_equal_synchronous(swe, solver):
    geo, h, hu, hv, b = swe.init_domain(0, 192, 160, 4, None)
    rng = np.random.default_rng(5)
    inputs = []
    for k in range(5):
        hk = (h * (1 + 0.05 * k)).astype(np.float32)
        huk = (hu + rng.normal(0, 0.1, hu.shape)).astype(np.float32)
        inputs.append([pinned(a) for a in (hk, huk, hv, b)])

    def domain():
        D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver)
        D.upload(*inputs[0])
        D.exchange_bathymetry()
        return D

    D = domain()
    ref = []
    for k in range(5):
        D.upload(*inputs[k])
        D.step(2)
        ref.append(D.download()[:3])
    D.close()

    D = domain()
    outs = [[pinned(np.zeros_like(h)) for _ in range(3)] for _ in range(5)]
    for k in range(5):
        D.upload_async(*inputs[k])
        D.step(2)
        D.download_async(outs[k])
    D.sync()
    assert D.status() == 0
    D.close()
    for k in range(5):
        for a, r, name in zip(outs[k], ref[k], "h hu hv".split()):
            assert_bitwise(a, r, "step %d %s" % (k, name))
