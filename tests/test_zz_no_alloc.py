"""The allocation-free single-block step (swe_gpu_step_block_noalloc) against
the library's regular entry point (a domain handle stepped with
swe_gpu_step), through the C ABI, on two calls in a row.

Callers that cannot allocate device memory (GPU memory owned by another
allocator, latency-critical loops) use this entry point: it keeps its scratch
in a fixed device array instead of calling cudaMalloc.  The tolerance is the
one every GPU parity test here uses: bit-for-bit equality.  This file is
collected last so a failure here stops a -x run only after all other tests."""
import numpy as np
import pytest

from helpers import assert_bitwise

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("solver,semantics,scenario,params,nx,ny", [
    (4, 0, 1, [], 300, 260),                                  # HLLE, unsplit, ragged tiles
    (2, 0, 12, [3, 50000.0], 96, 64),                          # augmented solver, wet/dry shoreline
    (3, 1, 10, [1000.0, 100.0, 15.0, 10.0, 0.0], 128, 128),   # hybrid, split step
    (1, 0, 10, [1000.0, 120.0, 12.0, 6.0, 0.0], 150, 90),     # f-wave, unsplit
    (4, 1, 10, [1000.0, 150.0, 14.0, 7.0, 0.0], 200, 300),    # HLLE, split step over two row tiles
])
def test_noalloc_step_matches_domain_step(swe, solver, semantics, scenario, params, nx, ny):
    geo, h, hu, hv, b = swe.init_domain(scenario, nx, ny, 1, params)
    ld = ny + 2
    # regular entry point: a domain handle (allocates its own buffers)
    D = swe.Domain([nx], [ny], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver, semantics=semantics)
    D.upload(h, hu, hv, b)
    dts_ref = []
    states_ref = []
    for _ in range(2):
        D.set_ghost_layer()
        D.compute_fluxes()
        dts_ref.append(D.max_timestep())
        D.update_unknowns()
        # the allocation-free step leaves the next step's ghost ring in its
        # output; the domain shows the same after an explicit setGhostLayer
        D.set_ghost_layer()
        states_ref.append(D.download())
    D.close()

    # allocation-free entry point on caller-owned device arrays, two calls in a row
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    cur = [dev(h), dev(hu), dev(hv)]
    bd = dev(b)
    nxt = [torch.empty_like(cur[0]) for _ in range(3)]
    torch.cuda.synchronize()
    for call in range(2):
        dt = swe.step_block_noalloc(solver, semantics, nx, ny, geo["dx"], geo["dy"], geo["boundary"], ld,
                                    [t.data_ptr() for t in cur] + [bd.data_ptr()], [t.data_ptr() for t in nxt])
        torch.cuda.synchronize()
        assert np.float32(dt) == np.float32(dts_ref[call]), (call, dt, dts_ref[call])
        for t, ref, k in zip(nxt, states_ref[call][:3], ("h", "hu", "hv")):
            assert_bitwise(t.cpu().numpy(), ref, "call %d %s" % (call, k))
        cur, nxt = nxt, cur


def test_noalloc_rejects_oversized_block(swe):
    """Blocks beyond the fixed scratch capacity fail with a clear error (no GPU work)."""
    z = torch.zeros(16, device="cuda")
    p = z.data_ptr()
    with pytest.raises(swe.SweGpuError) as e:
        swe.step_block_noalloc(4, 0, 100000, 100000, 1.0, 1.0, [0, 0, 0, 0], 100002, [p] * 4, [p] * 3)
    assert "at most" in str(e.value)
