"""The multi-rank helpers of bench.py (N independent replicas, one rank per
GPU under torchrun) on CPU: world size 2 over gloo, rendezvous on 127.0.0.1.
Each rank must see the same world, the barrier must hold, and the timing
reduction must be the maximum over the ranks."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "SWE_BENCH_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_init()
    try:
        bench.dist_barrier(w)
        # a per-rank "time" and the value the bench prints: cells of all ranks / max time
        t = 1.0 + 0.5 * r
        tmax = bench.dist_max(t, w)
        out.put((r, w, local, tmax))
        bench.dist_barrier(w)
    finally:
        dist.destroy_process_group()


def test_replica_helpers_over_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    codes = [p.exitcode for p in procs]
    for p in procs:
        if p.is_alive():
            p.kill()
    assert codes == [0, 0], codes
    res = sorted(out.get(timeout=10) for _ in range(world))
    assert [r for r, *_ in res] == [0, 1]
    assert all(w == 2 for _, w, _, _ in res)
    assert all(loc == r for r, _, loc, _ in res)
    assert all(tmax == 1.5 for *_, tmax in res)  # the slowest rank's time on every rank
