"""Benchmark of the GB300 block step.

Workload (default): the synthetic tsunami at 2048 x 2048 cells as 4 x 4 blocks
of 512^2 (100 km box, b = -2000 + 500 sin cos + seeded noise, Gaussian bump),
HLLE solver, unsplit step (the path swe_benchmark_mpi runs), global time
stepping.  One bench step = one time step (ghost layer + fluxes/dt + update)
of the whole domain.  Metric: cell-updates/s (higher is better).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--arith fast|exact]

gb300 arm: the fast-arithmetic step (one launch per step; the bit-exact step
is reported beside it); state resident in HBM; L2 (126 MB) is flushed by
writing 256 MB between timed steps (the 2048^2 state, 67 MB, would otherwise
stay in L2); each step is timed with CUDA events on the library's stream.
`e2e` runs the same steps through the C ABI on host buffers: upload h, hu,
hv, b from pinned memory, step, download h, hu, hv, timed on the host clock.
`roofline` is the step kernel's algorithmic bytes (28 B/cell) over its
event-timed duration.  `cpu_baseline` times the reference's own stock CPU
benchmark driver (swe_benchmark_mpioverdecomp, built on this host from the
staged reference sources) on all host cores for a bounded span, or, without
those sources, the oracle (the CPU restatement of the reference's block code).
reference arm: the same CPU leg, one bounded sample per step.
Multi-GPU: replicas only (independent copies, no collective in the step);
value = all ranks' cell updates / max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "swe-ppm_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

N_CELLS_SIDE = 2048
N_BLOCKS = 16
SEED = 20261203
BYTES_PER_CELL = 28  # read h, hu, hv, b; write h, hu, hv (FP32)
METRIC = "cell-updates/s at 2048^2 (plain fused path, HLLE, unsplit step)"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def workload_config(extra=None):
    cfg = {"workload": "synthetic tsunami 2048x2048 as 4x4 blocks of 512^2, HLLE, unsplit step, GTS",
           "cells": N_CELLS_SIDE * N_CELLS_SIDE, "blocks": "4x4", "block_cells": "512x512", "solver": "hlle",
           "semantics": "unsplit (SWE_DimensionalSplittingMpi)", "seed": SEED,
           "l2": "flushed between timed steps (256 MB write)"}
    if extra:
        cfg.update(extra)
    return cfg


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def setup_domain(swe, device, n=N_CELLS_SIDE, solver=None, arithmetic=None):
    solver = swe.HLLE if solver is None else solver
    arithmetic = swe.FAST if arithmetic is None else arithmetic
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_TSUNAMI, n, n, N_BLOCKS, [n, SEED, 100000.0])
    tile_rows = int(os.environ.get("SWE_TILE_ROWS", "0"))
    tile_cols = int(os.environ.get("SWE_TILE_COLS", "0"))
    speed_pass = int(os.environ.get("SWE_SPEED_PASS", "0"))  # 1: evaluate every edge in the speed pass
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver,
                   tile_rows=tile_rows, tile_cols=tile_cols, device=device, speed_pass=speed_pass,
                   arithmetic=arithmetic)
    D.upload(h, hu, hv, b)
    D.exchange_bathymetry()
    return D, geo, (h, hu, hv, b)


def timed_steps(D, stream, flush, steps):
    """`steps` steps, L2 flushed before each, CUDA events around each step on
    the library's stream; returns the milliseconds of every step"""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for e0, e1 in ev:
            flush.zero_()
            e0.record(stream)
            D.step(1)
            e1.record(stream)
    stream.synchronize()
    return [e0.elapsed_time(e1) for e0, e1 in ev]


def kernel_times(D, stream, flush, steps):
    """the reference's call sequence, L2 flushed before each step, events
    between the calls: mean ms of setGhostLayer, computeNumericalFluxes and
    updateUnknowns (the fast step: the ghost ring and the dt come from the
    previous launch, so the first two launch nothing)"""
    import torch
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(steps)]
    with torch.cuda.stream(stream):
        for e in ev:
            flush.zero_()
            e[0].record(stream)
            D.set_ghost_layer()
            e[1].record(stream)
            D.compute_fluxes()
            e[2].record(stream)
            D.update_unknowns()
            e[3].record(stream)
    stream.synchronize()
    return {k: statistics.mean(e[i].elapsed_time(e[i + 1]) for e in ev) for i, k in
            enumerate(("ghost", "speed", "update"))}


def accuracy_measure(swe, device, steps=100):
    """Error of the GPU steps against the FP64 oracle of the same scheme on
    the benchmark's workload (2048^2 tsunami, HLLE, unsplit), after `steps`
    steps from the initial state: relative L1 and max |dh| of the fast step,
    of the bit-exact step (identical to the FP32 oracle, the reference's own
    float arithmetic), and mass drift in FP64 of all three.  The tsunami stays
    wet (no dry clamp) and its bump does not reach the outflow sides in this
    time, so mass is conserved up to round-off."""
    import oracle
    oracle.build()
    out = {}
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_TSUNAMI, N_CELLS_SIDE, N_CELLS_SIDE, N_BLOCKS,
                                        [N_CELLS_SIDE, SEED, 100000.0])
    m = []
    off = 0
    for k in range(len(geo["nx_cols"]) * len(geo["ny_rows"])):
        nx, ny = geo["nx_cols"][k // len(geo["ny_rows"])], geo["ny_rows"][k % len(geo["ny_rows"])]
        a = np.zeros((nx + 2, ny + 2), bool)
        a[1:-1, 1:-1] = True
        m.append(a.ravel())
    m = np.concatenate(m)
    states = {}
    for name, arith in (("fast", swe.FAST), ("exact", swe.EXACT)):
        D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"],
                       solver=swe.HLLE, device=device, arithmetic=arith)
        D.upload(h, hu, hv, b)
        D.exchange_bathymetry()
        D.step(steps)
        D.sync()
        states[name] = D.download()[0][m].astype(np.float64)
        D.close()
    R = oracle.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=oracle.HLLE,
                      precision=64)
    R.set_state(h, hu, hv, b)
    R.bathymetry_ghosts()
    R.step_parallel(steps)
    h64 = R.get_state(np.float64)[0][m]
    m0 = float(np.sum(h[m].astype(np.float64)))
    out = {"workload": "tsunami 2048^2 as 4x4 blocks of 512^2, HLLE, unsplit, %d steps from the initial state" % steps,
           "against": "FP64 oracle (CPU restatement of the reference's block code in double)", "steps": steps}
    for name in ("fast", "exact"):
        d = states[name] - h64
        out[name] = {"rel_l1_h": float(np.abs(d).sum() / np.abs(h64).sum()),
                     "rel_linf_h": float(np.abs(d).max() / np.abs(h64).max()), "max_abs_dh": float(np.abs(d).max()),
                     "mass_drift_rel": float(abs(states[name].sum() - m0) / m0)}
    out["exact"]["note"] = "bit-identical to the FP32 oracle (the reference's float arithmetic)"
    out["fp64_mass_drift_rel"] = float(abs(h64.sum() - m0) / m0)
    out["clamp_mass"] = float(R.clamp_mass)  # depth the FP64 run's dry clamp added
    return out


def cpu_baseline(seconds=12.0):
    """The oracle on all host cores (one OpenMP thread per block), a bounded
    number of steps of the same 2048^2 workload."""
    import oracle
    import swe_gb300 as swe
    oracle.build()
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_TSUNAMI, N_CELLS_SIDE, N_CELLS_SIDE, N_BLOCKS,
                                        [N_CELLS_SIDE, SEED, 100000.0])
    R = oracle.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=oracle.HLLE)
    R.set_state(h, hu, hv, b)
    R.bathymetry_ghosts()
    t0 = time.perf_counter()
    _, threads = R.step_parallel(1)  # also calibrates
    t1 = time.perf_counter()
    per = max(t1 - t0, 1e-3)
    n = max(1, min(10000, int(seconds / per)))
    t0 = time.perf_counter()
    R.step_parallel(n)
    el = time.perf_counter() - t0
    cells = N_CELLS_SIDE * N_CELLS_SIDE
    return {"value": cells * n / el, "unit": "cell-updates/s", "cores": int(threads), "kind": "port",
            "sample": "%d steps of the 2048^2 workload (oracle, OpenMP over 16 blocks), %.1f s" % (n, el),
            "seconds_per_step": el / n}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("SWE_BENCH_BACKEND", "") != "gloo" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def dist_max(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def host_cpu():
    """(cores usable, CPU model) of this host"""
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    model = "unknown"
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return int(cores), model


def reference_binary():
    """The reference's stock overdecomposed driver (src/examples/swe_mpi_overdecomp.cpp
    with its blocks, release flags and OpenMP), built from its sources on this
    host by oracle/ref/Makefile; None where the sources are absent."""
    import oracle
    try:
        if not oracle.reference_available():
            oracle.stage_reference()
        if oracle.reference_available():
            return oracle.build_reference_perf()
    except Exception as e:
        log("reference build failed:", e)
    return None


def reference_run(binary, duration, blocks=N_BLOCKS, cells=N_CELLS_SIDE, lts=0.0):
    """One run of the stock driver at cells^2 over `blocks` blocks for
    `duration` simulated seconds on every host core (lts > 0: local time
    stepping with intervals of `lts` s, its -l); returns (cell-updates, wall
    seconds).  Cell-updates come from the driver's own log (FLOP_COUNT /
    270, src/tools/Collector.hpp:129-142, 270 flop per cell-update at
    src/blocks/SWE_DimensionalSplittingMpi.cpp:458).  Its WALL_TIME column is
    not usable: the driver folds the blocks' collectors into its own with a
    minimum over wall time (src/tools/Collector.hpp:42-43), and the blocks
    never run that counter, so the log holds 0; the wall time is taken around
    the process instead, and the set-up cost is removed by the caller."""
    import tempfile
    cores, _ = host_cpu()
    with tempfile.TemporaryDirectory() as tmp:
        base = os.path.join(tmp, "ref")
        env = dict(os.environ, OMP_NUM_THREADS=str(cores))
        t0 = time.perf_counter()
        r = subprocess.run([binary, "-x", str(cells), "-y", str(cells), "-b", str(blocks), "-t", repr(float(duration)),
                            "-n", "1", "-o", base, "-w", "0", "-l", repr(float(lts))], capture_output=True, text=True,
                           env=env,
                           cwd=tmp)
        el = time.perf_counter() - t0
        if r.returncode != 0:
            raise RuntimeError("reference driver failed: " + r.stderr[-500:])
        rows = open(base + ".log").read().strip().splitlines()
        flop = float(rows[-1].split(",")[1])
    return flop / 270.0, el


def port_tsunami_state():
    """The tsunami workload's shape for the oracle port, built with numpy
    alone (the CPU legs load no product library): 2048^2 over 100 km as 4 x 4
    blocks of 512^2 in the blocks' Float2D layout with ghost rings, sinusoidal
    bathymetry around -2000 m with seeded noise, still water and a 5 m bump.
    The cost of a wet step does not depend on the values."""
    n, nb = N_CELLS_SIDE, 4
    m = n // nb
    L = 100000.0
    dx = L / n
    rng = np.random.default_rng(SEED)
    xc = (np.arange(n) + 0.5) * dx
    X, Y = np.meshgrid(xc, xc, indexing="ij")
    bath = -2000.0 + 500.0 * np.sin(2 * np.pi * X / L) * np.cos(2 * np.pi * Y / L) + rng.normal(0.0, 20.0, (n, n))
    cx, cy = rng.uniform(0.3 * L, 0.7 * L, 2)
    eta = 5.0 * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * 5000.0 ** 2))
    fields = [eta - bath, np.zeros((n, n)), np.zeros((n, n)), bath]
    parts = [[], [], [], []]
    for k in range(nb * nb):
        px, py = k // nb, k % nb
        for i, f in enumerate(fields):
            blk = np.zeros((m + 2, m + 2), np.float32)
            blk[1:-1, 1:-1] = f[px * m:(px + 1) * m, py * m:(py + 1) * m]
            blk[0, :], blk[-1, :] = blk[1, :], blk[-2, :]
            blk[:, 0], blk[:, -1] = blk[:, 1], blk[:, -2]
            parts[i].append(blk.ravel())
    geo = dict(dx=dx, dy=dx, nx_cols=[m] * nb, ny_rows=[m] * nb, boundary=[0] * 4)
    return (geo,) + tuple(np.concatenate(p) for p in parts)


def run_reference(args, world, rank):
    """The reference's own CPU path on the host cores: its stock
    overdecomposed driver (swe_benchmark_mpioverdecomp: 16 blocks of 512^2,
    OpenMP over the blocks, HLLE -- the solver its build selects) timed as
    built from its sources on this host.  Each step is one run over a short
    simulated span; the cost of a run that only sets up and takes a few steps
    is subtracted.  Without the sources, the oracle (a line-by-line
    restatement of the reference's block code) on all host cores."""
    if rank != 0:
        return 0
    cores, model = host_cpu()
    binary = reference_binary()
    if binary:
        span = float(os.environ.get("SWE_REF_SPAN", "0.5"))
        u0, w0 = reference_run(binary, 0.02)  # set-up and the first steps
        for _ in range(max(args.warmup, 1) - 1):
            reference_run(binary, 0.02)
        rates, secs = [], []
        for _ in range(args.steps):
            u, w = reference_run(binary, span)
            rates.append((u - u0) / max(w - w0, 1e-6))
            secs.append(w - w0)
        value = statistics.median(rates)
        sample = ("%d runs of the stock swe_benchmark_mpioverdecomp -x %d -y %d -b %d -t %g (its radial-bathymetry dam "
                  "break, HLLE), minus a -t 0.02 run's set-up; %d OpenMP threads on %s" % (
                      args.steps, N_CELLS_SIDE, N_CELLS_SIDE, N_BLOCKS, span, cores, model))
        kind = "reference"
        ms_per_step = 1e3 * N_CELLS_SIDE * N_CELLS_SIDE / value
    else:
        import oracle
        oracle.build()
        geo, h, hu, hv, b = port_tsunami_state()
        R = oracle.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"],
                          solver=oracle.HLLE)
        R.set_state(h, hu, hv, b)
        R.bathymetry_ghosts()
        threads = 1
        for _ in range(max(args.warmup, 3)):
            _, threads = R.step_parallel(1)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            R.step_parallel(1)
            times.append(time.perf_counter() - t0)
        per = sum(times) / len(times)
        value = N_CELLS_SIDE * N_CELLS_SIDE / per
        ms_per_step = 1e3 * per
        cores = int(threads)
        kind = "port"
        sample = "%d full time steps of the 2048^2 workload, oracle with OpenMP over 16 blocks on %d threads (%s)" % (
            args.steps, threads, model)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config({"parallelism": "host cores"}),
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": int(cores), "kind": kind,
                             "sample": sample, "cpu_model": model},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def lts_fp64_proxy(swe, device, n=256, duration=200.0):
    """Error and mass of local time stepping against the FP64 oracle, on a
    coarser copy of the benchmark's set-up (n^2 as 8x8 blocks, the same 50 km
    shoreline ramp and bump, 1 s intervals, `duration` s): the FP64 oracle of
    the 2048^2 run would take minutes on the host."""
    import oracle
    oracle.build()
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_SHORELINE, n, n, 64, [SEED, 50000.0])
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=swe.HLLE,
                   device=device, lts_max_timestep=1.0, duration=duration)
    D.upload(h, hu, hv, b)
    D.exchange_bathymetry()
    D.lts_advance(duration)
    g = D.download()[0].astype(np.float64)
    D.close()
    res = {}
    for p in (32, 64):
        R = oracle.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=oracle.HLLE,
                          precision=p, lts_max_timestep=1.0, duration=duration)
        R.set_state(h, hu, hv, b)
        R.bathymetry_ghosts()
        for _ in range(int(round(duration))):
            R.lts_interval()
        res[p] = (R.get_state(np.float64)[0], R.clamp_mass)
    m = []
    for k in range(64):
        nx, ny = geo["nx_cols"][k // 8], geo["ny_rows"][k % 8]
        a = np.zeros((nx + 2, ny + 2), bool)
        a[1:-1, 1:-1] = True
        m.append(a.ravel())
    m = np.concatenate(m)
    h64 = res[64][0][m]
    m0 = float(np.sum(h[m].astype(np.float64)))
    return {"workload": "%dx%d as 8x8 blocks, same ramp and bump, %g s" % (n, n, duration),
            "rel_l1_h_gpu": float(np.abs(g[m] - h64).sum() / np.abs(h64).sum()),
            "rel_l1_h_fp32_oracle": float(np.abs(res[32][0][m] - h64).sum() / np.abs(h64).sum()),
            "max_abs_dh_gpu": float(np.abs(g[m] - h64).max()),
            "mass_change_rel_gpu": float((g[m].sum() - m0) / m0),
            "mass_change_rel_fp64": float((h64.sum() - m0) / m0),
            "clamp_mass_rel_fp64": float(res[64][1] / m0),
            "note": "outflow sides: mass change = outflow through the sides + depth the dry clamp added"}


def lts_measure(swe, device, duration=200.0):
    """Local time stepping at 2048^2 as 8x8 blocks of 256^2 over a 50 km
    shoreline ramp (bathymetry -4000 m to +50 m across x, seeded Gaussian
    bump), HLLE, synchronisation intervals of 1 s: blocks step at 2^k
    substeps per interval.  The first interval is the warm-up; the rest up to
    `duration` s simulated are timed (host clock around the device-driven
    interval loop); cell-updates summed over the blocks' own steps."""
    n, nb = 2048, 64
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_SHORELINE, n, n, nb, [SEED, 50000.0])
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=swe.HLLE,
                   device=device, lts_max_timestep=1.0, duration=duration)
    D.upload(h, hu, hv, b)
    D.exchange_bathymetry()
    D.lts_advance(1.0)
    cells = np.array([geo["nx_cols"][k // len(geo["ny_rows"])] * geo["ny_rows"][k % len(geo["ny_rows"])]
                      for k in range(nb)], dtype=np.float64)
    s0 = D.block_steps()
    t0 = time.perf_counter()
    done, t = D.lts_advance(duration)
    el = time.perf_counter() - t0
    s1 = D.block_steps()
    _, _, iters, per_interval = D.lts_state()
    status = D.status()
    updates = float(np.dot(cells, (s1 - s0).astype(np.float64)))
    D.close()
    levels = sorted(set(int(v) for v in per_interval))
    # the global step (exact arithmetic, as local time stepping uses) on the
    # same domain: 40 back-to-back steps between CUDA events
    import torch
    G = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=swe.HLLE,
                   device=device)
    G.upload(h, hu, hv, b)
    G.exchange_bathymetry()
    gs = torch.cuda.Stream()
    G.set_stream(gs.cuda_stream)
    with torch.cuda.stream(gs):
        G.step(5)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(gs)
        G.step(40)
        e1.record(gs)
        gs.synchronize()
    global_rate = float(cells.sum()) * 40 / (1e-3 * e0.elapsed_time(e1))
    G.close()
    return {"workload": "local time stepping, shoreline ramp 2048x2048 as 8x8 blocks of 256^2, HLLE, 1 s intervals, "
                        "%g s simulated" % duration,
            "value": updates / el, "unit": "cell-updates/s (sum over blocks of cells x own steps)",
            "intervals": done, "t_end": t, "seconds": el, "block_steps_per_interval": levels,
            "mean_steps_per_block_interval": float(np.mean((s1 - s0) / max(1, done))), "device_status": status,
            "global_step_same_domain": {"value": global_rate, "unit": "cell-updates/s",
                                        "note": "exact global time stepping on the same 8x8 blocks, 40 steps back to back"},
            "ratio_to_global_step": updates / el / global_rate,
            "fp64_proxy": lts_fp64_proxy(swe, device, duration=duration)}


def ensemble_measure(swe, device, steps=100, count=256):
    """Batched ensemble: 256 independent radial dam breaks (nx, ny uniform in
    64, 96, ..., 1024; radius U(0.05, 0.3) L; inner height U(5, 20) m, outer
    U(1, 5) m; b = 0; one seed) in one handle, tile shape chosen by the tuner,
    100 steps each at its own CFL dt, captured-graph replay (swe_gpu_advance),
    in both arithmetics.  Cell-updates summed over the instances.  Accuracy:
    the first 8 instances against the FP64 oracle after the same steps."""
    import torch
    import oracle
    inst, states = swe.dam_break_ensemble(count, seed=SEED)
    cells = np.array([nx * ny for nx, ny, *_ in inst], dtype=np.float64)
    out = {"workload": "256 radial dam breaks, nx, ny in 64..1024, HLLE, unsplit, own dt each, graph replay",
           "unit": "cell-updates/s (sum over instances)", "cells": int(cells.sum())}
    finals = {}
    for name, arith in (("exact", swe.EXACT), ("fast", swe.FAST)):
        E = swe.Ensemble(inst, solver=swe.HLLE, device=device, arithmetic=arith)
        E.upload(*[np.concatenate([st[i] for st in states]) for i in range(4)])
        E.exchange_bathymetry()
        rows, cols, _ = E.autotune(trial_steps=3)
        E.upload(*[np.concatenate([st[i] for st in states]) for i in range(4)])
        E.advance(1e30, max_steps=16)  # warm-up (graph capture)
        stream = torch.cuda.Stream()
        E.set_stream(stream.cuda_stream)
        s0 = E.group_state()[2].astype(np.int64)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            n, _ = E.advance(1e30, max_steps=steps)
            e1.record(stream)
            stream.synchronize()
        ms = e0.elapsed_time(e1)
        s1 = E.group_state()[2].astype(np.int64)
        updates = float(np.dot(cells, (s1 - s0).astype(np.float64)))
        finals[name] = (E.download()[0], int(s1[0]))
        E.close()
        out[name] = {"value": updates / (ms * 1e-3), "steps": int(n), "ms": ms, "tile_rows": rows, "tile_cols": cols}
    out["value"] = max(out["exact"]["value"], out["fast"]["value"])
    # accuracy of the first instances after the same number of steps (the
    # warm-up's 16 plus the timed ones)
    oracle.build()
    errs = {"fast": [], "exact": []}
    linf = {"fast": [], "exact": []}
    mass = {"fast": [], "exact": [], "fp64": []}
    clamp = 0.0
    off = 0
    for i in range(8):
        nx, ny, dx, dy, bnd = inst[i]
        sz = (nx + 2) * (ny + 2)
        R = oracle.Domain([nx], [ny], dx, dy, outer=bnd, solver=oracle.HLLE, precision=64)
        R.set_state(*states[i])
        R.bathymetry_ghosts()
        R.step(finals["fast"][1])
        h64 = R.get_state(np.float64)[0]
        clamp += float(R.clamp_mass)
        a = np.zeros((nx + 2, ny + 2), bool)
        a[1:-1, 1:-1] = True
        a = a.ravel()
        m0 = float(np.sum(states[i][0][a].astype(np.float64)))
        mass["fp64"].append(abs(float(h64[a].sum()) - m0) / m0)
        for name in ("fast", "exact"):
            g = finals[name][0][off:off + sz].astype(np.float64)
            errs[name].append(float(np.abs(g[a] - h64[a]).sum() / np.abs(h64[a]).sum()))
            linf[name].append(float(np.abs(g[a] - h64[a]).max() / np.abs(h64[a]).max()))
            mass[name].append(abs(float(g[a].sum()) - m0) / m0)
        off += sz
    out["fp64_first8"] = {"steps": finals["fast"][1], "rel_l1_h_fast_max": max(errs["fast"]),
                          "rel_l1_h_exact_max": max(errs["exact"]), "rel_linf_h_fast_max": max(linf["fast"]),
                          "rel_linf_h_exact_max": max(linf["exact"]), "mass_change_rel_fast_max": max(mass["fast"]),
                          "mass_change_rel_exact_max": max(mass["exact"]), "mass_change_rel_fp64_max": max(mass["fp64"]),
                          "clamp_mass_fp64": clamp,
                          "note": "mass change: flow through open sides plus depth the dry clamp added"}
    return out


def drivers_measure():
    """The driver executable (swe-ppm_gb300/_build/swe_gb300, the reference
    drivers' flags) on two of the reference's run lines, timed by the
    driver's own wall clock around its checkpoint loop, which includes the
    asynchronous snapshots and the NetCDF writes (-w 1, one file per block,
    as the reference's WALL_TIME covers its writer): the 256^2 radial dam
    break with the hybrid solver to 10 s in 5 checkpoints, and the 2048^2
    tsunami as 4 x 4 blocks to 80 s in 20 checkpoints in both arithmetics."""
    import shutil
    import tempfile
    exe = os.path.join(ROOT, "swe-ppm_gb300", "_build", "swe_gb300")
    runs = {
        "radial_dam_break_256_hybrid_10s": ["-t", "10", "-n", "5", "-x", "256", "-y", "256", "--scenario",
                                            "radial_dam_break", "--solver", "hybrid"],
        "tsunami_2048_80s_fast": ["-t", "80", "-n", "20", "-x", "2048", "-y", "2048", "--blocks", "16", "--scenario",
                                  "tsunami", "--solver", "hlle", "--arithmetic", "fast"],
        "tsunami_2048_80s_exact": ["-t", "80", "-n", "20", "-x", "2048", "-y", "2048", "--blocks", "16", "--scenario",
                                   "tsunami", "--solver", "hlle"],
    }
    out = {"note": "wall clock of the driver's checkpoint loop, NetCDF output included"}
    tmp = tempfile.mkdtemp(prefix="swe_drivers_")
    try:
        for name, args in runs.items():
            r = subprocess.run([exe] + args + ["-w", "1", "-o", os.path.join(tmp, name)], capture_output=True,
                               text=True, timeout=900)
            vals = {}
            for line in r.stdout.splitlines():
                if ":" in line:
                    k, v = line.split(":", 1)
                    vals[k.strip()] = v.strip()
            if r.returncode != 0 or "Wall Time" not in vals:
                out[name] = {"error": (r.stderr or r.stdout)[-300:]}
                continue
            files = [f for f in os.listdir(tmp) if f.startswith(name) and f.endswith(".nc")]
            out[name] = {"wall_s": float(vals["Wall Time"].rstrip("s")), "steps": int(vals["Steps"]),
                         "cell_updates_per_s": float(vals["Cell updates"].split("/")[0]),
                         "netcdf_bytes": int(sum(os.path.getsize(os.path.join(tmp, f)) for f in files))}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return out


def split_measure(swe, device, steps=20):
    """The split step (SWE_DimensionalSplitting: x-sweep over the ghost rows,
    dt from the x-sweep's speeds, y-sweep with dt/dx) on the same tsunami
    2048^2 as one block (the reference's split block is a single block), HLLE,
    maximum reduction of dt.  CUDA events around `steps` steps after warm-up,
    L2 flushed between steps."""
    import torch
    n = N_CELLS_SIDE
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_TSUNAMI, n, n, 1, [n, SEED, 100000.0])
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=swe.HLLE,
                   semantics=swe.SPLIT, device=device)
    stream = torch.cuda.Stream()
    D.set_stream(stream.cuda_stream)
    D.upload(h, hu, hv, b)
    D.exchange_bathymetry()
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        for _ in range(5):
            flush.zero_()
            D.step(1)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for e0, e1 in ev:
            flush.zero_()
            e0.record(stream)
            D.step(1)
            e1.record(stream)
    stream.synchronize()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev) / steps
    status = D.status()
    D.close()
    return {"workload": "split step (SWE_DimensionalSplitting), tsunami 2048x2048 as one block, HLLE",
            "value": n * n / (ms * 1e-3), "unit": "cell-updates/s", "ms_per_step": ms, "device_status": status}


def surrogate_measure(swe, device, steps=10, err_steps=120):
    """MLP surrogate of the augmented Riemann solver at 4096^2: the shoreline
    ramp (bathymetry -4000 m to +50 m across 50 km, seeded Gaussian bump) as
    4x4 blocks of 1024^2, unsplit.  Training data: about 1e7 wet-edge states
    with their augmented-solver net updates, logged from augmented-solver runs
    of the benchmark's configurations 1 and 2 (the 256^2 radial dam break, every
    edge at 20 instants; the 2048^2 tsunami as 4x4 blocks, every 8th edge at 6
    instants) and of this workload (every 64th edge at 4 instants); 8 epochs
    of Adam on the device.  Timed (CUDA events, `steps` steps after warm-up): the augmented
    solver's default step (each edge solved once into the edge buffers), its
    two-pass step (speed pass + update pass, each edge solved twice), and the
    surrogate step.  Accuracy: each solver runs `err_steps` steps from the
    start state with its own dt; the L1 distance of its water heights to the
    augmented solver's trajectory, interpolated to the same time."""
    import torch
    n, nb = 4096, 16
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_SHORELINE, n, n, nb, [SEED, 50000.0])
    st = (h, hu, hv, b)
    stream = torch.cuda.Stream()

    def make(solver, speed_pass=0):
        D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver,
                       device=device, speed_pass=speed_pass)
        D.set_stream(stream.cuda_stream)
        D.upload(*st)
        D.exchange_bathymetry()
        return D

    E, T = [], []

    def log_run(D, logs, every, stride):
        for _ in range(logs):
            D.step(every)
            e, t = D.log_edges(stride=stride, capacity=1 << 21)
            E.append(e)
            T.append(t)
        D.close()

    for scen, nn, nblk, params, logs, every, stride in (
            (swe.SCENARIO_RADIAL_DAM_BREAK, 256, 1, None, 20, 2, 1),
            (swe.SCENARIO_TSUNAMI, 2048, 16, [2048, SEED, 100000.0], 6, 10, 8)):
        g2, *s2 = swe.init_domain(scen, nn, nn, nblk, params)
        D2 = swe.Domain(g2["nx_cols"], g2["ny_rows"], g2["dx"], g2["dy"], boundary=g2["boundary"],
                        solver=swe.AUGRIE, device=device)
        D2.set_stream(stream.cuda_stream)
        D2.upload(*s2)
        D2.exchange_bathymetry()
        log_run(D2, logs, every, stride)
    log_run(make(swe.AUGRIE), 4, 10, 64)
    E, T = np.concatenate(E, axis=1), np.concatenate(T, axis=1)
    m = swe.Surrogate(seed=SEED)
    epochs = 8
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = m.train(E, T, epochs=epochs, batch=8192, lr=2e-3, seed=SEED)
    train_s = time.perf_counter() - t0

    def timed(D, fn):
        fn(D, 3)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            fn(D, steps)
            e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / steps

    cells = float(n * n)
    rates = {}
    D = make(swe.AUGRIE)
    rates["augmented_step"] = cells / (1e-3 * timed(D, lambda D, k: D.step(k)))
    D.close()
    D = make(swe.AUGRIE, speed_pass=1)
    rates["augmented_two_pass_step"] = cells / (1e-3 * timed(D, lambda D, k: D.step(k)))
    D.close()
    D = make(swe.AUGRIE)
    ms_sur = timed(D, lambda D, k: D.surrogate_step(m, k, count=False))
    rates["surrogate_step"] = cells / (1e-3 * ms_sur)
    used = D.surrogate_step(m, 1)
    nedges = D.surrogate_edge_count()
    D.close()

    def interior(D):
        a = D.download()[0]
        return a  # whole domain in host order, ghosts included; compared at equal time below

    ends = {}
    for name, solver in (("fwave", swe.FWAVE), ("hlle", swe.HLLE), ("surrogate", swe.AUGRIE)):
        D = make(solver)
        if name == "surrogate":
            D.surrogate_step(m, err_steps, count=False)
        else:
            D.step(err_steps)
        ends[name] = (D.time()[0], interior(D).astype(np.float64))
        D.close()
    # augmented trajectory around each end time
    D = make(swe.AUGRIE)
    targets = sorted((t, k) for k, (t, _) in ends.items())
    errs, prev, t_prev, dt_last = {}, None, D.time()[0], 0.0
    while targets:
        t_next = targets[0][0]
        if dt_last == 0.0 or t_next - t_prev < 3.0 * dt_last:
            prev = interior(D).astype(np.float64)
        D.step(1)
        t_now = D.time()[0]
        dt_last, t_cur = t_now - t_prev, t_prev
        t_prev = t_now
        while targets and t_now >= targets[0][0]:
            t_x, k = targets.pop(0)
            cur = interior(D).astype(np.float64)
            w = (t_x - t_cur) / (t_now - t_cur)
            ref = (1 - w) * prev + w * cur
            errs[k] = float(np.abs(ends[k][1] - ref).sum() / cells)
    D.close()
    fp64 = surrogate_fp64_proxy(swe, m, device)
    batched = ensemble_surrogate_measure(swe, m, device, stream)
    m.close()
    flop_edge = 2 * (6 * 64 + 2 * 64 * 64 + 64 * 4)
    return {"workload": "surrogate of the augmented solver, shoreline ramp 4096x4096 as 4x4 blocks of 1024^2, unsplit",
            "unit": "cell-updates/s", "rates": rates,
            "speedup_vs_augmented_step": rates["surrogate_step"] / rates["augmented_step"],
            "surrogate_edge_fraction": used / nedges,
            "mlp_flop_per_edge": flop_edge,
            "mlp_tflops_over_step": nedges * flop_edge / (1e-3 * ms_sur) / 1e12,
            "l1_error_per_cell_vs_augmented": errs, "error_steps": err_steps, "fp64_proxy": fp64,
            "batched": batched,
            "training": {"edges": int(E.shape[1]), "epochs": epochs, "batch": 8192, "seconds": train_s,
                         "edges_per_s": epochs * E.shape[1] / train_s, "loss_first_epoch": float(losses[0]),
                         "loss_last_epoch": float(losses[-1])}}


def ensemble_surrogate_measure(swe, m, device, stream, steps=10, err_steps=100, count=256):
    """The batched + surrogate form: the ensemble workload (256 radial dam
    breaks, nx, ny in 64..1024, b = 0, one seed) with the augmented solver
    in one handle, stepped by the surrogate (swe_gpu_surrogate_step on the
    ensemble) against the augmented solver's own batched step.  Timed like
    the single-domain rates (CUDA events, `steps` steps after 3 warm-up
    steps).  Accuracy: after err_steps steps (each instance at its own dt),
    the relative L1 distance of h to the augmented solver's batched run,
    largest and median over the instances, and for the four smallest
    instances the relative L1 and L-infinity distances to the FP64 oracle's
    augmented solver after the same steps."""
    import torch
    inst, states = swe.dam_break_ensemble(count, seed=SEED)
    cells = float(sum(nx * ny for nx, ny, *_ in inst))

    def make():
        E = swe.Ensemble(inst, solver=swe.AUGRIE, device=device)
        E.set_stream(stream.cuda_stream)
        E.upload(*[np.concatenate([st[i] for st in states]) for i in range(4)])
        E.exchange_bathymetry()
        return E

    def timed(E, fn):
        fn(E, 3)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            fn(E, steps)
            e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / steps

    rates = {}
    E = make()
    rates["augmented_ensemble_step"] = cells / (1e-3 * timed(E, lambda E, k: E.step(k)))
    E.close()
    E = make()
    rates["surrogate_ensemble_step"] = cells / (1e-3 * timed(E, lambda E, k: E.surrogate_step(m, k, count=False)))
    used = E.surrogate_step(m, 1)
    nedges = E.surrogate_edge_count()
    E.close()
    h = {}
    status = 0
    for name in ("augmented", "surrogate"):
        E = make()
        if name == "surrogate":
            E.surrogate_step(m, err_steps, count=False)
        else:
            E.step(err_steps)
        h[name] = E.download()[0].astype(np.float64)
        status |= E.status()
        E.close()
    offs = np.cumsum([0] + [(nx + 2) * (ny + 2) for nx, ny, *_ in inst])
    rel = []
    for k, (nx, ny, *_) in enumerate(inst):
        a = h["augmented"][offs[k]:offs[k + 1]].reshape(nx + 2, ny + 2)[1:-1, 1:-1]
        b_ = h["surrogate"][offs[k]:offs[k + 1]].reshape(nx + 2, ny + 2)[1:-1, 1:-1]
        rel.append(float(np.abs(b_ - a).sum() / np.abs(a).sum()))
    import oracle
    oracle.build()
    fp64 = {"surrogate": [], "augmented": []}
    small = sorted(range(len(inst)), key=lambda k: inst[k][0] * inst[k][1])[:4]
    for k in small:
        nx, ny, dx, dy, bnd = inst[k]
        R = oracle.Domain([nx], [ny], dx, dy, outer=bnd, solver=oracle.AUGRIE, precision=64)
        R.set_state(*states[k])
        R.bathymetry_ghosts()
        R.step(err_steps)
        ref = R.get_state(np.float64)[0].reshape(nx + 2, ny + 2)[1:-1, 1:-1]
        for name in fp64:
            g = h[name][offs[k]:offs[k + 1]].reshape(nx + 2, ny + 2)[1:-1, 1:-1]
            fp64[name].append((float(np.abs(g - ref).sum() / np.abs(ref).sum()),
                               float(np.abs(g - ref).max() / np.abs(ref).max())))
    return {"workload": "%d radial dam breaks, nx, ny in 64..1024, augmented solver, unsplit, own dt each" % count,
            "unit": "cell-updates/s (sum over instances)", "cells": int(cells), "rates": rates,
            "speedup_vs_augmented_ensemble_step": rates["surrogate_ensemble_step"] / rates["augmented_ensemble_step"],
            "surrogate_edge_fraction": used / nedges, "error_steps": err_steps,
            "rel_l1_h_vs_augmented_max": max(rel), "rel_l1_h_vs_augmented_median": float(np.median(rel)),
            "fp64_smallest4": {"instances": [list(inst[k][:2]) for k in small], "steps": err_steps,
                               "rel_l1_h_surrogate_max": max(e[0] for e in fp64["surrogate"]),
                               "rel_linf_h_surrogate_max": max(e[1] for e in fp64["surrogate"]),
                               "rel_l1_h_augmented_max": max(e[0] for e in fp64["augmented"]),
                               "rel_linf_h_augmented_max": max(e[1] for e in fp64["augmented"])},
            "device_status": status}


def surrogate_fp64_proxy(swe, m, device, n=512, duration=300.0):
    """The surrogate against the FP64 oracle on a coarser copy of the 4096^2
    set-up (n^2 as 4x4 blocks, the same 50 km shoreline ramp and bump) to
    `duration` s simulated: the FP64 oracle of the 4096^2 run would take
    hours on the host.  Relative L1 and L-infinity water-height errors of the
    surrogate step and of the plain augmented-solver step (both on the GPU,
    each with its own dt) against the oracle's augmented solver in double,
    interpolated linearly to each run's end time between the two oracle steps
    around it; mass change of each run (outflow sides: outflow plus the
    depth the dry clamp added)."""
    import oracle
    oracle.build()
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_SHORELINE, n, n, 16, [SEED, 50000.0])
    mask = []
    for k in range(16):
        a = np.zeros((geo["nx_cols"][k // 4] + 2, geo["ny_rows"][k % 4] + 2), bool)
        a[1:-1, 1:-1] = True
        mask.append(a.ravel())
    mask = np.concatenate(mask)

    def run(surr):
        D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"],
                       solver=swe.AUGRIE, device=device)
        D.upload(h, hu, hv, b)
        D.exchange_bathymetry()
        steps = 0
        while D.time()[0] < duration:
            if surr:
                D.surrogate_step(m, 1, count=False)
            else:
                D.step(1)
            steps += 1
        t_end = D.time()[0]
        g = D.download()[0].astype(np.float64)[mask]
        status = D.status()
        D.close()
        return t_end, g, steps, status

    runs = {"surrogate": run(True), "augmented_gpu": run(False)}
    R = oracle.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"],
                      solver=oracle.AUGRIE, precision=64)
    R.set_state(h, hu, hv, b)
    R.bathymetry_ghosts()
    targets = sorted((v[0], k) for k, v in runs.items())
    refs, t, prev, ref_steps = {}, 0.0, R.get_state(np.float64)[0][mask], 0
    while targets:
        dts, _ = R.step_parallel(1)
        ref_steps += 1
        cur = R.get_state(np.float64)[0][mask]
        t_new = t + float(dts[0])
        while targets and t_new >= targets[0][0]:
            t_x, k = targets.pop(0)
            w = (t_x - t) / (t_new - t)
            refs[k] = (1 - w) * prev + w * cur
        t, prev = t_new, cur
    m0 = float(np.sum(h[mask].astype(np.float64)))
    out = {"workload": "%dx%d as 4x4 blocks, the same shoreline ramp and bump, %g s" % (n, n, duration),
           "oracle_steps": ref_steps}
    for k, (t_end, g, steps, status) in runs.items():
        r = refs[k]
        out[k] = {"t_end": t_end, "steps": steps, "rel_l1_h": float(np.abs(g - r).sum() / np.abs(r).sum()),
                  "rel_linf_h": float(np.abs(g - r).max() / np.abs(r).max()),
                  "mass_change_rel": float((g.sum() - m0) / m0), "device_status": status}
    out["mass_change_rel_fp64"] = float((refs["surrogate"].sum() - m0) / m0)
    return out


def profile_lts(seconds):
    """small case for launch lists of local time stepping: the bench's lts
    workload (shoreline ramp 2048^2 as 8x8 blocks of 256^2, HLLE, 1 s
    intervals), one warm-up interval, then `seconds` intervals"""
    import swe_gb300 as swe
    n, nb = 2048, 64
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_SHORELINE, n, n, nb, [SEED, 50000.0])
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=swe.HLLE,
                   lts_max_timestep=1.0, duration=200.0)
    D.upload(h, hu, hv, b)
    D.exchange_bathymetry()
    D.lts_advance(1.0)
    _, _, it0, _ = D.lts_state()
    t0 = time.perf_counter()
    done, _ = D.lts_advance(1.0 + seconds)
    el = time.perf_counter() - t0
    _, _, it1, _ = D.lts_state()
    log("lts intervals", done, "inner iterations", it1 - it0, "us per iteration", 1e6 * el / max(1, it1 - it0),
        "device status", D.status())
    D.close()
    return 0


def profile_surrogate(n):
    """small case for captures of the surrogate kernels: the shoreline ramp on
    one n x n block, a surrogate trained for 3 epochs on every 8th wet edge of
    an augmented-solver state after 10 steps, then 4 surrogate steps"""
    import swe_gb300 as swe
    geo, h, hu, hv, b = swe.init_domain(swe.SCENARIO_SHORELINE, n, n, 1, [SEED, 50000.0])

    def make(solver):
        D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver)
        D.upload(h, hu, hv, b)
        D.exchange_bathymetry()
        return D

    A = make(swe.AUGRIE)
    A.step(10)
    E, T = A.log_edges(stride=8, capacity=1 << 20)
    A.close()
    m = swe.Surrogate(seed=1)
    m.train(E, T, epochs=3, batch=8192, lr=2e-3, seed=1)
    D = make(swe.AUGRIE)
    used = D.surrogate_step(m, 4)
    log("surrogate edge fraction", used / (4 * D.surrogate_edge_count()))
    D.close()
    m.close()
    return 0


def reference_lts_rate():
    """The reference's own local time stepping on the host cores at the
    shape of the lts workload: the stock overdecomposed driver at 2048^2 as
    8 x 8 blocks with 1 s intervals (-b 64 -l 1) on its own scenario (the
    radial-bathymetry dam break, HLLE).  A run always completes whole
    intervals, so the rate is the difference of a 2 s and a 1 s run."""
    binary = reference_binary()
    if not binary:
        return None
    cores, model = host_cpu()
    u1, w1 = reference_run(binary, 1.0, blocks=64, lts=1.0)
    u2, w2 = reference_run(binary, 2.0, blocks=64, lts=1.0)
    return {"value": (u2 - u1) / max(w2 - w1, 1e-6), "unit": "cell-updates/s (its log's FLOP_COUNT / 270)",
            "cores": cores, "cpu_model": model, "kind": "reference",
            "sample": "stock swe_benchmark_mpioverdecomp -x 2048 -y 2048 -b 64 -l 1 (its radial-bathymetry dam "
                      "break, HLLE), the second 1 s interval: a -t 2 run minus a -t 1 run, %d OpenMP threads" % cores}


def cpu_reference_baseline(args):
    """cpu_baseline of the gb300 line: the reference's stock driver on the
    host cores (a bounded sample), else the oracle port"""
    binary = reference_binary()
    cores, model = host_cpu()
    if binary:
        span = float(os.environ.get("SWE_REF_SPAN", "0.5"))
        u0, w0 = reference_run(binary, 0.02)
        rates = []
        for _ in range(3):
            u, w = reference_run(binary, span)
            rates.append((u - u0) / max(w - w0, 1e-6))
        return {"value": statistics.median(rates), "unit": "cell-updates/s", "cores": cores, "kind": "reference",
                "cpu_model": model,
                "sample": "3 runs of the stock swe_benchmark_mpioverdecomp -x 2048 -y 2048 -b 16 -t %g (its radial-"
                          "bathymetry dam break, HLLE) minus a -t 0.02 run's set-up, %d OpenMP threads" % (span, cores)}
    base = cpu_baseline(float(os.environ.get("SWE_CPU_BASELINE_SECONDS", "12")))
    base["cpu_model"] = model
    return base


def run_gb300(args, world, rank, local):
    import torch
    import swe_gb300 as swe
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.cells
    solvers = {"hlle": swe.HLLE, "fwave": swe.FWAVE, "augrie": swe.AUGRIE, "hybrid": swe.HYBRID}
    solver = solvers[args.profile_solver] if args.profile else swe.HLLE
    # the headline path: fast arithmetic (one launch per step); --arith exact
    # runs the bit-exact two-launch step instead
    arith = swe.EXACT if args.arith == "exact" or solver in (swe.AUGRIE, swe.HYBRID) else swe.FAST
    D, geo, host = setup_domain(swe, local, n, solver, arith)
    stream = torch.cuda.Stream(dev)  # a real stream handle: the library launches on it
    assert stream.cuda_stream != 0
    D.set_stream(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    cells = n * n

    with torch.cuda.stream(stream), ClockSampler(local) as clk:
        # warm-up: W steps, and at least ~1.5 s of the same load so the clock
        # samples (taken every 200 ms) describe the timed kernels
        t_end = time.perf_counter() + (0.0 if args.profile else 1.5)
        i = 0
        while i < max(args.warmup, 3) or time.perf_counter() < t_end:
            flush.zero_()
            D.step(1)
            i += 1
            if i % 64 == 0:
                stream.synchronize()
        stream.synchronize()
        dist_barrier(world)

        # timed region: exactly K steps, L2 flushed before each, CUDA events
        # around each step on the library's stream
        stream.synchronize()
        dist_barrier(world)
        launches0 = D.launch_count()
        step_ms = timed_steps(D, stream, flush, args.steps)
        dist_barrier(world)
        launches = D.launch_count() - launches0
    total_ms = dist_max(sum(step_ms), world)
    ms_per_step = total_ms / args.steps
    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_run": True, "cells": cells, "ms_per_step": ms_per_step}), flush=True)
        D.close()
        return 0

    kt = kernel_times(D, stream, flush, args.steps)
    status = D.status()

    # end to end through the C ABI on host buffers: upload h, hu, hv, b from
    # pinned memory, one step, download h, hu, hv; host clock around it all
    pinned = [torch.from_numpy(a).pin_memory() for a in host]
    outs = [torch.empty(host[0].shape, dtype=torch.float32).pin_memory() for _ in range(3)]
    pn = [p.numpy() for p in pinned]
    on = [o.numpy() for o in outs]
    e2e_steps = max(3, min(args.steps, 20))
    for _ in range(2):
        D.upload(*pn)
        D.step(1)
        D.download_into(on)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        D.upload(*pn)
        D.step(1)
        D.download_into(on)
    e2e_sync_s = dist_max((time.perf_counter() - t0) / e2e_steps, world)
    # the same per-step transfers through the asynchronous calls: step k's
    # download (second stream) overlaps step k+1's upload
    for _ in range(2):
        D.upload_async(*pn)
        D.step(1)
        D.download_async(on)
    D.sync()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        D.upload_async(*pn)
        D.step(1)
        D.download_async(on)
    D.sync()
    e2e_s = dist_max((time.perf_counter() - t0) / e2e_steps, world)
    h2d = sum(p.nbytes for p in pn)
    d2h = sum(o.nbytes for o in on)
    D.close()

    # the bit-exact step (identical to the reference's float arithmetic) on
    # the same workload, for comparison
    exact = None
    if arith == swe.FAST:
        E, _, _ = setup_domain(swe, local, n, solver, swe.EXACT)
        E.set_stream(stream.cuda_stream)
        with torch.cuda.stream(stream):
            for _ in range(max(args.warmup, 3)):
                flush.zero_()
                E.step(1)
        ems = timed_steps(E, stream, flush, args.steps)
        ekt = kernel_times(E, stream, flush, args.steps)
        E.close()
        exact = {"ms_per_step": sum(ems) / len(ems), "value": cells / (1e-3 * sum(ems) / len(ems)),
                 "unit": "cell-updates/s", "kernel_ms": ekt,
                 "roofline_frac_update": BYTES_PER_CELL * cells / (ekt["update"] * 1e-3) / 1e9 / peaks()[0],
                 "arithmetic": "IEEE division and square root, no contraction: bit-identical to the oracle"}

    hbm, peak_kind = peaks()
    algo_bytes = BYTES_PER_CELL * cells
    t_kernel = kt["update"] + kt["speed"]  # fast: the one step kernel (compute_fluxes launches nothing)
    achieved = algo_bytes / (t_kernel * 1e-3) / 1e9
    step_achieved = algo_bytes / (ms_per_step * 1e-3) / 1e9
    traffic, warp_inst = None, None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            prof = json.load(f)
        key = "fast_kernel" if arith == swe.FAST else "update_kernel"
        traffic = prof.get(key + "_dram_bytes_per_launch")
        warp_inst = prof.get(key + "_warp_instructions_per_launch")
    except Exception:
        pass
    sms = torch.cuda.get_device_properties(dev).multi_processor_count

    acc = accuracy_measure(swe, local) if rank == 0 else None
    lts = lts_measure(swe, local)
    ens = ensemble_measure(swe, local)
    sur = surrogate_measure(swe, local) if rank == 0 else None
    split = split_measure(swe, local) if rank == 0 else None
    drivers = drivers_measure() if rank == 0 else None
    base = cpu_reference_baseline(args) if rank == 0 else None
    if rank == 0:
        try:
            lts["cpu_reference"] = reference_lts_rate()
        except Exception as e:
            log("reference lts run failed:", e)
    clocks = clk.summary()
    issue = None
    if warp_inst and clocks.get("sm_mhz"):
        # warp instructions of one launch (ncu) per second against one
        # instruction per SM sub-partition per cycle
        issue_peak = sms * 4 * clocks["sm_mhz"] * 1e6
        issue_achieved = warp_inst / (t_kernel * 1e-3)
        issue = {"warp_instructions_per_launch": warp_inst, "achieved": issue_achieved, "peak": issue_peak,
                 "unit": "warp instructions/s", "frac": issue_achieved / issue_peak,
                 "peak_from": "%d SMs x 4 sub-partitions x %.0f MHz (median SM clock under load)" % (sms, clocks["sm_mhz"])}
    if rank == 0:
        kname = "fastStepKernel<HLLE> (one launch per step)" if arith == swe.FAST else "sweepKernel<HLLE,unsplit,update>"
        line = {
            "metric": METRIC, "value": world * cells / (ms_per_step * 1e-3), "unit": "cell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded tsunami scenario, shapes of the 2048^2 benchmark)",
            "config": workload_config({"parallelism": "replicas x%d" % world if world > 1 else "1 GPU",
                                       "arithmetic": "fast (approximate rcp/rsqrt/sqrt, FMA; results equal to the "
                                                     "reference to FP32 round-off, see accuracy)"
                                       if arith == swe.FAST else "exact (bit-identical to the reference's float "
                                                                 "arithmetic)"}),
            "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved,
                         "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "peak_kind": peak_kind,
                         "traffic": traffic, "algorithmic_bytes_per_launch": algo_bytes,
                         "step_achieved": step_achieved, "step_frac": step_achieved / hbm, "issue": issue},
            "kernel_ms": kt,
            "exact": exact,
            "accuracy": acc,
            "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample", "cpu_model")},
            "e2e": {"value": world * cells / e2e_s, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "calls": "upload_async, step, download_async; sync at the end",
                    "synchronous_value": world * cells / e2e_sync_s},
            "clocks": clocks, "gpu_launches": launches, "device_status": status,
            "lts": lts, "ensemble": ens, "surrogate": sur, "split": split, "drivers": drivers,
        }
        print(json.dumps(line), flush=True)
    dist_barrier(world)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--arith", default="fast", choices=["fast", "exact"],
                    help="arithmetic of the timed step (fast: one launch per step, FP32 round-off; exact: bit-identical)")
    ap.add_argument("--cells", type=int, default=N_CELLS_SIDE, help="cells per side (profiling cases only)")
    ap.add_argument("--profile", action="store_true", help="timed steps only (for ncu captures)")
    ap.add_argument("--profile-solver", default="hlle", choices=["hlle", "fwave", "augrie", "hybrid"],
                    help="solver of the --profile run (the bench itself always runs HLLE)")
    ap.add_argument("--profile-surrogate", type=int, default=0, metavar="N",
                    help="only the surrogate step on an N x N shoreline (for ncu captures)")
    ap.add_argument("--profile-lts", type=float, default=0.0, metavar="SECONDS",
                    help="only local time stepping, SECONDS simulated after a warm-up interval (for ncu captures)")
    args = ap.parse_args()
    if args.profile_surrogate:
        return profile_surrogate(args.profile_surrogate)
    if args.profile_lts > 0:
        return profile_lts(args.profile_lts)
    world, rank, local = dist_init()
    if args.impl == "reference":
        rc = run_reference(args, world, rank)
    else:
        rc = run_gb300(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
