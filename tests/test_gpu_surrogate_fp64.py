"""Accuracy of the solvers on the shoreline ramp against an FP64 reference:
the augmented Riemann solver of the oracle in double precision, 256^2 as 4x4
blocks over 50 km, 300 s of simulated time (about 760 steps).  Runs on the GPU: the
augmented solver (FP32), the f-wave and HLLE solvers, and the MLP surrogate
trained on edges logged from the augmented solver's run.  Each run picks its
own dt, so each is compared with the FP64 trajectory interpolated to the
run's final time (mean |h - h_FP64| over the interior cells); the figures are
printed as one JSON line.  On this smooth deep-water case FP32 rounding, not
the choice of solver, dominates the distance to the FP64 run."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make(swe, geo, st, solver):
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver)
    D.upload(*st)
    D.exchange_bathymetry()
    return D


def interior(h, geo):
    cols, rows = geo["nx_cols"], geo["ny_rows"]
    out, off = [], 0
    for k in range(len(cols) * len(rows)):
        nx, ny = cols[k // len(rows)], rows[k % len(rows)]
        out.append(np.asarray(h[off:off + (nx + 2) * (ny + 2)], np.float64).reshape(nx + 2, ny + 2)[1:-1, 1:-1].ravel())
        off += (nx + 2) * (ny + 2)
    return np.concatenate(out)


def test_solvers_against_fp64_augmented_solver(swe, oracle_mod):
    n, nb, t_end = 256, 16, 300.0
    max_steps = 5000
    geo, h, hu, hv, b = swe.init_domain(12, n, n, nb, [20261203, 50000.0])
    st = (h, hu, hv, b)
    A = make(swe, geo, st, swe.AUGRIE)
    E, T = [], []
    for _ in range(8):
        A.step(80)
        e, t = A.log_edges(stride=1, capacity=1 << 21)
        E.append(e)
        T.append(t)
    A.close()
    m = swe.Surrogate(seed=11)
    losses = m.train(np.concatenate(E, axis=1), np.concatenate(T, axis=1), epochs=10, batch=8192, lr=2e-3, seed=12)
    assert losses[-1] < losses[0]

    ends, used = {}, [0, 0]
    for name, solver in (("augmented_fp32", swe.AUGRIE), ("fwave", swe.FWAVE), ("hlle", swe.HLLE),
                         ("surrogate", swe.AUGRIE)):
        D = make(swe, geo, st, solver)
        if name == "surrogate":
            for _ in range(max_steps):
                if not D.time()[0] < t_end:
                    break
                used[0] += D.surrogate_step(m, 1)
                used[1] += D.surrogate_edge_count()
            assert not D.time()[0] < t_end
        else:
            D.advance(t_end)
        assert D.status() == 0
        ends[name] = (D.time()[0], interior(D.download()[0], geo))
        D.close()
    m.close()

    R = oracle_mod.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], outer=geo["boundary"], solver=2,
                          precision=64)
    R.set_state(*st)
    R.bathymetry_ghosts()
    targets = sorted((t, k) for k, (t, _) in ends.items())
    err, prev, dt_last, steps, t1 = {}, None, 0.0, 0, 0.0  # the FP64 clock: the sum of its dts
    while targets:
        assert steps < max_steps, "the FP64 run does not reach t = %g" % targets[0][0]
        t0 = t1
        if dt_last == 0.0 or targets[0][0] - t0 < 3.0 * dt_last:
            prev = interior(R.get_state(np.float64)[0], geo)
        dt_last = float(R.step(1)[0])
        steps += 1
        t1 = t0 + dt_last
        assert t1 > t0
        while targets and t1 >= targets[0][0]:
            t_x, k = targets.pop(0)
            cur = interior(R.get_state(np.float64)[0], geo)
            w = (t_x - t0) / (t1 - t0)
            err[k] = float(np.mean(np.abs(ends[k][1] - ((1 - w) * prev + w * cur))))
    print(json.dumps({"case": "shoreline ramp 256^2 (4x4 blocks), t = 300 s", "fp64_steps": steps,
                      "mean_abs_h_error_m": err, "surrogate_edge_fraction": used[0] / max(1, used[1])}))
    assert all(np.isfinite(v) for v in err.values())
    # In deep, smooth water the solvers differ by less than FP32 rounding
    # accumulates over the run (measured: all four within 2.8e-3 .. 3.7e-3 m
    # of the FP64 run), so the bar is the FP32 augmented solver's own error:
    # the surrogate must be as accurate as running the solver it replaces.
    assert err["surrogate"] <= 1.5 * err["augmented_fp32"], err
    assert max(err.values()) <= 3.0 * min(err.values()), err
