"""The MLP surrogate on a domain: the edge-buffer step with the augmented
solver on every edge must equal the augmented solver's own step bit for bit
(so the edge tiling, the stored net updates, dt and the cell update are
exact); the edge-state logger must log the step's edge states with the
oracle's augmented-solver net updates; a surrogate trained on logged edges
on a strong dam break must stay closer to the augmented solver's run than
the f-wave solver does."""
import numpy as np
import pytest

from helpers import assert_bitwise

pytestmark = pytest.mark.gpu


def make(swe, geo, st, solver, speed_pass=0):
    D = swe.Domain(geo["nx_cols"], geo["ny_rows"], geo["dx"], geo["dy"], boundary=geo["boundary"], solver=solver,
                   speed_pass=speed_pass)
    D.upload(*st)
    D.exchange_bathymetry()
    return D


CASES = [
    ("radial_dam_break", 0, 160, 128, 4, None),
    ("half_domain_dry", 3, 96, 80, 1, None),
    ("shoreline", 12, 192, 192, 4, [5.0, 50000.0]),
    ("tsunami", 11, 256, 256, 4, [256, 7.0, 100000.0]),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_default_augmented_step_equals_two_pass_step(swe, case):
    """The default step of an augmented-solver domain (each edge solved once
    into the edge buffers) against the two-pass step, with advance() and the
    split API, ghost rings included."""
    name, sid, nx, ny, nb, params = case
    geo, h, hu, hv, b = swe.init_domain(sid, nx, ny, nb, params)
    st = (h, hu, hv, b)
    outs = []
    for sp in (1, 0):
        D = make(swe, geo, st, swe.AUGRIE, speed_pass=sp)
        D.advance(1e30, max_steps=9)
        dts = []
        for _ in range(4):
            D.set_ghost_layer()
            D.compute_fluxes()
            dts.append(D.max_timestep())
            D.update_unknowns()
        outs.append((D.download(), D.time(), np.asarray(dts, np.float32)))
        assert D.status() == 0
        D.close()
    (a, ta, da), (b_, tb, db) = outs
    assert ta[1] == tb[1] == 13 and np.float32(ta[0]) == np.float32(tb[0])
    assert_bitwise(da, db, "dt")
    for x, y, k in zip(a, b_, "h hu hv b".split()):
        assert_bitwise(x, y, k)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_augmented_solver_through_edge_buffers_is_bitwise(swe, case):
    name, sid, nx, ny, nb, params = case
    geo, h, hu, hv, b = swe.init_domain(sid, nx, ny, nb, params)
    st = (h, hu, hv, b)
    A = make(swe, geo, st, swe.AUGRIE, speed_pass=1)  # two passes, every edge solved in both
    A.step(12)
    ref = A.download()
    tref, nref = A.time()
    A.close()
    S = make(swe, geo, st, swe.AUGRIE, speed_pass=1)
    used = S.surrogate_step(None, 7)
    S.step(5)  # two-pass steps continue from the edge-buffer path's state
    out = S.download()
    t, n = S.time()
    assert S.status() == 0
    S.close()
    assert used == 0 and n == nref == 12
    assert np.float32(t) == np.float32(tref)
    for a, r, k in zip(out, ref, "h hu hv b".split()):
        assert_bitwise(a, r, k)


def test_log_edges_matches_oracle(swe, oracle_mod):
    geo, h, hu, hv, b = swe.init_domain(11, 128, 96, 1, [128, 7.0, 100000.0])
    D = make(swe, geo, (h, hu, hv, b), swe.AUGRIE)
    D.step(3)
    n_all = D.surrogate_edge_count()
    assert n_all == 129 * 96 + 128 * 97
    e1, t1 = D.log_edges(stride=1, capacity=1 << 20)
    e7, t7 = D.log_edges(stride=7, capacity=1000)
    st = D.download()
    D.close()
    assert e1.shape[1] == n_all  # the tsunami basin is wet everywhere
    ref = oracle_mod.solve_edges(2, *e1)
    for k in range(4):
        assert_bitwise(t1[k], ref[k], "target %d" % k)
    # the first tile: x-edges (0|1) of rows 1..96, from the state after setGhostLayer
    H = st[0].reshape(130, 98)
    assert_bitwise(e1[1, :96], H[1, 1:97], "right cells")
    assert_bitwise(e1[0, :96], H[0, 1:97], "left ghosts (outflow copies)")
    assert_bitwise(H[0, 1:97], H[1, 1:97], "outflow ghost")
    # stride: every 7th slot of the padded tile order, capacity honoured
    assert e7.shape[1] == 1000
    assert np.isin(e7[0], e1[0]).all()


def interior(D, nx, ny):
    return D.download()[0].reshape(nx + 2, ny + 2)[1:-1, 1:-1].astype(np.float64)


def run_until(D, nx, ny, T, stepper):
    traj = [(D.time()[0], interior(D, nx, ny))]
    while traj[-1][0] < T:
        stepper(D)
        traj.append((D.time()[0], interior(D, nx, ny)))
    return traj


def state_at(traj, t):
    """linear interpolation in time of a trajectory"""
    ts = np.array([x[0] for x in traj])
    k = min(max(int(np.searchsorted(ts, t)) - 1, 0), len(ts) - 2)
    w = (t - ts[k]) / (ts[k + 1] - ts[k])
    return (1 - w) * traj[k][1] + w * traj[k + 1][1]


def test_trained_surrogate_on_a_strong_dam_break(swe):
    """Train on edges logged from an augmented-solver run of a radial dam
    break (20 m onto 0.5 m, a transonic rarefaction the Roe-speed f-wave
    solver resolves as an expansion shock), then run the same start state with
    the surrogate and with the f-wave solver up to t = 6 s.  Each solver picks
    its own dt, so each run is compared with the augmented solver's trajectory
    interpolated to the run's final time: the surrogate (with its gate and
    fallback) stays closer than the f-wave solver, and conserves the water
    volume (the front stays inside the domain)."""
    n = 192
    geo, h, hu, hv, b = swe.init_domain(10, n, n, 1, [1000.0, 150.0, 20.0, 0.5, 0, 0, 0])
    st = (h, hu, hv, b)
    A = make(swe, geo, st, swe.AUGRIE)
    E, T = [], []
    for _ in range(8):
        A.step(8)
        e, t = A.log_edges(stride=1, capacity=1 << 21)
        E.append(e)
        T.append(t)
    A.close()
    E, T = np.concatenate(E, axis=1), np.concatenate(T, axis=1)
    m = swe.Surrogate(seed=4)
    losses = m.train(E, T, epochs=40, batch=4096, lr=2e-3, seed=5)
    assert losses[-1] < 0.2 * losses[0], losses
    t_end = 6.0
    A = make(swe, geo, st, swe.AUGRIE)
    ref = run_until(A, n, n, 1.05 * t_end, lambda D: D.step(1))
    A.close()
    used = [0, 0]

    def sur_step(D):
        used[0] += D.surrogate_step(m, 1)
        used[1] += D.surrogate_edge_count()

    err = {}
    for name, solver, stepper in (("fwave", swe.FWAVE, lambda D: D.step(1)), ("sur", swe.AUGRIE, sur_step)):
        D = make(swe, geo, st, solver)
        tr = run_until(D, n, n, t_end, stepper)
        assert D.status() == 0
        D.close()
        t, hh = tr[-1]
        err[name] = float(np.abs(hh - state_at(ref, t)).sum())
        if name == "sur":
            v0 = tr[0][1].sum()
            assert abs(hh.sum() - v0) <= 1e-5 * v0
    m.close()
    assert used[0] > 0
    assert err["sur"] < err["fwave"], (err, used[0] / used[1])
