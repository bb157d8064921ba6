"""Batched ensembles: independent simulations of different sizes, each with its
own CFL time step, stepped together in one handle.  Every instance must be
bit-identical to the same simulation run alone (and, for small ones, to the
oracle); retiling and the tile-shape tuner must not change any result."""
import numpy as np
import pytest

from helpers import assert_bitwise

pytestmark = pytest.mark.gpu


def alone(swe, inst, st, solver, nsteps, semantics=0):
    nx, ny, dx, dy, bnd = inst
    D = swe.Domain([nx], [ny], dx, dy, boundary=bnd, solver=solver, semantics=semantics)
    D.upload(*st)
    D.exchange_bathymetry()
    D.step(nsteps)
    out = D.download()
    t, n = D.time()
    assert D.status() == 0
    D.close()
    return out, t


def ensemble(swe, inst, states, solver, nsteps, semantics=0, **kw):
    E = swe.Ensemble(inst, solver=solver, semantics=semantics, **kw)
    E.upload(*[np.concatenate([s[i] for s in states]) for i in range(4)])
    E.exchange_bathymetry()
    E.step(nsteps)
    out = E.download()
    t, dt, steps = E.group_state()
    assert E.status() == 0
    E.close()
    return out, t, steps


def split_blocks(E_out, inst):
    offs = np.cumsum([0] + [(nx + 2) * (ny + 2) for nx, ny, *_ in inst])
    return [[a[offs[k]:offs[k + 1]] for a in E_out] for k in range(len(inst))]


@pytest.mark.parametrize("solver", [4, 1, 2, 3])
def test_ensemble_equals_instances_alone(swe, solver):
    inst, states = swe.dam_break_ensemble(10, seed=5, sizes=np.arange(64, 257, 32))
    out, t, steps = ensemble(swe, inst, states, solver, 25)
    assert (steps == 25).all()
    for k, blk in enumerate(split_blocks(out, inst)):
        ref, tref = alone(swe, inst[k], states[k], solver, 25)
        assert np.float32(t[k]) == np.float32(tref), "instance %d clock" % k
        for a, b_, name in zip(blk, ref, "h hu hv b".split()):
            assert_bitwise(a, b_, "instance %d %s" % (k, name))


def test_ensemble_small_instances_match_oracle(swe, oracle_mod):
    inst, states = swe.dam_break_ensemble(4, seed=9, sizes=[64, 96])
    out, _, _ = ensemble(swe, inst, states, 4, 20)
    for k, blk in enumerate(split_blocks(out, inst)):
        nx, ny, dx, dy, bnd = inst[k]
        R = oracle_mod.Domain([nx], [ny], dx, dy, outer=bnd, solver=4)
        R.set_state(*states[k])
        R.bathymetry_ghosts()
        R.step(20)
        ref = R.get_state()
        for a, b_, name in zip(blk[:3], ref[:3], "h hu hv".split()):
            assert_bitwise(a, b_, "instance %d %s" % (k, name))


def test_ensemble_advance_stops_each_instance_at_its_target(swe):
    inst, states = swe.dam_break_ensemble(6, seed=2, sizes=np.arange(64, 193, 32))
    E = swe.Ensemble(inst, solver=4)
    E.upload(*[np.concatenate([s[i] for s in states]) for i in range(4)])
    E.exchange_bathymetry()
    E.advance(2.0)
    t, _, steps = E.group_state()
    out = E.download()
    E.close()
    assert (t >= 2.0).all()
    for k, blk in enumerate(split_blocks(out, inst)):
        nx, ny, dx, dy, bnd = inst[k]
        D = swe.Domain([nx], [ny], dx, dy, boundary=bnd, solver=4)
        D.upload(*states[k])
        D.exchange_bathymetry()
        n, tk = D.advance(2.0)
        ref = D.download()
        D.close()
        assert n == steps[k] and np.float32(tk) == np.float32(t[k])
        for a, b_, name in zip(blk, ref, "h hu hv b".split()):
            assert_bitwise(a, b_, "instance %d %s" % (k, name))


def test_retile_and_autotune_keep_results(swe):
    inst, states = swe.dam_break_ensemble(8, seed=3, sizes=np.arange(64, 321, 32))
    base, _, _ = ensemble(swe, inst, states, 4, 12)
    E = swe.Ensemble(inst, solver=4)
    E.upload(*[np.concatenate([s[i] for s in states]) for i in range(4)])
    E.exchange_bathymetry()
    E.step(4)
    E.retile(64, 8)
    E.step(4)
    rows, cols, ms = E.autotune(trial_steps=3)
    assert rows % 32 == 0 and ms > 0
    E.step(4)
    out = E.download()
    _, _, steps = E.group_state()
    E.close()
    assert (steps == 12).all()
    for a, b_, name in zip(out, base, "h hu hv b".split()):
        assert_bitwise(a, b_, name)


def test_ensemble_of_split_steps(swe):
    inst, states = swe.dam_break_ensemble(5, seed=4, sizes=np.arange(64, 161, 32))
    out, _, _ = ensemble(swe, inst, states, 3, 10, semantics=1)
    for k, blk in enumerate(split_blocks(out, inst)):
        ref, _ = alone(swe, inst[k], states[k], 3, 10, semantics=1)
        for a, b_, name in zip(blk, ref, "h hu hv b".split()):
            assert_bitwise(a, b_, "instance %d %s" % (k, name))


def test_ensemble_surrogate_step_equals_instances_alone(swe):
    """The batched + surrogate form: an augmented-solver ensemble stepped by
    the MLP surrogate (swe_gpu_surrogate_step on the ensemble handle) is,
    instance by instance, bit-identical to each simulation's own surrogate
    run; without a network the same call is the ensemble's augmented step."""
    inst, states = swe.dam_break_ensemble(6, seed=7, sizes=np.arange(64, 193, 32))
    nx, ny, dx, dy, bnd = inst[0]
    A = swe.Domain([nx], [ny], dx, dy, boundary=bnd, solver=swe.AUGRIE)
    A.upload(*states[0])
    A.exchange_bathymetry()
    A.step(4)
    e, tg = A.log_edges(stride=1, capacity=1 << 18)
    A.close()
    m = swe.Surrogate(seed=3)
    m.train(e, tg, epochs=4, batch=2048, lr=2e-3, seed=3)
    nsteps = 12

    def batched(model, plain=False):
        E = swe.Ensemble(inst, solver=swe.AUGRIE)
        E.upload(*[np.concatenate([s[i] for s in states]) for i in range(4)])
        E.exchange_bathymetry()
        used = 0
        if plain:
            E.step(nsteps)
        else:
            used = E.surrogate_step(model, nsteps)
        out = E.download()
        t, dt, steps = E.group_state()
        assert E.status() == 0
        E.close()
        return out, t, used

    out, t, used = batched(m)
    assert used > 0
    for k, blk in enumerate(split_blocks(out, inst)):
        nx, ny, dx, dy, bnd = inst[k]
        D = swe.Domain([nx], [ny], dx, dy, boundary=bnd, solver=swe.AUGRIE)
        D.upload(*states[k])
        D.exchange_bathymetry()
        D.surrogate_step(m, nsteps)
        ref = D.download()
        tref, _ = D.time()
        assert D.status() == 0
        D.close()
        assert np.float32(t[k]) == np.float32(tref), "instance %d clock" % k
        for a, b_, name in zip(blk, ref, "h hu hv b".split()):
            assert_bitwise(a, b_, "instance %d %s" % (k, name))
    m.close()
    out0, t0, _ = batched(None)
    out1, t1, _ = batched(None, plain=True)
    assert_bitwise(np.asarray(t0, np.float32), np.asarray(t1, np.float32), "clocks")
    for a, b_, name in zip(out0, out1, "h hu hv b".split()):
        assert_bitwise(a, b_, name)
