"""Batched quenches (dyn_batch_*): every quench of a batch against the same
quench run alone through the mixed-precision single-quench path (same stage
arithmetic, same device-side controller decisions: bit-identical histories),
the stopping rules, capacity, rollback, state upload and the autotuner."""
import numpy as np
import pytest

import dynamite_gb300 as D
from conftest import load_golden
from helpers import STATE_FIELDS, grid_from, model_from, rel_err, state_from

pytestmark = pytest.mark.gpu

MIXED_TRAJ_TOL = 1e-6   # a different gather tile only reorders the compensated FP32 sums


def _quench(grid_idx, m: D.Model, **kw):
    return D.Quench(grid=grid_idx, p=m.p, p2=m.p2, lam=m.lam, T0=m.T0, Gamma=m.Gamma, delta_t_min=m.delta_t_min,
                    delta_max=m.delta_max, **kw)


def _single(grid, m: D.Model, nsteps, rollback=False, tmax=0.0, upload=None, ctl=None, precision="mixed"):
    s = D.Simulation(grid, m, precision=precision)
    if upload is None:
        s.init()
    else:
        s.upload(upload)
        s.set_controller(**ctl)
    tr = s.run(nsteps, tmax=tmax, gpu_rollback=rollback)
    return s, tr


def _assert_same_state(a: D.State, b: D.State):
    for f in STATE_FIELDS:
        np.testing.assert_array_equal(getattr(a, f), getattr(b, f), err_msg=f)


def _grids():
    g32, g64 = load_golden(32), load_golden(64)
    return [grid_from(g32, D.Grid), grid_from(g64, D.Grid)], model_from(g32, D.Model), model_from(g64, D.Model)


def test_batch_equals_single_quenches(product_built):
    grids, m32, m64 = _grids()
    ma = D.Model(p=3, p2=4, lam=0.3, Gamma=0.9)
    mb = D.Model(p=3, p2=4, lam=0.7, Gamma=0.45)
    specs = [(0, m32, 70), (1, ma, 55), (0, mb, 40), (1, m32, 64)]
    b = D.Batch(grids, [_quench(gi, m, max_steps=n) for gi, m, n in specs], ticks_per_launch=16, precision="mixed")
    b.run(100_000)
    for q, (gi, m, n) in enumerate(specs):
        inf = b.info(q)
        assert inf["status"] == "max_steps" and inf["steps"] == n and inf["n"] == n + 1
        s, tr = _single(grids[gi], m, n)
        _assert_same_state(b.download(q), s.download())
        assert inf["energy"] == tr["energy"][-1]
        c = s.controller
        assert (inf["delta_t"], inf["method"], inf["loop"], inf["delta"]) == (c["delta_t"], c["method"], c["loop"],
                                                                              c["delta"])


def test_batch_generic_exponents(product_built):
    """Quenches with different (p, p2) in one batch take the runtime-exponent kernels."""
    grids, m32, m64 = _grids()
    specs = [(0, m32, 50), (1, m64, 50), (0, D.Model(p=3, p2=0, lam=1.0, Gamma=0.7), 35)]
    b = D.Batch(grids, [_quench(gi, m, max_steps=n) for gi, m, n in specs], precision="mixed")
    b.run(100_000)
    for q, (gi, m, n) in enumerate(specs):
        s, _ = _single(grids[gi], m, n)
        _assert_same_state(b.download(q), s.download())


def test_batch_stopping_time_and_capacity(product_built):
    grids, m32, _ = _grids()
    s, tr = _single(grids[0], m32, 90)
    t_stop = float(tr["t"][60])  # time reached by step 61; the quench stops once t >= t_stop
    b = D.Batch(grids, [_quench(0, m32, t_stop=t_stop), _quench(0, m32, capacity=25),
                        _quench(1, m32, max_steps=10)], precision="mixed")
    b.run(100_000)
    i0, i1, i2 = b.info(0), b.info(1), b.info(2)
    assert i0["status"] == "done" and i0["t"] >= t_stop
    st0 = b.download(0)
    assert st0.t1grid[-2] < t_stop
    ref = s.download()
    np.testing.assert_array_equal(st0.t1grid, ref.t1grid[: st0.n])
    assert i1["status"] == "full" and i1["n"] == 25
    np.testing.assert_array_equal(b.download(1).QK, ref.QK[: 25 * grids[0].L])
    assert i2["status"] == "max_steps"
    # new limits restart a stopped quench where it stopped
    b.set_limits(2, max_steps=25)
    assert b.info(2)["status"] == "running"
    b.run(100_000)
    s2, _ = _single(grids[1], m32, 25)
    _assert_same_state(b.download(2), s2.download())


def test_batch_rollback_matches_single(product_built):
    """delta_max small enough that steps are rejected: the device-side rollback
    (simulation_runner.cpp:280-304) against dyn_run's."""
    grids, m32, _ = _grids()
    m = D.Model(p=3, p2=4, lam=0.5, Gamma=0.6, delta_max=1e-13)
    b = D.Batch(grids, [_quench(0, m, max_steps=80), _quench(1, m, max_steps=60)], gpu_rollback=True,
                precision="mixed")
    b.run(100_000)
    for q, (gi, n) in enumerate([(0, 80), (1, 60)]):
        s, tr = _single(grids[gi], m, n, rollback=True)
        _assert_same_state(b.download(q), s.download())
        assert b.info(q)["loop"] == s.controller["loop"]
    assert b.info(0)["n"] < 81  # some steps were rolled back


@pytest.mark.parametrize("precision", ["mixed", "mixed_df"])
def test_batch_upload_continues_like_single(product_built, precision):
    g = load_golden(32)
    grids, m32, _ = _grids()
    mid = state_from(g, "mid", D.State)
    ctl = dict(delta_t=float(mid.t1grid[-1] - mid.t1grid[-2]), method=1, delta=1e-11, delta_old=2e-11, loop=40)
    b = D.Batch(grids, [_quench(0, m32, max_steps=5), _quench(1, m32, max_steps=5)], precision=precision)
    b.upload(0, mid, **ctl)
    b.set_limits(0, max_steps=30)
    b.run(100_000)
    s, _ = _single(grids[0], m32, 30, upload=mid, ctl=ctl, precision=precision)
    _assert_same_state(b.download(0), s.download())


def test_batch_autotuned_tiles(product_built):
    """The autotuner's pick reorders the FP32 partial sums only."""
    L = 128
    grid = D.grid.generate(L, Tmax=1e3)
    models = [D.Model(p=3, p2=4, lam=lam, Gamma=gm) for lam, gm in ((0.3, 0.5), (0.5, 0.6), (0.7, 0.9))]
    b = D.Batch([grid], [_quench(0, m, max_steps=40) for m in models], precision="mixed")
    b.run(20)  # tune on a live state
    pick = b.tune(reps=3)
    assert pick["threads"] in (128, 256) and pick["targets"] in (1, 2) and pick["ms_gather"] > 0
    b.run(100_000)
    for q, m in enumerate(models):
        s, tr = _single(grid, m, 40)
        sa, sb = b.download(q), s.download()
        if sa.n == sb.n and np.array_equal(sa.t1grid, sb.t1grid):
            assert rel_err(sa.QK, sb.QK) < MIXED_TRAJ_TOL
            assert rel_err(sa.rvec, sb.rvec) < MIXED_TRAJ_TOL
        assert abs(b.info(q)["energy"] - tr["energy"][-1]) <= MIXED_TRAJ_TOL * abs(tr["energy"][-1])


@pytest.mark.parametrize("precision", ["mixed", "mixed_df"])
def test_batch_periodic_sparsify_equals_single(product_built, precision):
    """The reference driver's periodic sparsify (every 20 loops here) inside a batch: each
    quench pauses at the end of the loop, the host compacts its history, the controller
    and planner resume on the device; the result equals dyn_run with the same cadence."""
    grids, m32, m64 = _grids()
    kw = dict(vars(m32))
    kw["delta_max"] = 1e-7
    m = D.Model(**kw)
    kw2 = dict(vars(m64))
    kw2["delta_max"] = 1e-7
    m2 = D.Model(**kw2)
    specs = [(0, m, 70), (1, m2, 45)]
    for variant, serk2 in (("gpu", False), ("cpu", False), ("gpu", True)):
        b = D.Batch(grids, [_quench(gi, mm, max_steps=n) for gi, mm, n in specs], ticks_per_launch=16,
                    sparsify_every=20, sparsify_variant=variant, precision=precision, use_serk2=serk2)
        b.run(100_000)
        if serk2:
            assert b.info(0)["method"] >= 3  # climbed past SSPRK(10,4)
        for q, (gi, mm, n) in enumerate(specs):
            inf = b.info(q)
            assert inf["status"] == "max_steps" and inf["steps"] == n
            s = D.Simulation(grids[gi], mm, precision=precision)
            s.init()
            tr = s.run(n, sparsify_every=20, sparsify_variant=variant, use_serk2=serk2)
            st = s.download()
            assert st.t1grid.size < n + 1  # rows were dropped
            _assert_same_state(b.download(q), st)
            c = s.controller
            assert (inf["delta_t"], inf["method"], inf["loop"]) == (c["delta_t"], c["method"], c["loop"])
            assert inf["energy"] == tr["energy"][-1]
        b.close()


def test_batch_df_equals_single_df(product_built):
    """The (hi, lo) form in a batch: every quench equals the same quench run alone in that form."""
    grids, m32, m64 = _grids()
    specs = [(0, m32, 50), (1, m64, 35)]
    b = D.Batch(grids, [_quench(gi, m, max_steps=n) for gi, m, n in specs], ticks_per_launch=16, precision="mixed_df")
    b.run(100_000)
    for q, (gi, m, n) in enumerate(specs):
        s = D.Simulation(grids[gi], m, precision="mixed_df")
        s.init()
        tr = s.run(n)
        _assert_same_state(b.download(q), s.download())
        assert b.info(q)["energy"] == tr["energy"][-1]
    b.close()
