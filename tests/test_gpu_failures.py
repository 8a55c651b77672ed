"""Failure detection on the GPU path, made on the host (no device fault, trap or hang):

* a history with a NaN is refused at upload (DYN_ERR_INVALID) and the context keeps
  its previous state;
* a finite state whose model terms overflow (C ~ 1e200, so f'(C) is infinite) gives a
  non-finite error estimate at the first step: dyn_run stops with DYN_ERR_NONFINITE
  instead of letting its controller act on NaN (the reference's loop would go on, every
  comparison false);
* the same state in one quench of a batch stops that quench with status "failed" while
  the other quench runs to its step limit and equals its single run.
"""
import numpy as np
import pytest

import dynamite_gb300 as D
from dynamite_gb300 import _lib
from conftest import load_golden
from helpers import grid_from, model_from, state_from

pytestmark = pytest.mark.gpu


def test_nan_history_refused_at_upload(product_built):
    g = load_golden(32)
    s = D.Simulation(grid_from(g, D.Grid), model_from(g, D.Model))
    good = state_from(g, "mid", D.State)
    s.upload(good)
    n = s.n
    for field in ("QK", "dQR", "rvec"):
        bad = state_from(g, "mid", D.State)
        setattr(bad, field, np.array(getattr(bad, field), copy=True))  # the fixture's arrays stay clean
        getattr(bad, field)[3] = np.nan
        with pytest.raises(_lib.DynError) as e:
            s.upload(bad)
        assert e.value.status == _lib.DYN_ERR_INVALID
    assert s.n == n
    np.testing.assert_array_equal(s.download().QK, good.QK)


def _overflowing(g):
    st = state_from(g, "mid", D.State)
    L = g["grid_theta"].size
    st.QK = np.array(st.QK, copy=True)
    st.QK[-L:] *= 1e200        # finite, but f'(C) = 3 lam C^2 + ... overflows
    return st


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overflow_stops_the_driver_loop(product_built, precision):
    g = load_golden(32)
    s = D.Simulation(grid_from(g, D.Grid), model_from(g, D.Model), precision=precision)
    s.upload(_overflowing(g))
    s.set_controller(float(g["rk54_dt"][0]), 1)
    n = s.n
    with pytest.raises(_lib.DynError) as e:
        s.run(5)
    assert e.value.status == _lib.DYN_ERR_NONFINITE
    assert s.n == n + 1          # the one step that produced it, nothing after
    # the context stays usable: a good state runs again
    s.upload(state_from(g, "mid", D.State))
    s.set_controller(float(g["rk54_dt"][0]), 1)
    s.run(2)
    assert np.isfinite(s.download().QK).all()


def test_overflow_fails_one_batch_quench(product_built):
    g = load_golden(32)
    grid, m = grid_from(g, D.Grid), model_from(g, D.Model)
    kw = dict(p=m.p, p2=m.p2, lam=m.lam, T0=m.T0, Gamma=m.Gamma, delta_t_min=m.delta_t_min,
              delta_max=m.delta_max, max_steps=6)
    b = D.Batch([grid], [D.Quench(grid=0, **kw), D.Quench(grid=0, **kw)], ticks_per_launch=8, precision="mixed")
    b.upload(0, _overflowing(g), delta_t=float(g["rk54_dt"][0]), method=1)
    b.run(10_000)
    i0, i1 = b.info(0), b.info(1)
    assert i0["status"] == "failed" and i0["steps"] == 1
    assert i1["status"] == "max_steps" and i1["steps"] == 6
    s = D.Simulation(grid, m, precision="mixed")
    s.init()
    s.run(6)
    np.testing.assert_array_equal(b.download(1).QK, s.download().QK)
    b.close()
