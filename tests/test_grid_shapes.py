"""Grid shapes other than the golden poly-9 grids: stencil depth 8 (interp_order 7)
at L = 72 (partial tiles in the gather and the epilogue), depth 6 (interp_order 5)
at L = 96, and Floater-Hormann (-m rational) stencils of order 5 on 12-point
windows at L = 80, all from the native generator (bit-identical to the
reference's).  They take the generic-depth instantiations of every kernel family
(FP64 and mixed gathers, the batch, the log-space form, the adjoint's generic B2
path), which the depth-10 golden cases never reach.

Not every (L, depth) at Tmax = 1e3 gives a usable grid: with L = 44, 45 or 48 the
reference itself produces NaN within 60 steps, and with L = 40 at depth 8 C(t, t')
exceeds 1 and rounding differences grow about 30-fold every 10 steps, so two
correct implementations drift apart; those are not test cases."""
import numpy as np
import pytest

import oracle as O
from helpers import rel_err

SHAPES = [(72, 7), (96, 5), (80, -5)]  # a negative order: -m rational, FH order 5 on 12-point windows
STEPS = 60


def _grids(L, order):
    import dynamite_gb300 as D
    if order < 0:
        g = D.grid.generate(L, Tmax=1e3, interp_order=-order, method="rational", fh_window=12)
    else:
        g = D.grid.generate(L, Tmax=1e3, interp_order=order)
    og = O.Grid(L, g.theta, g.phi1, g.phi2, g.integ, g.indsA1, g.wA1, g.indsA2, g.wA2, g.indsB2, g.wB2)
    return g, og


MODEL = dict(p=3, p2=4, lam=0.5, Gamma=0.6)


@pytest.mark.parametrize("L,order", SHAPES)
def test_oracle_matches_reference_on_other_depths(product_built, oracle_built, L, order):
    if not O.Reference.available():
        pytest.skip("compiled reference not present")
    import dynamite_gb300 as D
    g, og = _grids(L, order)
    ref_grid = (O.Reference.grid(L, Tmax=1e3, interp_order=-order, method="rational", fh_window=12) if order < 0
                else O.Reference.grid(L, Tmax=1e3, interp_order=order))
    for f in ("theta", "indsA1", "wA1", "indsB2", "wB2"):
        np.testing.assert_array_equal(getattr(g, f), getattr(ref_grid, f), err_msg=f)
    p = O.Port(og, O.Model(**MODEL), search_mode=0, threads=4)
    p.init_state()
    tp = p.run(STEPS)
    ref = O.Reference(og, O.Model(**MODEL), threads=1)
    ref.init_state()
    tr = ref.run(STEPS)
    a, b = p.get_state(), ref.get_state()
    np.testing.assert_array_equal(a.t1grid, b.t1grid)
    np.testing.assert_array_equal(a.QK, b.QK)
    np.testing.assert_array_equal(tp["energy"], tr["energy"])
    assert g.depth == (12 if order < 0 else order + 1) and np.isfinite(a.QK).all()


@pytest.mark.gpu
@pytest.mark.parametrize("L,order", SHAPES)
def test_gpu_forms_on_other_depths(product_built, L, order):
    """FP64 and log-space runs against the oracle on the GPU run's schedule; the two
    mixed forms against the FP64 run; a two-quench batch against the single run."""
    import dynamite_gb300 as D
    g, og = _grids(L, order)
    s = D.Simulation(g, D.Model(**MODEL))
    s.init()
    tr = s.run(STEPS)
    sched = (tr["dt"], tr["method"])
    p = O.Port(og, O.Model(**MODEL), search_mode=1, threads=4)
    p.init_state()
    tp = p.run(STEPS, schedule=sched)
    a, b = s.download(), p.get_state()
    np.testing.assert_array_equal(a.t1grid, b.t1grid)
    for k in ("QK", "QR", "rvec"):
        assert rel_err(getattr(a, k), getattr(b, k)) < 1e-10, k
    assert rel_err(tr["energy"], tp["energy"]) < 1e-10
    # log-space response
    sl = D.Simulation(g, D.Model(**MODEL), log_response=True)
    sl.init()
    sl.run(STEPS, schedule=sched)
    pl = O.Port(og, O.Model(**MODEL), search_mode=1, threads=4, log_response=True)
    pl.init_state()
    pl.run(STEPS, schedule=sched)
    assert rel_err(sl.download().QK, pl.get_state().QK) < 1e-10
    # mixed forms
    for prec in ("mixed", "mixed_df"):
        sm = D.Simulation(g, D.Model(**MODEL), precision=prec)
        sm.init()
        sm.run(STEPS, schedule=sched)
        c = sm.download()
        assert rel_err(c.QK, a.QK) < 1e-6 and rel_err(c.QR, a.QR) < 1e-6, prec
    # batch of two quenches on this grid against the same quenches alone (mixed form)
    qs = [D.Quench(grid=0, p=3, p2=4, lam=lam, Gamma=0.6, max_steps=40, capacity=64) for lam in (0.3, 0.5)]
    bt = D.Batch([g], qs, ticks_per_launch=16, precision="mixed")
    bt.run(100_000)
    for q, lam in enumerate((0.3, 0.5)):
        ss = D.Simulation(g, D.Model(p=3, p2=4, lam=lam, Gamma=0.6), precision="mixed")
        ss.init()
        ss.run(40)
        st, sb = ss.download(), bt.download(q)
        np.testing.assert_array_equal(sb.t1grid, st.t1grid)
        np.testing.assert_array_equal(sb.QK, st.QK)
    bt.close()


@pytest.mark.gpu
def test_gpu_adjoint_on_depth_8(product_built):
    """dE/dGamma through the adjoint's generic-depth B2 path against central differences."""
    import dynamite_gb300 as D
    g, _ = _grids(72, 7)
    m = D.Model(**MODEL)
    s = D.Simulation(g, m)
    s.init()
    fw = s.adjoint_forward(30)
    sched = (fw["dt"], fw["method"])
    grad, stats = s.adjoint_backward(w_energy=1.0)
    assert stats["recompute_mismatch"] == 0
    h = 1e-5
    vals = []
    for sgn in (+1, -1):
        kw = dict(MODEL)
        kw["Gamma"] = MODEL["Gamma"] * (1 + sgn * h)
        f = D.Simulation(g, D.Model(**kw))
        f.init()
        f.run(30, schedule=sched)
        vals.append(f.energy())
    fd = (vals[0] - vals[1]) / (2 * h * MODEL["Gamma"])
    floor = 50 * np.finfo(np.float64).eps * abs(vals[0]) / (h * MODEL["Gamma"])  # the FD's rounding
    assert abs(grad[0] - fd) <= 1e-5 * abs(fd) + floor, (grad[0], fd)
