"""Discrete adjoint of the FP64 pipeline (dyn_adjoint_forward/backward):
gradients of E(t_f), C(t_f, t_f/2) and r(t_f) with respect to Gamma (the
bath temperature) and lambda against central finite differences (h = 1e-5,
relative) of the FP64 forward on the same frozen step schedule."""
import numpy as np
import pytest

import dynamite_gb300 as D
from conftest import load_golden
from helpers import grid_from, model_from

pytestmark = pytest.mark.gpu

FD_TOL = 1e-5   # relative agreement adjoint vs central differences
H = 1e-5        # relative FD step
EPS = np.finfo(np.float64).eps


def _agree(a, f, J, p):
    """|adjoint - FD| within FD_TOL relative, or within the FD's own rounding
    floor (50 eps |J| / (H |p|)) for derivatives far smaller than J / p."""
    return abs(a - f) <= FD_TOL * abs(f) + 50 * EPS * abs(J) / (H * abs(p))


def _objectives(s: D.Simulation, cK):
    st = s.download()
    L = s.L
    last = st.QK[-L:]
    return {"E": s.energy(), "C": float(cK @ last), "r": float(st.rvec[-1])}


def _fd(grid, model, sched, cK):
    out = {"J": None}
    for name, base in (("Gamma", model.Gamma), ("lam", model.lam)):
        vals = []
        for sgn in (+1, -1):
            kw = dict(vars(model))
            kw[name] = base * (1 + sgn * H)
            s = D.Simulation(grid, D.Model(**kw))
            s.init()
            s.run(len(sched[0]), schedule=sched)
            vals.append(_objectives(s, cK))
            s.close()
        out[name] = {k: (vals[0][k] - vals[1][k]) / (2 * H * base) for k in vals[0]}
        out["J"] = vals[0]
    return out


def _check(grid, model, nsteps):
    s = D.Simulation(grid, model)
    s.init()
    fw = s.adjoint_forward(nsteps)
    sched = (fw["dt"], fw["method"])
    cK = D.grid.lagrange_weights(grid.theta, 0.5)
    gE, stats = s.adjoint_backward(w_energy=1.0)
    assert stats["recompute_mismatch"] == 0  # the reverse sweep recomputes the forward bit for bit
    adj = {"E": gE, "C": s.adjoint_backward(c_K=cK)[0], "r": s.adjoint_backward(w_r=1.0)[0]}
    # the reverse sweep leaves the forward's history in place
    ref = D.Simulation(grid, model)
    ref.init()
    ref.run(nsteps, schedule=sched)
    np.testing.assert_array_equal(s.download().QK, ref.download().QK)
    fd = _fd(grid, model, sched, cK)
    for obj in ("E", "C", "r"):
        for k, name in enumerate(("Gamma", "lam")):
            a, f = adj[obj][k], fd[name][obj]
            assert _agree(a, f, fd["J"][obj], getattr(model, name)), (obj, name, a, f)
    return s


def test_adjoint_matches_fd_small(product_built):
    g = load_golden(32)
    _check(grid_from(g, D.Grid), model_from(g, D.Model), 40)


def test_adjoint_matches_fd_ssprk_and_l64(product_built):
    """L=64 run long enough for the controller to use both RK54 and SSPRK(10,4)."""
    g = load_golden(64)
    m = D.Model(p=3, p2=4, lam=0.3, Gamma=0.7)
    grid = grid_from(g, D.Grid)
    s = D.Simulation(grid, m)
    s.init()
    s.set_controller(delta_t=0.02, method=2)  # start on SSPRK(10,4)
    fw = s.adjoint_forward(30)
    assert set(np.unique(fw["method"])) >= {2}
    cK = D.grid.lagrange_weights(grid.theta, 0.5)
    gE = s.adjoint_backward(w_energy=1.0)[0]
    sched = (fw["dt"], fw["method"])
    for k, name in enumerate(("Gamma", "lam")):
        vals = []
        for sgn in (+1, -1):
            kw = dict(vars(m))
            kw[name] = getattr(m, name) * (1 + sgn * H)
            t = D.Simulation(grid, D.Model(**kw))
            t.init()
            t.set_controller(delta_t=0.02, method=2)
            t.run(30, schedule=sched)
            vals.append(t.energy())
        f = (vals[0] - vals[1]) / (2 * H * getattr(m, name))
        assert _agree(gE[k], f, vals[0], getattr(m, name)), (name, gE[k], f)


def test_adjoint_requires_recorded_forward(product_built):
    g = load_golden(32)
    s = D.Simulation(grid_from(g, D.Grid), model_from(g, D.Model))
    s.init()
    with pytest.raises(D.DynError):
        s.adjoint_backward(w_energy=1.0)
    s.adjoint_forward(5)
    s.update()  # the history moves on: the recorded forward no longer applies
    with pytest.raises(D.DynError):
        s.adjoint_backward(w_energy=1.0)


def test_adjoint_history_gradient_matches_fd(product_built):
    """dJ/d(uploaded initial history) on a 3-step sweep, spot-checked entry by entry."""
    g = load_golden(32)
    grid, model = grid_from(g, D.Grid), model_from(g, D.Model)
    L = grid.L
    base = D.Simulation(grid, model)
    base.init()
    sched = (np.full(2, 2e-3), np.full(2, 1, dtype=np.int32))
    base.run(2, schedule=sched)
    st0 = base.download()
    sd = (np.full(3, 2e-3), np.full(3, 1, dtype=np.int32))
    s = D.Simulation(grid, model)
    s.upload(st0)
    s.adjoint_forward(3, schedule=sd)
    s.adjoint_backward(w_r=1.0)
    hg = s.adjoint_history_grad(st0.n)
    fields = ("t1grid", "dtr", "QK", "QR", "dQK", "dQR", "rvec", "drvec")
    for field, k in (("QK", L + 3), ("QR", 2 * L + 7), ("dQK", 2 * L + 11), ("dQR", L + 5), ("rvec", 1),
                     ("drvec", 2)):
        vals = []
        for sg in (+1, -1):
            p = D.State(*[getattr(st0, f).copy() for f in fields])
            getattr(p, field)[k] += sg * 1e-7
            t = D.Simulation(grid, model)
            t.upload(p)
            t.run(3, schedule=sd)
            vals.append(float(t.download().rvec[-1]))
        f = (vals[0] - vals[1]) / 2e-7
        a = getattr(hg, field)[k]
        assert abs(a - f) <= 1e-4 * abs(f) + 1e-8, (field, k, a, f)
