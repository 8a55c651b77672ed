"""Log-space response interpolation, the reference's -R option
(index_vec.cu:185-226 for A1/A2, index_vec.cu:456-530 for B1,
index_mat.cu:149-227 for B2): QK is gathered as in the linear form, QR as the
exponential of the same stencil / Hermite interpolation applied to log QR
(with the derivatives dQR / QR), wherever every value it rests on is
positive, and linearly elsewhere.

The oracle's log-space gathers restate the reference's CPU form
(index_vec.cpp:24-57, 82-104, 117-131; index_mat.cpp:44-63, 72-86) and are
pinned to the compiled reference's own outputs (tests/golden/golden_log_L64.npz,
made by tests/golden/make_golden.py) and by known answers: a history whose QR is
the exponential of a polynomial is gathered exactly in log space (the poly-9
A1/A2 stencils in theta; the cubic and quadratic Hermite forms in time for
B1/B2), which the linear form cannot do.  The GPU tests hold the CUDA path to
the golden vectors and to the oracle."""
import os
import platform

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN, load_golden
from helpers import STATE_FIELDS, grid_from, model_from, rel_err, state_from

# the reference sums the A1/A2 logs in long double: 80-bit on x86-64, 128-bit on aarch64
EXACT_HOST = platform.machine() in ("x86_64", "AMD64")


def load_log_golden() -> dict:
    with np.load(os.path.join(GOLDEN, "golden_log_L64.npz")) as f:
        return {k: f[k] for k in f.files}

# A1/A2 case: three rows, the last one QR = exp(QA(theta))
QA = lambda x: -3.0 * x + 0.7 * x ** 3 - 0.2 * x ** 9
# B1/B2 case: every column of row k holds QR = exp(q(t_k)); q quadratic, so the
# cubic and the quadratic (last-interval) Hermite branches are both exact
T_ROWS = np.array([0.0, 0.1, 0.25, 0.45, 0.7, 1.0, 1.4, 1.9, 2.5, 3.2, 4.0, 5.0])
q = lambda t: -0.3 * t + 0.02 * t ** 2
dq = lambda t: -0.3 + 0.04 * t


def _ratio(t):
    r = np.zeros(t.size)
    r[2:] = (t[2:] - t[1:-1]) / (t[1:-1] - t[:-2])
    return r


def last_row_state(cls, theta):
    L, n = theta.size, 3
    t = np.array([0.0, 0.5, 1.0])
    return cls(t, _ratio(t), np.tile(0.5 * theta, n), np.tile(np.exp(QA(theta)), n), np.zeros(n * L),
               np.zeros(n * L), np.full(n, 0.6), np.zeros(n))


def time_history_state(cls, L):
    """dQR of row k is h_k times the derivative at t_{k-1}, as the stored
    derivative columns pair with the row before them."""
    t = T_ROWS
    n = t.size
    R = np.exp(q(t))
    dR = np.zeros(n)
    dR[1:] = np.diff(t) * dq(t[:-1]) * R[:-1]
    K = np.cos(t)
    dK = np.zeros(n)
    dK[1:] = -np.diff(t) * np.sin(t[:-1])
    return cls(t, _ratio(t), np.repeat(K, L), np.repeat(R, L), np.repeat(dK, L), np.repeat(dR, L),
               np.full(n, 0.6), np.zeros(n))


def positive_history(cls, theta, n=60, Tm=0.6, t_hi=50.0):
    """A smooth history with QR = 1 / (Tm (t + 1)) > 0 everywhere (QK as in the
    stage-timing history), where the log and linear forms differ."""
    t = np.concatenate([[0.0], np.logspace(-5, np.log10(t_hi), n - 1)])
    tc = t[:, None]
    QK = (theta[None, :] * tc + 1.0) / (tc + 1.0)
    QR = np.broadcast_to(1.0 / (Tm * (tc + 1.0)), QK.shape).copy()
    h = np.diff(t, prepend=0.0)[:, None]
    tp = np.concatenate([[0.0], t[:-1]])[:, None]
    dQK = h * (theta[None, :] - 1.0) / (tp + 1.0) ** 2
    dQR = np.broadcast_to(-h / (Tm * (tp + 1.0) ** 2), QK.shape).copy()
    return cls(t, _ratio(t), QK.ravel(), QR.ravel(), dQK.ravel(), dQR.ravel(), np.ones(n), np.zeros(n))


def port_for(g, log_response, search_mode=1):
    return O.Port(grid_from(g, O.Grid), model_from(g, O.Model), search_mode=search_mode, threads=4,
                  log_response=log_response)


def rel_elem(a, b):
    return float(np.max(np.abs(a / b - 1.0)))


# ------------------------------------------------------------------ oracle (CPU)
def test_oracle_log_a1_a2_reproduce_exp_of_polynomial(oracle_built):
    g = load_golden(64)
    p = port_for(g, True)
    theta, phi1, phi2 = g["grid_theta"], g["grid_phi1"], g["grid_phi2"]
    p.set_state(last_row_state(O.State, theta))
    p.interpolate()
    assert rel_elem(p.interp(1), np.exp(QA(phi1))) < 1e-11
    assert rel_elem(p.interp(3), np.exp(QA(phi2))) < 1e-11
    # QK stays linear: the linear form's values bit for bit
    lin = port_for(g, False)
    lin.set_state(last_row_state(O.State, theta))
    lin.interpolate()
    np.testing.assert_array_equal(p.interp(0), lin.interp(0))
    np.testing.assert_array_equal(p.interp(2), lin.interp(2))


def test_oracle_log_b1_b2_reproduce_exp_of_quadratic_in_time(oracle_built):
    g = load_golden(32)
    L = 32
    T = T_ROWS[-1]
    out = {}
    for logr in (True, False):
        p = port_for(g, logr)
        p.set_state(time_history_state(O.State, L))
        p.interpolate()
        out[logr] = (p.interp(5).reshape(L, L), p.interp(7))
    want_b1 = np.broadcast_to(np.exp(q(g["grid_theta"] * T))[:, None], (L, L))
    want_b2 = np.exp(q(g["grid_phi2"] * T))
    assert rel_elem(out[True][0], want_b1) < 1e-12
    assert rel_elem(out[True][1], want_b2) < 1e-11  # the wB2 stencils sum to 1 within ~1e-12
    # the linear form interpolates exp(q) with an O(h^4) error: the test discriminates
    assert rel_elem(out[False][0], want_b1) > 1e-7
    assert rel_elem(out[False][1], want_b2) > 1e-7


def test_oracle_log_falls_back_to_linear_where_a_value_is_not_positive(oracle_built):
    g = load_golden(32)
    L, m = 32, g["grid_wA1"].size // (32 * 32)
    st = last_row_state(O.State, g["grid_theta"])
    j0 = 13
    st.QR[2 * L + j0] = -0.01
    vals = {}
    for logr in (True, False):
        p = port_for(g, logr)
        p.set_state(st)
        p.interpolate()
        vals[logr] = p.interp(1)
    i0 = g["grid_indsA1"].astype(np.int64)
    covers = (i0 <= j0) & (j0 < i0 + m)
    assert covers.any() and (~covers).any()
    np.testing.assert_array_equal(vals[True][covers], vals[False][covers])
    assert np.all(vals[True][~covers] > 0.0)


def test_oracle_log_step_differs_from_linear_step(oracle_built):
    """On a history with curvature in log QR the two forms give different steps
    (so the GPU step test below exercises the log-space branches)."""
    g = load_golden(64)
    out = {}
    for logr in (True, False):
        p = port_for(g, logr)
        p.set_state(positive_history(O.State, g["grid_theta"]))
        p.interpolate()
        out[logr] = (p.update(1, 1e-3), p.get_state())
    assert rel_err(out[True][1].QK, out[False][1].QK) > 1e-6
    assert np.isfinite(out[True][0]) and out[True][0] > 0.0


def _same(a, b, what):
    if EXACT_HOST:
        np.testing.assert_array_equal(a, b, err_msg=what)
    else:
        assert rel_err(a, b) < 1e-14, what


def test_oracle_log_matches_reference_golden(oracle_built):
    """Interpolation, QKstep/QRstep and one RK54 step on a history with curvature
    in log QR, and the reference controller's 80-step log-space run from t = 0."""
    g, lg = load_golden(64), load_log_golden()
    p = port_for(g, True, search_mode=0)
    st = state_from(lg, "pos", O.State, with_pos=False)
    p.set_state(st)
    p.interpolate()
    for w in (1, 3, 5, 7):
        _same(p.interp(w), lg[f"pos_interp{w}"], f"interp {w}")
    _same(p.qkstep(), lg["pos_qk"], "qk")
    _same(p.qrstep(), lg["pos_qr"], "qr")
    p.set_state(st)
    p.interpolate()
    err = p.update(1, 1e-3)
    b = p.get_state()
    for k in STATE_FIELDS:
        _same(getattr(b, k), lg[f"pos_rk54_{k}"], k)
    _same(np.array([err]), lg["pos_rk54_err"], "err")
    p = port_for(g, True, search_mode=0)
    p.init_state()
    tr = p.run(lg["ltraj_dt"].size)
    for k in ("dt", "method", "t", "energy"):
        _same(tr[k], lg[f"ltraj_{k}"], k)
    b = p.get_state()
    for k in ("t1grid", "QK", "QR", "rvec"):
        _same(getattr(b, k), lg[f"ltraj_final_{k}"], k)


@pytest.mark.skipif(not O.Reference.available(), reason="compiled reference not present")
def test_oracle_log_matches_compiled_reference_on_the_known_answer_states(oracle_built):
    g = load_golden(64)
    ref = O.Reference(grid_from(g, O.Grid), model_from(g, O.Model), threads=1, log_response=True)
    p = port_for(g, True, search_mode=0)
    for st in (last_row_state(O.State, g["grid_theta"]), time_history_state(O.State, 64),
               state_from(g, "mid", O.State)):
        for x in (ref, p):
            x.set_state(st)
            x.interpolate()
        for w in range(16):
            np.testing.assert_array_equal(p.interp(w), ref.interp(w), err_msg=f"interp {w}")


def test_log_response_is_fp64_only(product_built):
    """Rejected before any CUDA call: the mixed forms have no log-space gathers."""
    import dynamite_gb300 as D
    from dynamite_gb300 import _lib
    g = load_golden(32)
    for prec in ("mixed", "mixed_df"):
        with pytest.raises(_lib.DynError, match="log-space"):
            D.Simulation(grid_from(g, D.Grid), model_from(g, D.Model), precision=prec, log_response=True)


# ------------------------------------------------------------------ CUDA path
STEP_TOL = 1e-12
TRAJ_TOL = 1e-10


def sim_for(g, **kw):
    import dynamite_gb300 as D
    return D.Simulation(grid_from(g, D.Grid), model_from(g, D.Model), log_response=True, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("L", (32, 64))
def test_gpu_log_interpolation_matches_oracle(product_built, L):
    """Reference-order gathers: A1/A2 QK bit for bit; B1/B2 QK within 1e-15 (the
    reference's log-space B1 kernel folds (w^2 + w^3) / ratio into one
    coefficient, its linear CPU form divides last); QR and Sigma arrays within
    1e-13 (CUDA's log/exp against the host libm's)."""
    import dynamite_gb300 as D
    g = load_golden(L)
    s = sim_for(g)
    s.upload(state_from(g, "mid", D.State))
    s.interpolate()
    p = port_for(g, True, search_mode=0)
    p.set_state(state_from(g, "mid", O.State))
    p.interpolate()
    for w in (0, 2):
        np.testing.assert_array_equal(s.interp(w), p.interp(w), err_msg=f"interp {w}")
    for w in (4, 6):
        assert rel_err(s.interp(w), p.interp(w)) < 1e-15, w
    for w in (1, 3, 5, 7, 8, 9, 11, 12, 13, 14, 15):
        assert rel_err(s.interp(w), p.interp(w)) < 1e-13, w


@pytest.mark.gpu
def test_gpu_log_matches_reference_golden(product_built):
    """The CUDA path against the compiled reference's log-space outputs: the
    reference-order gathers and RHS, the fused RK54 step, and the reference
    controller's schedule replayed from t = 0."""
    import dynamite_gb300 as D
    g, lg = load_golden(64), load_log_golden()
    s = sim_for(g)
    s.upload(state_from(lg, "pos", D.State, with_pos=False))
    s.interpolate()
    # the reference's CPU form sums the A1/A2 logs in long double, its CUDA form
    # and this one in double: ~1.5e-13 apart on this history (poly-9 weights)
    for w in (1, 3, 5, 7):
        assert rel_err(s.interp(w), lg[f"pos_interp{w}"]) < 1e-12, w
    hK, hR = s.QKRstep()
    assert rel_err(hK, lg["pos_qk"]) < 1e-12
    assert rel_err(hR, lg["pos_qr"]) < 1e-12
    s.upload(state_from(lg, "pos", D.State, with_pos=False))
    r = s.update(1, 1e-3)
    a = s.download()
    np.testing.assert_array_equal(a.t1grid, lg["pos_rk54_t1grid"])
    for k in ("QK", "QR", "dQK", "dQR", "rvec"):
        assert rel_err(getattr(a, k), lg[f"pos_rk54_{k}"]) < STEP_TOL, k
    assert abs(r.delta - lg["pos_rk54_err"][0]) < 5e-14  # a difference of two embedded solutions
    s.init()
    tr = s.run(lg["ltraj_dt"].size, schedule=(lg["ltraj_dt"], lg["ltraj_method"]))
    a = s.download()
    np.testing.assert_array_equal(a.t1grid, lg["ltraj_final_t1grid"])
    for k in ("QK", "QR", "rvec"):
        assert rel_err(getattr(a, k), lg[f"ltraj_final_{k}"]) < TRAJ_TOL, k
    assert rel_err(tr["energy"], lg["ltraj_energy"]) < TRAJ_TOL


@pytest.mark.gpu
def test_gpu_log_known_answers(product_built):
    import dynamite_gb300 as D
    g = load_golden(32)
    L, T = 32, T_ROWS[-1]
    s = sim_for(g)
    s.upload(time_history_state(D.State, L))
    s.interpolate()
    assert rel_elem(s.interp(5).reshape(L, L), np.exp(q(g["grid_theta"] * T))[:, None]) < 1e-12
    assert rel_elem(s.interp(7), np.exp(q(g["grid_phi2"] * T))) < 1e-11
    s.upload(last_row_state(D.State, g["grid_theta"]))
    s.interpolate()
    assert rel_elem(s.interp(1), np.exp(QA(g["grid_phi1"]))) < 1e-10  # FMA sums on the coarse L=32 grid


@pytest.mark.gpu
@pytest.mark.parametrize("L", (32, 64))
@pytest.mark.parametrize("tag,method", [("rk54", 1), ("ssp", 2)])
def test_gpu_log_fused_step_matches_oracle(product_built, L, tag, method):
    import dynamite_gb300 as D
    g = load_golden(L)
    dt = float(g[f"{tag}_dt"][0])
    s = sim_for(g)
    s.upload(state_from(g, "mid", D.State))
    r = s.update(method, dt)
    p = port_for(g, True)
    st = state_from(g, "mid", O.State)
    p.set_state(st)
    p.interpolate(st.posB1xOld, st.posB2xOld, True)  # the step starts from the state's own interpolation
    delta = p.update(method, dt)
    a, b = s.download(), p.get_state()
    np.testing.assert_array_equal(a.t1grid, b.t1grid)
    for k in ("QK", "QR", "dQK", "dQR", "rvec"):
        assert rel_err(getattr(a, k), getattr(b, k)) < STEP_TOL, k
    assert abs(r.delta - delta) < 5e-14


@pytest.mark.gpu
def test_gpu_log_fused_step_on_positive_history(product_built):
    import dynamite_gb300 as D
    g = load_golden(64)
    s = sim_for(g)
    s.upload(positive_history(D.State, g["grid_theta"]))
    r = s.update(1, 1e-3)
    p = port_for(g, True)
    p.set_state(positive_history(O.State, g["grid_theta"]))
    p.interpolate()
    delta = p.update(1, 1e-3)
    a, b = s.download(), p.get_state()
    np.testing.assert_array_equal(a.t1grid, b.t1grid)
    for k in ("QK", "QR", "dQK", "dQR", "rvec"):
        assert rel_err(getattr(a, k), getattr(b, k)) < STEP_TOL, k
    assert abs(r.delta - delta) < 5e-14


@pytest.mark.gpu
@pytest.mark.parametrize("L", (64, 512))
def test_gpu_log_trajectory_matches_oracle(product_built, L):
    """From t = 0 over the oracle's replay of the GPU run's schedule; L = 512 on
    the production grid (poly-9, Tmax 1e5)."""
    import dynamite_gb300 as D
    if L == 64:
        g = load_golden(L)
        grid, model = grid_from(g, D.Grid), model_from(g, D.Model)
        og, om = grid_from(g, O.Grid), model_from(g, O.Model)
        steps = 40
    else:
        grid = D.grid.generate(L)
        model, om = D.Model(p=3, p2=4, lam=0.5, Gamma=0.6), O.Model(p=3, p2=4, lam=0.5, Gamma=0.6)
        og = O.Grid(L, grid.theta, grid.phi1, grid.phi2, grid.integ, grid.indsA1, grid.wA1, grid.indsA2,
                    grid.wA2, grid.indsB2, grid.wB2)
        steps = 12
    s = D.Simulation(grid, model, log_response=True)
    s.init()
    tr = s.run(steps)
    p = O.Port(og, om, search_mode=1, threads=0, log_response=True)
    p.init_state()
    tp = p.run(steps, schedule=(tr["dt"], tr["method"]))
    a, b = s.download(), p.get_state()
    np.testing.assert_array_equal(a.t1grid, b.t1grid)
    for k in ("QK", "QR", "rvec"):
        assert rel_err(getattr(a, k), getattr(b, k)) < TRAJ_TOL, k
    assert rel_err(tr["energy"], tp["energy"]) < TRAJ_TOL


@pytest.mark.gpu
def test_gpu_log_adjoint_rejected(product_built):
    from dynamite_gb300 import _lib
    g = load_golden(32)
    s = sim_for(g)
    s.init()
    with pytest.raises(_lib.DynError, match="linear-domain"):
        s.adjoint_forward(4)
