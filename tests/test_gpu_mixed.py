"""Mixed-precision form (FP32 gathers and convolutions with compensated sums;
r(t), time, C(t,t), the error norm and every O(L) quantity in FP64) against
the FP64 path and the oracle."""
import numpy as np
import pytest

import oracle as O
import dynamite_gb300 as D
from conftest import load_golden
from helpers import STATE_FIELDS, grid_from, model_from, rel_err, state_from

pytestmark = pytest.mark.gpu

MIXED_RHS_TOL = 1e-4     # one RHS: a cancelling sum of FP32 terms, relative to max |h|
MIXED_TRAJ_TOL = 1e-6    # energy / C after a fixed-schedule run, relative


@pytest.mark.parametrize("L", [32, 64])
def test_mixed_rhs_vs_reference(product_built, L):
    g = load_golden(L)
    s = D.Simulation(grid_from(g, D.Grid), model_from(g, D.Model), precision="mixed")
    s.upload(state_from(g, "mid", D.State))
    hK, hR = s.rhs()
    assert rel_err(hK, g["mid_qk"]) < MIXED_RHS_TOL
    assert rel_err(hR, g["mid_qr"]) < MIXED_RHS_TOL


@pytest.mark.parametrize("L", [32, 64])
def test_mixed_trajectory_vs_reference(product_built, L):
    g = load_golden(L)
    s = D.Simulation(grid_from(g, D.Grid), model_from(g, D.Model), precision="mixed")
    s.init()
    tr = s.run(g["traj_dt"].size, schedule=(g["traj_dt"], g["traj_method"]))
    st = s.download()
    np.testing.assert_array_equal(st.t1grid, g["traj_final_t1grid"])  # time stays FP64
    assert rel_err(tr["energy"], g["traj_energy"]) < MIXED_TRAJ_TOL
    assert rel_err(st.QK, g["traj_final_QK"]) < MIXED_TRAJ_TOL
    assert rel_err(st.rvec, g["traj_final_rvec"]) < MIXED_TRAJ_TOL


def test_mixed_large_grid_vs_fp64(product_built):
    """L=512, the FP64 run's schedule replayed in mixed precision."""
    L = 512
    grid = D.grid.generate(L)
    m = D.Model(p=3, p2=4, lam=0.5, Gamma=0.6)
    a = D.Simulation(grid, m)
    b = D.Simulation(grid, m, precision="mixed")
    a.init()
    b.init()
    ta = a.run(300)
    tb = b.run(300, schedule=(ta["dt"], ta["method"]))
    sa, sb = a.download(), b.download()
    np.testing.assert_array_equal(sa.t1grid, sb.t1grid)
    assert rel_err(tb["energy"], ta["energy"]) < MIXED_TRAJ_TOL
    assert rel_err(sb.QK, sa.QK) < MIXED_TRAJ_TOL
    assert rel_err(sb.rvec, sa.rvec) < MIXED_TRAJ_TOL
    # C(t,t) (theta = 1 column) stays at its FP64 value to within the FP64 error
    L_ = L
    diag_a = sa.QK.reshape(-1, L_)[:, -1]
    diag_b = sb.QK.reshape(-1, L_)[:, -1]
    assert np.max(np.abs(diag_a - diag_b)) < 1e-6


def test_mixed_sparsify_and_graph_replay(product_built):
    g = load_golden(32)
    s = D.Simulation(grid_from(g, D.Grid), model_from(g, D.Model), precision="mixed", use_graph=True)
    s.upload(state_from(g, "traj_final", D.State))
    n = s.sparsifyNscale(float(g["spars_threshold"][0]), "gpu")
    assert n < g["traj_final_t1grid"].size
    dt = float(g["traj_dt"][-1])
    r1 = s.update(1, dt)
    r2 = s.update(1, dt)
    assert np.isfinite([r1.delta, r2.delta, r2.energy]).all()


MIXED_DF_TOL = 1e-8   # (hi, lo) inputs: the frozen FP32 roundings removed


@pytest.mark.parametrize("L", [32, 64])
def test_mixed_df_trajectory_vs_reference(product_built, L):
    g = load_golden(L)
    s = D.Simulation(grid_from(g, D.Grid), model_from(g, D.Model), precision="mixed_df")
    s.init()
    tr = s.run(g["traj_dt"].size, schedule=(g["traj_dt"], g["traj_method"]))
    st = s.download()
    np.testing.assert_array_equal(st.t1grid, g["traj_final_t1grid"])
    assert rel_err(tr["energy"], g["traj_energy"]) < MIXED_DF_TOL
    assert rel_err(st.QK, g["traj_final_QK"]) < MIXED_DF_TOL
    assert rel_err(st.rvec, g["traj_final_rvec"]) < MIXED_DF_TOL


def test_mixed_df_large_grid_vs_fp64(product_built):
    """L=512, 300 steps of the FP64 run's schedule in the (hi, lo) form."""
    grid = D.grid.generate(512)
    m = D.Model(p=3, p2=4, lam=0.5, Gamma=0.6)
    a = D.Simulation(grid, m)
    b = D.Simulation(grid, m, precision="mixed_df")
    a.init()
    b.init()
    ta = a.run(300)
    tb = b.run(300, schedule=(ta["dt"], ta["method"]))
    sa, sb = a.download(), b.download()
    assert rel_err(tb["energy"], ta["energy"]) < MIXED_DF_TOL
    assert rel_err(sb.QK, sa.QK) < MIXED_DF_TOL
    assert rel_err(sb.QR, sa.QR) < MIXED_DF_TOL


def test_df_beyond_the_default_shared_memory(product_built):
    """The (hi, lo) form stages 2 (L + 2) float2 of the newest row, more than the 48 KB
    default from L = 3071 on (the kernels raise their limit per device).  At L = 3200 a
    short run alone and in a batch agrees with the FP64 form and with each other."""
    L = 3200
    grid = D.grid.generate(L)
    m = D.Model(p=3, p2=4, lam=0.5, Gamma=0.6)
    a = D.Simulation(grid, m, history_capacity=16)
    a.init()
    a.run(4)
    b = D.Simulation(grid, m, precision="mixed_df", history_capacity=16)
    b.init()
    b.run(4)
    qa, qb = a.download().QK, b.download().QK
    assert rel_err(qb, qa) < 1e-8
    bt = D.Batch([grid], [D.Quench(max_steps=4, capacity=16)], precision="mixed_df", ticks_per_launch=8)
    bt.run(1000)
    np.testing.assert_array_equal(bt.download(0).QK, qb)
    bt.close()


def test_df_controller_and_sparsify_follow_fp64(product_built):
    """What makes the (hi, lo) form a free-running replacement for FP64 at delta_max 1e-10
    (mixed p-spin lam = 0.5, T = 0.6, L = 512, 3000 steps from t = 0): (1) its own
    step-size controller takes the FP64 form's steps -- its stage derivatives carry no
    stage-to-stage FP32 rounding noise for the embedded error estimate to read -- and
    (2) one sparsify pass over the same history keeps FP64's rows.  Both up to
    decisions that sit within rounding of a threshold: the free runs end within 1e-3 of
    each other in t (measured 9e-5), and the keep lists may differ in a borderline row
    (over 4e5 steps at L=512 with four sparsify events: 147,283 rows kept against
    147,284).  (The plain mixed form meets neither: its free steps stay ~1000x below
    FP64's and its sparsify keeps far more rows.)"""
    grid = D.grid.generate(512)
    m = D.Model(p=3, p2=4, lam=0.5, Gamma=0.6)
    N = 3000
    runs, states = {}, {}
    for prec in ("fp64", "mixed_df"):
        s = D.Simulation(grid, m, precision=prec, history_capacity=N + 64)
        s.init()
        runs[prec] = s.run(N)
        s.close()
        assert np.count_nonzero(runs[prec]["dt"]) == N
    t_fp64 = runs["fp64"]["t"][-1]
    assert abs(runs["mixed_df"]["t"][-1] - t_fp64) < 1e-3 * t_fp64
    sched = (runs["fp64"]["dt"], runs["fp64"]["method"])
    for prec in ("fp64", "mixed_df"):
        s = D.Simulation(grid, m, precision=prec, history_capacity=N + 64)
        s.init()
        s.run(N, schedule=sched)
        s.sparsifyNscale(1e-10)
        states[prec] = s.download()
        s.close()
    kept, kept_df = states["fp64"].t1grid, states["mixed_df"].t1grid
    assert kept.size < 0.95 * (N + 1)  # rows were dropped
    assert abs(kept_df.size - kept.size) <= 2
    assert np.isin(kept, kept_df).mean() > 0.999
