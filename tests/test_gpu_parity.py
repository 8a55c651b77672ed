"""CUDA path vs the oracle (GPU).

Bit-exact where the reference computes integers or where the CUDA kernel
uses the reference's operation order (materialized interpolation, QKRstep,
r, dr, energy, positions, sparsify keep lists); within stated tolerances
where the fused kernels reassociate sums (fused RHS: 1e-12 relative; one RK
step: 1e-12; fixed-schedule trajectories: 1e-10, the parity bar for the
plain FP64 form).
"""
import numpy as np
import pytest

import oracle as O
import dynamite_gb300 as D
from conftest import load_golden
from helpers import STATE_FIELDS, grid_from, model_from, rel_err, state_from

pytestmark = pytest.mark.gpu

SIZES = (32, 64)
RHS_TOL = 1e-12      # fused RHS vs reference-order RHS, relative to max |h|
STEP_TOL = 1e-12     # one RK step, relative to max |state|
TRAJ_TOL = 1e-10     # fixed-schedule trajectory, relative


def sim_for(g, **kw):
    return D.Simulation(grid_from(g, D.Grid), model_from(g, D.Model), **kw)


def port_for(g, search_mode=1):
    return O.Port(grid_from(g, O.Grid), model_from(g, O.Model), search_mode=search_mode, threads=4)


@pytest.mark.parametrize("L", SIZES)
def test_interpolation_bit_exact(product_built, L):
    g = load_golden(L)
    s = sim_for(g)
    s.upload(state_from(g, "mid", D.State))
    s.interpolate()
    for w in range(16):
        if w == 10:
            continue  # SigmaKA2: the reference CPU interpolate leaves it unset
        np.testing.assert_array_equal(s.interp(w), g[f"mid_interp{w}"], err_msg=f"interp {w}")
    np.testing.assert_array_equal(s.interp(16), g["mid_interp16"], err_msg="rInt")
    # positions: bit-identical to the reference's bsearchPosSorted
    p = port_for(g, search_mode=0)
    p.set_state(state_from(g, "mid", O.State))
    p.interpolate()
    np.testing.assert_array_equal(s.interp(17), p.interp(17))
    np.testing.assert_array_equal(s.interp(18), p.interp(18))


@pytest.mark.parametrize("L", SIZES)
def test_rhs_and_scalars_bit_exact(product_built, L):
    g = load_golden(L)
    s = sim_for(g)
    st = state_from(g, "mid", D.State)
    s.upload(st)
    s.interpolate()
    hK, hR = s.QKRstep()
    np.testing.assert_array_equal(hK, g["mid_qk"])
    np.testing.assert_array_equal(hR, g["mid_qr"])
    assert s.rstep() == g["mid_rstep"][0]
    n = st.n
    qK, qR = st.QK[(n - 1) * L:], st.QR[(n - 1) * L:]
    assert s.drstep2(qK, qR, hK, hR, st.t1grid[-1]) == g["mid_drstep2"][0]
    assert s.energy() == g["mid_energy"][0]


@pytest.mark.parametrize("L", SIZES)
def test_fused_rhs(product_built, L):
    g = load_golden(L)
    s = sim_for(g)
    s.upload(state_from(g, "mid", D.State))
    hK, hR = s.rhs()
    assert rel_err(hK, g["mid_qk"]) < RHS_TOL
    assert rel_err(hR, g["mid_qr"]) < RHS_TOL


@pytest.mark.parametrize("L", SIZES)
def test_fused_rhs_at_t0(product_built, L):
    g = load_golden(L)
    s = sim_for(g)
    s.init()
    hK, hR = s.rhs()
    assert rel_err(hK, g["t0_qk"]) < RHS_TOL
    assert rel_err(hR, g["t0_qr"]) < RHS_TOL
    st = s.download()
    for k in STATE_FIELDS:
        np.testing.assert_array_equal(getattr(st, k), g[f"t0_{k}"], err_msg=k)


@pytest.mark.parametrize("L", SIZES)
@pytest.mark.parametrize("tag,method", [("rk54", 1), ("ssp", 2)])
@pytest.mark.parametrize("graph", [False, True])
def test_single_step(product_built, L, tag, method, graph):
    g = load_golden(L)
    s = sim_for(g, use_graph=graph)
    dt = float(g[f"{tag}_dt"][0])
    for _ in range(2 if graph else 1):  # second pass replays the captured graph
        s.upload(state_from(g, "mid", D.State))
        r = s.update(method, dt)
    st = s.download()
    n = st.n
    for k in ("QK", "QR", "dQK", "dQR"):
        assert rel_err(getattr(st, k), g[f"{tag}_{k}"]) < STEP_TOL, k
    np.testing.assert_array_equal(st.t1grid, g[f"{tag}_t1grid"])
    np.testing.assert_array_equal(st.dtr, g[f"{tag}_dtr"])
    assert rel_err(st.rvec, g[f"{tag}_rvec"]) < STEP_TOL
    assert rel_err(st.drvec, g[f"{tag}_drvec"]) < 1e-11
    assert abs(r.delta - g[f"{tag}_err"][0]) < 5e-14  # error estimate is itself ~1e-14
    assert r.t == g[f"{tag}_t1grid"][-1]
    assert r.qk0 == st.QK[(n - 1) * L]


@pytest.mark.parametrize("L", SIZES)
def test_trajectory_fixed_schedule(product_built, L):
    """Replay the reference run's step sizes and methods from t = 0."""
    g = load_golden(L)
    s = sim_for(g)
    s.init()
    sched = (g["traj_dt"], g["traj_method"])
    tr = s.run(g["traj_dt"].size, schedule=sched)
    st = s.download()
    np.testing.assert_array_equal(st.t1grid, g["traj_final_t1grid"])
    for k in ("QK", "QR", "dQK", "dQR", "rvec"):
        assert rel_err(getattr(st, k), g[f"traj_final_{k}"]) < TRAJ_TOL, k
    assert rel_err(tr["energy"], g["traj_energy"]) < TRAJ_TOL
    np.testing.assert_array_equal(tr["t"], g["traj_t"])


@pytest.mark.parametrize("L", SIZES)
def test_trajectory_free_controller(product_built, L):
    """With its own controller the GPU run makes the reference's decisions
    except where the error estimate sits within rounding of a threshold."""
    g = load_golden(L)
    s = sim_for(g)
    s.init()
    tr = s.run(g["traj_dt"].size)
    same = tr["dt"] == g["traj_dt"]
    if not same.all():
        k = int(np.argmin(same))
        d = g["traj_delta"][k - 1]
        dmax = float(g["model"][6])
        near = min(abs(d - dmax), abs(d - 2 * dmax), abs(d - 1.1 * g["traj_delta"][k - 2])) / dmax
        assert near < 1e-3, f"schedules diverge at step {k} away from a threshold"
    else:
        st = s.download()
        assert rel_err(st.QK, g["traj_final_QK"]) < TRAJ_TOL


@pytest.mark.parametrize("q", [2, 4])
def test_serk2_step(product_built, q):
    g = load_golden(32)
    s = sim_for(g)
    p = port_for(g, search_mode=1)
    st = state_from(g, "mid", D.State)
    s.upload(st)
    p.set_state(state_from(g, "mid", O.State))
    dt = 4 * float(g["rk54_dt"][0])
    r = s.SERK2(q, dt)
    e = p.update(D.serk2_method(q), dt)
    a, b = s.download(), p.get_state()
    np.testing.assert_array_equal(a.t1grid, b.t1grid)
    for k in ("QK", "QR", "dQK", "dQR", "rvec", "drvec"):
        assert rel_err(getattr(a, k), getattr(b, k)) < STEP_TOL, k
    assert abs(r.delta - e) < 5e-14


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("L", SIZES)
def test_sparsify_keep_lists_exact(product_built, L, variant):
    g = load_golden(L)
    s = sim_for(g)
    p = port_for(g)
    thr = float(g["spars_threshold"][0])
    s.upload(state_from(g, "traj_final", D.State))
    p.set_state(state_from(g, "traj_final", O.State))
    n_gpu = s.sparsifyNscale(thr, ["cpu", "cuda_host", "gpu"][variant])
    n_port, _ = p.sparsify(thr, variant)
    assert n_gpu == n_port
    a, b = s.download(), p.get_state()
    for k in STATE_FIELDS:
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k), err_msg=k)
    if variant == 0:
        for k in STATE_FIELDS:
            np.testing.assert_array_equal(getattr(a, k), g[f"spars_{k}"], err_msg=k)


def test_sparsify_then_step(product_built):
    g = load_golden(32)
    s = sim_for(g)
    p = port_for(g)
    thr = float(g["spars_threshold"][0])
    s.upload(state_from(g, "traj_final", D.State))
    p.set_state(state_from(g, "traj_final", O.State))
    s.sparsifyNscale(thr, "gpu")
    p.sparsify(thr, 2)
    p.interpolate()
    dt = float(g["traj_dt"][-1])
    s.update(1, dt)
    p.update(1, dt)
    a, b = s.download(), p.get_state()
    assert rel_err(a.QK, b.QK) < STEP_TOL


def test_rollback(product_built):
    g = load_golden(32)
    s = sim_for(g)
    s.upload(state_from(g, "traj_final", D.State))
    n = s.n
    s.rollbackState(5)
    assert s.n == n - 5
    st = s.download()
    np.testing.assert_array_equal(st.t1grid, g["traj_final_t1grid"][: n - 5])
    c = s.controller
    assert c["delta_t"] == st.t1grid[-1] - st.t1grid[-2]


@pytest.mark.parametrize("L", [128, 512])
def test_fixed_schedule_large_grid(product_built, L):
    """Production-sized grids (poly-9, Tmax 1e5): GPU vs the oracle (binary
    search, the CUDA path's positions) over a short run from t = 0."""
    grid = D.grid.generate(L)
    m = D.Model(p=3, p2=4, lam=0.5, Gamma=0.6)
    s = D.Simulation(grid, m)
    s.init()
    steps = 12 if L == 512 else 40
    tr = s.run(steps)
    og = O.Grid(L, grid.theta, grid.phi1, grid.phi2, grid.integ, grid.indsA1, grid.wA1, grid.indsA2, grid.wA2,
                grid.indsB2, grid.wB2)
    p = O.Port(og, O.Model(p=3, p2=4, lam=0.5, Gamma=0.6), search_mode=1, threads=0)
    p.init_state()
    tp = p.run(steps, schedule=(tr["dt"], tr["method"]))
    a, b = s.download(), p.get_state()
    np.testing.assert_array_equal(a.t1grid, b.t1grid)
    for k in ("QK", "QR", "rvec"):
        assert rel_err(getattr(a, k), getattr(b, k)) < TRAJ_TOL, k
    assert rel_err(tr["energy"], tp["energy"]) < TRAJ_TOL


def test_polynomial_history_is_reproduced(product_built):
    """Size-independent property at L=512: the poly-9 A1/A2 stencils are exact
    for polynomials of degree <= 9 in theta, so a last history row C = P(theta)
    is gathered to P(phi1) and P(phi2) (the reference's own stencil invariant,
    src/grid/test_interpolation_weights.cpp:36-66)."""
    L = 512
    grid = D.grid.generate(L)
    s = D.Simulation(grid, D.Model())
    th = grid.theta
    P = lambda x: 0.3 + 0.2 * x - 0.1 * x ** 3 + 0.05 * x ** 7
    Q = lambda x: 1.0 - 0.4 * x ** 2 + 0.01 * x ** 9
    n = 3
    t = np.array([0.0, 0.5, 1.0])
    st = D.State(t, np.array([0.0, 0.0, 1.0]), np.tile(P(th), n), np.tile(Q(th), n), np.zeros(n * L),
                 np.zeros(n * L), np.full(n, 0.6), np.zeros(n))
    s.upload(st)
    s.interpolate()
    assert np.max(np.abs(s.interp(0) - P(grid.phi1))) < 1e-12
    assert np.max(np.abs(s.interp(1) - Q(grid.phi1))) < 1e-12
    assert np.max(np.abs(s.interp(2) - P(grid.phi2))) < 1e-12
    assert np.max(np.abs(s.interp(3) - Q(grid.phi2))) < 1e-12


def _spars_model(g, M):
    """The golden model with a delta_max at which sparsify drops rows of a short run."""
    kw = dict(vars(model_from(g, M)))
    kw["delta_max"] = 1e-7
    return M(**kw)


@pytest.mark.parametrize("variant", [0, 2])
def test_periodic_sparsify_fixed_schedule(product_built, variant):
    """dyn_run's periodic block (simulation_runner.cpp:148-237) against the oracle: the
    oracle runs its own controller with a sparsify every 20 loops, the GPU replays
    that schedule with the same cadence; time grids and keep decisions bit-exact."""
    g = load_golden(32)
    p = O.Port(grid_from(g, O.Grid), _spars_model(g, O.Model), search_mode=1, threads=4)
    p.init_state()
    tr = p.run(70, sparsify_every=20, sparsify_variant=variant)
    s = D.Simulation(grid_from(g, D.Grid), _spars_model(g, D.Model))
    s.init()
    tg = s.run(70, schedule=(tr["dt"], tr["method"]), sparsify_every=20,
               sparsify_variant=["cpu", "cuda_host", "gpu"][variant])
    a, b = s.download(), p.get_state()
    assert a.t1grid.size < 71
    np.testing.assert_array_equal(a.t1grid, b.t1grid)
    np.testing.assert_array_equal(a.dtr, b.dtr)
    for k in ("QK", "QR", "dQK", "dQR", "rvec", "drvec"):
        assert rel_err(getattr(a, k), getattr(b, k)) < TRAJ_TOL, k
    assert rel_err(tg["energy"], tr["energy"]) < TRAJ_TOL


def test_periodic_sparsify_free_controller(product_built):
    """A free run with the cadence (sparsify, then the step-halving rule, then the
    usual adaptation) makes the oracle's decisions, except where an error estimate
    sits within rounding of a threshold."""
    g = load_golden(32)
    p = O.Port(grid_from(g, O.Grid), _spars_model(g, O.Model), search_mode=1, threads=4)
    p.init_state()
    tr = p.run(70, sparsify_every=20, sparsify_variant=2)
    s = D.Simulation(grid_from(g, D.Grid), _spars_model(g, D.Model))
    s.init()
    tg = s.run(70, sparsify_every=20, sparsify_variant="gpu")
    same = (tg["dt"] == tr["dt"]) & (tg["method"] == tr["method"])
    if not same.all():
        k = int(np.argmin(same))
        d, dmax = tr["delta"][k - 1], 1e-7
        near = min(abs(d - dmax), abs(d - 2 * dmax), abs(d - dmax / 2), abs(d - 1.1 * tr["delta"][k - 2])) / dmax
        assert near < 1e-3, f"schedules diverge at step {k} away from a threshold"
    else:
        a, b = s.download(), p.get_state()
        np.testing.assert_array_equal(a.t1grid, b.t1grid)
        assert rel_err(a.QK, b.QK) < TRAJ_TOL
        c = s.controller
        assert (c["delta_t"], c["method"]) == p.controller()


def test_periodic_block_sweep_counts(product_built):
    """sparsify_sweeps (simulation_runner.cpp:163-187): 0 runs the block without a
    pass (no row dropped, the step still halves), -1 ("auto", the reference's
    default) is one pass on a device less than half full."""
    g = load_golden(32)
    p = O.Port(grid_from(g, O.Grid), _spars_model(g, O.Model), search_mode=1, threads=4)
    p.init_state()
    tr = p.run(70, sparsify_every=20, sparsify_sweeps=0)
    assert p.get_state().t1grid.size == 71 and tr["dt"][20] == 0.5 * tr["dt"][19]
    s = D.Simulation(grid_from(g, D.Grid), _spars_model(g, D.Model))
    s.init()
    tg = s.run(70, sparsify_every=20, sparsify_sweeps=0)
    np.testing.assert_array_equal(tg["dt"], tr["dt"])
    np.testing.assert_array_equal(s.download().t1grid, p.get_state().t1grid)
    runs = []
    for sweeps in (-1, 1):
        s = D.Simulation(grid_from(g, D.Grid), _spars_model(g, D.Model))
        s.init()
        s.run(70, sparsify_every=20, sparsify_sweeps=sweeps)
        runs.append(s.download())
    assert runs[0].t1grid.size < 71
    np.testing.assert_array_equal(runs[0].t1grid, runs[1].t1grid)
    np.testing.assert_array_equal(runs[0].QK, runs[1].QK)


def test_periodic_sparsify_serk2_climb(product_built):
    """use_serk2 (the reference's default on its GPU loop, simulation_runner.cpp:222-229):
    every periodic halving moves a method past RK54 one SERK2 level up.  The free GPU
    run makes the oracle's method and step choices, except where an error estimate
    sits within rounding of a threshold."""
    g = load_golden(32)
    p = O.Port(grid_from(g, O.Grid), _spars_model(g, O.Model), search_mode=1, threads=4)
    p.init_state()
    tr = p.run(100, sparsify_every=20, sparsify_variant=2, use_serk2=True)
    assert tr["method"].max() >= 4  # SSPRK(10,4) -> SERK2(2) -> SERK2(4) ...
    s = D.Simulation(grid_from(g, D.Grid), _spars_model(g, D.Model))
    s.init()
    tg = s.run(100, sparsify_every=20, sparsify_variant="gpu", use_serk2=True)
    same = (tg["dt"] == tr["dt"]) & (tg["method"] == tr["method"])
    if not same.all():
        k = int(np.argmin(same))
        d, dmax = tr["delta"][k - 1], 1e-7
        near = min(abs(d - dmax), abs(d - 2 * dmax), abs(d - dmax / 2), abs(d - 1.1 * tr["delta"][k - 2])) / dmax
        assert near < 1e-3, f"schedules diverge at step {k} away from a threshold"
    else:
        a, b = s.download(), p.get_state()
        np.testing.assert_array_equal(a.t1grid, b.t1grid)
        assert rel_err(a.QK, b.QK) < TRAJ_TOL
        assert (s.controller["delta_t"], s.controller["method"]) == p.controller()


def test_checkpoint_resume_continues_bit_for_bit(product_built, tmp_path):
    """A run saved to RG-Evo's data.bin and loaded into a fresh context continues exactly
    as the original (the loader's delta_t_ratio rebuild leaves the rows the stencils use
    unchanged)."""
    from dynamite_gb300 import checkpoint as ck
    g = load_golden(32)
    a = sim_for(g)
    a.init()
    a.run(40)
    c = a.controller
    st = a.download()
    m = model_from(g, D.Model)
    path = str(tmp_path / "data.bin")
    ck.save(path, st, ck.CheckpointParams(m.p, m.p2, m.lam, m.T0, m.Gamma, c["delta"], c["delta_t"], c["loop"],
                                          a.energy()))
    back, prm = ck.load(path)
    np.testing.assert_array_equal(back.dtr[2:], st.dtr[2:])
    b = sim_for(g)
    b.upload(back)
    b.set_controller(prm.delta_t, c["method"], prm.delta, c["delta_old"], prm.loop)
    ta, tb = a.run(15), b.run(15)
    np.testing.assert_array_equal(ta["dt"], tb["dt"])
    sa, sb = a.download(), b.download()
    for k in ("t1grid", "QK", "QR", "dQK", "dQR", "rvec", "drvec"):
        np.testing.assert_array_equal(getattr(sa, k), getattr(sb, k), err_msg=k)


@pytest.mark.parametrize("L", SIZES)
def test_compressed_outputs_hold_the_reference_b1_interpolation(product_built, L, tmp_path):
    """A save's QK_compressed / QR_compressed of the mid state: the reference's own
    B1 arrays at fresh positions, bit for bit."""
    from dynamite_gb300 import checkpoint as ck
    g = load_golden(L)
    s = sim_for(g)
    s.upload(state_from(g, "mid", D.State))
    s.save_compressed(str(tmp_path))
    qk, qr, t = ck.load_compressed(str(tmp_path))
    np.testing.assert_array_equal(qk.ravel(), g["mid_interp4"])
    np.testing.assert_array_equal(qr.ravel(), g["mid_interp5"])
    np.testing.assert_array_equal(t, np.array([float(f"{x:.16f}") for x in g["mid_t1grid"][-1] * g["grid_theta"]]))
    assert s.t == g["mid_t1grid"][-1]


def test_energy_history_as_the_reference_saves_it(product_built):
    """computeEnergyHistoryKernel (io_output.cu:61-122) restated in numpy: E_k = -t_k (sum_j
    w_j f'(QK[k,j]) QR[k,j] + f'(QK[k,0]) / T0) over every row of a mid-run history."""
    g = load_golden(32)
    s = sim_for(g)
    st = state_from(g, "traj_final", D.State)
    s.upload(st)
    e = s.energy_history()
    m = model_from(g, D.Model)
    L = 32
    QK, QR = st.QK.reshape(-1, L), st.QR.reshape(-1, L)
    fp = lambda q: m.lam * m.p * q ** (m.p - 1) + (1 - m.lam) * m.p2 * q ** (m.p2 - 1)
    w = g["grid_integ"]
    ref = -st.t1grid * ((fp(QK) * QR * w[None, :]).sum(axis=1) + fp(QK[:, 0]) / m.T0)
    assert e.shape == ref.shape
    assert np.max(np.abs(e - ref)) <= 1e-13 * np.max(np.abs(ref))
