"""dyn_rhs_noalloc: the fused right-hand side for callers that cannot
allocate device memory (they own every buffer; the kernels' scratch is a
fixed device array inside the library).  Checked through the C ABI against
the existing dyn_rhs entry point on two different states, two calls in a
row, so the second call also shows that the shared scratch carries nothing
over from the first.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import dynamite_gb300 as D
from dynamite_gb300 import _lib
from conftest import load_golden
from helpers import grid_from, model_from, rel_err, state_from

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12  # same bar as the fused-RHS parity tests


def _device(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _args(torch, grid, model, st, out, keep):
    L, n = grid.L, st.n
    f64, i32 = torch.float64, torch.int32
    bufs = dict(
        theta=_device(torch, grid.theta, f64), phi2=_device(torch, grid.phi2, f64),
        integ=_device(torch, grid.integ, f64),
        indsA1y=_device(torch, grid.indsA1, i32), indsA2y=_device(torch, grid.indsA2, i32),
        indsB2y=_device(torch, grid.indsB2, i32),
        weightsA1y=_device(torch, grid.wA1, f64), weightsA2y=_device(torch, grid.wA2, f64),
        weightsB2y=_device(torch, grid.wB2, f64),
        KR=_device(torch, np.stack([st.QK, st.QR], axis=-1), f64),
        dKR=_device(torch, np.stack([st.dQK, st.dQR], axis=-1), f64),
        t1grid=_device(torch, st.t1grid, f64), delta_t_ratio=_device(torch, st.dtr, f64),
        rvec=_device(torch, st.rvec, f64), drvec=_device(torch, st.drvec, f64),
    )
    keep.append(bufs)
    a = _lib.NoAllocRHS(model.p, model.p2, model.lam, model.T0, model.Gamma, L, grid.depth, n, 0)
    for k, v in bufs.items():
        setattr(a, k, v.data_ptr())
    a.out = out.data_ptr()
    return a


def _check(torch, grid, model, st, hK, hR, keep, what):
    out = torch.empty((grid.L, 2), dtype=torch.float64, device="cuda")
    out.fill_(float("nan"))
    args = _args(torch, grid, model, st, out, keep)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.lib().dyn_rhs_noalloc(C.byref(args), stream), "dyn_rhs_noalloc")
    torch.cuda.synchronize()
    res = out.cpu().numpy()
    assert np.isfinite(res).all(), what
    assert rel_err(res[:, 0], hK) < RHS_TOL, what
    assert rel_err(res[:, 1], hR) < RHS_TOL, what


def test_rhs_noalloc_matches_rhs_on_two_calls():
    torch = pytest.importorskip("torch")
    g = load_golden(64)
    grid, model = grid_from(g, D.Grid), model_from(g, D.Model)
    sim = D.Simulation(grid, model)
    out = torch.empty((grid.L, 2), dtype=torch.float64, device="cuda")
    keep = []
    for prefix in ("mid", "traj_final"):
        st = state_from(g, prefix, D.State)
        sim.upload(st)
        hK, hR = sim.rhs()
        out.fill_(float("nan"))
        args = _args(torch, grid, model, st, out, keep)
        stream = torch.cuda.current_stream().cuda_stream
        status = _lib.lib().dyn_rhs_noalloc(C.byref(args), stream)
        _lib.check(status, "dyn_rhs_noalloc")
        torch.cuda.synchronize()
        res = out.cpu().numpy()
        assert np.isfinite(res).all()
        assert rel_err(res[:, 0], hK) < RHS_TOL, prefix
        assert rel_err(res[:, 1], hR) < RHS_TOL, prefix
        if prefix == "mid":
            # and the reference's own QKstep/QRstep of that state (the golden fixture)
            assert rel_err(res[:, 0], g["mid_qk"]) < RHS_TOL
            assert rel_err(res[:, 1], g["mid_qr"]) < RHS_TOL


@pytest.mark.parametrize("L", [512, 1024])
def test_rhs_noalloc_at_production_sizes(L):
    """The scratch layout at the sizes it is sized for: L = 512 (4 targets per thread,
    2 chunks per row) and L = 1024 (the largest length, 4 chunks per row), on a state
    of 40 steps from t = 0 on the poly-9 grid, two calls in a row, against dyn_rhs."""
    torch = pytest.importorskip("torch")
    grid = D.grid.generate(L)
    model = D.Model(p=3, p2=4, lam=0.5, Gamma=0.6)
    sim = D.Simulation(grid, model)
    sim.init()
    sim.run(40)
    st = sim.download()
    hK, hR = sim.rhs()
    keep = []
    for call in range(2):
        _check(torch, grid, model, st, hK, hR, keep, f"L={L} call {call}")
    sim.close()


def test_rhs_noalloc_rejects_sizes_beyond_its_scratch():
    a = _lib.NoAllocRHS(3, 4, 0.5, 1e50, 0.6, 2048, 10, 10, 0)
    assert _lib.lib().dyn_rhs_noalloc(C.byref(a), None) == -1
    assert b"DYN_NOALLOC_MAX_LEN" in _lib.lib().dyn_last_error()
    b = _lib.NoAllocRHS(3, 4, 0.5, 1e50, 0.6, 64, 10, 20000, 0)
    assert _lib.lib().dyn_rhs_noalloc(C.byref(b), None) == -1
    assert b"DYN_NOALLOC_MAX_ROWS" in _lib.lib().dyn_last_error()
    # a one-row history (its B1/B2 clamps would point at row 1) and an unknown search
    c = _lib.NoAllocRHS(3, 4, 0.5, 1e50, 0.6, 64, 10, 1, 0)
    assert _lib.lib().dyn_rhs_noalloc(C.byref(c), None) == -1
    assert b"rows" in _lib.lib().dyn_last_error()
    d = _lib.NoAllocRHS(3, 4, 0.5, 1e50, 0.6, 64, 10, 10, 2)
    assert _lib.lib().dyn_rhs_noalloc(C.byref(d), None) == -1
    assert b"search" in _lib.lib().dyn_last_error()
