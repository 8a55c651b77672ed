"""The device-resident state exchange of the RG-Evo drop-in layer (GPU).

dynamite_gb300/shim/rgevo_shim.cu keeps RG-Evo's thrust vectors (separate n x len
arrays QKv, QRv, dQKv, dQRv and the n-vectors t1grid, delta_t_ratio, rvec, drvec) as the
driver's record and moves state with dyn_state_upload_dev, dyn_state_rows_load_dev,
dyn_state_rows_store_dev, dyn_get_interp_dev and dyn_interp_b1_dev.  Here torch device
tensors stand in for those vectors and the layer's protocol runs step by step:

* every step re-loads the newest row, steps, grows the arrays by one row and stores it
  (updateGPU); the arrays then hold exactly the history dyn_run builds on the same
  schedule, bit for bit;
* shrinking the arrays by hand and re-uploading them (what rollbackState does to the
  vectors) continues exactly as dyn_rollback does;
* the interpolation arrays and the B1 pair copied device to device equal the host
  copies of dyn_get_interp bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

import dynamite_gb300 as D
from dynamite_gb300 import _lib
from conftest import load_golden
from helpers import grid_from, model_from, state_from

pytestmark = pytest.mark.gpu

FIELDS = ("t1grid", "dtr", "QK", "QR", "dQK", "dQR", "rvec", "drvec")


class SimArrays:
    """RG-Evo's d_* vectors, as torch tensors that grow by whole rows."""

    def __init__(self, torch, st, L):
        self.torch, self.L = torch, L
        self.a = {f: torch.as_tensor(np.ascontiguousarray(getattr(st, f)), dtype=torch.float64, device="cuda").clone()
                  for f in FIELDS}

    @property
    def n(self):
        return self.a["t1grid"].numel()

    def resize(self, n):
        for f in FIELDS:
            per = self.L if f in ("QK", "QR", "dQK", "dQR") else 1
            t = self.a[f]
            if n * per <= t.numel():
                self.a[f] = t[: n * per].clone()
            else:
                self.a[f] = self.torch.cat([t, self.torch.zeros(n * per - t.numel(), dtype=t.dtype, device=t.device)])

    def dev(self):
        a = self.a
        return _lib.StateDev(self.n, a["t1grid"].data_ptr(), a["dtr"].data_ptr(), a["QK"].data_ptr(),
                             a["QR"].data_ptr(), a["dQK"].data_ptr(), a["dQR"].data_ptr(), a["rvec"].data_ptr(),
                             a["drvec"].data_ptr())

    def host(self):
        return {f: self.a[f].cpu().numpy() for f in FIELDS}


def _step(lib, h, sim, method, dt):
    """The layer's updateGPU: newest row re-loaded, one step, the new row stored, the B1
    pair refreshed for the driver's saves."""
    st = sim.dev()
    _lib.check(lib.dyn_state_rows_load_dev(h, sim.n - 1, 1, C.byref(st)), "rows_load_dev")
    r = _lib.StepResult()
    _lib.check(lib.dyn_update(h, method, dt, C.byref(r)), "dyn_update")
    sim.resize(sim.n + 1)
    st = sim.dev()
    _lib.check(lib.dyn_state_rows_store_dev(h, sim.n - 1, 1, C.byref(st)), "rows_store_dev")
    b1 = sim.torch.empty(2 * sim.L * sim.L, dtype=sim.torch.float64, device="cuda")
    _lib.check(lib.dyn_interp_b1_dev(h, b1.data_ptr(), b1[sim.L * sim.L:].data_ptr()), "dyn_interp_b1_dev")
    return r.delta


def test_dropin_protocol_reproduces_dyn_run(product_built):
    torch = pytest.importorskip("torch")
    g = load_golden(32)
    grid, model = grid_from(g, D.Grid), model_from(g, D.Model)
    L = grid.L
    start = state_from(g, "mid", D.State)
    ref = D.Simulation(grid, model)
    ref.upload(start)
    ref.set_controller(float(g["rk54_dt"][0]), 1)
    tr = ref.run(12)
    a = ref.download()

    lay = D.Simulation(grid, model)
    sim = SimArrays(torch, start, L)
    lib = _lib.lib()
    st = sim.dev()
    _lib.check(lib.dyn_state_upload_dev(lay._h, C.byref(st)), "dyn_state_upload_dev")
    deltas = [_step(lib, lay._h, sim, int(m), float(dt)) for dt, m in zip(tr["dt"], tr["method"])]
    np.testing.assert_array_equal(np.array(deltas), tr["delta"])
    b = sim.host()
    for f in FIELDS:
        np.testing.assert_array_equal(b[f], getattr(a, f), err_msg=f)

    # rollbackState shrinks the vectors; the layer re-uploads them and goes on as dyn_rollback does
    sim.resize(sim.n - 5)
    st = sim.dev()
    _lib.check(lib.dyn_state_upload_dev(lay._h, C.byref(st)), "dyn_state_upload_dev")
    ref.rollbackState(5)
    dt = float(tr["dt"][-1])
    for _ in range(3):
        _step(lib, lay._h, sim, 1, dt)
    ref.run(3, schedule=(np.full(3, dt), np.ones(3, dtype=np.int32)))
    a, b = ref.download(), sim.host()
    for f in FIELDS:
        np.testing.assert_array_equal(b[f], getattr(a, f), err_msg=f)
    ref.close()
    lay.close()


def test_interpolation_arrays_device_to_device(product_built):
    torch = pytest.importorskip("torch")
    g = load_golden(64)
    grid, model = grid_from(g, D.Grid), model_from(g, D.Model)
    L = grid.L
    s = D.Simulation(grid, model)
    s.upload(state_from(g, "mid", D.State))
    lib = _lib.lib()
    qk = torch.empty(L * L, dtype=torch.float64, device="cuda")
    qr = torch.empty(L * L, dtype=torch.float64, device="cuda")
    # the B1 pair alone (what the layer refreshes after each step) ...
    _lib.check(lib.dyn_interp_b1_dev(s._h, qk.data_ptr(), qr.data_ptr()), "dyn_interp_b1_dev")
    b1 = (qk.cpu().numpy(), qr.cpu().numpy())
    # ... equals the reference-order interpolation's B1 arrays and the golden fixture
    s.interpolate()
    np.testing.assert_array_equal(b1[0], s.interp(4))
    np.testing.assert_array_equal(b1[1], s.interp(5))
    np.testing.assert_array_equal(b1[0], g["mid_interp4"])
    out = torch.empty(L * L, dtype=torch.float64, device="cuda")
    for w in (0, 3, 6, 7, 9, 15, 18):
        _lib.check(lib.dyn_get_interp_dev(s._h, w, out.data_ptr()), "dyn_get_interp_dev")
        np.testing.assert_array_equal(out.cpu().numpy(), s.interp(w), err_msg=str(w))
    s.close()
