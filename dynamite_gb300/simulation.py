"""The reference's hot-path interface, on the GB300 path.

`Simulation` owns one native context (include/dyn.h) and exposes the
reference's operations under their reference names:

=====================  =====================================================
reference (file:line)  here
=====================  =====================================================
interpolateGPU         Simulation.interpolate (interpolation_core.cu:63-159)
QKstep / QRstep        Simulation.QKstep / QRstep (time_steps.cpp:27-100)
QKRstepGPU             Simulation.QKRstep (time_steps.cu:327-408)
rstepGPU               Simulation.rstep (time_steps.cu:410-472)
drstep2GPU             Simulation.drstep2 (time_steps.cu:564-639)
energyGPU              Simulation.energy (time_steps.cu:641-674)
updateGPU / update     Simulation.update (runge_kutta.cu:607-615)
RK54GPU / SSPRK104GPU  Simulation.RK54 / SSPRK104 / SERK2
sparsifyNscaleGPU      Simulation.sparsifyNscale (sparsify_utils.cu:199-290)
rollbackState          Simulation.rollbackState (simulation_control.cpp:14)
runSimulation loop     Simulation.run (simulation_runner.cpp:125-304)
tailFitBlendCPU/GPU    Simulation.tail_fit (tail_fit.cpp:46-262)
-R (log response)      Simulation(..., log_response=True) (index_vec.cpp:24-131)
computeEnergyHistory   Simulation.energy_history (io_output.cu:61-122)
saveCompressedData     Simulation.save_compressed (io_save_compressed.cpp:17-63)
=====================  =====================================================

Every numeric call goes to the CUDA library; nothing here computes on the
CPU beyond argument marshalling.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .grid import Grid

METHODS = {"RK54": 1, "SSPRK104": 2}
SPARSIFY = {"cpu": 0, "cuda_host": 1, "gpu": 2}
SEARCH = {"binary": 0, "lower_bound": 1}


@dataclass
class Model:
    """f(q) = lam q^p + (1-lam) q^p2 (math_ops.cpp:23-37), bath Gamma, start T0."""

    p: int = 3
    p2: int = 4
    lam: float = 0.5
    T0: float = 1e50
    Gamma: float = 0.6
    delta_t_min: float = 1e-5
    delta_max: float = 1e-10


@dataclass
class State:
    t1grid: np.ndarray
    dtr: np.ndarray
    QK: np.ndarray
    QR: np.ndarray
    dQK: np.ndarray
    dQR: np.ndarray
    rvec: np.ndarray
    drvec: np.ndarray
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.t1grid.size)


@dataclass
class StepResult:
    delta: float
    t: float
    r: float
    energy: float
    qk0: float
    dr: float


def serk2_method(q: int) -> int:
    """rk->init value of SERK2(q) (runge_kutta.cu:274-297: init = 2 + q/2)."""
    return 2 + q // 2


class Simulation:
    def __init__(self, grid: Grid, model: Model, precision: str = "fp64", search: str = "binary",
                 device: int = 0, use_graph: bool = True, history_capacity: int = 0, stream: int | None = None,
                 log_response: bool = False):
        self.grid = grid
        self.model = model
        self.L = grid.L
        self._h = C.c_void_p()
        cfg = _lib.Config(model.p, model.p2, model.lam, model.T0, model.Gamma, grid.L, grid.depth,
                          model.delta_t_min, model.delta_max, {"fp64": 0, "mixed": 1, "mixed_df": 2}[precision],
                          SEARCH[search], history_capacity, device, stream, int(use_graph), int(log_response))
        self._keep = [np.ascontiguousarray(a) for a in (grid.theta, grid.phi2, grid.integ)]
        i64 = [np.ascontiguousarray(a, dtype=np.int64) for a in (grid.indsA1, grid.indsA2, grid.indsB2)]
        w = [np.ascontiguousarray(a, dtype=np.float64) for a in (grid.wA1, grid.wA2, grid.wB2)]
        tb = _lib.Tables(_lib.ptr(self._keep[0]), _lib.ptr(self._keep[1]), _lib.ptr(self._keep[2]),
                         *[a.ctypes.data_as(_lib.i64p) for a in i64], *[_lib.ptr(a) for a in w])
        _lib.check(_lib.lib().dyn_ctx_create(C.byref(cfg), C.byref(tb), C.byref(self._h)), "dyn_ctx_create")

    # ---------------------------------------------------------------- state
    def close(self):
        if self._h:
            _lib.lib().dyn_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def init(self, delta_t: float = 0.0):
        """t = 0 state (initialization.cpp:204-222)."""
        _lib.check(_lib.lib().dyn_state_init(self._h, delta_t), "dyn_state_init")

    @property
    def n(self) -> int:
        v = C.c_size_t()
        _lib.check(_lib.lib().dyn_state_rows(self._h, C.byref(v)), "dyn_state_rows")
        return int(v.value)

    def upload(self, st) -> None:
        a = [np.ascontiguousarray(getattr(st, f), dtype=np.float64)
             for f in ("t1grid", "dtr", "QK", "QR", "dQK", "dQR", "rvec", "drvec")]
        sc = _lib.StateC(a[0].size, *[_lib.ptr(x) for x in a])
        _lib.check(_lib.lib().dyn_state_upload(self._h, C.byref(sc)), "dyn_state_upload")

    def download(self) -> State:
        n, L = self.n, self.L
        arrs = [np.empty(n), np.empty(n), np.empty(n * L), np.empty(n * L), np.empty(n * L), np.empty(n * L),
                np.empty(n), np.empty(n)]
        sc = _lib.StateC(n, *[_lib.ptr(x) for x in arrs])
        _lib.check(_lib.lib().dyn_state_download(self._h, C.byref(sc)), "dyn_state_download")
        return State(*arrs)

    @property
    def controller(self) -> dict:
        c = _lib.Controller()
        _lib.check(_lib.lib().dyn_controller_get(self._h, C.byref(c)), "dyn_controller_get")
        return dict(delta_t=c.delta_t, delta=c.delta, delta_old=c.delta_old, loop=c.loop, method=c.method)

    def set_controller(self, delta_t: float, method: int, delta: float = 1.0, delta_old: float = 0.0, loop: int = 0):
        c = _lib.Controller(delta_t, delta, delta_old, loop, method)
        _lib.check(_lib.lib().dyn_controller_set(self._h, C.byref(c)), "dyn_controller_set")

    # ---------------------------------------------------------- hot path
    def interpolate(self, posB1x=None, posB2x=None) -> None:
        a = None if posB1x is None else np.ascontiguousarray(posB1x, dtype=np.float64)
        b = None if posB2x is None else np.ascontiguousarray(posB2x, dtype=np.float64)
        _lib.check(_lib.lib().dyn_interpolate(self._h, _lib.ptr(a), _lib.ptr(b)), "dyn_interpolate")

    def interp(self, which: int) -> np.ndarray:
        out = np.empty(self.L if which in (16, 17) else self.L * self.L)
        _lib.check(_lib.lib().dyn_get_interp(self._h, which, _lib.ptr(out)), "dyn_get_interp")
        return out

    def QKRstep(self):
        hK, hR = np.empty(self.L), np.empty(self.L)
        _lib.check(_lib.lib().dyn_qkr_step(self._h, _lib.ptr(hK), _lib.ptr(hR)), "dyn_qkr_step")
        return hK, hR

    def QKstep(self):
        return self.QKRstep()[0]

    def QRstep(self):
        return self.QKRstep()[1]

    def rhs(self):
        """Right-hand side of the current state by the fused stage kernels."""
        hK, hR = np.empty(self.L), np.empty(self.L)
        _lib.check(_lib.lib().dyn_rhs(self._h, _lib.ptr(hK), _lib.ptr(hR)), "dyn_rhs")
        return hK, hR

    def rstep(self) -> float:
        v = C.c_double()
        _lib.check(_lib.lib().dyn_rstep(self._h, C.byref(v)), "dyn_rstep")
        return v.value

    def drstep2(self, qK, qR, dqK, dqR, t: float) -> float:
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (qK, qR, dqK, dqR)]
        v = C.c_double()
        _lib.check(_lib.lib().dyn_drstep2(self._h, *[_lib.ptr(x) for x in a], t, C.byref(v)), "dyn_drstep2")
        return v.value

    def energy(self) -> float:
        v = C.c_double()
        _lib.check(_lib.lib().dyn_energy(self._h, C.byref(v)), "dyn_energy")
        return v.value

    def energy_history(self) -> np.ndarray:
        """E at every history row as RG-Evo writes it with a save (io_output.cu:61-122)."""
        out = np.empty(self.n)
        _lib.check(_lib.lib().dyn_energy_history(self._h, _lib.ptr(out), out.size), "dyn_energy_history")
        return out

    def save_compressed(self, dir_path: str) -> None:
        """The compressed outputs of a save (io_save_compressed.cpp:17-63): the B1
        interpolation QKB1/QRB1 of the current state (reference-order gathers at
        fresh positions, as the reference holds them after a step) and t theta."""
        from .checkpoint import save_compressed
        self.interpolate()
        save_compressed(dir_path, self.interp(4), self.interp(5), self.grid.theta, self.t)

    @property
    def t(self) -> float:
        """The current time (t1grid of the newest row)."""
        v = C.c_double()
        _lib.check(_lib.lib().dyn_state_time(self._h, C.byref(v)), "dyn_state_time")
        return v.value

    def tail_fit(self, last_rollback_loop: int = -1000) -> dict:
        """One QK tail fit of the newest row (tailFitBlendCPU, tail_fit.cpp:46-262);
        the window and the smoothed alpha carry over between calls."""
        info = _lib.TailInfo()
        _lib.check(_lib.lib().dyn_tail_fit(self._h, last_rollback_loop, C.byref(info)), "dyn_tail_fit")
        return dict(alpha_raw=info.alpha_raw, alpha=info.alpha, j0=info.j0, applied=bool(info.applied))

    def tail_fit_reset(self) -> None:
        _lib.check(_lib.lib().dyn_tail_fit_reset(self._h), "dyn_tail_fit_reset")

    def update(self, method: int | None = None, delta_t: float | None = None) -> StepResult:
        c = self.controller
        m = c["method"] if method is None else method
        dt = c["delta_t"] if delta_t is None else delta_t
        r = _lib.StepResult()
        _lib.check(_lib.lib().dyn_update(self._h, m, dt, C.byref(r)), "dyn_update")
        return StepResult(r.delta, r.t, r.r, r.energy, r.qk0, r.dr)

    def RK54(self, delta_t: float) -> StepResult:
        return self.update(1, delta_t)

    def SSPRK104(self, delta_t: float) -> StepResult:
        return self.update(2, delta_t)

    def SERK2(self, q: int, delta_t: float) -> StepResult:
        return self.update(serk2_method(q), delta_t)

    def run(self, nsteps: int, schedule=None, tmax: float = 0.0, gpu_rollback: bool = False,
            sparsify_every: int = 0, sparsify_sweeps: int = -1, sparsify_variant: str = "gpu",
            tail_fit: bool = False, use_serk2: bool = False) -> dict:
        """The driver loop (simulation_runner.cpp:125-304): `nsteps` controller iterations
        (or until t >= tmax); with `sparsify_every` > 0 the periodic sparsify of the
        reference (every that many loops; the reference uses 100000), whose step halving
        with `use_serk2` also climbs one SERK2 level; with `tail_fit` the QK tail fit
        after every step (the reference's --tail-fit)."""
        out = {k: np.zeros(nsteps) for k in ("dt", "delta", "t", "energy", "qk0", "r")}
        meth = np.zeros(nsteps, dtype=np.int32)
        sd = sm = None
        if schedule is not None:
            sd = np.ascontiguousarray(schedule[0], dtype=np.float64)
            sm = np.ascontiguousarray(schedule[1], dtype=np.int32)
        rp = _lib.RunParams(nsteps, tmax, _lib.ptr(sd), None if sm is None else sm.ctypes.data_as(_lib.ip),
                            int(gpu_rollback), _lib.ptr(out["dt"]), meth.ctypes.data_as(_lib.ip),
                            _lib.ptr(out["delta"]), _lib.ptr(out["t"]), _lib.ptr(out["energy"]),
                            _lib.ptr(out["qk0"]), _lib.ptr(out["r"]), sparsify_every, sparsify_sweeps,
                            SPARSIFY[sparsify_variant], int(tail_fit), int(use_serk2))
        last = _lib.StepResult()
        _lib.check(_lib.lib().dyn_run(self._h, C.byref(rp), C.byref(last)), "dyn_run")
        out["method"] = meth
        return out

    # ------------------------------------------------------ discrete adjoint
    def adjoint_forward(self, nsteps: int, schedule=None, tmax: float = 0.0) -> dict:
        """`run` (no rollback) that records its step schedule for `adjoint_backward`."""
        out = {k: np.zeros(nsteps) for k in ("dt", "delta", "t", "energy", "qk0", "r")}
        meth = np.zeros(nsteps, dtype=np.int32)
        sd = sm = None
        if schedule is not None:
            sd = np.ascontiguousarray(schedule[0], dtype=np.float64)
            sm = np.ascontiguousarray(schedule[1], dtype=np.int32)
        rp = _lib.RunParams(nsteps, tmax, _lib.ptr(sd), None if sm is None else sm.ctypes.data_as(_lib.ip), 0,
                            _lib.ptr(out["dt"]), meth.ctypes.data_as(_lib.ip), _lib.ptr(out["delta"]),
                            _lib.ptr(out["t"]), _lib.ptr(out["energy"]), _lib.ptr(out["qk0"]), _lib.ptr(out["r"]))
        last = _lib.StepResult()
        _lib.check(_lib.lib().dyn_adjoint_forward(self._h, C.byref(rp), C.byref(last)), "dyn_adjoint_forward")
        out["method"] = meth
        return out

    def adjoint_backward(self, w_energy: float = 0.0, w_r: float = 0.0, c_K=None, c_R=None, c_dK=None, c_dR=None,
                         w_dr: float = 0.0):
        """Gradient (d/dGamma, d/dlambda) of w_energy E(t_f) + c_K . C(t_f, theta t_f) + w_r r(t_f)
        (+ c_R . R, c_dK . dQK, c_dR . dQR, w_dr drvec of the final row) over the recorded forward;
        returns (grad, stats)."""
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (c_K, c_R, c_dK, c_dR)]
        obj = _lib.AdjointObjective(w_energy, w_r, *[_lib.ptr(a) for a in arrs], w_dr)
        g = np.zeros(2)
        st = _lib.AdjointStats()
        _lib.check(_lib.lib().dyn_adjoint_backward(self._h, C.byref(obj), _lib.ptr(g), C.byref(st)),
                   "dyn_adjoint_backward")
        return g, dict(ms_forward=st.ms_forward, ms_backward=st.ms_backward, device_bytes=int(st.device_bytes),
                       steps=st.steps, recompute_mismatch=int(st.recompute_mismatch))

    def adjoint_history_grad(self, n_start: int) -> State:
        """dJ/d(initial history rows [0, n_start)) from the last adjoint_backward."""
        L = self.L
        arrs = [np.zeros(n_start), np.zeros(n_start), np.empty(n_start * L), np.empty(n_start * L),
                np.empty(n_start * L), np.empty(n_start * L), np.empty(n_start), np.empty(n_start)]
        sc = _lib.StateC(n_start, *[_lib.ptr(x) for x in arrs])
        _lib.check(_lib.lib().dyn_adjoint_history_grad(self._h, C.byref(sc)), "dyn_adjoint_history_grad")
        return State(*arrs)

    def sparsifyNscale(self, threshold: float, variant: str = "gpu") -> int:
        v = C.c_size_t()
        _lib.check(_lib.lib().dyn_sparsify(self._h, threshold, SPARSIFY[variant], C.byref(v)), "dyn_sparsify")
        return int(v.value)

    def rollbackState(self, n: int) -> None:
        _lib.check(_lib.lib().dyn_rollback(self._h, n), "dyn_rollback")

    def last_row(self, qK: np.ndarray | None = None, qR: np.ndarray | None = None):
        """C(t, theta t) and R(t, theta t) of the newest row into host buffers."""
        qK = np.empty(self.L) if qK is None else qK
        qR = np.empty(self.L) if qR is None else qR
        _lib.check(_lib.lib().dyn_last_row(self._h, _lib.ptr(qK), _lib.ptr(qR)), "dyn_last_row")
        return qK, qR

    def profile_stage(self, reps: int = 20):
        """Average device milliseconds of the (gather+convolution, epilogue) kernels."""
        a, b = C.c_float(), C.c_float()
        _lib.check(_lib.lib().dyn_profile_stage(self._h, reps, C.byref(a), C.byref(b)), "dyn_profile_stage")
        return a.value, b.value

    def sync(self):
        _lib.check(_lib.lib().dyn_sync(self._h), "dyn_sync")

    # device-array entry points (for callers that own device memory)
    def conv_dev(self, kind: int, f_ptr: int, g_ptr: int, n: int, t: float, out_ptr: int):
        _lib.check(_lib.lib().dyn_conv_dev(self._h, kind, f_ptr, g_ptr, n, t, out_ptr), "dyn_conv_dev")

    def search_dev(self, list_ptr: int, nlist: int, elem_ptr: int, nelem: int, out_ptr: int):
        _lib.check(_lib.lib().dyn_search_dev(self._h, list_ptr, nlist, elem_ptr, nelem, out_ptr), "dyn_search_dev")


def probe_fp64(device: int = 0) -> float:
    """Measured FP64 FMA throughput of the device in GFLOP/s."""
    v = C.c_double()
    _lib.check(_lib.lib().dyn_probe_fp64(device, C.byref(v)), "dyn_probe_fp64")
    return v.value
