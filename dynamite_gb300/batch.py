"""Batched quenches on one GPU (include/dyn.h, `dyn_batch_*`).

The reference runs one quench per process (simulation_runner.cpp:125-304);
`Batch` advances many quenches together, each with its own model, grid,
history, step controller (the one `Simulation.run` applies) and stopping rule,
in the arithmetic of `Simulation(precision="mixed_df")` (the default: its free
controller and sparsify decisions match the FP64 form's) or of
`Simulation(precision="mixed")`.

    b = Batch([grid512], [Quench(grid=0, Gamma=0.6, lam=0.5, t_stop=1e4)])
    b.run(max_ticks=10_000)
    b.info(0)["t"], b.download(0).QK

With `sparsify_every` > 0 every quench takes the reference driver's periodic
sparsify (simulation_runner.cpp:148-237) after each loop that is a multiple
of it: it pauses at that step's end and the host compacts its history between
graph replays.

`mixed_length_quenches` draws the 64-quench workload (temperatures on [0.4, 1.0],
lambda in {0.3, 0.5, 0.7}, grid length from {256, 512, 1024}, stopping times
log-uniform on [1e4, 1e7]) from `mt19937_64` with a fixed seed.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .grid import Grid
from .simulation import SEARCH, SPARSIFY, State

STATUS = {0: "running", 1: "done", 2: "max_steps", 3: "full", 4: "sparsify", 5: "failed"}


@dataclass
class Quench:
    grid: int = 0
    p: int = 3
    p2: int = 4
    lam: float = 0.5
    T0: float = 1e50
    Gamma: float = 0.6
    delta_t_min: float = 1e-5
    delta_max: float = 1e-10
    delta_t: float = 0.0
    t_stop: float = 0.0
    max_steps: int = 0
    capacity: int = 4096


class Batch:
    def __init__(self, grids: list[Grid], quenches: list[Quench], search: str = "binary", gpu_rollback: bool = False,
                 ticks_per_launch: int = 32, threads: int = 128, targets: int = 1, ctas_per_sm: int = 0,
                 device: int = 0, stream: int | None = None, sparsify_every: int = 0, sparsify_sweeps: int = -1,
                 sparsify_variant: str = "gpu", precision: str = "mixed_df", use_serk2: bool = False):
        self.grids = grids
        self.quenches = list(quenches)
        self._h = C.c_void_p()
        keep = []
        gs = (_lib.BatchGrid * len(grids))()
        for k, g in enumerate(grids):
            f64 = [np.ascontiguousarray(a, dtype=np.float64) for a in (g.theta, g.phi2, g.integ, g.wA1, g.wA2, g.wB2)]
            i64 = [np.ascontiguousarray(a, dtype=np.int64) for a in (g.indsA1, g.indsA2, g.indsB2)]
            keep += f64 + i64
            tb = _lib.Tables(_lib.ptr(f64[0]), _lib.ptr(f64[1]), _lib.ptr(f64[2]),
                             *[a.ctypes.data_as(_lib.i64p) for a in i64], *[_lib.ptr(a) for a in f64[3:]])
            gs[k] = _lib.BatchGrid(g.L, g.depth, tb)
        qs = (_lib.BatchQuench * len(quenches))()
        for k, q in enumerate(quenches):
            qs[k] = _lib.BatchQuench(q.grid, q.p, q.p2, q.lam, q.T0, q.Gamma, q.delta_t_min, q.delta_max, q.delta_t,
                                     q.t_stop, q.max_steps, q.capacity)
        cfg = _lib.BatchConfig(device, stream, SEARCH[search], int(gpu_rollback), ticks_per_launch, threads, targets,
                               ctas_per_sm, sparsify_every, sparsify_sweeps, SPARSIFY[sparsify_variant],
                               {"mixed": 1, "mixed_df": 2}[precision], int(use_serk2))
        _lib.check(_lib.lib().dyn_batch_create(C.byref(cfg), gs, len(grids), qs, len(quenches), C.byref(self._h)),
                   "dyn_batch_create")
        del keep  # the tables were copied to the device

    def close(self):
        if self._h:
            _lib.lib().dyn_batch_destroy(self._h)
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

    def __len__(self) -> int:
        return len(self.quenches)

    def run(self, max_ticks: int) -> int:
        """Advance until no quench runs or `max_ticks` stages have run; returns the ticks run."""
        t = C.c_longlong()
        _lib.check(_lib.lib().dyn_batch_run(self._h, int(max_ticks), C.byref(t)), "dyn_batch_run")
        return int(t.value)

    def enqueue(self, ticks: int) -> None:
        """Enqueue `ticks` ticks on the batch's stream without waiting."""
        _lib.check(_lib.lib().dyn_batch_enqueue(self._h, int(ticks)), "dyn_batch_enqueue")

    def sync(self) -> None:
        """Wait for enqueued ticks and refresh the quench infos."""
        _lib.check(_lib.lib().dyn_batch_sync(self._h), "dyn_batch_sync")

    def last_row(self, q: int, qK: np.ndarray | None = None, qR: np.ndarray | None = None):
        """C(t, theta t) and R(t, theta t) of quench q's newest row."""
        L = self.grids[self.quenches[q].grid].L
        qK = np.empty(L) if qK is None else qK
        qR = np.empty(L) if qR is None else qR
        _lib.check(_lib.lib().dyn_batch_last_row(self._h, q, _lib.ptr(qK), _lib.ptr(qR)), "dyn_batch_last_row")
        return qK, qR

    def info(self, q: int) -> dict:
        i = _lib.BatchInfo()
        _lib.check(_lib.lib().dyn_batch_get_info(self._h, q, C.byref(i)), "dyn_batch_get_info")
        return dict(status=STATUS[i.status], method=i.method, loop=i.loop, steps=int(i.steps), n=int(i.n), t=i.t,
                    delta_t=i.delta_t, delta=i.delta, delta_old=i.delta_old, energy=i.energy, r=i.r, qk0=i.qk0)

    def infos(self) -> list[dict]:
        return [self.info(q) for q in range(len(self))]

    def total_steps(self) -> int:
        return sum(self.info(q)["steps"] for q in range(len(self)))

    def set_limits(self, q: int, t_stop: float = 0.0, max_steps: int = 0) -> None:
        _lib.check(_lib.lib().dyn_batch_set_limits(self._h, q, t_stop, int(max_steps)), "dyn_batch_set_limits")

    def upload(self, q: int, st: State, delta_t: float, method: int, delta: float = 1.0, delta_old: float = 0.0,
               loop: int = 0) -> None:
        a = [np.ascontiguousarray(getattr(st, f), dtype=np.float64)
             for f in ("t1grid", "dtr", "QK", "QR", "dQK", "dQR", "rvec", "drvec")]
        sc = _lib.StateC(a[0].size, *[_lib.ptr(x) for x in a])
        ctl = _lib.Controller(delta_t, delta, delta_old, loop, method)
        _lib.check(_lib.lib().dyn_batch_upload(self._h, q, C.byref(sc), C.byref(ctl)), "dyn_batch_upload")

    def download(self, q: int) -> State:
        n = self.info(q)["n"]
        L = self.grids[self.quenches[q].grid].L
        arrs = [np.empty(n), np.empty(n), np.empty(n * L), np.empty(n * L), np.empty(n * L), np.empty(n * L),
                np.empty(n), np.empty(n)]
        sc = _lib.StateC(n, *[_lib.ptr(x) for x in arrs])
        _lib.check(_lib.lib().dyn_batch_download(self._h, q, C.byref(sc)), "dyn_batch_download")
        return State(*arrs)

    def tune(self, reps: int = 5) -> dict:
        """Autotuner: time every gather tile shape on the current states, keep the fastest."""
        t, k, c = C.c_int(), C.c_int(), C.c_int()
        ms = C.c_float()
        _lib.check(_lib.lib().dyn_batch_tune(self._h, reps, C.byref(t), C.byref(k), C.byref(c), C.byref(ms)),
                   "dyn_batch_tune")
        return dict(threads=t.value, targets=k.value, ctas_per_sm=c.value, ms_gather=ms.value)

    def profile(self, reps: int = 10) -> float:
        """Average device time (ms) of one gather launch over all running quenches."""
        ms = C.c_float()
        _lib.check(_lib.lib().dyn_batch_profile(self._h, reps, C.byref(ms)), "dyn_batch_profile")
        return ms.value


# ------------------------------------------------------------ workload draws
class MT19937_64:
    """std::mt19937_64 (the C++ standard's 64-bit Mersenne Twister parameters)."""

    N, M = 312, 156
    MATRIX_A = 0xB5026F5AA96619E9
    UPPER, LOWER = 0xFFFFFFFF80000000, 0x7FFFFFFF
    MASK = (1 << 64) - 1

    def __init__(self, seed: int = 5489):
        self.mt = [0] * self.N
        self.mt[0] = seed & self.MASK
        for i in range(1, self.N):
            self.mt[i] = (6364136223846793005 * (self.mt[i - 1] ^ (self.mt[i - 1] >> 62)) + i) & self.MASK
        self.idx = self.N

    def _twist(self):
        mt = self.mt
        for i in range(self.N):
            x = (mt[i] & self.UPPER) | (mt[(i + 1) % self.N] & self.LOWER)
            xa = x >> 1
            if x & 1:
                xa ^= self.MATRIX_A
            mt[i] = mt[(i + self.M) % self.N] ^ xa
        self.idx = 0

    def __call__(self) -> int:
        if self.idx >= self.N:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & self.MASK

    def uniform(self) -> float:
        """53-bit uniform on [0, 1)."""
        return (self() >> 11) * (1.0 / 9007199254740992.0)


def mixed_length_quenches(n: int = 64, seed: int = 20261203, lengths=(256, 512, 1024), capacity: int = 4096,
                     max_steps: int = 0):
    """The batched-quench workload: quench b has temperature Gamma_b = 0.4 + 0.6 b/(n-1),
    lambda cycling through {0.3, 0.5, 0.7}, grid length lengths[x % 3] and stopping time
    10**(4 + 3u) with x, u drawn from mt19937_64(seed).  Returns (lengths per quench, quenches
    with `grid` = index into sorted(set(lengths)))."""
    rng = MT19937_64(seed)
    Ls, qs = [], []
    for b in range(n):
        L = lengths[rng() % len(lengths)]
        u = rng.uniform()
        Ls.append(L)
        qs.append(Quench(grid=-1, p=3, p2=4, lam=(0.3, 0.5, 0.7)[b % 3], Gamma=0.4 + 0.6 * b / max(n - 1, 1),
                         t_stop=10.0 ** (4.0 + 3.0 * u), capacity=capacity, max_steps=max_steps))
    order = sorted(set(Ls))
    for L, q in zip(Ls, qs):
        q.grid = order.index(L)
    return order, qs
