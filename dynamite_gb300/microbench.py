"""Stage-kernel microbench on a synthetic two-time history (no dynamics).

The history is the smooth two-time function of the L=512 kernel microbench:
C(t, t') = exp(-|ln(t+1) - ln(t'+1)|) = (t'+1)/(t+1) for t' <= t and
R(t, t') = -(1/T) dC/dt' = -1/(T (t+1)), on rows t_0 = 0 and t_k
log-spaced on [1e-5, 1e6]; row k holds C(t_k, theta_j t_k), R(t_k, theta_j t_k),
the staggered derivatives (t_k - t_{k-1}) d/dt C(t, theta_j t) at t_{k-1}
(same for R), delta_t_ratio from the t_k, r = 1, dr = 0.

    python -m dynamite_gb300.microbench --form fp64  --L 512 --rows 4096 --reps 20
    python -m dynamite_gb300.microbench --form mixed --L 512 --rows 4096 --reps 20
    python -m dynamite_gb300.microbench --form batch --L 512 --rows 1500 --quenches 64 --reps 3

`fp64` / `mixed` time the single-quench gather+convolution kernel and the
epilogue (one right-hand side at t = t_{n-1}); `batch` times the batched
gather over `quenches` copies of the history.  Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from .grid import Grid
from .simulation import State


def synthetic_history(grid: Grid, n: int, T: float = 0.6, t_lo: float = 1e-5, t_hi: float = 1e6) -> State:
    th = np.asarray(grid.theta, dtype=np.float64)
    t = np.concatenate([[0.0], np.logspace(np.log10(t_lo), np.log10(t_hi), n - 1)])
    tc = t[:, None]
    QK = (th[None, :] * tc + 1.0) / (tc + 1.0)
    QR = np.broadcast_to(-1.0 / (T * (tc + 1.0)), QK.shape).copy()
    dt = np.diff(t, prepend=0.0)[:, None]
    tp = np.concatenate([[0.0], t[:-1]])[:, None]
    dQK = dt * (th[None, :] - 1.0) / (tp + 1.0) ** 2
    dQR = np.broadcast_to(dt / (T * (tp + 1.0) ** 2), QK.shape).copy()
    dtr = np.zeros(n)
    dtr[2:] = (t[2:] - t[1:-1]) / (t[1:-1] - t[:-2])
    return State(t, dtr, QK.ravel(), QR.ravel(), dQK.ravel(), dQR.ravel(), np.ones(n), np.zeros(n))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--form", choices=["fp64", "mixed", "batch"], default="batch")
    ap.add_argument("--L", type=int, default=512)
    ap.add_argument("--rows", type=int, default=4096)
    ap.add_argument("--quenches", type=int, default=16)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--T", type=float, default=0.6)
    a = ap.parse_args(argv)
    from . import build as B
    B.build()
    from . import grid as G
    from .batch import Batch, Quench
    from .simulation import Model, Simulation

    grid = G.generate(a.L)
    st = synthetic_history(grid, a.rows, a.T)
    t = st.t1grid
    out = {"form": a.form, "L": a.L, "rows": a.rows}
    if a.form in ("fp64", "mixed"):
        s = Simulation(grid, Model(p=3, p2=4, lam=0.5, Gamma=a.T), precision=a.form, history_capacity=a.rows + 2)
        s.upload(st)
        ms_main, ms_epi = s.profile_stage(reps=a.reps)
        out.update(ms_main=ms_main, ms_epilogue=ms_epi)
        s.close()
    else:
        qs = [Quench(grid=0, p=3, p2=4, lam=(0.3, 0.5, 0.7)[b % 3], Gamma=0.4 + 0.6 * b / max(a.quenches - 1, 1),
                     capacity=a.rows + 2) for b in range(a.quenches)]
        bt = Batch([grid], qs)
        for q in range(a.quenches):
            bt.upload(q, st, delta_t=0.01 * (t[-1] - t[-2]), method=1)
        out.update(quenches=a.quenches, ms_gather=bt.profile(reps=a.reps))
        bt.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
