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

    python -m dynamite_gb300.microbench --form adjoint --L 512 --steps 20
    python -m dynamite_gb300.microbench --form mixed_error --L 1024 --steps 5000
    python -m dynamite_gb300.microbench --form long --L 512 --steps 400000 --tmax 1e6

`fp64` / `mixed` time the single-quench gather+convolution kernel and the
epilogue (one right-hand side at t = t_{n-1}); `batch` times the batched
gather over `quenches` copies of the history; `adjoint` runs the FP64
forward of the mixed p-spin quench (lam=0.5, T=0.6) from t=0 for `steps`
steps with its schedule recorded, then one reverse sweep for d E(t_f) /
d(T, lam), and reports both wall times; `mixed_error` runs the FP64 form of
that quench for `steps` steps and replays its step schedule in the mixed
form, then reports the relative error of the mixed run per observable:
energy over the run, r(t), C and R over the whole history, the equal-time
C(t, t), and at the final time t_f C(t_f/2, t_f) and R(t_f, t_f/2); `long`
runs the FP64 form from t=0 to `tmax` (at most `steps` steps) with the
reference driver's periodic sparsify every 100000 loops, then the mixed
form on that step schedule, and reports steps, wall times, history sizes and
the final-time observables of both.
Prints one JSON line.
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


def mixed_error(grid: Grid, nsteps: int, T: float = 0.6, lam: float = 0.5, tmax: float = 0.0,
                precision: str = "mixed") -> dict:
    """Mixed form against the FP64 form on the FP64 run's step schedule (see module doc);
    with tmax > 0 the FP64 run stops at t >= tmax (nsteps is then a cap)."""
    import time
    from .grid import lagrange_weights
    from .simulation import Model, Simulation
    L = grid.L
    m = Model(p=3, p2=4, lam=lam, Gamma=T)
    a = Simulation(grid, m, history_capacity=nsteps + 64)
    b = Simulation(grid, m, precision=precision, history_capacity=nsteps + 64)
    a.init()
    b.init()
    t0 = time.perf_counter()
    ta = a.run(nsteps, tmax=tmax)
    t1 = time.perf_counter()
    done = int(np.count_nonzero(ta["dt"]))
    ta = {k: v[:done] for k, v in ta.items()}
    tb = b.run(done, schedule=(ta["dt"], ta["method"]))
    t2 = time.perf_counter()
    nsteps = done
    sa, sb = a.download(), b.download()
    a.close()
    b.close()
    QA, QB = sa.QK.reshape(-1, L), sb.QK.reshape(-1, L)
    RA, RB = sa.QR.reshape(-1, L), sb.QR.reshape(-1, L)
    t = sa.t1grid
    w = lagrange_weights(grid.theta, 0.5)
    # C(t_f/2, t_f) = C(t_f, theta t_f) at theta = 1/2 (C symmetric), R(t_f, t_f/2) likewise
    c_a, c_b = float(w @ QA[-1]), float(w @ QB[-1])
    r_a, r_b = float(w @ RA[-1]), float(w @ RB[-1])
    rel = lambda x, y: float(np.max(np.abs(x - y)) / np.max(np.abs(y)))
    return {"form": "mixed_error", "precision": precision, "L": L, "steps": nsteps, "t_final": float(t[-1]),
            "T": T, "lam": lam,
            "history_rows": int(t.size), "s_fp64": t1 - t0, "s_mixed": t2 - t1,
            "time_grid_identical": bool(np.array_equal(sa.t1grid, sb.t1grid)),
            "energy": rel(tb["energy"], ta["energy"]), "r": rel(sb.rvec, sa.rvec), "C_history": rel(QB, QA),
            "R_history": rel(RB, RA), "C_equal_time_abs": float(np.max(np.abs(QB[:, -1] - QA[:, -1]))),
            "C_tf_half_tf": abs(c_b - c_a) / abs(c_a), "R_tf_tf_half": abs(r_b - r_a) / abs(r_a)}


def long_run(grid: Grid, nmax: int, tmax: float, T: float = 0.6, lam: float = 0.5, every: int = 100000,
             precision: str = "mixed") -> dict:
    """FP64 run to tmax with the periodic sparsify, then the mixed form on its schedule."""
    import time
    from .grid import lagrange_weights
    from .simulation import Model, Simulation
    L = grid.L
    m = Model(p=3, p2=4, lam=lam, Gamma=T)
    w = lagrange_weights(grid.theta, 0.5)
    out = {"form": "long", "L": L, "tmax": tmax, "T": T, "lam": lam, "sparsify_every": every}
    sched = None
    for prec in ("fp64", precision):
        s = Simulation(grid, m, precision=prec, history_capacity=min(nmax, every) + 64)
        s.init()
        t0 = time.perf_counter()
        if sched is None:
            tr = s.run(nmax, tmax=tmax, sparsify_every=every)
            done = int(np.count_nonzero(tr["dt"]))
            sched = (tr["dt"][:done], tr["method"][:done])
        else:
            tr = s.run(sched[0].size, schedule=sched, sparsify_every=every)
        sec = time.perf_counter() - t0
        st = s.download()
        last_K, last_R = st.QK[-L:], st.QR[-L:]
        out[prec] = {"steps": int(sched[0].size), "seconds": sec, "steps_per_s": sched[0].size / sec,
                     "t_final": float(st.t1grid[-1]), "history_rows": int(st.t1grid.size), "energy": s.energy(),
                     "r": float(st.rvec[-1]), "C_tf_half_tf": float(w @ last_K), "R_tf_tf_half": float(w @ last_R)}
        s.close()
    a, b = out["fp64"], out[precision]
    out["mixed_rel_err"] = {k: abs(b[k] - a[k]) / abs(a[k]) for k in ("energy", "r", "C_tf_half_tf", "R_tf_tf_half")}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--form", choices=["fp64", "mixed", "batch", "adjoint", "mixed_error", "long"], default="batch")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--tune", action="store_true", help="batch: autotune the gather tile first")
    ap.add_argument("--tmax", type=float, default=0.0, help="mixed_error: run the FP64 form to t >= tmax")
    ap.add_argument("--precision", choices=["mixed", "mixed_df"], default="mixed",
                    help="mixed_error / long / fp64 stage timing: the mixed form to compare")
    ap.add_argument("--L", type=int, default=512)
    ap.add_argument("--rows", type=int, default=4096)
    ap.add_argument("--quenches", type=int, default=16)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--T", type=float, default=0.6)
    ap.add_argument("--log-response", action="store_true", help="fp64 stage timing: QR gathers in log space")
    a = ap.parse_args(argv)
    from . import build as B
    B.build()
    from . import grid as G
    from .batch import Batch, Quench
    from .simulation import Model, Simulation

    grid = G.generate(a.L)
    if a.form == "adjoint":
        s = Simulation(grid, Model(p=3, p2=4, lam=0.5, Gamma=a.T), history_capacity=a.steps + 16)
        s.init()
        fw = s.adjoint_forward(a.steps)
        g, stats = s.adjoint_backward(w_energy=1.0)
        s.close()
        print(json.dumps({"form": "adjoint", "L": a.L, "steps": a.steps, "t_final": float(fw["t"][-1]),
                          "dE_dT": float(g[0]), "dE_dlam": float(g[1]), **stats}))
        return
    if a.form == "long":
        print(json.dumps(long_run(grid, a.steps, a.tmax, a.T, precision=a.precision)))
        return
    if a.form == "mixed_error":
        print(json.dumps(mixed_error(grid, a.steps, a.T, tmax=a.tmax, precision=a.precision)))
        return
    st = synthetic_history(grid, a.rows, a.T)
    t = st.t1grid
    out = {"form": a.form, "L": a.L, "rows": a.rows}
    if a.form in ("fp64", "mixed"):
        prec = a.form if a.form == "fp64" else a.precision
        logr = a.log_response and prec == "fp64"
        s = Simulation(grid, Model(p=3, p2=4, lam=0.5, Gamma=a.T), precision=prec, history_capacity=a.rows + 2,
                       log_response=logr)
        if logr:  # QR > 0 everywhere, so the log-space branches run: QR -> -QR, dQR -> -dQR
            st = State(st.t1grid, st.dtr, st.QK, -st.QR, st.dQK, -st.dQR, st.rvec, st.drvec)
        s.upload(st)
        ms_main, ms_epi = s.profile_stage(reps=a.reps)
        out.update(ms_main=ms_main, ms_epilogue=ms_epi, log_response=logr)
        s.close()
    else:
        qs = [Quench(grid=0, p=3, p2=4, lam=(0.3, 0.5, 0.7)[b % 3], Gamma=0.4 + 0.6 * b / max(a.quenches - 1, 1),
                     capacity=a.rows + 2) for b in range(a.quenches)]
        bt = Batch([grid], qs, precision=a.precision)
        for q in range(a.quenches):
            bt.upload(q, st, delta_t=0.01 * (t[-1] - t[-2]), method=1)
        if a.tune:
            out.update(tile=bt.tune(reps=3))
        out.update(quenches=a.quenches, precision=a.precision, ms_gather=bt.profile(reps=a.reps))
        bt.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
