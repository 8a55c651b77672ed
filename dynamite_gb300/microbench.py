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
    python -m dynamite_gb300.microbench --form decades --L 1024 --tmax 1e7 --wall 1500
    python -m dynamite_gb300.microbench --form batch_job --tscale 1e-3 --wall 1200

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
the final-time observables of both; `decades` runs one quench in the FP64, mixed and
(hi, lo) forms side by side (the mixed forms on the FP64 schedule, periodic block with the
SERK2 climb) and reports, at every decade t_d of the run, E(t_d), r(t_d), R(t_d, t_d/2) and
C(2 t_d, t_d) of each form with the mixed forms' relative errors.
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


def sparsify_probe(grid: Grid, nsteps: int, T: float = 0.6, lam: float = 0.5,
                   thresholds=(1e-10, 1e-9, 1e-8, 1e-7)) -> dict:
    """How many rows one sparsify pass keeps on the same history computed in each form: the
    FP64 form runs `nsteps` controller steps (no sparsify), the mixed forms replay its
    schedule; each form's history then goes through one sparsify pass (reference GPU variant)
    at each threshold, restarting from the unsparsified history every time."""
    from .simulation import Model, Simulation
    m = Model(p=3, p2=4, lam=lam, Gamma=T)
    out = {"form": "sparsify_probe", "L": grid.L, "steps": nsteps, "T": T, "lam": lam, "kept": {}}
    sched = None
    for prec in ("fp64", "mixed", "mixed_df"):
        s = Simulation(grid, m, precision=prec, history_capacity=nsteps + 64)
        s.init()
        if sched is None:
            tr = s.run(nsteps)
            done = int(np.count_nonzero(tr["dt"]))
            sched = (tr["dt"][:done], tr["method"][:done])
            out["t_final"] = float(tr["t"][done - 1])
        else:
            s.run(sched[0].size, schedule=sched)
        st = s.download()
        out["rows"] = int(st.t1grid.size)
        kept = {}
        for thr in thresholds:
            s.upload(st)
            kept[f"{thr:g}"] = s.sparsifyNscale(thr)
        out["kept"][prec] = kept
        s.close()
    return out


DECADE_FORMS = ("fp64", "mixed", "mixed_df", "fp64_full", "mixed_df_full")


def decades(grid: Grid, tmax: float, wall: float, T: float = 0.6, lam: float = 0.5, every: int = 100000,
            use_serk2: bool = True, chunk: int = 2000, out_path: str | None = None,
            forms: tuple = ("fp64", "mixed", "mixed_df")) -> dict:
    """One quench in several forms.  "fp64" runs its own controller with the reference GPU
    loop's periodic block (sparsify every `every` loops, SERK2 climb); "mixed" and "mixed_df"
    replay its step schedule chunk by chunk with the same cadence (their own sparsify flags);
    "fp64_full" and "mixed_df_full" replay it with no sparsify at all, so that their
    difference is the (hi, lo) form's arithmetic alone and "fp64" against "fp64_full" is what
    the reference's own sparsify changes.  At every decade t_d = 1, 10, ... up to tmax the run
    stops at the first step reaching t_d and at the first reaching 2 t_d; per form it records
    E(t_d) and r(t_d), R(t_d, t_d/2) = QR of the row at t_d evaluated at theta = (t_d/2)/t, and
    C(2 t_d, t_d) = QK of the row at 2 t_d at theta = t_d/t (a 10-point Lagrange functional of
    the row, the same on every form).  Errors are relative: a "_full" form against
    "fp64_full", the other forms against "fp64", and "sparsify_rel_err" is "fp64" against
    "fp64_full".  Stops early after `wall` seconds; with out_path every finished decade is
    appended there as one JSON line."""
    import time
    from .grid import lagrange_weights
    from .simulation import Model, Simulation
    m = Model(p=3, p2=4, lam=lam, Gamma=T)
    names = ("fp64",) + tuple(f for f in forms if f != "fp64")
    for f in names:
        if f not in DECADE_FORMS:
            raise ValueError(f"unknown form {f}")
    sims = {k: Simulation(grid, m, precision=k.replace("_full", ""), history_capacity=4096) for k in names}
    for s in sims.values():
        s.init()
    secs = dict.fromkeys(names, 0.0)
    steps = 0
    events = []
    d = 1.0
    while d <= tmax:
        events += [(d, "E", d), (2 * d, "C", d)]
        d *= 10.0
    events.sort()
    rec = {}
    t_now = 0.0
    t_start = time.perf_counter()
    kw = dict(sparsify_every=every, use_serk2=use_serk2)
    from ._lib import DYN_ERR_NONFINITE, DynError
    stopped = None
    while events and time.perf_counter() - t_start < wall and stopped is None:
        target = events[0][0]
        t0 = time.perf_counter()
        try:
            tr = sims["fp64"].run(chunk, tmax=target, **kw)
        except DynError as e:
            if e.status != DYN_ERR_NONFINITE:
                raise
            stopped = {"form": "fp64", "near_step": steps}
            break
        secs["fp64"] += time.perf_counter() - t0
        done = int(np.count_nonzero(tr["dt"]))
        if done == 0:
            break
        sched = (tr["dt"][:done], tr["method"][:done])
        res = {"fp64": tr}
        for k in names[1:]:
            t0 = time.perf_counter()
            try:
                res[k] = sims[k].run(done, schedule=sched,
                                     **(dict(kw, sparsify_every=0) if k.endswith("_full") else kw))
            except DynError as e:
                if e.status != DYN_ERR_NONFINITE:
                    raise
                stopped = {"form": k, "near_step": steps}
            secs[k] += time.perf_counter() - t0
        if stopped is not None:
            break
        steps += done
        t_now = float(tr["t"][done - 1])
        while events and t_now >= events[0][0]:
            _, kind, td = events.pop(0)
            vals = {}
            for k in names:
                qK, qR = sims[k].last_row()
                if kind == "E":
                    vals[k] = {"E": float(res[k]["energy"][done - 1]), "r": float(res[k]["r"][done - 1]),
                               "R_t_thalf": float(lagrange_weights(grid.theta, 0.5 * td / t_now) @ qR)}
                else:
                    vals[k] = {"C_2t_t": float(lagrange_weights(grid.theta, td / t_now) @ qK)}
            e = rec.setdefault(td, {"t": td, "steps_at_t": None, "rows": None})
            if kind == "E":
                e.update(steps_at_t=steps, rows={k: sims[k].n for k in names})
            for k in names:
                e.setdefault(k, {}).update(vals[k])
            if kind == "C":
                for k in names[1:]:
                    b = "fp64_full" if k.endswith("_full") and "fp64_full" in names else "fp64"
                    if k != b:
                        e[k + "_rel_err"] = {q: abs(e[k][q] - e[b][q]) / abs(e[b][q]) for q in e[b]}
                if "fp64_full" in names:
                    e["sparsify_rel_err"] = {q: abs(e["fp64"][q] - e["fp64_full"][q]) / abs(e["fp64_full"][q])
                                             for q in e["fp64"]}
                if out_path:
                    with open(out_path, "a") as fh:
                        fh.write(json.dumps(dict(e, seconds=dict(secs), steps=steps)) + "\n")
    for s in sims.values():
        s.close()
    return {"form": "decades", "L": grid.L, "T": T, "lam": lam, "sparsify_every": every, "use_serk2": use_serk2,
            "steps": steps, "t_reached": t_now if steps else 0.0, "seconds": secs, "nonfinite": stopped,
            "steps_per_s": {k: steps / v for k, v in secs.items() if v > 0},
            "decades": [rec[k] for k in sorted(rec)]}


def batch_job(tscale: float, wall: float, every: int = 100000, use_serk2: bool = True, chunk: int = 256,
              max_gb: float = 150.0, precision: str = "mixed_df", **batch_kw) -> dict:
    """The mixed-L batch run as a whole job: the 64 quenches of mixed_length_quenches (T on
    [0.4, 1.0], lam 0.3/0.5/0.7, L from {256, 512, 1024} and t_stop log-uniform on
    [1e4, 1e7], both drawn from mt19937_64) with every t_stop multiplied by `tscale`, the
    periodic block of the reference GPU loop (sparsify every `every` loops, SERK2 climb) and
    the gather tile the autotuner picks after the first ticks; run until every quench has
    stopped (or `wall` seconds).  History capacity per quench from the step count a quench
    needs to reach its t_stop (about 424 t^0.577 steps for the mixed p-spin at T = 0.6, with
    a 1.5 margin); the job is refused above `max_gb` of history memory.  `batch_kw` goes to
    Batch (device, stream)."""
    import time
    from . import grid as G
    from .batch import Batch, mixed_length_quenches
    lengths, qs = mixed_length_quenches(n=64)
    need = 0.0
    for q in qs:
        q.t_stop *= tscale
        q.capacity = int(1.5 * 424.0 * q.t_stop ** 0.577) + 2048
        # FP64 (QK, QR), (dQK, dQR) + their FP32 mirrors (+ the low parts of (QK, QR))
        need += q.capacity * lengths[q.grid] * (56.0 if precision == "mixed_df" else 48.0)
    if need / 1e9 > max_gb:
        raise ValueError(f"batch job needs {need / 1e9:.0f} GB of history, above {max_gb} GB: lower tscale")
    grids = [G.generate(L) for L in lengths]
    bt = Batch(grids, qs, ticks_per_launch=32, sparsify_every=every, use_serk2=use_serk2, precision=precision,
               **batch_kw)
    t0 = time.perf_counter()
    ticks = bt.run(512)
    tile = bt.tune(reps=3)
    while time.perf_counter() - t0 < wall:
        k = bt.run(chunk * 32)
        ticks += k
        if k < chunk * 32:
            break
    sec = time.perf_counter() - t0
    infos = bt.infos()
    bt.close()
    per_L = {}
    for q, i in zip(qs, infos):
        d = per_L.setdefault(str(lengths[q.grid]), {"quenches": 0, "steps": 0})
        d["quenches"] += 1
        d["steps"] += i["steps"]
    total = sum(i["steps"] for i in infos)
    status = {}
    for i in infos:
        status[i["status"]] = status.get(i["status"], 0) + 1
    reached = [i["t"] / q.t_stop for q, i in zip(qs, infos)]
    return {"form": "batch_job", "precision": precision, "quenches": len(qs), "tscale": tscale,
            "t_stop_range": [min(q.t_stop for q in qs), max(q.t_stop for q in qs)], "sparsify_every": every,
            "use_serk2": use_serk2, "tile": tile, "ticks": ticks, "seconds": sec, "rk_steps": total,
            "steps_per_s": total / sec, "per_L": per_L, "status": status,
            "t_over_t_stop_range": [min(reached), max(reached)], "history_gb": need / 1e9,
            "max_rows": max(i["n"] for i in infos)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--form", choices=["fp64", "mixed", "batch", "adjoint", "mixed_error", "long", "decades", "batch_job",
                                       "sparsify_probe"],
                    default="batch")
    ap.add_argument("--wall", type=float, default=600.0, help="decades / batch_job: stop after this many seconds")
    ap.add_argument("--tscale", type=float, default=1e-3, help="batch_job: factor on every stopping time")
    ap.add_argument("--out", default=None, help="decades: append each finished decade to this file")
    ap.add_argument("--forms", default="fp64,mixed,mixed_df",
                    help="decades: comma-separated forms out of " + ",".join(DECADE_FORMS))
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--tune", action="store_true", help="batch: autotune the gather tile first")
    ap.add_argument("--tmax", type=float, default=0.0, help="mixed_error: run the FP64 form to t >= tmax")
    ap.add_argument("--precision", choices=["mixed", "mixed_df"], default="mixed",
                    help="mixed_error / long / batch / batch_job / fp64 stage timing: the mixed form")
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
    if a.form == "batch_job":
        print(json.dumps(batch_job(a.tscale, a.wall, precision=a.precision)))
        return
    if a.form == "sparsify_probe":
        print(json.dumps(sparsify_probe(grid, a.steps, a.T)))
        return
    if a.form == "decades":
        print(json.dumps(decades(grid, a.tmax, a.wall, a.T, out_path=a.out, forms=tuple(a.forms.split(",")))))
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
