"""Generate the golden vectors in tests/golden/ by running the reference itself.

The reference DYNAMITE CPU implementation is compiled from its own sources by
oracle/Makefile (oracle/_ref/libdynref.so, IEEE build, single thread) and driven
through the harness in oracle/ref_harness.cpp.  The vectors pin both the C
restatement (oracle/dyn_oracle.c) and the CUDA path.

    python tests/golden/make_golden.py        # needs the reference sources

Cases (one .npz per grid size):
  grid       tables from the reference generator (poly-9, spline order 5)
  t0_*       t=0 state and its first interpolation / right-hand side
  mid_*      state after an adaptive RK54 run (40 controller iterations),
             interpolation at fresh (binary-search) positions, QKstep/QRstep,
             rstep, drstep2, energy
  rk54_*     one RK54 step from the mid state
  ssp_*      one SSPRK(10,4) step from the mid state
  traj_*     the reference controller run from t=0: per-step dt, method,
             error, time, energy, and the final history
  spars_*    sparsifyNscale (CPU-only build variant) of the trajectory state

golden_log_L64.npz: the log-space response option (-R, config.log_response_interp)
on the grid and model of golden_L64.npz:
  pos_*      a history with QR > 0 and curvature in log QR (positive_history),
             its interpolation (QR arrays 1, 3, 5, 7), QKstep/QRstep, and one
             RK54 step of 1e-3 (pos_rk54_*)
  ltraj_*    the reference controller run from t=0 with the option on

golden_tail_L64.npz: the QK tail fit (--tail-fit, tailFitBlendCPU) on the grid
and model of golden_L64.npz, in one process (the fit keeps its state in statics):
  tft_*      the reference controller run from t=0 with the fit after every
             update (400 steps): per-step records, final t1grid/rvec, the last
             row, and per-row sums of QK and QR
  tfs_*      then single fits: state A (the mid state of golden_L64.npz with its
             newest row's tail replaced by tail_row(theta)) fitted twice; state B
             (A plus one row, tfB_*) fitted, then with the rollback loop set to 5,
             then back to -1000; the newest QK row after each fit
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [
    # L, Tmax, model, trajectory steps
    (32, 10.0, O.Model(p=3, p2=4, lam=0.5, T0=1e50, Gamma=0.6), 120),
    (64, 100.0, O.Model(p=3, p2=0, lam=0.5, T0=1e50, Gamma=0.8), 80),
]


def state_dict(prefix: str, st: O.State) -> dict:
    return {f"{prefix}_{k}": getattr(st, k) for k in
            ("t1grid", "dtr", "QK", "QR", "dQK", "dQR", "rvec", "drvec", "posB1xOld", "posB2xOld")}


def make(L: int, Tmax: float, model: O.Model, nsteps: int) -> dict:
    out = {}
    g = O.Reference.grid(L, Tmax=Tmax)
    for k in ("theta", "phi1", "phi2", "integ", "indsA1", "wA1", "indsA2", "wA2", "indsB2", "wB2"):
        out[f"grid_{k}"] = getattr(g, k)
    out["model"] = np.array([model.p, model.p2, model.lam, model.T0, model.Gamma, model.delta_t_min,
                             model.delta_max, Tmax])
    ref = O.Reference(g, model, threads=1)

    # t = 0
    ref.init_state()
    out.update(state_dict("t0", ref.get_state()))
    for w in range(17):
        out[f"t0_interp{w}"] = ref.interp(w)
    out["t0_qk"] = ref.qkstep()
    out["t0_qr"] = ref.qrstep()

    # trajectory with the reference controller
    ref.init_state()
    tr = ref.run(nsteps)
    for k, v in tr.items():
        out[f"traj_{k}"] = v
    out.update(state_dict("traj_final", ref.get_state()))

    # mid state: first 40 iterations of the same run
    ref.init_state()
    ref.run(40)
    mid = ref.get_state()
    out.update(state_dict("mid", mid))
    out["mid_ctl"] = np.array([O.Reference.lib().dynref_get_delta_t()], dtype=np.float64)
    ref.interpolate()  # fresh positions (binary search)
    for w in range(17):
        out[f"mid_interp{w}"] = ref.interp(w)
    out["mid_qk"] = ref.qkstep()
    out["mid_qr"] = ref.qrstep()
    out["mid_rstep"] = np.array([ref.rstep()])
    st = ref.get_state()
    n = st.n
    qK, qR = st.QK[(n - 1) * L:], st.QR[(n - 1) * L:]
    out["mid_drstep2"] = np.array([ref.drstep2(qK, qR, out["mid_qk"], out["mid_qr"], st.t1grid[-1])])
    out["mid_energy"] = np.array([ref.energy(st.t1grid[-1])])

    dt = float(out["mid_ctl"][0])
    for tag, method in (("rk54", 1), ("ssp", 2)):
        ref.set_state(mid)
        ref.interpolate(mid.posB1xOld, mid.posB2xOld, True)
        err = ref.update(method, dt)
        out[f"{tag}_dt"] = np.array([dt])
        out[f"{tag}_err"] = np.array([err])
        out.update(state_dict(tag, ref.get_state()))

    # sparsify the trajectory state (CPU-only build variant)
    final = O.State(*(out[f"traj_final_{k}"] for k in
                      ("t1grid", "dtr", "QK", "QR", "dQK", "dQR", "rvec", "drvec", "posB1xOld", "posB2xOld")))
    thr = float(np.quantile(_indicators(final, L), 0.5))
    ref.set_state(final)
    ref.sparsify(thr)
    out["spars_threshold"] = np.array([thr])
    out.update(state_dict("spars", ref.get_state()))
    return out


def _indicators(st: O.State, L: int) -> np.ndarray:
    """Node error indicators (sparsify_utils.cpp:19-56), to pick a threshold that drops about half."""
    t = st.t1grid
    QK, QR, dQK, dQR = (a.reshape(-1, L) for a in (st.QK, st.QR, st.dQK, st.dQR))
    vals = []
    for i in range(2, t.size - 1):
        td1, td2, td3 = t[i - 1] - t[i - 2], t[i] - t[i - 2], t[i + 1] - t[i]
        v = 0.0
        for X, dX in ((QK, dQK), (QR, dQR)):
            v += np.abs(td2 / 12.0 * (2 * (X[i] - X[i - 2]) - td2 * (dX[i - 1] / td1 + dX[i + 1] / td3))).sum()
        vals.append(v)
    return np.array(vals)


def positive_history(theta: np.ndarray, n: int = 60, T: float = 0.6, t_hi: float = 50.0) -> O.State:
    """QK = (theta t + 1) / (t + 1), QR = 1 / (T (t + 1)) on rows t = 0 and
    logspace(1e-5, t_hi); row k's derivative columns hold h_k times the
    derivative at t_{k-1}."""
    t = np.concatenate([[0.0], np.logspace(-5, np.log10(t_hi), n - 1)])
    tc = t[:, None]
    QK = (theta[None, :] * tc + 1.0) / (tc + 1.0)
    QR = np.broadcast_to(1.0 / (T * (tc + 1.0)), QK.shape).copy()
    h = np.diff(t, prepend=0.0)[:, None]
    tp = np.concatenate([[0.0], t[:-1]])[:, None]
    dQK = h * (theta[None, :] - 1.0) / (tp + 1.0) ** 2
    dQR = np.broadcast_to(-h / (T * (tp + 1.0) ** 2), QK.shape).copy()
    dtr = np.zeros(n)
    dtr[2:] = (t[2:] - t[1:-1]) / (t[1:-1] - t[:-2])
    return O.State(t, dtr, QK.ravel(), QR.ravel(), dQK.ravel(), dQR.ravel(), np.ones(n), np.zeros(n))


def make_log(L: int, Tmax: float, model: O.Model, nsteps: int) -> dict:
    out = {}
    g = O.Reference.grid(L, Tmax=Tmax)
    ref = O.Reference(g, model, threads=1, log_response=True)
    st = positive_history(g.theta)
    out.update({k: v for k, v in state_dict("pos", st).items() if v is not None})
    ref.set_state(st)
    ref.interpolate()
    for w in (1, 3, 5, 7):
        out[f"pos_interp{w}"] = ref.interp(w)
    out["pos_qk"] = ref.qkstep()
    out["pos_qr"] = ref.qrstep()
    ref.set_state(st)
    ref.interpolate()
    out["pos_rk54_err"] = np.array([ref.update(1, 1e-3)])
    out.update(state_dict("pos_rk54", ref.get_state()))
    ref.init_state()
    tr = ref.run(nsteps)
    for k, v in tr.items():
        out[f"ltraj_{k}"] = v
    out.update(state_dict("ltraj_final", ref.get_state()))
    return out


TAIL_ALPHA = 3.0


def tail_row(theta: np.ndarray, qk: np.ndarray) -> np.ndarray:
    """The newest row with its second half replaced by 1 - a (1 - theta)^2 (1 + 1e-5 sin 7 theta)."""
    out = qk.copy()
    h = theta.size // 2
    th = theta[h:]
    out[h:] = 1.0 - TAIL_ALPHA * (1.0 - th) ** 2 * (1.0 + 1e-5 * np.sin(7.0 * th))
    return out


def tail_states(mid: O.State, theta: np.ndarray) -> tuple:
    """State A (mid with tail_row in its newest row) and B (A plus one row)."""
    L = theta.size
    QK = mid.QK.copy()
    QK[-L:] = tail_row(theta, QK[-L:])
    a = O.State(mid.t1grid.copy(), mid.dtr.copy(), QK, mid.QR.copy(), mid.dQK.copy(), mid.dQR.copy(),
                mid.rvec.copy(), mid.drvec.copy())
    t = mid.t1grid
    tn = t[-1] + 0.5 * (t[-1] - t[-2])
    rowK = 0.999 * QK[-L:] + 0.001
    b = O.State(np.append(t, tn), np.append(mid.dtr, 0.5), np.concatenate([QK, rowK]),
                np.concatenate([mid.QR, mid.QR[-L:]]), np.concatenate([mid.dQK, mid.dQK[-L:]]),
                np.concatenate([mid.dQR, mid.dQR[-L:]]), np.append(mid.rvec, mid.rvec[-1]),
                np.append(mid.drvec, mid.drvec[-1]))
    return a, b


def make_tail(L: int, Tmax: float, model: O.Model, mid: O.State, nsteps: int = 400) -> dict:
    out = {}
    g = O.Reference.grid(L, Tmax=Tmax)
    ref = O.Reference(g, model, threads=1)
    ref.set_tail_fit(True)
    ref.init_state()
    tr = ref.run(nsteps)
    for k, v in tr.items():
        out[f"tft_{k}"] = v
    st = ref.get_state()
    out["tft_t1grid"] = st.t1grid
    out["tft_rvec"] = st.rvec
    out["tft_QK_last"] = st.QK[-L:]
    out["tft_QR_last"] = st.QR[-L:]
    out["tft_rowsum_QK"] = st.QK.reshape(-1, L).sum(axis=1)
    out["tft_rowsum_QR"] = st.QR.reshape(-1, L).sum(axis=1)
    a, b = tail_states(mid, g.theta)
    rows = []
    ref.set_state(a)
    for _ in range(2):
        ref.tail_fit()
        rows.append(ref.get_state().QK[-L:])
    ref.set_state(b)
    for rb in (-1000, 5, -1000):
        O.Reference.lib().dynref_set_rollback_loop(rb)
        ref.tail_fit()
        rows.append(ref.get_state().QK[-L:])
    out["tfs_QK"] = np.array(rows)
    return out


def main():
    if not O.Reference.available():
        O.build(reference=True)
    for L, Tmax, model, nsteps in CASES:
        data = make(L, Tmax, model, nsteps)
        path = os.path.join(HERE, f"golden_L{L}.npz")
        np.savez_compressed(path, **data)
        print(path, os.path.getsize(path))
    L, Tmax, model, nsteps = CASES[1]
    path = os.path.join(HERE, f"golden_log_L{L}.npz")
    np.savez_compressed(path, **make_log(L, Tmax, model, nsteps))
    print(path, os.path.getsize(path))
    with np.load(os.path.join(HERE, f"golden_L{L}.npz")) as f:
        mid = O.State(*(f[f"mid_{k}"] for k in ("t1grid", "dtr", "QK", "QR", "dQK", "dQR", "rvec", "drvec")))
    path = os.path.join(HERE, f"golden_tail_L{L}.npz")
    np.savez_compressed(path, **make_tail(L, Tmax, model, mid))
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
