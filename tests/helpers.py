"""Shared helpers for the parity tests (fixtures -> oracle/product objects)."""
import numpy as np

STATE_FIELDS = ("t1grid", "dtr", "QK", "QR", "dQK", "dQR", "rvec", "drvec")


def grid_from(g: dict, cls):
    L = g["grid_theta"].size
    return cls(L, *(g[f"grid_{k}"] for k in
                    ("theta", "phi1", "phi2", "integ", "indsA1", "wA1", "indsA2", "wA2", "indsB2", "wB2")))


def model_from(g: dict, cls):
    p, p2, lam, T0, Gamma, dtmin, dmax, _ = g["model"]
    return cls(p=int(p), p2=int(p2), lam=float(lam), T0=float(T0), Gamma=float(Gamma),
               delta_t_min=float(dtmin), delta_max=float(dmax))


def state_from(g: dict, prefix: str, cls, with_pos=True):
    args = [g[f"{prefix}_{k}"] for k in STATE_FIELDS]
    st = cls(*args)
    if with_pos and hasattr(st, "posB1xOld"):
        st.posB1xOld = g[f"{prefix}_posB1xOld"]
        st.posB2xOld = g[f"{prefix}_posB2xOld"]
    return st


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)
