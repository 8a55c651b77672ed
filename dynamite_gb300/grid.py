"""Stencil/quadrature tables: generation (native) and the RG-Evo text format.

`generate` is the reference's `RG-Evo grid` (grid_cli.cpp:35-258, poly and
rational methods) done by the native generator in the library; `load`/`save`
read and write `Grid_data/<L>/` as the reference does (io_input.cpp:90-110,
grid_io.cpp:26-263, with the position grids and grid_params.txt the reference
checks for, initialization.cpp:40-62), so tables interchange with RG-Evo in both
directions.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class Grid:
    L: int
    theta: np.ndarray
    phi1: np.ndarray
    phi2: np.ndarray
    integ: np.ndarray
    indsA1: np.ndarray
    wA1: np.ndarray
    indsA2: np.ndarray
    wA2: np.ndarray
    indsB2: np.ndarray
    wB2: np.ndarray
    params: dict | None = None  # generation parameters (set by generate)

    @property
    def depth(self) -> int:
        return self.wA1.size // (self.L * self.L)


_CACHE: dict = {}


def generate(L: int, Tmax: float = 1e5, spline_order: int = 5, interp_order: int = 9,
             alpha: float = 0.0, delta: float = 0.0, cache: bool = True, method: str = "poly",
             fh_window: int = 0) -> Grid:
    """`RG-Evo grid -L L -M Tmax -s spline_order -m method -o interp_order [-f fh_window]`:
    method "poly" (local barycentric, depth interp_order + 1) or "rational" (local
    Floater-Hormann of order interp_order on windows of max(interp_order + 1, fh_window)
    points).  The reference's "bspline" tables (global weights, start index -1) are
    metadata its own solver cannot read, so they are not generated."""
    if method not in ("poly", "rational"):
        raise ValueError(f"unknown stencil method {method!r} (poly | rational)")
    key = (L, Tmax, spline_order, interp_order, alpha, delta, method, fh_window)
    if cache and key in _CACHE:
        return _CACHE[key]
    rational = method == "rational"
    m = _lib.lib().dyn_grid_rational_depth(L, interp_order, fh_window) if rational else interp_order + 1
    L2 = L * L
    th, it = np.empty(L), np.empty(L)
    p1, p2 = np.empty(L2), np.empty(L2)
    i1, i2, i3 = (np.empty(L2, dtype=np.int64) for _ in range(3))
    w1, w2, w3 = (np.empty(L2 * m) for _ in range(3))
    i64 = lambda a: a.ctypes.data_as(_lib.i64p)
    tail = (_lib.ptr(th), _lib.ptr(p1), _lib.ptr(p2), _lib.ptr(it), i64(i1), _lib.ptr(w1), i64(i2), _lib.ptr(w2),
            i64(i3), _lib.ptr(w3))
    if rational:
        st = _lib.lib().dyn_grid_generate_rational(L, Tmax, spline_order, interp_order, fh_window, alpha, delta, *tail)
    else:
        st = _lib.lib().dyn_grid_generate(L, Tmax, spline_order, interp_order, alpha, delta, *tail)
    _lib.check(st, "dyn_grid_generate")
    params = dict(len=L, Tmax=Tmax, spline_order=spline_order, interp_method=method, interp_order=max(1, interp_order),
                  fh_stencil=m if rational else 0, alpha=alpha, delta=delta)
    g = Grid(L, th, p1, p2, it, i1, w1, i2, w2, i3, w3, params)
    if cache:
        _CACHE[key] = g
    return g


def positions(L: int, Tmax: float = 1e5, alpha: float = 0.0, delta: float = 0.0):
    """posA1y, posA2y, posB2y (generate_pos_grids, pos_grid.cpp:111-205): the 1-based
    fractional theta index of phi1, phi2 and theta_i / phi2, each L*L."""
    out = [np.empty(L * L) for _ in range(3)]
    _lib.check(_lib.lib().dyn_grid_positions(L, Tmax, alpha, delta, *[_lib.ptr(a) for a in out]),
               "dyn_grid_positions")
    return tuple(out)


def validate(directory: str, L: int, Tmax: float = 1e5, spline_order: int = 5, alpha: float = 0.0,
             delta: float = 0.0) -> dict:
    """`RG-Evo grid -V`: regenerate theta, phi1, phi2 and int.dat and compare them with the
    files in `directory` (phi_grid.cpp:38-72 at 5e-16, integration.cpp:208-227 at 1e-7,
    absolute).  A missing or mis-sized file fails the check."""
    out = dict(ok=False, max_abs_diff=np.inf, mismatches=-1, max_abs_diff_int=np.inf, mismatches_int=-1)
    try:
        th = _read(os.path.join(directory, "theta.dat"))
        p1 = _read(os.path.join(directory, "phi1.dat"))
        p2 = _read(os.path.join(directory, "phi2.dat"))
        wi = _read(os.path.join(directory, "int.dat"))
    except OSError:
        return out
    if th.size != L or p1.size != L * L or p2.size != L * L or wi.size != L:
        return out
    g = generate(L, Tmax, spline_order, 1, alpha, delta, cache=False)
    d = np.abs(np.concatenate([g.theta - th, g.phi1 - p1, g.phi2 - p2]))
    di = np.abs(g.integ - wi)
    out.update(max_abs_diff=float(d.max()), mismatches=int((d > 5e-16).sum()), max_abs_diff_int=float(di.max()),
               mismatches_int=int((di > 1e-7).sum()))
    out["ok"] = out["mismatches"] == 0 and out["mismatches_int"] == 0
    return out


def _read(path: str, dtype=np.float64) -> np.ndarray:
    with open(path, "r") as fh:
        return np.array(fh.read().split(), dtype=dtype)


def check(g: Grid) -> None:
    """Raise ValueError unless the tables are complete and usable: every array of the size
    its length L implies (weights L*L*depth with one depth for the three families), and
    the host-side table check of the library (dyn_check_tables: theta on [0, 1] ending at
    1, stencil starts within [0, L - depth], phi2 within [0, 1] ending at 1, finite
    weights).  The reference reads the same files with no check (io_input.cpp:90-110)."""
    L, L2 = g.L, g.L * g.L
    sizes = dict(theta=L, integ=L, phi1=L2, phi2=L2, indsA1=L2, indsA2=L2, indsB2=L2)
    for name, n in sizes.items():
        a = getattr(g, name)
        if a.size != n:
            raise ValueError(f"grid L={L}: {name} holds {a.size} values, expected {n}")
    if g.wA1.size % L2 or g.wA1.size // L2 < 2:
        raise ValueError(f"grid L={L}: weightsA1y holds {g.wA1.size} values, not L*L*depth with depth >= 2")
    m = g.wA1.size // L2
    for name in ("wA2", "wB2"):
        if getattr(g, name).size != L2 * m:
            raise ValueError(f"grid L={L}: {name} holds {getattr(g, name).size} values, expected {L2 * m}")
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (g.theta, g.phi2, g.integ, g.wA1, g.wA2, g.wB2)]
    i64 = [np.ascontiguousarray(a, dtype=np.int64) for a in (g.indsA1, g.indsA2, g.indsB2)]
    tb = _lib.Tables(_lib.ptr(keep[0]), _lib.ptr(keep[1]), _lib.ptr(keep[2]), *[a.ctypes.data_as(_lib.i64p) for a in i64],
                     *[_lib.ptr(a) for a in keep[3:]])
    if _lib.lib().dyn_check_tables(L, m, tb) != _lib.DYN_OK:
        raise ValueError(f"grid L={L}: " + _lib.lib().dyn_last_error().decode(errors="replace"))


def load(directory: str) -> Grid:
    """Read Grid_data/<L>/ as written by `RG-Evo grid`; a missing, truncated or
    inconsistent table raises (OSError for a missing file, ValueError otherwise)."""
    th = _read(os.path.join(directory, "theta.dat"))
    L = th.size
    if L < 4:
        raise ValueError(f"{directory}: theta.dat holds {L} values (at least 4 needed)")
    p1_path = os.path.join(directory, "phi1.dat")
    p1 = _read(p1_path) if os.path.exists(p1_path) else np.zeros(L * L)
    g = Grid(L, th, p1, _read(os.path.join(directory, "phi2.dat")), _read(os.path.join(directory, "int.dat")),
             _read(os.path.join(directory, "indsA1y.dat"), np.int64), _read(os.path.join(directory, "weightsA1y.dat")),
             _read(os.path.join(directory, "indsA2y.dat"), np.int64), _read(os.path.join(directory, "weightsA2y.dat")),
             _read(os.path.join(directory, "indsB2y.dat"), np.int64), _read(os.path.join(directory, "weightsB2y.dat")))
    check(g)
    return g


def save(g: Grid, directory: str) -> None:
    """Write the tables in RG-Evo's layout (17 digits after the point)."""
    os.makedirs(directory, exist_ok=True)
    L = g.L

    def vec(name, a):
        np.savetxt(os.path.join(directory, name), a, fmt="%.17e")

    def mat(name, a, fmt="%.17e"):
        np.savetxt(os.path.join(directory, name), a.reshape(L, L), fmt=fmt, delimiter="\t")

    vec("theta.dat", g.theta)
    vec("int.dat", g.integ)
    mat("phi1.dat", g.phi1)
    mat("phi2.dat", g.phi2)
    for name, inds, w in (("A1y", g.indsA1, g.wA1), ("A2y", g.indsA2, g.wA2), ("B2y", g.indsB2, g.wB2)):
        mat(f"inds{name}.dat", inds, fmt="%d")
        vec(f"weights{name}.dat", w)
    if g.params is None:
        return
    # the position grids and the provenance file (grid_io.cpp:159-228)
    p = g.params
    for name, a in zip(("posA1y.dat", "posA2y.dat", "posB2y.dat"), positions(L, p["Tmax"], p["alpha"], p["delta"])):
        mat(name, a)
    lines = ["# DYNAMITE grid generation parameters", f"len={L}", f"Tmax={p['Tmax']:.17e}",
             f"spline_order={p['spline_order']}", f"interp_method={p['interp_method']}",
             f"interp_order={p['interp_order']}"]
    if p["fh_stencil"] > 0:
        lines.append(f"fh_stencil={p['fh_stencil']}")
    lines += [f"alpha={p['alpha']:.17e}", f"delta={p['delta']:.17e}",
              f"subdir={os.path.basename(os.path.normpath(directory))}"]
    with open(os.path.join(directory, "grid_params.txt"), "w") as fh:
        fh.write("\n".join(lines) + "\n")


def lagrange_weights(theta, x: float, npts: int = 10):
    """Weights c with c . f(theta) = the degree npts-1 Lagrange interpolant of f at x on the
    npts theta nodes nearest x (the C(t, x t) functional of a history row)."""
    th = np.asarray(theta, dtype=np.float64)
    k0 = int(np.clip(np.searchsorted(th, x) - npts // 2, 0, th.size - npts))
    nodes = th[k0:k0 + npts]
    c = np.zeros(th.size)
    for a in range(npts):
        others = np.delete(nodes, a)
        c[k0 + a] = np.prod((x - others) / (nodes[a] - others))
    return c
