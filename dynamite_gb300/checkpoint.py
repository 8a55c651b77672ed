"""RG-Evo's binary checkpoint `data.bin` (io_save_binary.cpp:66-99, read back by
io_input.cpp:112-175), so states move between the reference and this library:
resume a reference run here, or hand one of ours back to RG-Evo.  Also the
"compressed" outputs a save writes beside it (io_save_compressed.cpp:17-63) and
the per-step log correlation.txt (simulation_runner.cpp:83-91, 326-340).

Layout (native byte order, as the reference writes it with `ofstream::write`):

    int32   header version (1)
    uint64  n  (rows of t1grid)          uint64 L
    int32   p        int32 p2
    float64 lambda, T0, Gamma, delta, delta_t
    int32   loop
    float64 energy
    float64 t1grid[n], QK[n*L], QR[n*L], dQK[n*L], dQR[n*L], rvec[n], drvec[n]

delta_t_ratio is not stored: the reader rebuilds it as the reference's loader
does (io_input.cpp:169-172): entries 0 and 1 are 0, entry i >= 2 is
(t_i - t_{i-1}) / (t_{i-1} - t_{i-2}).
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass

import numpy as np

from .simulation import State

_HEAD = struct.Struct("=iQQiidddddid")  # version, n, L, p, p2, lambda, T0, Gamma, delta, delta_t, loop, energy


@dataclass
class CheckpointParams:
    p: int
    p2: int
    lam: float
    T0: float
    Gamma: float
    delta: float       # controller error of the last step
    delta_t: float     # next step size
    loop: int
    energy: float      # E at the last row (the writer's own evaluation)


def delta_t_ratio(t1grid: np.ndarray) -> np.ndarray:
    """The ratio column as the reference's binary loader rebuilds it."""
    t = np.asarray(t1grid, dtype=np.float64)
    r = np.zeros(t.size)
    if t.size > 2:
        r[2:] = (t[2:] - t[1:-1]) / (t[1:-1] - t[:-2])
    return r


def save(path: str, state: State, params: CheckpointParams) -> None:
    n = int(np.asarray(state.t1grid).size)
    L = int(np.asarray(state.QK).size // max(n, 1))
    with open(path, "wb") as fh:
        fh.write(_HEAD.pack(1, n, L, params.p, params.p2, params.lam, params.T0, params.Gamma, params.delta,
                            params.delta_t, params.loop, params.energy))
        for name, count in (("t1grid", n), ("QK", n * L), ("QR", n * L), ("dQK", n * L), ("dQR", n * L),
                            ("rvec", n), ("drvec", n)):
            a = np.ascontiguousarray(getattr(state, name), dtype=np.float64)
            if a.size != count:
                raise ValueError(f"{name}: {a.size} values, the layout needs {count}")
            fh.write(a.tobytes())


def load(path: str) -> tuple[State, CheckpointParams]:
    with open(path, "rb") as fh:
        raw = fh.read()
    if len(raw) < _HEAD.size:
        raise ValueError("truncated checkpoint header")
    ver, n, L, p, p2, lam, T0, Gamma, delta, delta_t, loop, energy = _HEAD.unpack_from(raw, 0)
    if ver != 1:
        raise ValueError(f"unsupported checkpoint version {ver}")
    need = _HEAD.size + 8 * (3 * n + 4 * n * L)
    if len(raw) < need:
        raise ValueError(f"truncated checkpoint: {len(raw)} bytes, the header promises {need}")
    off = _HEAD.size
    arrays = {}
    for name, count in (("t1grid", n), ("QK", n * L), ("QR", n * L), ("dQK", n * L), ("dQR", n * L),
                        ("rvec", n), ("drvec", n)):
        arrays[name] = np.frombuffer(raw, dtype=np.float64, count=count, offset=off).copy()
        off += 8 * count
    st = State(arrays["t1grid"], delta_t_ratio(arrays["t1grid"]), arrays["QK"], arrays["QR"], arrays["dQK"],
               arrays["dQR"], arrays["rvec"], arrays["drvec"])
    return st, CheckpointParams(p, p2, lam, T0, Gamma, delta, delta_t, loop, energy)


def save_compressed(dir_path: str, QKB1: np.ndarray, QRB1: np.ndarray, theta: np.ndarray, t_last: float) -> None:
    """QK_compressed / QR_compressed (uint64 rows, uint64 cols, then the L x L B1
    interpolation, row i = theta_i t) and t1_compressed.txt (t theta_i, fixed with
    16 decimals), as io_save_compressed.cpp:17-63 writes them."""
    L = int(np.asarray(theta).size)
    for name, a in (("QK_compressed", QKB1), ("QR_compressed", QRB1)):
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size != L * L:
            raise ValueError(f"{name}: {a.size} values, the layout needs {L * L}")
        with open(os.path.join(dir_path, name), "wb") as fh:
            fh.write(struct.pack("=QQ", L, L))
            fh.write(a.tobytes())
    with open(os.path.join(dir_path, "t1_compressed.txt"), "w") as fh:
        fh.writelines(f"{t_last * th:.16f}\n" for th in np.asarray(theta, dtype=np.float64))


def load_compressed(dir_path: str) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(QKB1, QRB1, t theta) from the three compressed files."""
    out = []
    for name in ("QK_compressed", "QR_compressed"):
        with open(os.path.join(dir_path, name), "rb") as fh:
            raw = fh.read()
        if len(raw) < 16:
            raise ValueError(f"{name}: truncated header")
        rows, cols = struct.unpack_from("=QQ", raw, 0)
        if len(raw) != 16 + 8 * rows * cols:
            raise ValueError(f"{name}: {len(raw)} bytes, the header promises {16 + 8 * rows * cols}")
        out.append(np.frombuffer(raw, dtype=np.float64, offset=16).reshape(rows, cols).copy())
    t = np.loadtxt(os.path.join(dir_path, "t1_compressed.txt"), dtype=np.float64, ndmin=1)
    return out[0], out[1], t


def append_correlation(path: str, t, energy, qk0) -> None:
    """Append `t<TAB>E<TAB>QK(t,0)` lines with 14 fixed decimals to correlation.txt, as the
    reference's loop logs every step (simulation_runner.cpp:83-91, 326-340); the
    arrays are `Simulation.run`'s "t", "energy" and "qk0" records."""
    t, energy, qk0 = (np.atleast_1d(np.asarray(a, dtype=np.float64)) for a in (t, energy, qk0))
    if not (t.size == energy.size == qk0.size):
        raise ValueError("t, energy and qk0 must have the same length")
    with open(path, "a") as fh:
        fh.writelines(f"{a:.14f}\t{b:.14f}\t{c:.14f}\n" for a, b, c in zip(t, energy, qk0))
