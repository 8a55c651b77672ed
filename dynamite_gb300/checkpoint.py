"""RG-Evo's binary checkpoint `data.bin` (io_save_binary.cpp:66-99, read back by
io_input.cpp:112-175), so states move between the reference and this library:
resume a reference run here, or hand one of ours back to RG-Evo.

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
