"""RG-Evo's data.bin checkpoint (io_save_binary.cpp:66-99, io_input.cpp:112-175): the
byte layout the reference writes, a round trip, the loader's delta_t_ratio rule, and
rejection of damaged files (no GPU)."""
import struct

import numpy as np
import pytest

from dynamite_gb300 import checkpoint as ck
from dynamite_gb300.simulation import State

from conftest import load_golden
from helpers import STATE_FIELDS, state_from


def _params():
    return ck.CheckpointParams(p=3, p2=4, lam=0.5, T0=1e50, Gamma=0.6, delta=3e-11, delta_t=2.5e-3, loop=120,
                               energy=-0.75)


def test_layout_matches_the_reference_writer(tmp_path):
    g = load_golden(32)
    st = state_from(g, "traj_final", State, with_pos=False)
    path = tmp_path / "data.bin"
    ck.save(str(path), st, _params())
    raw = path.read_bytes()
    n, L = st.t1grid.size, 32
    # io_save_binary.cpp:66-80: version, t1grid size, len, p, p2, lambda, T0, Gamma, delta, delta_t, loop, energy
    ver, = struct.unpack_from("=i", raw, 0)
    nn, ll = struct.unpack_from("=QQ", raw, 4)
    p, p2 = struct.unpack_from("=ii", raw, 20)
    lam, T0, Gamma, delta, dt = struct.unpack_from("=ddddd", raw, 28)
    loop, = struct.unpack_from("=i", raw, 68)
    energy, = struct.unpack_from("=d", raw, 72)
    assert (ver, nn, ll, p, p2, loop) == (1, n, L, 3, 4, 120)
    assert (lam, T0, Gamma, delta, dt, energy) == (0.5, 1e50, 0.6, 3e-11, 2.5e-3, -0.75)
    # :83-98: t1grid, QK, QR, dQK, dQR, rvec, drvec
    assert len(raw) == 80 + 8 * (3 * n + 4 * n * L)
    np.testing.assert_array_equal(np.frombuffer(raw, np.float64, n, 80), st.t1grid)
    np.testing.assert_array_equal(np.frombuffer(raw, np.float64, n, 80 + 8 * (n + 4 * n * L) + 8 * n), st.drvec)


def test_round_trip_and_ratio_rule(tmp_path):
    g = load_golden(64)
    st = state_from(g, "traj_final", State, with_pos=False)
    path = str(tmp_path / "data.bin")
    ck.save(path, st, _params())
    back, prm = ck.load(path)
    for f in STATE_FIELDS:
        if f != "dtr":
            np.testing.assert_array_equal(getattr(back, f), getattr(st, f), err_msg=f)
    assert prm == _params()
    # io_input.cpp:169-172: entries 0 and 1 are zero, the rest from the time grid
    t = st.t1grid
    assert back.dtr[0] == 0.0 and back.dtr[1] == 0.0
    np.testing.assert_array_equal(back.dtr[2:], (t[2:] - t[1:-1]) / (t[1:-1] - t[:-2]))


def test_damaged_files_rejected(tmp_path):
    g = load_golden(32)
    st = state_from(g, "traj_final", State, with_pos=False)
    path = tmp_path / "data.bin"
    ck.save(str(path), st, _params())
    raw = path.read_bytes()
    (tmp_path / "short.bin").write_bytes(raw[:-8])
    with pytest.raises(ValueError):
        ck.load(str(tmp_path / "short.bin"))
    (tmp_path / "v2.bin").write_bytes(struct.pack("=i", 2) + raw[4:])
    with pytest.raises(ValueError):
        ck.load(str(tmp_path / "v2.bin"))
    bad = State(st.t1grid, st.dtr, st.QK[:-1], st.QR, st.dQK, st.dQR, st.rvec, st.drvec)
    with pytest.raises(ValueError):
        ck.save(str(tmp_path / "x.bin"), bad, _params())


def test_compressed_outputs_layout_and_round_trip(tmp_path):
    """io_save_compressed.cpp:17-63: uint64 rows and cols, then L*L doubles of the B1
    interpolation; t1_compressed.txt holds t theta_i with 16 fixed decimals."""
    L = 8
    rng = np.random.default_rng(3)
    qk, qr = rng.standard_normal(L * L), rng.standard_normal(L * L)
    theta = np.linspace(0.0, 1.0, L)
    ck.save_compressed(str(tmp_path), qk, qr, theta, 12.5)
    raw = (tmp_path / "QK_compressed").read_bytes()
    assert struct.unpack_from("=QQ", raw, 0) == (L, L) and len(raw) == 16 + 8 * L * L
    np.testing.assert_array_equal(np.frombuffer(raw, dtype=np.float64, offset=16), qk)
    lines = (tmp_path / "t1_compressed.txt").read_text().splitlines()
    assert lines[0] == "0.0000000000000000" and lines[-1] == "12.5000000000000000"
    a, b, t = ck.load_compressed(str(tmp_path))
    np.testing.assert_array_equal(a.ravel(), qk)
    np.testing.assert_array_equal(b.ravel(), qr)
    np.testing.assert_array_equal(t, 12.5 * theta)
    with pytest.raises(ValueError):
        ck.save_compressed(str(tmp_path), qk[:-1], qr, theta, 1.0)
    (tmp_path / "QK_compressed").write_bytes(raw[:-8])
    with pytest.raises(ValueError):
        ck.load_compressed(str(tmp_path))


def test_correlation_log_format(tmp_path):
    """simulation_runner.cpp:83-91, 326-340: appended lines, std::fixed, 14 decimals."""
    path = str(tmp_path / "correlation.txt")
    ck.append_correlation(path, [1e-5, 2.5], [-0.125, -1.0 / 3.0], [1.0, 0.75])
    ck.append_correlation(path, 3.0, -0.5, 0.5)
    lines = open(path).read().splitlines()
    assert lines == ["0.00001000000000\t-0.12500000000000\t1.00000000000000",
                     "2.50000000000000\t-0.33333333333333\t0.75000000000000",
                     "3.00000000000000\t-0.50000000000000\t0.50000000000000"]
    with pytest.raises(ValueError):
        ck.append_correlation(path, [1.0, 2.0], [1.0], [1.0])
