"""Host-side failure detection (no GPU): damaged grid tables and model parameters are
refused by the C ABI before any CUDA call, and a damaged Grid_data directory is refused
by the loader.  The reference reads the same files and parameters unchecked
(io_input.cpp:90-110, config.cpp:21-229), so a bad stencil start there becomes an
out-of-range history read on the GPU; here it is DYN_ERR_INVALID with a reason.

The GPU-side outcomes (a state with NaN refused at upload, an overflowing state
stopping dyn_run with DYN_ERR_NONFINITE and a batch quench with status "failed") are
in test_gpu_failures.py."""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

from dynamite_gb300 import _lib


def _tables(g):
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (g.theta, g.phi2, g.integ, g.wA1, g.wA2, g.wB2)]
    i64 = [np.ascontiguousarray(a, dtype=np.int64) for a in (g.indsA1, g.indsA2, g.indsB2)]
    tb = _lib.Tables(_lib.ptr(keep[0]), _lib.ptr(keep[1]), _lib.ptr(keep[2]),
                     *[a.ctypes.data_as(_lib.i64p) for a in i64], *[_lib.ptr(a) for a in keep[3:]])
    return tb, keep, i64


def _damaged(g, what):
    """A copy of grid g with one defect."""
    import dataclasses
    h = dataclasses.replace(g, **{k: np.array(getattr(g, k), copy=True) for k in
                                  ("theta", "phi2", "integ", "indsA1", "indsA2", "indsB2", "wA1", "wA2", "wB2")})
    L, m = g.L, g.depth
    if what == "start_past_end":
        h.indsB2[L * L // 2] = L - m + 1       # the last tap would read column L
    elif what == "negative_start":
        h.indsA1[7] = -1
    elif what == "theta_not_ending_at_1":
        h.theta[-1] = 0.999
    elif what == "theta_decreasing":
        h.theta[5], h.theta[6] = h.theta[6], h.theta[5] + 1e-3
    elif what == "phi2_outside":
        h.phi2[3] = 1.5
    elif what == "nan_weight":
        h.wA2[11] = np.nan
    elif what == "inf_integ":
        h.integ[2] = np.inf
    return h


DEFECTS = ["start_past_end", "negative_start", "theta_not_ending_at_1", "theta_decreasing", "phi2_outside",
           "nan_weight", "inf_integ"]
REASONS = {"start_past_end": b"stencil start", "negative_start": b"stencil start", "theta_not_ending_at_1": b"theta",
           "theta_decreasing": b"theta", "phi2_outside": b"phi2", "nan_weight": b"weight", "inf_integ": b"int.dat"}


def test_good_tables_pass(product_built):
    g = product_built.grid.generate(32)
    tb, *_ = _tables(g)
    assert product_built.lib().dyn_check_tables(32, g.depth, C.byref(tb)) == 0


@pytest.mark.parametrize("what", DEFECTS)
def test_damaged_tables_rejected_by_check_and_create(product_built, what):
    D = product_built
    g = _damaged(D.grid.generate(32), what)
    L = D.lib()
    tb, *_ = _tables(g)
    assert L.dyn_check_tables(32, g.depth, C.byref(tb)) == _lib.DYN_ERR_INVALID
    assert REASONS[what] in L.dyn_last_error()
    # the context and the batch refuse the same tables before they touch a device
    with pytest.raises(_lib.DynError) as e:
        D.Simulation(g, D.Model())
    assert e.value.status == _lib.DYN_ERR_INVALID
    with pytest.raises(_lib.DynError) as e:
        D.Batch([g], [D.Quench()])
    assert e.value.status == _lib.DYN_ERR_INVALID
    assert REASONS[what] in L.dyn_last_error()


@pytest.mark.parametrize("bad", [dict(T0=0.0), dict(T0=-1.0), dict(Gamma=float("nan")), dict(lam=float("inf")),
                                 dict(p=-1), dict(p2=65)])
def test_bad_model_rejected_before_any_cuda_call(product_built, bad):
    D = product_built
    g = D.grid.generate(32)
    with pytest.raises(_lib.DynError) as e:
        D.Simulation(g, D.Model(**bad))
    assert e.value.status == _lib.DYN_ERR_INVALID


def test_damaged_grid_directory_rejected(product_built, tmp_path):
    """A Grid_data/<L>/ directory with a truncated weights file, a stencil start past the
    end, a non-numeric token or a missing file is refused by grid.load."""
    D = product_built
    g = D.grid.generate(32)
    good = str(tmp_path / "good")
    D.grid.save(g, good)
    back = D.grid.load(good)
    np.testing.assert_array_equal(back.indsB2, g.indsB2)

    def variant(name, edit):
        d = str(tmp_path / name)
        shutil.copytree(good, d)
        edit(d)
        return d

    def truncate(d):
        p = os.path.join(d, "weightsA2y.dat")
        lines = open(p).read().splitlines()
        open(p, "w").write("\n".join(lines[: len(lines) - 7]) + "\n")

    def bad_start(d):
        p = os.path.join(d, "indsA1y.dat")
        rows = open(p).read().splitlines()
        cols = rows[3].split("\t")
        cols[4] = str(32)
        rows[3] = "\t".join(cols)
        open(p, "w").write("\n".join(rows) + "\n")

    def garbage(d):
        p = os.path.join(d, "int.dat")
        lines = open(p).read().splitlines()
        lines[2] = "1.0e-3x"
        open(p, "w").write("\n".join(lines) + "\n")

    for name, edit, exc, msg in (("trunc", truncate, ValueError, "wA2"), ("start", bad_start, ValueError, "stencil"),
                                 ("garbage", garbage, ValueError, None),
                                 ("missing", lambda d: os.remove(os.path.join(d, "indsB2y.dat")), OSError, None)):
        with pytest.raises(exc) as e:
            D.grid.load(variant(name, edit))
        if msg:
            assert msg in str(e.value)


def test_status_codes_match_the_header():
    """The Python side's status constants are the header's."""
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    text = open(os.path.join(root, "include", "dyn.h")).read()
    codes = dict((k, int(v)) for k, v in re.findall(r"(DYN_ERR_\w+)\s*=\s*(-?\d+)", text))
    for k, v in codes.items():
        assert getattr(_lib, k) == v, k
    assert "DYN_ERR_TIMEOUT" not in codes
