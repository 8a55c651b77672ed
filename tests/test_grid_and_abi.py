"""Native grid generator vs the reference generator's tables, the RG-Evo text
format round trip, and the C-ABI library surface (no GPU)."""
import ctypes as C
import os
import platform
import re

import numpy as np
import pytest

from conftest import ROOT, load_golden

FIELDS = ("theta", "phi1", "phi2", "integ", "indsA1", "wA1", "indsA2", "wA2", "indsB2", "wB2")


@pytest.mark.parametrize("L,Tmax", [(32, 10.0), (64, 100.0)])
def test_generator_matches_reference_golden(product_built, L, Tmax):
    g = product_built.grid.generate(L, Tmax=Tmax, cache=False)
    gold = load_golden(L)
    exact = platform.machine() in ("x86_64", "AMD64")
    for f in FIELDS:
        a, b = getattr(g, f), gold[f"grid_{f}"]
        if f.startswith("inds") or exact:
            np.testing.assert_array_equal(a, b, err_msg=f)
        else:  # 128-bit long double on aarch64: last-bit differences only
            np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-13, err_msg=f)


def test_generator_invariants(product_built):
    """theta spans [0,1]; quadrature integrates 1; poly-9 stencils reproduce
    monomials up to degree 9 (the reference's own invariant,
    src/grid/test_interpolation_weights.cpp:36-66, tolerance 5e-13)."""
    g = product_built.grid.generate(128, Tmax=1e5, cache=False)
    L, m = g.L, g.depth
    assert g.theta[0] == 0.0 and g.theta[-1] == 1.0 and np.all(np.diff(g.theta) >= 0)
    assert abs(g.integ.sum() - 1.0) < 1e-12
    xq = g.phi1
    w = g.wA1.reshape(L * L, m)
    idx = g.indsA1[:, None] + np.arange(m)[None, :]
    for d in range(0, 10):
        approx = (w * g.theta[idx] ** d).sum(axis=1)
        assert np.max(np.abs(approx - xq ** d)) < 5e-13, d


@pytest.mark.parametrize("L,order,window", [(64, 9, 0), (80, 5, 12), (128, 9, 14)])
def test_rational_generator_matches_reference(product_built, oracle_built, L, order, window):
    """-m rational (Floater-Hormann stencils, grid_cli.cpp:104-141, 198-206) against the
    reference generator compiled here: every table bit for bit."""
    import oracle as O
    if not O.Reference.available():
        pytest.skip("compiled reference not present")
    g = product_built.grid.generate(L, Tmax=1e3, interp_order=order, method="rational", fh_window=window,
                                    cache=False)
    r = O.Reference.grid(L, Tmax=1e3, interp_order=order, method="rational", fh_window=window)
    assert g.depth == max(order + 1, window)
    for f in FIELDS:
        np.testing.assert_array_equal(getattr(g, f), getattr(r, f), err_msg=f)


def test_rational_stencils_reproduce_low_degree_polynomials(product_built):
    """A Floater-Hormann interpolant of order d reproduces polynomials of degree <= d
    (and the polynomial fallback, of degree m - 1 >= d, does too)."""
    L, d = 96, 5
    g = product_built.grid.generate(L, Tmax=1e3, interp_order=d, method="rational", fh_window=12, cache=False)
    m = g.depth
    w = g.wA2.reshape(L * L, m)
    idx = g.indsA2[:, None] + np.arange(m)[None, :]
    np.testing.assert_allclose(w.sum(axis=1), 1.0, atol=1e-13)
    for k in range(1, d + 1):
        assert np.max(np.abs((w * g.theta[idx] ** k).sum(axis=1) - g.phi2 ** k)) < 1e-11, k
    with pytest.raises(ValueError):
        product_built.grid.generate(32, method="bspline")


@pytest.mark.parametrize("L,Tmax,alpha,delta", [(32, 10.0, 0.0, 0.0), (128, 1e5, 0.0, 0.0), (96, 1e3, 0.3, 0.2)])
def test_position_grids_match_reference(product_built, oracle_built, L, Tmax, alpha, delta):
    """posA1y/posA2y/posB2y (pos_grid.cpp:111-205, the inverse theta map through 20 L
    samples and 12-node barycentric windows) bit for bit, with and without the
    index remap (alpha, delta)."""
    import oracle as O
    if not O.Reference.available():
        pytest.skip("compiled reference not present")
    ours = product_built.grid.positions(L, Tmax, alpha, delta)
    ref = O.Reference.grid_positions(L, Tmax, alpha, delta)
    for a, b, name in zip(ours, ref, ("posA1y", "posA2y", "posB2y")):
        np.testing.assert_array_equal(a, b, err_msg=name)


def test_saved_grid_directory_is_complete(product_built, tmp_path):
    """save() of a generated grid writes every file the reference's solver checks for
    before it runs (initialization.cpp:40-62) and grid_params.txt (grid_io.cpp:205-228)."""
    G = product_built.grid
    g = G.generate(32, Tmax=10.0, method="rational", fh_window=12, cache=False)
    d = tmp_path / "32"
    G.save(g, str(d))
    for f in ("theta.dat", "phi1.dat", "phi2.dat", "int.dat", "indsA1y.dat", "weightsA1y.dat", "indsA2y.dat",
              "weightsA2y.dat", "indsB2y.dat", "weightsB2y.dat", "posA1y.dat", "posA2y.dat", "posB2y.dat"):
        assert (d / f).exists(), f
    params = (d / "grid_params.txt").read_text().splitlines()
    assert params[:2] == ["# DYNAMITE grid generation parameters", "len=32"]
    assert "Tmax=1.00000000000000000e+01" in params and "interp_method=rational" in params
    assert "fh_stencil=12" in params and "subdir=32" in params
    pos = np.loadtxt(d / "posB2y.dat", delimiter="\t").ravel()
    np.testing.assert_array_equal(pos, G.positions(32, 10.0)[2])
    back = G.load(str(d))
    for f in FIELDS:
        np.testing.assert_array_equal(getattr(g, f), getattr(back, f), err_msg=f)


def test_validate_mode(product_built, tmp_path):
    """`RG-Evo grid -V` (grid_cli.cpp:235-256): a saved grid validates; a perturbed phi2 or
    int.dat entry, or a missing file, fails."""
    G = product_built.grid
    g = G.generate(32, Tmax=10.0, cache=False)
    d = tmp_path / "32"
    G.save(g, str(d))
    assert G.validate(str(d), 32, Tmax=10.0)["ok"]
    assert not G.validate(str(d), 32, Tmax=100.0)["ok"]
    phi2 = g.phi2.copy()
    phi2[5] += 1e-12
    np.savetxt(d / "phi2.dat", phi2.reshape(32, 32), fmt="%.17e", delimiter="\t")
    r = G.validate(str(d), 32, Tmax=10.0)
    assert not r["ok"] and r["mismatches"] == 1
    (d / "int.dat").unlink()
    assert not G.validate(str(d), 32, Tmax=10.0)["ok"]


def test_text_format_round_trip(product_built, tmp_path):
    g = product_built.grid.generate(32, Tmax=10.0, cache=False)
    product_built.grid.save(g, str(tmp_path))
    h = product_built.grid.load(str(tmp_path))
    for f in FIELDS:
        np.testing.assert_array_equal(getattr(g, f), getattr(h, f), err_msg=f)


def _declared_symbols():
    with open(os.path.join(ROOT, "include", "dyn.h")) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"^\s*(?:dyn_status|int|const char\*)\s+(dyn_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(product_built):
    lib = C.CDLL(product_built._lib.LIB_PATH)
    names = _declared_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.dyn_abi_version() == 5


def test_invalid_arguments_rejected_without_touching_the_gpu(product_built):
    L = product_built.lib()
    h = C.c_void_p()
    assert L.dyn_ctx_create(None, None, C.byref(h)) == -1
    assert b"null" in L.dyn_last_error()
    assert L.dyn_update(None, 1, 1e-3, None) == -1
    assert L.dyn_sparsify(None, 1e-10, 0, None) == -1
    assert L.dyn_tail_fit(None, -1000, None) == -1
    assert L.dyn_state_time(None, None) == -1
    # the generator: null tables and impossible sizes
    assert L.dyn_grid_generate(32, 10.0, 5, 9, 0.0, 0.0, *([None] * 10)) == -1
    assert L.dyn_grid_positions(2, 10.0, 0.0, 0.0, None, None, None) == -1
    assert L.dyn_grid_rational_depth(32, 9, 40) == 32 and L.dyn_grid_rational_depth(64, 5, 0) == 6


def test_missing_library_raises(monkeypatch, tmp_path):
    """No fallback: without the native library every numeric call fails loudly."""
    from dynamite_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(_lib.DynError):
        _lib.lib()


def test_batch_and_adjoint_arguments_rejected_without_touching_the_gpu(product_built):
    """Bad batch configurations and quenches, and adjoint calls on a null context, fail
    with DYN_ERR_INVALID before any CUDA call."""
    D = product_built
    from dynamite_gb300 import _lib
    g = D.grid.generate(32)
    for bad in (dict(p=1), dict(grid=3), dict(delta_max=0.0), dict(capacity=1)):
        with pytest.raises(_lib.DynError):
            D.Batch([g], [D.Quench(**bad)])
    with pytest.raises(KeyError):
        D.Batch([g], [D.Quench()], precision="fp64")       # batches run the mixed forms only
    # a sparsify variant out of range, through the C ABI
    cfg = _lib.BatchConfig(0, None, 0, 0, 32, 128, 1, 0, 100, 1, 7, 1)
    qs = (_lib.BatchQuench * 1)(_lib.BatchQuench(0, 3, 4, 0.5, 1e50, 0.6, 1e-5, 1e-10, 0.0, 0.0, 0, 64))
    gs = (_lib.BatchGrid * 1)()
    h = C.c_void_p()
    L = D.lib()
    assert L.dyn_batch_create(C.byref(cfg), gs, 1, qs, 1, C.byref(h)) == -1
    assert b"sparsify variant" in L.dyn_last_error()
    assert L.dyn_adjoint_forward(None, None, None) == -1
    assert L.dyn_adjoint_backward(None, None, None, None) == -1
    assert L.dyn_batch_run(None, 1, None) == -1


STRUCTS = [("Config", "dyn_config"), ("Tables", "dyn_tables"), ("StateC", "dyn_state"),
           ("Controller", "dyn_controller"), ("StepResult", "dyn_step_result"), ("RunParams", "dyn_run_params"),
           ("TailInfo", "dyn_tail_info"), ("NoAllocRHS", "dyn_noalloc_rhs"), ("BatchGrid", "dyn_batch_grid"),
           ("BatchQuench", "dyn_batch_quench"), ("BatchConfig", "dyn_batch_config"), ("BatchInfo", "dyn_batch_info"),
           ("AdjointObjective", "dyn_adjoint_objective"), ("AdjointStats", "dyn_adjoint_stats"),
           ("StateDev", "dyn_state_dev")]


def test_ctypes_structs_match_the_header(tmp_path):
    """Every ctypes mirror of an include/dyn.h struct has the C compiler's size and field
    offsets (a field added on one side only would shift the rest silently)."""
    import shutil
    import subprocess
    from dynamite_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    c_name = {"lam": "lambda"}  # Python keyword
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "dyn.h"', "int main(void) {"]
    for py, c in STRUCTS:
        lines.append(f'printf("{py} size %zu\\n", sizeof({c}));')
        for name, _ in getattr(_lib, py)._fields_:
            lines.append(f'printf("{py} {name} %zu\\n", offsetof({c}, {c_name.get(name, name)}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                                 text=True).stdout.splitlines())
    for py, _ in STRUCTS:
        S = getattr(_lib, py)
        assert int(got[f"{py} size"]) == C.sizeof(S), py
        for name, _ in S._fields_:
            assert int(got[f"{py} {name}"]) == getattr(S, name).offset, (py, name)
