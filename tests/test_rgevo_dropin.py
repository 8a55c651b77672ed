"""RG-Evo, the reference driver, built with this library in place of its hot path (no GPU).

`make -C oracle rgevo` compiles every reference source of RG-Evo's GPU build except
the hot-path CUDA files (src/{interpolation,convolution,EOMs,search,sparsify}/*.cu and
src/math/math_{ops,sigma}.cu, CMakeLists.txt:184-202), adds the drop-in layer
dynamite_gb300/shim/rgevo_shim.cu and links against libdynamite_gb300.so.  The link
succeeding is the check that the layer supplies every hot-path symbol the rest of
RG-Evo calls (interpolateGPU, updateGPU, the RK entry points and their init_*,
energyGPU, sparsifyNscaleGPU / sparsifyNscale and the device function DflambdaGPU);
the binary then starts and prints its version (`RG-Evo -v` needs no GPU).  Needs the
reference sources: the test is skipped where they are absent.  The state exchange the
layer makes on every call (dyn_state_upload_dev and friends) runs on the GPU in
test_gpu_state_dev.py.
"""
import os
import subprocess

import pytest

import oracle

REF = oracle.reference_dir()
pytestmark = pytest.mark.skipif(REF is None, reason="needs the reference sources (DYN_REFERENCE_DIR)")

EXE = os.path.join(oracle.HERE, "_ref", "rgevo", "RG-Evo")
# hot-path functions the rest of RG-Evo calls, now from the drop-in layer
CALLED = ["interpolateGPU(double const*, double const*, bool, StreamPool*)", "updateGPU(StreamPool*)",
          "RK54GPU(StreamPool*)", "SSPRK104GPU(StreamPool*)", "SERK2GPU(int, StreamPool*)", "init_RK54GPU()",
          "init_SSPRK104GPU()", "init_SERK2(int)", "sparsifyNscaleGPU(double, CUstream_st*)",
          "sparsifyNscale(double)"]
# kernels and helpers that live only in the hot-path CUDA files left out of the build
ABSENT = ["computeSparsifyFlags", "ConvAGPUKernel", "bsearch_interp_kernel", "computeSigmaKandRKernel",
          "diffNfloorKernel", "QKRstepGPU"]


@pytest.fixture(scope="module")
def rgevo(product_built):
    subprocess.run(["make", "-s", "-C", oracle.HERE, "rgevo", f"-j{os.cpu_count() or 4}"], check=True,
                   capture_output=True)
    return EXE


def _nm(*args):
    return subprocess.run(["nm", "-C", *args, EXE], check=True, capture_output=True, text=True).stdout


def test_rgevo_links_without_its_hot_path(rgevo):
    defined = _nm("--defined-only")
    for sig in CALLED:
        assert f" T {sig}" in defined, sig
    assert " T energyGPU(" in defined
    for name in ABSENT:
        assert name not in defined, name
    undefined = [ln.split()[-1] for ln in _nm("-u").splitlines() if ln.strip()]
    ours = [u for u in undefined if u.startswith("dyn_")]
    assert {"dyn_update", "dyn_ctx_create", "dyn_state_upload_dev", "dyn_sparsify"} <= set(ours)
    # nothing of the hot path is left unresolved: only the library's C ABI and system symbols
    assert not [u for u in undefined if not u.startswith("dyn_") and ("GPU" in u or "sparsify" in u.lower())]


def test_rgevo_starts(rgevo):
    # -v prints the version and leaves through the parser's "stop" path, status 1
    # (config.cpp:119-121, main.cpp:64-66; the reference's CI runs `RG-Evo -v || true`)
    r = subprocess.run([rgevo, "-v"], capture_output=True, text=True, timeout=60)
    assert r.returncode in (0, 1), r.stderr
    assert "DYNAMITE" in r.stdout and "Version" in r.stdout
    ldd = subprocess.run(["ldd", rgevo], capture_output=True, text=True).stdout
    assert "libdynamite_gb300.so" in ldd
