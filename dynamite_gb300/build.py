"""Build the native library libdynamite_gb300.so in-tree (nvcc, sm_103a).

    python -m dynamite_gb300.build

Translation units compile in parallel; one -gencode (compute_103a/sm_103a).
The output lands in dynamite_gb300/_build/ next to the sources, where the
package loads it from.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdynamite_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CU_SOURCES = ["dyn_kernels.cu", "dyn_api.cu", "dyn_mixed.cu", "dyn_batch.cu", "dyn_adjoint.cu", "dyn_noalloc.cu",
              "dyn_tail.cu"]
CXX_SOURCES = ["dyn_grid.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build dynamite_gb300")


def _sources():
    cu = [s for s in CU_SOURCES if os.path.exists(os.path.join(SRC, s))]
    cxx = [s for s in CXX_SOURCES if os.path.exists(os.path.join(SRC, s))]
    return cu, cxx


def _digest(files) -> str:
    h = hashlib.sha256()
    for f in sorted(files):
        with open(f, "rb") as fh:
            h.update(f.encode())
            h.update(fh.read())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(OUT, exist_ok=True)
    cu, cxx = _sources()
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(INCLUDE, "dyn.h")]
    stamp = os.path.join(OUT, "stamp")
    extra = os.environ.get("DYN_NVCC_EXTRA", "").split()  # e.g. -DDYN_BATCH_TPSM=1152 for tuning builds
    dig = _digest(deps) + os.uname().machine + " ".join(extra)
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        return LIB
    # host code: IEEE arithmetic as written (no FMA contraction on any host ISA), so the
    # host-side time grid matches the reference's -ffp-contract=off build everywhere
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp", "-Xcompiler", "-ffp-contract=off",
              f"-I{INCLUDE}"]
    jobs = []
    for s in cu:
        obj = os.path.join(OUT, s + ".o")
        jobs.append([nvcc, *ARCH, "-lineinfo", *common, *extra, "-c", os.path.join(SRC, s), "-o", obj])
    for s in cxx:
        obj = os.path.join(OUT, s + ".o")
        jobs.append([nvcc, *common, "-x", "c++", "-c", os.path.join(SRC, s), "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return cmd[-1]

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
