"""Build the package's native libraries in the tree (pydyn_gb300/_build/):

    libgbdyn.so   the CUDA kernels and the C ABI of include/gbdyn.h, sm_103a only, float64
                  with -fmad=false (no multiply-add contraction) and IEEE division/sqrt
    libgbmath.so  the host build of the transcendental functions the kernels use on the
                  device (exp, log, pow, sin, cos), compiled with -ffp-contract=off; the
                  reference's own libm twin hook (pydyn ops.use_libm) is pointed at it so that
                  the reference, the oracle and the device compute the same bits

Translation units compile in parallel; a unit is rebuilt when its source or a header is newer
than its object."""

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = [
    *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", f"-I{INCLUDE}",
]  # fmt: skip
CFLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-std=c11", f"-I{INCLUDE}"]

LIBGBDYN = OUT / "libgbdyn.so"
LIBGBMATH = OUT / "libgbmath.so"


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (Path(cand).exists() or cand == "nvcc"):
            return cand
    raise RuntimeError("pydyn_gb300.build: nvcc not found")


def _stale(target, sources):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def build(verbose=False):
    """Compile libgbdyn.so and libgbmath.so if any source changed; returns their paths."""
    OUT.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    units = sorted(CSRC.glob("*.cu"))
    nvcc = _nvcc()
    jobs = []
    for cu in units:
        obj = OUT / (cu.stem + ".o")
        if _stale(obj, [cu, *headers]):
            jobs.append([nvcc, *NVFLAGS, "-c", str(cu), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as pool:
        for r in pool.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    objs = [OUT / (cu.stem + ".o") for cu in units]
    if _stale(LIBGBDYN, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIBGBDYN), *map(str, objs)])
    math_src = CSRC / "gbmath.c"
    if math_src.exists() and _stale(LIBGBMATH, [math_src, CSRC / "gbmath.h"]):
        _run(["gcc", *CFLAGS, "-shared", "-o", str(LIBGBMATH), str(math_src), "-lm"])
    return LIBGBDYN, LIBGBMATH


if __name__ == "__main__":
    print(*build(verbose=True))
