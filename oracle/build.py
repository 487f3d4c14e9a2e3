"""ORACLE build recipe: compile oracle/src/*.c into oracle/_build/liboracle.so with gcc,
-O2 and no floating-point contraction (-ffp-contract=off), so that every element is the
IEEE result of the reference's own operation order on any host (x86-64 or aarch64).  The
per-column loops (convection, Calc_Kzz, the loss rates) run on every host thread (OpenMP):
columns are independent, so the bits do not depend on the thread count.
The transcendental functions are the package's gbmath.h (compiled in from its source), the
functions the reference is pointed at through its pydyn.ops.use_libm hook (as libgbmath.so)
when the golden fixtures are made."""

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "src"
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
CFLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-std=c11", "-Wall", "-fopenmp"]


def build():
    OUT.mkdir(exist_ok=True)
    srcs = sorted(SRC.glob("*.c"))
    heads = [*sorted(SRC.glob("*.h")), HERE.parent / "pydyn_gb300" / "csrc" / "gbmath.h", Path(__file__)]
    if LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime for s in [*srcs, *heads]):
        return LIB
    cmd = ["gcc", *CFLAGS, "-shared", "-o", str(LIB), *map(str, srcs), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build())
