"""Build recipe of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Compiles oracle/*.c with gcc into oracle/_build/libaxo.so, FP64 with
-ffp-contract=off so the arithmetic order of the restatement is the one
written in the sources.  Only tests/, __graft_entry__.smoke() and the
cpu-baseline leg of bench.py load the result.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libaxo.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(".c"))
    hdrs = [os.path.join(HERE, "axo.h"), os.path.join(ROOT, "include", "axgpu.h"),
            os.path.join(ROOT, "axion_grav_gb300", "csrc", "axg_detmath.h"),
            os.path.join(ROOT, "axion_grav_gb300", "csrc", "axg_ffchi2.h"), os.path.abspath(__file__)]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in srcs + hdrs):
            return LIB
    cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-I" + HERE, "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "axion_grav_gb300", "csrc"), *srcs, "-o", LIB + ".tmp", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
