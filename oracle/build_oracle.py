#!/usr/bin/env python3
"""Builds the C oracle (test infrastructure) into oracle/_build/libpct_oracle.so.

gcc, -O2, no FMA contraction, OpenMP for the per-history loops.  Runs on the
x86 container and on the Arm GPU host alike (no ISA-specific flags).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpct_oracle.so")


def build(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    src = os.path.join(HERE, "pct_oracle.c")
    deps = [src, os.path.join(HERE, "pct_oracle.h"), os.path.join(ROOT, "pct_gb300", "csrc", "pct_math.h"),
            os.path.join(ROOT, "pct_gb300", "csrc", "pct_geometry.h"), os.path.join(ROOT, "include", "pct.h")]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", "-Wall",
           "-I", HERE, "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "pct_gb300", "csrc"),
           src, "-o", LIB, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
