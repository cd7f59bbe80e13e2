#!/usr/bin/env python3
"""Builds the C oracle (test infrastructure) into oracle/_build/libpct_oracle.so,
and the host-only scan generator into oracle/_build/libpct_gen.so.

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
GEN_LIB = os.path.join(OUT_DIR, "libpct_gen.so")


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


def build_gen(verbose=False):
    """libpct_gen.so: pct_gb300/csrc/phantom.cpp (the seeded generator) on the host alone."""
    os.makedirs(OUT_DIR, exist_ok=True)
    csrc = os.path.join(ROOT, "pct_gb300", "csrc")
    srcs = [os.path.join(csrc, "phantom.cpp"), os.path.join(HERE, "gen_host.cpp")]
    deps = srcs + [os.path.join(csrc, h) for h in ("pct_math.h", "pct_geometry.h", "pct_internal.h")] + \
        [os.path.join(ROOT, "include", "pct.h")]
    if os.path.exists(GEN_LIB) and os.path.getmtime(GEN_LIB) >= max(os.path.getmtime(d) for d in deps):
        return GEN_LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", "-Wall",
           "-I", os.path.join(ROOT, "include"), "-I", csrc] + srcs + ["-o", GEN_LIB, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return GEN_LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
    print(build_gen(verbose="-v" in sys.argv))
