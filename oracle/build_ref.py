#!/usr/bin/env python3
"""Build the reference-kernel harness into oracle/_ref/ (test infrastructure only).

The unmodified reference translation unit
``src/pCT_Reconstruction_Data_Segments.cu`` (lynch829/pCT) is compiled with g++
as host C++.  The text is read from the reference checkout and streamed to the
compiler through stdin; no copy of it is written anywhere.  The only textual
change is the launch syntax: ``kernel<<<grid, block>>>(args)`` becomes
``PCT_LAUNCH(kernel, grid, block)(args)`` (oracle/ref/ref_launch.h), which runs
the kernel body once per (block, thread) of the grid, sequentially.  The
reference's host drivers then run unchanged on top of the emulated CUDA API,
and ``oracle/ref/ref_harness.inc`` calls them in the order of main().

Each geometry gets its own shared library because the reference fixes every
size at compile time (pCT_data.h:215-420).  The overrides below follow the
``#undef``/``#define`` scheme: the three reference headers are included first
(their include guards then make the .cu's own includes no-ops) and the macros
are redefined before the .cu body is seen.

Usage:  python oracle/build_ref.py [--ref /root/reference] [geometry ...]
Outputs: oracle/_ref/libpctref_<geometry>.so
"""
import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

# Geometries used by the golden fixtures.  Keys are reference macro names
# (pCT_data.h); values are the replacement token strings.
GEOMETRIES = {
    # Small grid for fast golden vectors: 64x64x4 voxels of 1x1x2.5 mm,
    # r = 3.2 cm, 90 gantry angles.
    "tiny": {
        "RECON_CYL_RADIUS": "3.2",
        "COLUMNS": "64",
        "ROWS": "64",
        "SSD_V_SIZE": "2.0",
        "SSD_T_SIZE": "12.0",
        "GANTRY_ANGLE_INTERVAL": "4.0",
        "ANGULAR_BIN_SIZE": "4.0",
    },
    # Water-cylinder scan: 200x200x8 at 1x1x2.5 mm, r = 10 cm, 4 degree steps.
    "cfg1": {
        "RECON_CYL_RADIUS": "10.0",
        "COLUMNS": "200",
        "ROWS": "200",
        "SSD_V_SIZE": "3.0",
        "GANTRY_ANGLE_INTERVAL": "4.0",
        "ANGULAR_BIN_SIZE": "4.0",
    },
    # The benchmark scan's grid: 256x256x32 at 1x1x2.5 mm, r = 12.8 cm,
    # 2 degree steps (180 angles).
    "cfg2": {
        "RECON_CYL_RADIUS": "12.8",
        "COLUMNS": "256",
        "ROWS": "256",
        "SSD_V_SIZE": "9.0",
        "GANTRY_ANGLE_INTERVAL": "2.0",
        "ANGULAR_BIN_SIZE": "2.0",
    },
    # Config 4's head-phantom grid: 320x320x64 at 0.8x0.8x2.5 mm, r = 12.8 cm,
    # 2 degree steps (180 angles).
    "cfg4": {
        "RECON_CYL_RADIUS": "12.8",
        "COLUMNS": "320",
        "ROWS": "320",
        "SSD_V_SIZE": "17.0",
        "GANTRY_ANGLE_INTERVAL": "2.0",
        "ANGULAR_BIN_SIZE": "2.0",
    },
    # Largest grid of the batched-scan family: 256x256x48 at 1x1x2.5 mm,
    # r = 12.8 cm, 2 degree steps (180 angles).
    "cfg3_256x48": {
        "RECON_CYL_RADIUS": "12.8",
        "COLUMNS": "256",
        "ROWS": "256",
        "SSD_V_SIZE": "13.0",
        "GANTRY_ANGLE_INTERVAL": "2.0",
        "ANGULAR_BIN_SIZE": "2.0",
    },
    # Smallest grid of the batched-scan family: 128x128x8 at 1x1x2.5 mm,
    # r = 6.4 cm, 2 degree steps (180 angles).
    "cfg3_128x8": {
        "RECON_CYL_RADIUS": "6.4",
        "COLUMNS": "128",
        "ROWS": "128",
        "SSD_V_SIZE": "3.0",
        "GANTRY_ANGLE_INTERVAL": "2.0",
        "ANGULAR_BIN_SIZE": "2.0",
    },
}

REF_TU = os.path.join("src", "pCT_Reconstruction_Data_Segments.cu")
# `kernel<<<grid, block>>>(args)` -> `PCT_LAUNCH(kernel, grid, block)(args)`:
# the harness turns that into a sequential walk over every (block, thread).
LAUNCH = re.compile(r"(\w+)\s*<<<([^<>]*)>>>")

# Reference configuration constants (pCT_config.h / pCT_data.h) that the
# harness sets at run time.  Each is renamed out of the way before the header
# defines it and then redeclared as a mutable global of the same type.
RUNTIME_FLAGS = [
    ("bool", "SC_ON"), ("bool", "MSC_ON"), ("bool", "SM_ON"),
    ("bool", "AVG_FILTER_HULL"), ("bool", "DEBUG_TEXT_ON"),
    ("bool", "EXIT_AFTER_FBP"),
    ("HULL_TYPES", "MLP_HULL"), ("INITIAL_ITERATE", "X_K0"),
    ("FILTER_TYPES", "FBP_FILTER"),
]
RUNTIME_STRINGS = ["INPUT_DIRECTORY", "OUTPUT_DIRECTORY", "INPUT_FOLDER", "OUTPUT_FOLDER"]


def transformed_source(ref_root, geometry):
    with open(os.path.join(ref_root, REF_TU), "r", encoding="latin-1") as f:
        text = f.read()
    # MSC_edge_detection_GPU (.cu:3569) reads its 3x3 neighbourhood and writes
    # its own voxel in place; run it as if a grid-wide barrier separated the
    # reads from the writes (its intended two-buffer semantics).
    text = re.sub(r"MSC_edge_detection_GPU\s*<<<([^<>]*)>>>",
                  lambda m: "PCT_LAUNCH_TWO_PHASE(MSC_edge_detection_GPU, %s)" % m.group(1), text)
    text = LAUNCH.sub(lambda m: "PCT_LAUNCH(%s, %s)" % (m.group(1), m.group(2)), text)
    head = ['#include "pct_ref_prelude.h"']
    for _, name in RUNTIME_FLAGS:
        head.append("#define %s pct_header_%s" % (name, name))
    for name in RUNTIME_STRINGS:
        head.append("#define %s pct_header_%s" % (name, name))
    head += ['#include "pCT_data.h"', '#include "pCT_functions.h"', '#include "pCT_config.h"']
    for typ, name in RUNTIME_FLAGS:
        head.append("#undef %s" % name)
        head.append("%s %s = pct_header_%s;" % (typ, name, name))
    for name in RUNTIME_STRINGS:
        head.append("#undef %s" % name)
        head.append("char %s[512];" % name)
    for name, value in GEOMETRIES[geometry].items():
        head.append("#undef %s" % name)
        head.append("#define %s %s" % (name, value))
    # Iteration count and DROP block size become run-time values too.
    head += ["#undef ITERATIONS", "int pct_ref_iterations = 1;", "#define ITERATIONS pct_ref_iterations",
             "#undef BLOCK_SIZE_RECON", "int pct_ref_block_size = 3200;",
             "#define BLOCK_SIZE_RECON pct_ref_block_size"]
    # Every array_2_disk of a float/int/bool array is captured at full precision.
    for t in ("float", "int", "bool"):
        head.append("template<> void array_2_disk<%s>( char*, const char*, const char*, %s*, "
                    "const int, const int, const int, const int, const bool );" % (t, t))
    head.append('#include "ref_launch.h"')
    head.append("#define main pct_reference_main")
    head.append("#define exit pct_reference_exit")
    head.append('#line 1 "%s"' % os.path.join(ref_root, REF_TU))
    tail = ["#undef main", "#undef exit", '#include "ref_harness.inc"']
    return "\n".join(head) + "\n" + text + "\n" + "\n".join(tail) + "\n"


def build(ref_root, geometry, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    src = transformed_source(ref_root, geometry)
    so = os.path.join(OUT, "libpctref_%s.so" % geometry)
    cmd = ["g++", "-std=c++14", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-w", "-fpermissive",
           "-I", os.path.join(HERE, "ref", "cuda_emul"),
           "-I", os.path.join(HERE, "ref"),
           "-I", os.path.join(ref_root, "include"),
           "-x", "c++", "-", "-o", so, "-fopenmp", "-lquadmath"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, input=src.encode("latin-1"), capture_output=True)
    if r.returncode != 0:
        sys.stderr.write(r.stderr.decode(errors="replace")[-20000:])
        raise SystemExit("reference harness build failed for %s" % geometry)
    return so


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("geometries", nargs="*", default=sorted(GEOMETRIES))
    a = ap.parse_args()
    if not os.path.isfile(os.path.join(a.ref, REF_TU)):
        print("reference sources not present at %s; nothing to build" % a.ref)
        return 0
    for g in a.geometries:
        print("built", build(a.ref, g))
    return 0


if __name__ == "__main__":
    sys.exit(main())
