"""In-tree build of libpct_gb300.so (CUDA kernels for sm_103a + host C++).

Every translation unit under pct_gb300/csrc is compiled by nvcc in parallel
with one -gencode (compute_103a/sm_103a) and linked into
pct_gb300/_lib/libpct_gb300.so.  Device code is compiled with -fmad=false and
host code with -ffp-contract=off: the kernels that must agree bit for bit with
the oracle rely on source-order IEEE arithmetic, and the fast FP32 kernels ask
for fused multiply-adds explicitly (fmaf / __fmaf_rn).

Objects are rebuilt only when their source or any header changed.
"""
import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pct_gb300")
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libpct_gb300.so")
COMPAT_SRC = os.path.join(PKG, "compat", "pct_functions_compat.cpp")
COMPAT_LIB = os.path.join(LIBDIR, "libpct_compat.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
          "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp,-O2",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers_digest():
    h = hashlib.sha256()
    for p in sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.h"))):
        with open(p, "rb") as f:
            h.update(p.encode() + f.read())
    return h.hexdigest()


def _compile(src, hdr_digest, extra, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    stamp = obj + ".stamp"
    with open(src, "rb") as f:
        digest = hashlib.sha256(f.read() + hdr_digest.encode() + " ".join(COMMON + extra).encode()).hexdigest()
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == digest:
        return obj, None
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, r.stderr + r.stdout
    with open(stamp, "w") as f:
        f.write(digest)
    return obj, None


def build(verbose=False, extra=None):
    """Compile and link; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    extra = list(extra or [])
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    hd = _headers_digest()
    errors = []
    objs = []
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for obj, err in ex.map(lambda s: _compile(s, hd, extra, verbose), srcs):
            objs.append(obj)
            if err:
                errors.append(err)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr + r.stdout)
    build_compat()
    return LIB


def build_compat():
    """libpct_compat.so: the reference's entry-point names over the C ABI (host C++ only)."""
    if (os.path.exists(COMPAT_LIB) and os.path.getmtime(COMPAT_LIB) >= os.path.getmtime(LIB)
            and os.path.getmtime(COMPAT_LIB) >= os.path.getmtime(COMPAT_SRC)):
        return COMPAT_LIB
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"), COMPAT_SRC,
           "-L", LIBDIR, "-lpct_gb300", "-Wl,-rpath,$ORIGIN", "-o", COMPAT_LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compat link failed:\n" + r.stderr + r.stdout)
    return COMPAT_LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
