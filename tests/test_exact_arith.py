"""Host checks of the exact-arithmetic identities that let the device code
replace binary64 operations without changing a bit of the results
(tests/arith/exact_arith_check.c): the corrected-reciprocal quotient of the
backprojection against IEEE division, the FMA product error against Dekker's
splitting, and the shared-reduction sine/cosine against the separate calls."""
import os
import platform
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _fma_flags():
    # hardware FMA for speed where the host has it; the results are the same
    # with libm's correctly rounded fma
    if platform.machine() in ("x86_64", "AMD64"):
        try:
            if " fma " in open("/proc/cpuinfo").read():
                return ["-mfma"]
        except OSError:
            pass
    return []


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_exact_arithmetic_identities(tmp_path):
    exe = str(tmp_path / "exact_arith_check")
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off"] + _fma_flags() + [
        "-I", os.path.join(ROOT, "pct_gb300", "csrc"), os.path.join(ROOT, "tests", "arith", "exact_arith_check.c"),
        "-o", exe, "-lm"]
    subprocess.run(cmd, check=True)
    res = subprocess.run([exe, "20000000"], capture_output=True, text=True, timeout=600)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
    lines = [l for l in res.stdout.splitlines() if l.strip()]
    assert len(lines) == 7
    assert all(l.endswith(" 0 differ") for l in lines), res.stdout


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_table_sine_cosine_correctly_rounded(tmp_path):
    """pct_sincos_cr, which builds the per-angle sine and cosine tables (gantry
    rotation, bin angles, backprojection, the tabulated MLP's trig table), is
    the correctly rounded sin and cos on every table argument of 0.5-6 degree
    grids and on random arguments (against 200-bit mpmath)."""
    mpmath = pytest.importorskip("mpmath")
    exe = str(tmp_path / "sincos_cr_check")
    subprocess.run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-I", os.path.join(ROOT, "pct_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "arith", "sincos_cr_check.c"), "-o", exe, "-lm"], check=True)
    out = subprocess.run([exe, "20000"], capture_output=True, text=True, check=True).stdout.split("\n")
    mpmath.mp.prec = 200
    bad = []
    for line in out:
        if not line.strip():
            continue
        x, s, c = (float.fromhex(v) for v in line.split())
        if float(mpmath.sin(mpmath.mpf(x))) != s or float(mpmath.cos(mpmath.mpf(x))) != c:
            bad.append(x)
    assert len(out) > 23000 and not bad, bad[:5]
