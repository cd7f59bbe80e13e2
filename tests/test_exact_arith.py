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
