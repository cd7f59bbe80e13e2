"""bench.py's reference arm on the host (no GPU): one JSON line with the
contract's keys, on one full DROP block of the cfg2 workload, without mapping
the CUDA library."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--histories", "150000",
           "--steps", "1", "--warmup", "0"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, res.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "histories/s per MLP+DROP iteration"
    assert d["unit"] == "histories*iterations/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert (d["n_gpus"], d["steps"], d["warmup"]) == (1, 1, 0)
    assert d["scaling"] == "weak" and d["vs_baseline"] is None
    assert d["data"].startswith("synthetic") and "cfg2" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["unit"] == d["unit"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # the arm runs the CPU restatement alone: no library of the product is mapped
    assert d["libraries_mapped"] and all(p.startswith("oracle" + os.sep) for p in d["libraries_mapped"]), \
        d["libraries_mapped"]
