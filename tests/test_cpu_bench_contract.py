"""The bench's reference arm runs on the host alone: its JSON line keeps the
contract (one line, the batch metric, a cpu_baseline and an e2e object, the
workload named by its sizes) on a small graph, without a GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line(built):
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--triples", "200000",
           "--entities", "20000", "--queries", "64", "--steps", "2", "--warmup", "1", "--cpu-sample", "32"]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, check=True).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "batched queries/s" and d["unit"] == "queries/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 1
    cb = d["cpu_baseline"]
    assert set(cb) >= {"value", "unit", "cores", "kind", "sample"} and cb["value"] == d["value"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    cfg = d["config"]
    assert cfg["triples"] == 200000 and cfg["queries"] == 64 and "workload" in cfg
