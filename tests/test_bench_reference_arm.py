"""bench.py --impl reference on CPU: the reference arm's JSON line.

The arm times the oracle (the CPU restatement of the reference path: element
loop, COO triplets, SparseArrays.sparse semantics, vector assembly) on the
host cores.  Here it runs on a 40 x 40 mesh, and the line must carry what the
bench contract asks of it: impl, metric, unit, the cpu_baseline
description (kind, cores, sample, single-thread figure) and an e2e entry
with no host-device bytes.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "40",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "elements/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 2 and line["config"]["elements"] == 2 * 40 * 40
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert cb["single_thread"]["cores"] == 1 and cb["single_thread"]["value"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
