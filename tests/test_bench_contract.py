"""The benchmark's reference arm runs on the host cores, so its JSON line can be
checked on the CPU: the keys and types of the line the comparison reads."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "plain_20k",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference"
    for key, kind in (("metric", str), ("value", float), ("unit", str), ("n_gpus", int), ("steps", int),
                      ("warmup", int), ("ms_per_step", float), ("higher_is_better", bool), ("scaling", str),
                      ("dtype", str), ("data", str), ("config", dict), ("cpu_baseline", dict), ("e2e", dict)):
        assert isinstance(line[key], kind), key
    assert line["n_gpus"] == 1 and line["gpus_used"] == 0 and line["steps"] == 2
    assert line["value"] > 0 and line["unit"] == "GFLOP/s" and line["higher_is_better"] is True
    assert line["config"]["workload"] == "plain_20k"
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["cores"] == 1 and cpu["kind"] in ("reference", "port")
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
