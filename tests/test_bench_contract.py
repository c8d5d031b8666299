"""The benchmark's reference arm runs on the host cores, so its JSON line can be
checked on the CPU: the keys and types of the line the comparison reads, and
that the arm never loads the solver library (its inputs come from the oracle
library's copy of the generator)."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

# runs bench.py in-process, then reports which in-tree shared objects it mapped
_PROBE = r"""
import runpy, sys, json
sys.argv = ["bench.py"] + sys.argv[1:]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    assert not e.code, e.code
maps = open("/proc/self/maps").read()
print("MAPPED " + json.dumps(sorted({l.split()[-1].rsplit("/", 1)[-1] for l in maps.splitlines()
                                      if l.endswith(".so") and ("_build" in l or "_ref" in l)})))
"""


def run_reference(*args):
    r = subprocess.run([sys.executable, "-c", _PROBE, "--impl", "reference", *args], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    mapped = json.loads([l for l in r.stdout.splitlines() if l.startswith("MAPPED ")][-1][len("MAPPED "):])
    return line, mapped


def check_common(line, mapped):
    assert line["impl"] == "reference"
    for key, kind in (("metric", str), ("value", float), ("unit", str), ("n_gpus", int), ("steps", int),
                      ("warmup", int), ("ms_per_step", float), ("higher_is_better", bool), ("scaling", str),
                      ("dtype", str), ("data", str), ("config", dict), ("cpu_baseline", dict), ("e2e", dict)):
        assert isinstance(line[key], kind), key
    assert "libcapsp.so" not in mapped, mapped
    assert "liboracle.so" in mapped, mapped
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["kind"] in ("reference", "port")
    assert cpu["host_cores"] >= cpu["cores"] >= 1
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_line():
    line, mapped = run_reference("--workload", "plain_20k", "--steps", "2", "--warmup", "1")
    check_common(line, mapped)
    assert line["n_gpus"] == 1 and line["gpus_used"] == 0 and line["steps"] == 2
    assert line["value"] > 0 and line["unit"] == "GFLOP/s" and line["higher_is_better"] is True
    assert line["config"]["workload"] == "plain_20k" and line["cpu_baseline"]["cores"] == 1


@pytest.mark.parametrize("workload", ["batched", "autograd"])
def test_reference_arm_forms_line(workload):
    extra = ["--nsys", "16"] if workload == "batched" else []
    line, mapped = run_reference("--workload", workload, "--steps", "1", "--warmup", "0", *extra)
    check_common(line, mapped)
    assert line["unit"] == ("solves/s" if workload == "batched" else "ms")
