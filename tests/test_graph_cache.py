"""CPU check of the CUDA-graph cache's invalidation logic (csrc/graph_cache.h).

The header is plain C++ templated on the graph handle type, so it is compiled
here with g++ against a fake handle that records its destruction.  The
sequence is the one that once replayed a graph pointing at freed scratch:
capture a 4-RHS solve, grow the scratch for 16 RHS, ask for the 4-RHS graph.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_graph_cache_invalidation(tmp_path):
    exe = tmp_path / "graph_cache_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "capellinisptrsv_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "graph_cache_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "graph cache ok" in r.stdout
