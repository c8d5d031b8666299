"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

# build the library (nvcc cross-compiles without a GPU) and the oracle before importing them
import __graft_entry__  # noqa: E402

__graft_entry__._build_module().build()

import oracle  # noqa: E402

oracle.build()

GOLDEN = ROOT / "tests" / "golden" / "golden.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


def _cuda_ok() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_ok():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def rel_inf_err(x, ref) -> float:
    """Relative infinity-norm error ||x - ref||_inf / ||ref||_inf."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.max(np.abs(ref)) if ref.size else 0.0
    num = np.max(np.abs(x - ref)) if ref.size else 0.0
    return float(num / den) if den > 0 else float(num)
