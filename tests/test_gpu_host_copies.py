"""capsp_solve_host with page-locked buffers: on the level schedule the row
kernel counts finished rows per segment of x, and a second stream copies each
segment to the host as soon as its count is complete, while the solve runs.
These tests check the results against the oracle on systems of several
segments (64k rows and more each), repeated calls with different right-hand
sides (a copy started on a stale count would return the previous x), several
right-hand sides, a CSC handle, and the paths that copy after the solve.

Tolerance: relative infinity-norm error <= 1e-12 in FP64.
"""
from __future__ import annotations

import numpy as np
import pytest

import capellinisptrsv_gb300 as cs
import oracle
from conftest import rel_inf_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def pinned(shape, seed):
    t = torch.from_numpy(np.random.default_rng(seed).standard_normal(shape)).pin_memory()
    return t, t.numpy()


@pytest.fixture(scope="module")
def banded():
    # 300k rows: 5 segments of 60k rows at the 64k-row minimum
    return cs.generate(n=300_000, kmin=1, kmax=7, band=20_000, seed=12)


@pytest.mark.parametrize("k", [1, 3])
def test_segmented_copies_match_oracle(banded, k):
    m = banded
    s = cs.TriangularSolver(m.rowptr, m.colidx, m.val)
    shape = (m.n, k) if k > 1 else (m.n,)
    xt, x = pinned(shape, 0)
    for seed in (1, 2, 3):
        bt, b = pinned(shape, seed)
        s.solve_host(b, x)
        assert rel_inf_err(x, oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)) <= TOL64, seed
    s.close()


def test_segmented_copies_csc_handle(banded):
    """A CSC handle solves over its transposed view, with the same copies."""
    m = banded
    cp, ri, cv = cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)
    s = cs.TriangularSolver(cp, ri, cv, fmt="csc")
    xt, x = pinned(m.n, 0)
    for seed in (4, 5):
        bt, b = pinned(m.n, seed)
        s.solve_host(b, x)
        assert rel_inf_err(x, oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)) <= TOL64
    s.close()


@pytest.mark.parametrize("how", ["natural", "syncfree_csc", "pageable"])
def test_copy_after_solve_paths(banded, how):
    """Natural schedule, column-driven CSC and pageable buffers copy x once
    after the solve."""
    m = banded
    if how == "syncfree_csc":
        cp, ri, cv = cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)
        s = cs.TriangularSolver(cp, ri, cv, fmt="csc", algorithm="syncfree_csc")
    else:
        s = cs.TriangularSolver(m.rowptr, m.colidx, m.val, schedule="natural" if how == "natural" else None)
    if how == "pageable":
        b = np.random.default_rng(6).standard_normal(m.n)
        x = np.empty_like(b)
    else:
        (_, b), (_, x) = pinned(m.n, 6), pinned(m.n, 0)
    s.solve_host(b, x)
    assert rel_inf_err(x, oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)) <= TOL64
    s.close()
