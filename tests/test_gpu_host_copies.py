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


def test_segmented_copies_mix_kernel(banded):
    """The mixed kernel (heavy 32-row groups warp-per-row at border 4) with the
    segmented copies: its warp-per-row chunks wait for b and count rows too."""
    m = banded
    s = cs.TriangularSolver(m.rowptr, m.colidx, m.val, algorithm="mix")
    s.set_mix_border(4)
    _, x = pinned(m.n, 0)
    for seed in (7, 8):
        _, b = pinned(m.n, seed)
        s.solve_host(b, x)
        assert rel_inf_err(x, oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)) <= TOL64
    assert s.info()["warp_occupy"] > 0.0
    s.close()


def test_segmented_copies_fp32(banded):
    m = banded
    v32 = m.val.astype(np.float32)
    s = cs.TriangularSolver(m.rowptr, m.colidx, v32)
    xt = torch.empty(m.n, dtype=torch.float32).pin_memory()
    bt = torch.from_numpy(np.random.default_rng(9).standard_normal(m.n).astype(np.float32)).pin_memory()
    s.solve_host(bt.numpy(), xt.numpy())
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, v32, bt.numpy())
    assert rel_inf_err(xt.numpy(), xo) <= 1e-5
    s.close()


def test_segmented_copies_wide_levels():
    """Ten levels of 40,000 rows (each row depends on 1-12 rows of the level
    before): the launch for levels of 32k rows and more, with the copies."""
    rng = np.random.default_rng(10)
    nb, w = 10, 40_000
    n = nb * w
    counts = np.concatenate([np.zeros(w, np.int64), rng.integers(1, 13, n - w)])
    # k distinct rows of the level before: base + t * step (mod w), t < k <= 12
    base = rng.integers(0, w, n)
    step = rng.integers(1, w // 12, n)
    offs = np.sort((base[:, None] + np.arange(12)[None, :] * step[:, None]) % w, axis=1)
    offs = np.where(np.arange(12)[None, :] < counts[:, None], offs, w)  # unused slots last
    offs.sort(axis=1)
    rows = np.arange(n)
    lo = (rows // w - 1) * w
    rp = np.concatenate([[0], np.cumsum(counts + 1)]).astype(np.int32)
    ci = np.empty(rp[-1], np.int32)
    val = np.empty(rp[-1])
    used = np.arange(12)[None, :] < counts[:, None]
    r_of = np.repeat(rows, counts)
    dep_pos = (rp[:-1][:, None] + np.arange(12)[None, :])[used]
    ci[dep_pos] = (lo[:, None] + offs)[used]
    val[dep_pos] = rng.uniform(-1, 1, dep_pos.size)
    diag = rp[1:] - 1
    ci[diag] = rows
    absum = np.zeros(n)
    np.add.at(absum, r_of, np.abs(val[dep_pos]))
    val[diag] = 1.0 + absum
    s = cs.TriangularSolver(rp, ci, val)
    assert s.info()["levels"] == nb
    _, x = pinned(n, 0)
    for seed in (11, 12):
        _, b = pinned(n, seed)
        s.solve_host(b, x)
        assert rel_inf_err(x, oracle.solve_csr_lower(rp, ci, val, b)) <= TOL64
    s.close()
