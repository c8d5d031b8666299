"""Batched form: many independent systems of uneven size with k right-hand
sides in one persistent launch (block-diagonal handle), with CUDA-graph replay
and the autotuner, against per-system oracle solves."""
from __future__ import annotations

import numpy as np
import pytest

import capellinisptrsv_gb300 as cs
import oracle
from conftest import rel_inf_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


@pytest.fixture(scope="module")
def batch():
    return cs.generate_batched(nsys=64, seed=0, nmin=500, nmax=8000)


@pytest.mark.parametrize("k", [1, 4, 16, 32])
def test_batched_matches_per_system_oracle(batch, k):
    m = batch
    b = np.random.default_rng(k).standard_normal((m.n, k))
    s = cs.TriangularSolver(t(m.rowptr), t(m.colidx), t(m.val), sys_rowoff=m.sys_rowoff)
    x = s.solve(t(b)).cpu().numpy()
    s.status()
    so = m.sys_rowoff
    worst = 0.0
    for i in range(0, len(so) - 1, 7):
        r0, r1 = so[i], so[i + 1]
        k0, k1 = m.rowptr[r0], m.rowptr[r1]
        rp = m.rowptr[r0:r1 + 1] - k0
        ci = m.colidx[k0:k1] - r0
        xo = oracle.solve_csr_lower(rp, ci, m.val[k0:k1], b[r0:r1])
        worst = max(worst, rel_inf_err(x[r0:r1], xo))
    assert worst <= 1e-12


def test_batched_graph_and_autotune(batch):
    m = batch
    k = 4
    b = t(np.random.default_rng(9).standard_normal((m.n, k)))
    s = cs.TriangularSolver(t(m.rowptr), t(m.colidx), t(m.val), sys_rowoff=m.sys_rowoff)
    ref = s.solve(b).cpu().numpy()
    x = torch.empty_like(b)
    st = torch.cuda.Stream()
    s.autotune(b, x, stream=st)
    with torch.cuda.stream(st):
        s.graph_solve(b, x, st)
        s.graph_solve(b, x, st)
    st.synchronize()
    assert rel_inf_err(x.cpu().numpy(), ref) <= 1e-12


def test_batched_rejects_cross_system_entries():
    m = cs.generate_batched(nsys=3, seed=1, nmin=50, nmax=80)
    ci = m.colidx.copy()
    r = int(m.sys_rowoff[1]) + 5       # a row of system 1
    ci[m.rowptr[r]] = 0                # points into system 0
    ci[m.rowptr[r]:m.rowptr[r + 1] - 1].sort()
    with pytest.raises(cs.CapspError):
        cs.TriangularSolver(m.rowptr, ci, m.val, sys_rowoff=m.sys_rowoff)


def test_graph_cache_after_scratch_growth(batch):
    """Graph-solve with 4 RHS, plain-solve with 16 (the handle's scratch grows
    and the memory the first capture points at is freed), graph-solve with 4
    again: the cache must have dropped the stale graph and recaptured."""
    m = batch
    rng = np.random.default_rng(21)
    b4 = rng.standard_normal((m.n, 4))
    b16 = rng.standard_normal((m.n, 16))
    s = cs.TriangularSolver(t(m.rowptr), t(m.colidx), t(m.val), sys_rowoff=m.sys_rowoff)
    st = torch.cuda.Stream()
    b4d, x4 = t(b4), torch.empty((m.n, 4), dtype=torch.float64, device=DEV)
    with torch.cuda.stream(st):
        s.graph_solve(b4d, x4, st)
    st.synchronize()
    assert s.info()["cached_graphs"] == 1
    x16 = s.solve(t(b16)).cpu().numpy()
    s.status()
    assert s.info()["cached_graphs"] == 0
    x4.fill_(0.0)
    with torch.cuda.stream(st):
        s.graph_solve(b4d, x4, st)
        s.graph_solve(b4d, x4, st)
    st.synchronize()
    s.status(st)
    assert s.info()["cached_graphs"] == 1
    x4h = x4.cpu().numpy()
    so = m.sys_rowoff
    for i in range(0, len(so) - 1, 9):
        r0, r1 = so[i], so[i + 1]
        k0, k1 = m.rowptr[r0], m.rowptr[r1]
        rp, ci, v = m.rowptr[r0:r1 + 1] - k0, m.colidx[k0:k1] - r0, m.val[k0:k1]
        assert rel_inf_err(x4h[r0:r1], oracle.solve_csr_lower(rp, ci, v, b4[r0:r1])) <= 1e-12
        assert rel_inf_err(x16[r0:r1], oracle.solve_csr_lower(rp, ci, v, b16[r0:r1])) <= 1e-12
    # settings that a capture bakes in drop the cache too
    s.set_timeout(5.0)
    assert s.info()["cached_graphs"] == 0


@pytest.mark.parametrize("algorithm", ["auto", "syncfree_csc"])
def test_graph_solve_csc_first_call(algorithm):
    """A CSC handle's first solve through graph replay: the publication
    scratch (transposed view) or the column visiting order and the
    sum-and-count words (column-driven) are built before the capture starts."""
    m = cs.generate("plain_20k", seed=0)
    cp, ri, cv = cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)
    s = cs.TriangularSolver(t(cp), t(ri), t(cv), fmt="csc", algorithm=algorithm)
    b = np.random.default_rng(3).standard_normal(m.n)
    bd, x = t(b), torch.empty(m.n, dtype=torch.float64, device=DEV)
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        s.graph_solve(bd, x, st)
        s.graph_solve(bd, x, st)
    st.synchronize()
    s.status(st)
    assert rel_inf_err(x.cpu().numpy(), oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)) <= 1e-12


def test_graph_cache_after_value_repointing():
    """Natural schedule: a captured solve reads the value array itself, so
    re-pointing the handle at new values must drop the cached graph (a stale
    replay would solve with the old values)."""
    m = cs.generate("plain_20k", seed=0)
    s = cs.TriangularSolver(t(m.rowptr), t(m.colidx), t(m.val), schedule="natural")
    b = np.random.default_rng(5).standard_normal(m.n)
    bd, x = t(b), torch.empty(m.n, dtype=torch.float64, device=DEV)
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        s.graph_solve(bd, x, st)
    st.synchronize()
    assert s.info()["cached_graphs"] == 1
    val2 = m.val * 1.5  # same structure, scaled values (still diagonally dominant)
    v2 = t(val2)
    s.refresh_values(v2)
    torch.cuda.synchronize()
    assert s.info()["cached_graphs"] == 0
    with torch.cuda.stream(st):
        s.graph_solve(bd, x, st)
    s.status(st)
    assert rel_inf_err(x.cpu().numpy(), oracle.solve_csr_lower(m.rowptr, m.colidx, val2, b)) <= 1e-12
    s.set_schedule("level")
    assert s.info()["cached_graphs"] == 0
