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
