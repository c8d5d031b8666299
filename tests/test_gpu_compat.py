"""The reference-compatible drivers keep the reference's contract: they build
b = L*ones themselves, time BENCH_REPEAT solves, validate against x_ref = ones
and report time / GFLOP/s / GB/s through out-parameters (solve_time = -1 on a
validation failure, -1 return on a non-square matrix)."""
from __future__ import annotations

import numpy as np
import pytest

import capellinisptrsv_gb300 as cs
import oracle
from conftest import rel_inf_err

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def few_repeats():
    old = cs.set_compat_repeat(3)
    yield
    cs.set_compat_repeat(old)


@pytest.fixture(scope="module")
def unit_L():
    """The reference's input pipeline: a general sparse A -> change2tran -> unit-valued L."""
    rng = np.random.default_rng(0)
    n = 30_000
    rows = [np.unique(rng.integers(max(0, i - 3000), n, size=6)) for i in range(n)]
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    ci = np.concatenate(rows).astype(np.int32)
    va = rng.uniform(-1, 1, len(ci))
    return cs.change2tran(n, rp, ci, va)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_wrtfst_and_twopart_drivers(unit_L, dtype):
    nnzL, rp, ci, v = unit_L
    v = v.astype(dtype)
    n = len(rp) - 1
    for fn in (cs.spts_syncfree_cuda_csr_wrt, cs.spts_syncfree_cuda_csr):
        ret, t, gf, bw = fn(rp, ci, v, n, n, nnzL)
        assert ret == 0 and t > 0 and gf > 0 and bw > 0


def test_mix_driver_reports_selector_stats(unit_L):
    nnzL, rp, ci, v = unit_L
    n = len(rp) - 1
    ret, t, gf, bw, pre, wo, eo = cs.spts_syncfree_cuda_csr_wrt_mix(rp, ci, v, n, n, nnzL)
    assert ret == 0 and t > 0 and pre >= 0
    _, _, wo_ref, eo_ref = cs.matrix_warp4(n, n, nnzL, rp, ci, v, border=10)
    assert (wo, eo) == (wo_ref, eo_ref)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_csc_driver_fills_x(dtype):
    m = cs.generate(n=40_000, kmin=1, kmax=6, band=4000, seed=2)
    val = m.val.astype(dtype)
    cp, ri, cv = cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, val)
    x_ref, b = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, val)
    x = np.zeros(m.n, dtype)
    ret, pre, t, gf, bw = cs.sptrsv_syncfree_cuda(cp, ri, cv, m.n, m.n, m.nnz, x, b, x_ref)
    assert ret == 0 and t > 0 and pre > 0
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, val, b)
    assert rel_inf_err(x, xo) <= (1e-12 if dtype == np.float64 else 1e-5)


def test_non_square_returns_minus_one(unit_L):
    nnzL, rp, ci, v = unit_L
    n = len(rp) - 1
    ret, *_ = cs.spts_syncfree_cuda_csr_wrt(rp, ci, v, n, n + 1, nnzL)
    assert ret == -1
