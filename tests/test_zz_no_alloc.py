"""capsp_csc_solve_noalloc_f64: the column-driven CSC solve on static device
scratch, for callers that may not allocate device memory (a host framework
that owns all of it through its own pool, or a latency-critical path where
cudaMalloc would synchronise the device).  It is called through the C ABI and
compared with the handle-based CSC solve of the same matrix (and with the
oracle) on two consecutive calls, which also shows that the scratch left by
one call does not leak into the next.  The file is collected last so that it
also runs after every other GPU test."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import capellinisptrsv_gb300 as cs
from capellinisptrsv_gb300 import _native as N
import oracle
from conftest import rel_inf_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEV = "cuda:0"
MAX_N = 65_536
TOL = 1e-12  # relative infinity-norm, FP64


def _fn():
    f = N.lib.capsp_csc_solve_noalloc_f64
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                  C.c_void_p]
    return f


def _csc(m):
    """Lower CSC of a lower CSR matrix (diagonal first in each column)."""
    return cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)


def _call(cp, ri, cv, b, x, n, nnz):
    st = torch.cuda.current_stream().cuda_stream
    return _fn()(cp.data_ptr(), ri.data_ptr(), cv.data_ptr(), n, nnz, b.data_ptr(), x.data_ptr(),
                 C.c_void_p(st))


@pytest.mark.parametrize("n", [20_000, MAX_N])
def test_noalloc_matches_handle_solve_twice(n):
    m = cs.generate(n=n, kind=N.GEN_UNIFORM_BAND, kmin=1, kmax=5, band=2000, seed=0)
    cp_h, ri_h, cv_h = _csc(m)
    b_h = cs.normal(m.n, seed=0, stream=7)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    cp, ri, cv, b = t(cp_h), t(ri_h), t(cv_h), t(b_h)
    ref = cs.TriangularSolver(cp, ri, cv, fmt="csc").solve(b).cpu().numpy()
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b_h)
    for _ in range(2):
        x = torch.full_like(b, float("nan"))
        assert _call(cp, ri, cv, b, x, m.n, m.nnz) == 0, N.last_error()
        xn = x.cpu().numpy()
        assert rel_inf_err(xn, ref) <= TOL
        assert rel_inf_err(xn, xo) <= TOL


def test_noalloc_rejects_rows_beyond_scratch():
    n = MAX_N + 1
    dummy = torch.zeros(4, dtype=torch.int32, device=DEV)
    vals = torch.zeros(4, dtype=torch.float64, device=DEV)
    st = torch.cuda.current_stream().cuda_stream
    rc = _fn()(dummy.data_ptr(), dummy.data_ptr(), vals.data_ptr(), n, n, vals.data_ptr(),
               vals[2:].data_ptr(), C.c_void_p(st))
    assert rc == N.ERR_INVALID
    assert "65536" in N.last_error()


def test_noalloc_rejects_malformed_column():
    # column 1 lacks its diagonal: caught on the device before the solve
    cp = torch.tensor([0, 2, 3, 4], dtype=torch.int32, device=DEV)
    ri = torch.tensor([0, 1, 2, 2], dtype=torch.int32, device=DEV)
    cv = torch.tensor([2.0, 1.0, 1.0, 3.0], dtype=torch.float64, device=DEV)
    b = torch.ones(3, dtype=torch.float64, device=DEV)
    x = torch.empty_like(b)
    assert _call(cp, ri, cv, b, x, 3, 4) == N.ERR_INVALID
    assert "column 1" in N.last_error()
