"""Full-size oracle parity for the deep, batched and differentiation workloads.

Each test runs one benchmark configuration at its stated size through the
C-ABI and compares it with the oracle (the reference's serial executor,
restated in C and pinned bit-for-bit by tests/test_oracle.py), the way the
reference validates every run it times
(CUDA/ourWrtFst/spts_syncfree_cuda_csr_wrt.h:187-201,
CUDA/SyncFree_csc/spts_syncfree_cuda2.h:245-264).

  * zipf_1m: n = 1,048,576, Zipf(1.8) dependency counts capped at 512, half
    of them in the previous 32 rows (~126k levels);
  * the batched workload: 2,048 systems (22.0 M rows, 187 M nonzeros), k in
    {1, 4, 16, 32} right-hand sides of N(0,1) values, autotuned and replayed
    from a CUDA graph as the benchmark runs it; every system is checked at
    k = 1 and 4, every fourth system at k = 16 and 32;
  * grad_1m: n = 1,048,576 with 16 right-hand sides through the autograd
    function, whose backward runs over the transposed view or column-driven:
    x, grad_b = L^{-T}(x - x*) and grad_val = -grad_b[row] x[col] against the
    serial forward, the serial adjoint and the oracle grad_val.
    (The finite-difference check runs at n = 20,000 in test_gpu_autograd.py:
    at 1M rows a central difference with h = 1e-6 is dominated by rounding.)

Tolerance: relative infinity-norm error <= 1e-12 in FP64.
"""
from __future__ import annotations

import numpy as np
import pytest

import capellinisptrsv_gb300 as cs
import oracle
from capellinisptrsv_gb300 import workloads as W
from conftest import rel_inf_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12
DEV = "cuda:0"


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def test_zipf_1m_full_size():
    m = cs.generate("zipf_1m", seed=0)
    assert m.n == 1_048_576
    _, b = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, m.val)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    s = cs.TriangularSolver(dev(m.rowptr), dev(m.colidx), dev(m.val))
    x = s.solve(dev(b)).cpu().numpy()
    s.status()
    assert s.info()["levels"] > 100_000
    assert rel_inf_err(x, xo) <= TOL64
    assert np.max(np.abs(x - 1.0)) <= 0.01  # the reference's own self-check (x_ref = ones)


@pytest.fixture(scope="module")
def full_batch():
    m = cs.generate_batched(2048, seed=0)
    assert len(m.sys_rowoff) == 2049 and m.n > 20_000_000
    s = cs.TriangularSolver(dev(m.rowptr), dev(m.colidx), dev(m.val), sys_rowoff=m.sys_rowoff)
    yield m, s
    s.close()


@pytest.mark.parametrize("k,stride", [(1, 1), (4, 1), (16, 4), (32, 4)])
def test_batched_full_size(full_batch, k, stride):
    m, s = full_batch
    b = cs.normal(m.n * k, seed=0, stream=1000 + k).reshape(m.n, k)
    b_d = dev(b if k > 1 else b[:, 0])
    x_d = torch.empty_like(b_d)
    st = torch.cuda.Stream()
    s.autotune(b_d, x_d, stream=st)
    x_d.zero_()
    with torch.cuda.stream(st):
        s.graph_solve(b_d, x_d, st)
        s.graph_solve(b_d, x_d, st)
    s.status(st)
    x = x_d.cpu().numpy().reshape(m.n, k)
    del b_d, x_d
    nsys = len(m.sys_rowoff) - 1
    worst, checked = 0.0, 0
    for sidx in range(0, nsys, stride):
        r0, r1, rp, ci, v = W.sub_system(m.rowptr, m.colidx, m.val, m.sys_rowoff, sidx)
        bs = b[r0:r1] if k > 1 else b[r0:r1, 0]
        xo = oracle.solve_csr_lower(rp, ci, v, bs).reshape(r1 - r0, k)
        worst = max(worst, rel_inf_err(x[r0:r1], xo))
        checked += 1
    assert checked == (nsys + stride - 1) // stride
    assert worst <= TOL64, worst


@pytest.mark.parametrize("algorithm", ["auto", "syncfree_csc"])
def test_grad_1m_full_size_16rhs(algorithm):
    """Backward over the transposed view plus the gradient pass (auto), or the
    column-driven transpose with the gradient fused (syncfree_csc)."""
    m = cs.generate("grad_1m", seed=0)
    n, k = m.n, 16
    assert n == 1_048_576
    b_h = cs.normal(n * k, seed=0, stream=1).reshape(n, k)
    xs_h = cs.normal(n * k, seed=0, stream=2).reshape(n, k)
    val = dev(m.val).requires_grad_(True)
    b = dev(b_h).requires_grad_(True)
    solver = cs.TriangularSolver(dev(m.rowptr), dev(m.colidx), val.detach(), algorithm=algorithm)
    x = cs.sptrsv(solver, val, b)
    loss = 0.5 * ((x - dev(xs_h)) ** 2).sum()
    loss.backward()
    solver.status()
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b_h)
    yo = oracle.solve_csr_transpose(m.rowptr, m.colidx, m.val, xo - xs_h)
    go = oracle.grad_val(m.rowptr, m.colidx, yo, xo)
    assert rel_inf_err(x.detach().cpu().numpy(), xo) <= TOL64
    assert rel_inf_err(b.grad.cpu().numpy(), yo) <= TOL64
    assert rel_inf_err(val.grad.cpu().numpy(), go) <= TOL64
