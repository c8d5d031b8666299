"""Differentiation form: torch.autograd.Function whose backward is the
transpose solve over the solver's transposed view plus the grad_val pass (or,
under "syncfree_csc", the column-driven transpose with grad_val fused).
Checked against the serial host adjoint (oracle BACKWARD executor), against
central finite differences along random directions (h = 1e-6), and with
torch.autograd.gradcheck."""
from __future__ import annotations

import numpy as np
import pytest

import capellinisptrsv_gb300 as cs
import oracle
from conftest import rel_inf_err

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def t(a, grad=False):
    x = torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    return x.requires_grad_(grad)


def test_backward_matches_serial_host_adjoint():
    m = cs.generate("grad_1m", n=100_000, seed=0)
    k = 16
    b = np.random.default_rng(0).standard_normal((m.n, k))
    xstar = np.random.default_rng(1).standard_normal((m.n, k))
    val = t(m.val, True)
    bt = t(b, True)
    solver = cs.TriangularSolver(t(m.rowptr), t(m.colidx), val.detach())
    x = cs.sptrsv(solver, val, bt)
    loss = 0.5 * ((x - t(xstar)) ** 2).sum()
    loss.backward()
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    go = xo - xstar
    yo = oracle.solve_csr_transpose(m.rowptr, m.colidx, m.val, go)
    gvo = oracle.grad_val(m.rowptr, m.colidx, yo, xo)
    assert rel_inf_err(x.detach().cpu().numpy(), xo) <= 1e-12
    assert rel_inf_err(bt.grad.cpu().numpy(), yo) <= 1e-12
    assert rel_inf_err(val.grad.cpu().numpy(), gvo) <= 1e-12


def test_central_finite_differences_64_directions():
    m = cs.generate("grad_1m", n=20_000, seed=1)
    k = 16
    rng = np.random.default_rng(2)
    b = rng.standard_normal((m.n, k))
    xstar = rng.standard_normal((m.n, k))
    solver = cs.TriangularSolver(t(m.rowptr), t(m.colidx), t(m.val))

    def loss_of(vv, bb):
        with torch.no_grad():
            x = cs.sptrsv(solver, vv, bb)
            return float(0.5 * ((x - t(xstar)) ** 2).sum())

    val = t(m.val, True)
    bt = t(b, True)
    x = cs.sptrsv(solver, val, bt)
    (0.5 * ((x - t(xstar)) ** 2).sum()).backward()
    gval, gb = val.grad.cpu().numpy(), bt.grad.cpu().numpy()
    h = 1e-6
    eps = np.finfo(np.float64).eps
    worst = 0.0
    for d in range(64):
        dv = rng.standard_normal(m.nnz)
        db = rng.standard_normal((m.n, k))
        fp = loss_of(t(m.val + h * dv), t(b + h * db))
        fm = loss_of(t(m.val - h * dv), t(b - h * db))
        fd = (fp - fm) / (2 * h)
        an = float(np.dot(gval, dv) + np.sum(gb * db))
        # central differences carry round-off ~ eps*|loss|/h (here |loss| ~ 1e5,
        # so ~0.04 absolute) plus O(h^2) truncation; allow 8x that floor
        noise = 8 * eps * (abs(fp) + abs(fm)) / (2 * h) + 1e-7 * abs(an)
        worst = max(worst, abs(fd - an) / noise)
    print(f"worst |FD - analytic| / noise floor over 64 directions: {worst:.3f}")
    assert worst < 1.0


def test_gradcheck_small():
    m = cs.generate(n=60, kmin=1, kmax=4, band=20, seed=3)
    solver = cs.TriangularSolver(t(m.rowptr), t(m.colidx), t(m.val))
    val = t(m.val, True)
    b = t(np.random.default_rng(0).standard_normal((m.n, 3)), True)
    # the backward accumulates with fp64 atomics: repeated backwards agree to
    # rounding, not bit for bit (nondet_tol)
    assert torch.autograd.gradcheck(lambda vv, bb: cs.sptrsv(solver, vv, bb), (val, b), eps=1e-6,
                                    atol=1e-7, rtol=1e-6, nondet_tol=1e-12)


def test_module_with_parameter_trains():
    m = cs.generate(n=2000, kmin=1, kmax=4, band=100, seed=4)
    from capellinisptrsv_gb300.autograd import DifferentiableTriangular
    op = DifferentiableTriangular(t(m.rowptr), t(m.colidx), t(m.val))
    b = t(np.random.default_rng(1).standard_normal((m.n, 2)))
    target = t(np.random.default_rng(2).standard_normal((m.n, 2)))
    opt = torch.optim.SGD(op.parameters(), lr=1e-3)
    losses = []
    for _ in range(5):
        opt.zero_grad()
        loss = 0.5 * ((op(b) - target) ** 2).sum()
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    assert losses[-1] < losses[0]


def test_two_forwards_share_a_solver():
    """Two forwards through one solver with different value tensors, then one
    backward: each backward must solve with its own forward's values (the
    solver is re-bound to them when another forward re-bound it since)."""
    m = cs.generate(n=20_000, kmin=1, kmax=6, band=500, seed=9)
    k = 4
    b = np.random.default_rng(3).standard_normal((m.n, k))
    v1, v2 = m.val, m.val * 1.25
    val1, val2 = t(v1, True), t(v2, True)
    solver = cs.TriangularSolver(t(m.rowptr), t(m.colidx), val1.detach())
    x1 = cs.sptrsv(solver, val1, t(b))
    x2 = cs.sptrsv(solver, val2, t(b))
    loss = (x1 ** 2).sum() + 3.0 * x2.sum()
    loss.backward()
    for v, val, g in ((v1, val1, 2.0 * x1.detach().cpu().numpy()), (v2, val2, np.full((m.n, k), 3.0))):
        xo = oracle.solve_csr_lower(m.rowptr, m.colidx, v, b)
        yo = oracle.solve_csr_transpose(m.rowptr, m.colidx, v, g)
        assert rel_inf_err(val.grad.cpu().numpy(), oracle.grad_val(m.rowptr, m.colidx, yo, xo)) <= 1e-12
