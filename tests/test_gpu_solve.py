"""GPU parity of the sync-free solves against the oracle (the reference's serial
executor restated in C, pinned bit-for-bit by tests/test_oracle.py).

Tolerances (relative infinity-norm error against the FP64 oracle):
  FP64: 1e-12          FP32: 1e-5 against the FP32 oracle
All calls go through the C-ABI (capellinisptrsv_gb300 binds it with ctypes).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import capellinisptrsv_gb300 as cs
import oracle
from conftest import rel_inf_err

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL64, TOL32 = 1e-12, 1e-5
DEV = "cuda:0"


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def solver_for(m, dtype=np.float64, on_device=True, **kw):
    val = m.val.astype(dtype)
    if on_device:
        return cs.TriangularSolver(dev(m.rowptr), dev(m.colidx), dev(val), **kw)
    return cs.TriangularSolver(m.rowptr, m.colidx, val, **kw)


@pytest.fixture(scope="module")
def plain20k():
    return cs.generate("plain_20k", seed=0)


SCHEDULES = ["level", "natural"]


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("alg", ["wrtfst", "twopart", "mix", "auto"])
@pytest.mark.parametrize("on_device", [True, False])
def test_plain_20k_fp64(plain20k, alg, on_device, schedule):
    m = plain20k
    _, b = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, m.val)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    s = solver_for(m, on_device=on_device, algorithm=alg, schedule=schedule)
    x = host(s.solve(dev(b)))
    s.status()
    assert rel_inf_err(x, xo) <= TOL64
    assert np.max(np.abs(x - 1.0)) <= 0.01  # the reference's own self-check (x_ref = ones)


def test_plain_20k_fp32_and_its_fp64_error(plain20k):
    m = plain20k
    v32 = m.val.astype(np.float32)
    _, b32 = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, v32)
    x32o = oracle.solve_csr_lower(m.rowptr, m.colidx, v32, b32)
    _, b64 = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, m.val)
    x64o = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b64)
    s = solver_for(m, np.float32)
    x = host(s.solve(dev(b32)))
    assert rel_inf_err(x, x32o) <= TOL32
    err64 = rel_inf_err(x, x64o)   # stated, not bounded by the FP32 tolerance alone
    print(f"FP32 result vs FP64 oracle: {err64:.3e}")
    assert err64 < 1e-4


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("rows_per_thread", [1, 2, 4])
@pytest.mark.parametrize("block", [64, 256, 512])
def test_launch_shapes(plain20k, rows_per_thread, block, schedule):
    m = plain20k
    b = cs.normal(m.n, seed=1)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    s = solver_for(m, schedule=schedule)
    s.set_tuning(rows_per_thread, block, 0)
    x = host(s.solve(dev(b)))
    assert rel_inf_err(x, xo) <= TOL64


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_deterministic_and_schedules_agree(plain20k, schedule):
    """Sums are taken in storage order whatever the arrival order: repeated solves
    and the write-first / two-phase schedules give identical bits."""
    m = plain20k
    b = dev(cs.normal(m.n, seed=2))
    s = solver_for(m, algorithm="wrtfst", schedule=schedule)
    x1, x2 = host(s.solve(b)), host(s.solve(b))
    s.set_algorithm("twopart")
    x3 = host(s.solve(b))
    assert np.array_equal(x1.view(np.uint64), x2.view(np.uint64))
    assert np.array_equal(x1.view(np.uint64), x3.view(np.uint64))


EDGE = ["single", "diagonal_only", "bidiagonal_chain", "stride64_chain", "dense_band_40", "row_512",
        "ragged_33", "full_lower_64"]


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("name", EDGE)
@pytest.mark.parametrize("alg", ["wrtfst", "twopart", "mix", "syncfree_csc"])
def test_edge_cases_against_golden(golden, name, alg, schedule):
    """Forward and transposed solves; the transposes walk the transposed view
    with the row kernel of `alg`, or (syncfree_csc) the stored rows as columns."""
    rp, ci, v = (golden[f"edge_{name}_{k}"] for k in ("rowptr", "colidx", "val"))
    n = len(rp) - 1
    b1 = np.random.default_rng(11).standard_normal(n)
    b4 = np.random.default_rng(12).standard_normal((n, 4))
    s = cs.TriangularSolver(dev(rp), dev(ci), dev(v), algorithm=alg, schedule=schedule)
    s.set_mix_border(4)
    assert rel_inf_err(host(s.solve(dev(b1))), golden[f"edge_{name}_x1"]) <= TOL64
    assert rel_inf_err(host(s.solve(dev(b4))), golden[f"edge_{name}_x4"]) <= TOL64
    assert rel_inf_err(host(s.solve_transpose(dev(b1))), golden[f"edge_{name}_y1"]) <= TOL64
    assert rel_inf_err(host(s.solve_transpose(dev(b4))), golden[f"edge_{name}_y4"]) <= TOL64
    s.status()


TRANSPOSE_PATHS = {"rows": "auto", "columns": "syncfree_csc"}


@pytest.mark.parametrize("path", list(TRANSPOSE_PATHS))
@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("nrhs", [1, 2, 3, 4, 8, 16, 32, 40])
def test_multi_rhs_forward_adjoint_grad(nrhs, schedule, path):
    """The transposes run over the transposed view (rows, then the gradient
    pass) or column-driven over the stored rows with the gradient fused."""
    m = cs.generate(n=30_000, kmin=1, kmax=9, band=3000, seed=nrhs)
    b = np.random.default_rng(nrhs).standard_normal((m.n, nrhs))
    g = np.random.default_rng(nrhs + 100).standard_normal((m.n, nrhs))
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    yo = oracle.solve_csr_transpose(m.rowptr, m.colidx, m.val, g)
    go = oracle.grad_val(m.rowptr, m.colidx, yo, xo)
    s = solver_for(m, schedule=schedule, algorithm=TRANSPOSE_PATHS[path])
    x = s.solve(dev(b))
    y, gv = s.solve_transpose_grad(dev(g), x)
    y2 = s.solve_transpose(dev(g))
    gv2 = s.grad_val(y2, x)
    s.status()
    assert rel_inf_err(host(x), xo) <= TOL64
    assert rel_inf_err(host(y), yo) <= TOL64
    assert rel_inf_err(host(y2), yo) <= TOL64
    assert rel_inf_err(host(gv), go) <= TOL64
    assert rel_inf_err(host(gv2), go) <= TOL64


@pytest.mark.parametrize("path", list(TRANSPOSE_PATHS))
@pytest.mark.parametrize("nrhs", [1, 4, 16])
def test_f32_forward_adjoint_grad(nrhs, path):
    """FP32 over the transposed view, and through the column kernel's 8-byte
    sum-and-count words, against the FP64 oracle."""
    m = cs.generate(n=30_000, kmin=1, kmax=9, band=3000, seed=60 + nrhs)
    shape = (m.n, nrhs) if nrhs > 1 else (m.n,)
    b = np.random.default_rng(nrhs).standard_normal(shape)
    g = np.random.default_rng(nrhs + 100).standard_normal(shape)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    yo = oracle.solve_csr_transpose(m.rowptr, m.colidx, m.val, g)
    go = oracle.grad_val(m.rowptr, m.colidx, yo, xo)
    s = solver_for(m, np.float32, algorithm=TRANSPOSE_PATHS[path])
    x = s.solve(dev(b.astype(np.float32)))
    y, gv = s.solve_transpose_grad(dev(g.astype(np.float32)), x)
    s.status()
    assert rel_inf_err(host(x), xo) <= TOL32
    assert rel_inf_err(host(y), yo) <= TOL32
    assert rel_inf_err(host(gv), go) <= TOL32


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_strided_rhs_layout(schedule):
    """ld > nrhs: a column slice of a wider buffer."""
    m = cs.generate(n=5000, kmin=1, kmax=5, band=500, seed=8)
    wide = np.random.default_rng(0).standard_normal((m.n, 7))
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, wide[:, 2:5])
    bt = dev(wide)
    xt = torch.full_like(bt, 123.0)
    s = solver_for(m, schedule=schedule)
    s.solve(bt[:, 2:5], xt[:, 2:5])
    out = host(xt)
    assert rel_inf_err(out[:, 2:5], xo) <= TOL64
    assert np.all(out[:, :2] == 123.0) and np.all(out[:, 5:] == 123.0)


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_wide_4m_full_size_fp64_and_fp32(schedule):
    """The 4M-row workload at full size against the oracle (it finishes in well under a second)."""
    m = cs.generate("wide_4m", seed=0)
    _, b = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, m.val)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    s = solver_for(m, schedule=schedule)
    x = host(s.solve(dev(b)))
    s.status()
    assert rel_inf_err(x, xo) <= TOL64
    v32 = m.val.astype(np.float32)
    _, b32 = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, v32)
    x32o = oracle.solve_csr_lower(m.rowptr, m.colidx, v32, b32)
    s32 = solver_for(m, np.float32, schedule=schedule)
    x32 = host(s32.solve(dev(b32)))
    assert rel_inf_err(x32, x32o) <= TOL32
    print(f"wide_4m FP32 vs FP64 oracle: {rel_inf_err(x32, xo):.3e}")


@pytest.mark.parametrize("path", list(TRANSPOSE_PATHS))
def test_wide_4m_full_size_csc(path):
    """The 4M-row workload as a CSC handle (the reference's SyncFree_csc input),
    solved over the transposed view or column by column, against the oracle."""
    m = cs.generate("wide_4m", seed=0)
    _, b = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, m.val)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    cp, ri, cv = cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)
    s = cs.TriangularSolver(dev(cp), dev(ri), dev(cv), fmt="csc", algorithm=TRANSPOSE_PATHS[path])
    x = host(s.solve(dev(b)))
    s.status()
    assert rel_inf_err(x, xo) <= TOL64
    assert np.max(np.abs(x - 1.0)) <= 1e-4  # the reference's own self-check (x_ref = ones)


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_zipf_mix_path(schedule):
    m = cs.generate("zipf_1m", seed=0, n=200_000)
    b = cs.normal(m.n, seed=3)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    s = solver_for(m, algorithm="mix", schedule=schedule)
    x = host(s.solve(dev(b)))
    s.status()
    info = s.info()
    assert info["warp_occupy"] > 0.0  # heavy groups went warp-per-row
    assert rel_inf_err(x, xo) <= TOL64


def test_zipf40_near_serial_chain():
    """The Zipf workload with its count floored at 38 (~40 off-diagonals per row,
    about 1.5 rows per level): AUTO, FP64, against the oracle."""
    m = cs.generate("zipf40_1m", seed=0, n=60_000)
    b = cs.normal(m.n, seed=40)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    s = solver_for(m)
    for _ in range(2):
        x = host(s.solve(dev(b)))
        s.status()
        assert rel_inf_err(x, xo) <= TOL64
    assert s.info()["levels"] > m.n // 2


@pytest.mark.parametrize("k", [1, 4])
def test_auto_deep_matrix_gives_every_row_a_warp(k):
    """Levels narrower than 32 rows: AUTO runs every row warp-per-row (the row's
    newest dependency folded last), single and multi-RHS."""
    m = cs.generate("zipf_1m", seed=0, n=200_000)
    b = cs.normal(m.n * k, seed=31).reshape(m.n, k) if k > 1 else cs.normal(m.n, seed=31)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    s = solver_for(m)
    for _ in range(2):
        x = host(s.solve(dev(b)))
        s.status()
        assert rel_inf_err(x, xo) <= TOL64
    if k == 1:  # info() describes the single-RHS launch
        assert s.info()["warp_occupy"] == pytest.approx(1.0)


@pytest.mark.parametrize("schedule", SCHEDULES)
@pytest.mark.parametrize("k", [1, 2])
def test_upper_csr_warp_per_row(schedule, k):
    """Upper CSR through the warp-per-row kernel (border 1: every row), where the
    natural schedule's newest dependency is the first stored entry."""
    m = cs.generate(n=20_000, kmin=1, kmax=12, band=700, seed=6)
    cp, ri, cv = cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)
    g = cs.normal(m.n * k, seed=32).reshape(m.n, k) if k > 1 else cs.normal(m.n, seed=32)
    yo = oracle.solve_csr_transpose(m.rowptr, m.colidx, m.val, g)
    s = cs.TriangularSolver(dev(cp), dev(ri), dev(cv), uplo="upper", algorithm="mix", schedule=schedule)
    s.set_mix_border(1)
    y = host(s.solve(dev(g)))
    s.status()
    assert rel_inf_err(y, yo) <= TOL64


@pytest.mark.parametrize("path", list(TRANSPOSE_PATHS))
@pytest.mark.parametrize("schedule", SCHEDULES)
def test_upper_csr_and_csc_paths(schedule, path):
    """Upper-triangular CSR (backward substitution) and CSC handles, forward
    and transposed, against the oracle on the same matrix.  A CSC solve walks
    the transposed view (rows) or the stored columns (the warp-per-column
    kernel); so does the transpose of the upper CSR handle."""
    m = cs.generate(n=20_000, kmin=1, kmax=6, band=900, seed=5)
    cp, ri, cv = cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)
    b = cs.normal(m.n, seed=6)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)   # L x = b
    yo = oracle.solve_csr_transpose(m.rowptr, m.colidx, m.val, b)  # L^T y = b
    # CSC of L == CSR of U = L^T (diagonal first in each row)
    alg = TRANSPOSE_PATHS[path]
    up = cs.TriangularSolver(dev(cp), dev(ri), dev(cv), uplo="upper", schedule=schedule, algorithm=alg)
    assert rel_inf_err(host(up.solve(dev(b))), yo) <= TOL64
    assert rel_inf_err(host(up.solve_transpose(dev(b))), xo) <= TOL64
    csc = cs.TriangularSolver(dev(cp), dev(ri), dev(cv), fmt="csc", schedule=schedule, algorithm=alg)
    assert rel_inf_err(host(csc.solve(dev(b))), xo) <= TOL64
    assert rel_inf_err(host(csc.solve_transpose(dev(b))), yo) <= TOL64
    b4 = np.random.default_rng(4).standard_normal((m.n, 4))
    assert rel_inf_err(host(csc.solve(dev(b4))),
                       oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b4)) <= TOL64
    up.status()
    csc.status()
    assert (csc.info()["algorithm"] == 4) == (path == "columns")


def test_set_values_refreshes(plain20k):
    """New values reach both views: the forward's and, once built, the
    transposed view's level values."""
    m = plain20k
    s = solver_for(m)
    b = cs.normal(m.n, seed=7)
    s.solve_transpose(dev(b))  # builds the transposed view with the old values
    v2 = m.val * 1.5
    s.set_values(dev(v2))
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, v2, b)
    assert rel_inf_err(host(s.solve(dev(b))), xo) <= TOL64
    yo = oracle.solve_csr_transpose(m.rowptr, m.colidx, v2, b)
    assert rel_inf_err(host(s.solve_transpose(dev(b))), yo) <= TOL64
    v3 = m.val * 0.75
    s.refresh_values(dev(v3))
    yo = oracle.solve_csr_transpose(m.rowptr, m.colidx, v3, b)
    assert rel_inf_err(host(s.solve_transpose(dev(b))), yo) <= TOL64


def test_solve_host_buffers(plain20k):
    m = plain20k
    s = solver_for(m, on_device=False)
    b = cs.normal((m.n * 2), seed=8).reshape(m.n, 2)
    x = s.solve_host(b)
    assert rel_inf_err(x, oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)) <= TOL64


@pytest.mark.parametrize("k", [1, 3])
def test_solve_host_pinned_buffers_in_place(plain20k, k):
    """Page-locked host buffers are solved in place (no staging copies)."""
    m = plain20k
    s = solver_for(m, on_device=False)
    b = cs.normal(m.n * k, seed=18).reshape(m.n, k) if k > 1 else cs.normal(m.n, seed=18)
    bh = torch.from_numpy(np.ascontiguousarray(b)).pin_memory()
    xh = torch.full_like(bh, float("nan")).pin_memory()
    for _ in range(2):
        s.solve_host(bh.numpy(), xh.numpy())
        assert rel_inf_err(xh.numpy(), oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)) <= TOL64


@pytest.mark.parametrize("k", [1, 2])
def test_solve_host_pinned_buffers_wide_levels(k):
    """Two levels of 35,000 rows (wider than the 32k rows at which a single
    right-hand side is copied rather than read in place), pinned buffers."""
    n = 70_000
    rng = np.random.default_rng(41)
    odd = np.arange(n) % 2 == 1
    rowptr = np.concatenate([[0], np.cumsum(np.where(odd, 2, 1))]).astype(np.int32)
    colidx = np.empty(rowptr[-1], np.int32)
    val = np.empty(rowptr[-1])
    off = rng.uniform(-1, 1, n)
    colidx[rowptr[:-1][odd]] = np.arange(n)[odd] - 1
    val[rowptr[:-1][odd]] = off[odd]
    colidx[rowptr[1:] - 1] = np.arange(n)
    val[rowptr[1:] - 1] = 1 + np.where(odd, np.abs(off), 0)
    assert cs.matrix_layer(n, n, len(colidx), rowptr, colidx)[0] == 2
    s = cs.TriangularSolver(rowptr, colidx, val)
    b = cs.normal(n * k, seed=42).reshape(n, k) if k > 1 else cs.normal(n, seed=42)
    bh = torch.from_numpy(np.ascontiguousarray(b)).pin_memory()
    xh = torch.full_like(bh, float("nan")).pin_memory()
    for _ in range(2):
        s.solve_host(bh.numpy(), xh.numpy())
        assert rel_inf_err(xh.numpy(), oracle.solve_csr_lower(rowptr, colidx, val, b)) <= TOL64


def test_graph_replay_and_autotune(plain20k):
    m = plain20k
    s = solver_for(m)
    b = dev(cs.normal(m.n, seed=9))
    x = torch.empty_like(b)
    st = torch.cuda.Stream()
    ms = s.autotune(b, x, stream=st)
    assert ms > 0
    with torch.cuda.stream(st):
        for _ in range(3):
            s.graph_solve(b, x, st)
    st.synchronize()
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, host(b))
    assert rel_inf_err(host(x), xo) <= TOL64


def test_invalid_matrices_are_rejected():
    rp = np.array([0, 1, 3], np.int32)
    bad_ci = np.array([0, 1, 0], np.int32)  # row 1: diagonal not last
    v = np.ones(3)
    with pytest.raises(cs.CapspError) as e:
        cs.TriangularSolver(rp, bad_ci, v)
    assert e.value.status == 1
    with pytest.raises(cs.CapspError):
        cs.TriangularSolver(dev(rp), dev(bad_ci), dev(v))
    with pytest.raises(cs.CapspError):  # zero diagonal
        cs.TriangularSolver(rp, np.array([0, 0, 1], np.int32), np.array([1.0, 1.0, 0.0]))


@pytest.mark.parametrize("schedule", SCHEDULES)
def test_timeout_is_reported_and_context_survives(plain20k, schedule):
    """A row that never publishes (debug hook): its dependants' waits run out
    after 20 ms, the solve reports TIMEOUT, and the next solve is clean."""
    m = plain20k
    s = solver_for(m, schedule=schedule)
    b = dev(cs.normal(m.n, seed=10))
    s.debug_stuck_row(5000, timeout_s=0.02)
    x = s.solve(b)
    with pytest.raises(cs.CapspError) as e:
        s.status()
    assert e.value.status == 2
    xh = host(x)
    assert np.isnan(xh).any()
    s.debug_stuck_row(-1, timeout_s=10.0)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, host(b))
    assert rel_inf_err(host(s.solve(b)), xo) <= TOL64
    s.status()


def test_hop_latency_probe_runs():
    lat_warp = cs.hop_latency(n=20_000, stride=1)
    lat_l2 = cs.hop_latency(n=20_000, stride=256)
    print(f"hop latency: in-warp {lat_warp:.0f} ns, cross-warp {lat_l2:.0f} ns")
    assert lat_warp > 0 and lat_l2 > 0


def test_level_schedule_reports_levels(plain20k):
    m = plain20k
    s = solver_for(m)
    info = s.info()
    assert info["schedule"] == 1
    assert info["levels"] == cs.matrix_layer(m.n, m.n, m.nnz, m.rowptr, m.colidx)[0]


def test_l2_policy_modes_bit_identical(plain20k):
    """The L2 policy changes caching only: the three modes give the same bits,
    and leaving the window modes restores the process's persisting carve-out."""
    m = plain20k
    _, b = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, m.val)
    s = solver_for(m)
    bd = dev(b)
    ref = host(s.solve(bd))
    for mode in ("window+hints", "window", "hints"):
        s.set_l2_policy(mode)
        assert np.array_equal(host(s.solve(bd)), ref), mode
    s.status()
    assert rel_inf_err(ref, oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)) <= TOL64


def _two_wide_levels(n=200_000, seed=5):
    """Rows < n/2 have no dependencies; row i >= n/2 depends on i - n/2 - 7
    (when that exists) and i - n/2: two levels of n/2 rows, the wide-level
    launch shape (levels of 32k rows and more: 16 warps per SM)."""
    rng = np.random.default_rng(seed)
    h = n // 2
    i = np.arange(n)
    far = (i >= h + 7)
    near = (i >= h)
    cnt = 1 + far + near
    rp = np.zeros(n + 1, np.int64)
    rp[1:] = np.cumsum(cnt)
    ci = np.empty(rp[-1], np.int32)
    v = np.empty(rp[-1])
    off1 = rng.uniform(-1, 1, n)
    off2 = rng.uniform(-1, 1, n)
    k = rp[:-1].copy()
    ci[k[far]] = i[far] - h - 7
    v[k[far]] = off1[far]
    k[far] += 1
    ci[k[near]] = i[near] - h
    v[k[near]] = off2[near]
    k[near] += 1
    ci[k] = i
    v[k] = 1.0 + np.where(far, np.abs(off1), 0.0) + np.where(near, np.abs(off2), 0.0)
    return cs.CSRMatrix(n, rp.astype(np.int32), ci, v)


@pytest.mark.parametrize("k,ld", [(1, 1), (3, 5), (16, 16), (40, 41)])
def test_wide_levels_strided_multi_block_rhs(k, ld):
    """Two levels of 100k rows: strided right-hand sides, several 32-RHS
    blocks (k = 40), and columns past nrhs left untouched."""
    m = _two_wide_levels()
    s = solver_for(m)
    assert s.info()["levels"] == 2
    rng = np.random.default_rng(k)
    b = np.zeros((m.n, ld))
    b[:, :k] = rng.standard_normal((m.n, k))
    bd = dev(b)
    xd = torch.full_like(bd, 7.0)
    N = cs._native
    N.check(N.lib.capsp_solve(s._h, C.c_void_p(bd.data_ptr()), C.c_void_p(xd.data_ptr()), k, ld,
                              C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    s.status()
    x = host(xd)
    xo = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, np.ascontiguousarray(b[:, :k]))
    assert rel_inf_err(x[:, :k].reshape(m.n, k), xo.reshape(m.n, k)) <= TOL64
    assert np.all(x[:, k:] == 7.0)  # columns past nrhs untouched


@pytest.mark.parametrize("nrhs", [1, 4])
def test_csc_transpose_grad(nrhs):
    """The backward of a CSC handle: y = L^-T g over its stored columns (rows
    of L^T), then grad_val over the CSC entries (column j, row idx[k]):
    grad_val[k] = -sum_r y[idx[k], r] x[j, r]."""
    m = cs.generate(n=20_000, kmin=1, kmax=9, band=800, seed=13)
    cp, ri, cv = cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)
    shape = (m.n, nrhs) if nrhs > 1 else (m.n,)
    g = np.random.default_rng(14).standard_normal(shape)
    x = np.random.default_rng(15).standard_normal(shape)
    yo = oracle.solve_csr_transpose(m.rowptr, m.colidx, m.val, g)
    s = cs.TriangularSolver(dev(cp), dev(ri), dev(cv), fmt="csc")
    y, gv = s.solve_transpose_grad(dev(g), dev(x))
    s.status()
    col = np.repeat(np.arange(m.n), np.diff(cp))
    y2, x2 = yo.reshape(m.n, -1), x.reshape(m.n, -1)
    go = -np.einsum("kr,kr->k", y2[ri], x2[col])
    assert rel_inf_err(host(y), yo) <= TOL64
    assert rel_inf_err(host(gv), go) <= TOL64
