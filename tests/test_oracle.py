"""The oracle (oracle/oracle.c) is pinned bit-for-bit to the reference's serial
executor: against the committed golden vectors (produced by the reference
itself, tests/golden/make_golden.py) and, where the reference sources are
present, against oracle/_ref live."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

import capellinisptrsv_gb300 as cs
import oracle


def sha(a) -> np.ndarray:
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), dtype=np.uint8)


EDGE = ["single", "diagonal_only", "bidiagonal_chain", "stride64_chain", "dense_band_40", "row_512",
        "ragged_33", "full_lower_64"]


def edge_rhs(n):
    return np.random.default_rng(11).standard_normal(n), np.random.default_rng(12).standard_normal((n, 4))


def test_generator_pinned(golden):
    m = cs.generate("plain_20k", seed=0)
    assert m.nnz == int(golden["plain_20k_nnz"][0])
    assert m.digest() == int(golden["plain_20k_digest"][0])


@pytest.mark.parametrize("t,dt", [("f64", np.float64), ("f32", np.float32)])
def test_plain_20k_matches_reference(golden, t, dt):
    m = cs.generate("plain_20k", seed=0)
    val = m.val.astype(dt)
    _, b = cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, val)
    assert np.array_equal(sha(b), golden[f"plain_20k_b_{t}_sha"]), "get_x_b differs from the reference"
    x = oracle.solve_csr_lower(m.rowptr, m.colidx, val, b)
    assert np.array_equal(x[:64], golden[f"plain_20k_x_{t}_head"])
    assert np.array_equal(sha(x), golden[f"plain_20k_x_{t}_sha"])


def test_plain_20k_multi_rhs_forward_and_adjoint(golden):
    m = cs.generate("plain_20k", seed=0)
    rhs = np.random.default_rng(3).standard_normal((m.n, 3))
    x = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, rhs)
    y = oracle.solve_csr_transpose(m.rowptr, m.colidx, m.val, rhs)
    assert np.array_equal(sha(x), golden["plain_20k_x_rhs3_sha"])
    assert np.array_equal(sha(y), golden["plain_20k_y_rhs3_sha"])


@pytest.mark.parametrize("name", EDGE)
def test_edge_cases_match_reference(golden, name):
    rp, ci, v = (golden[f"edge_{name}_{k}"] for k in ("rowptr", "colidx", "val"))
    b1, b4 = edge_rhs(len(rp) - 1)
    assert np.array_equal(oracle.solve_csr_lower(rp, ci, v, b1), golden[f"edge_{name}_x1"])
    assert np.array_equal(oracle.solve_csr_lower(rp, ci, v, b4), golden[f"edge_{name}_x4"])
    assert np.array_equal(oracle.solve_csr_transpose(rp, ci, v, b1), golden[f"edge_{name}_y1"])
    assert np.array_equal(oracle.solve_csr_transpose(rp, ci, v, b4), golden[f"edge_{name}_y4"])


def test_oracle_matches_live_reference():
    ref = oracle.ref()
    if ref is None:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    for seed in range(3):
        m = cs.generate(n=3000, kmin=0, kmax=9, band=300, seed=seed)
        rhs = np.random.default_rng(seed).standard_normal((m.n, 2))
        for dt in (np.float64, np.float32):
            v, bb = m.val.astype(dt), rhs.astype(dt)
            assert np.array_equal(oracle.solve_csr_lower(m.rowptr, m.colidx, v, bb),
                                  ref.solve_csr_lower(m.rowptr, m.colidx, v, bb))
            assert np.array_equal(oracle.solve_csr_transpose(m.rowptr, m.colidx, v, bb),
                                  ref.solve_csr_transpose(m.rowptr, m.colidx, v, bb))


def test_oracle_solution_is_a_solution():
    m = cs.generate(n=5000, kmin=1, kmax=8, band=500, seed=4)
    xt = np.random.default_rng(0).standard_normal((m.n, 2))
    b = cs.spmv(m, xt)
    x = oracle.solve_csr_lower(m.rowptr, m.colidx, m.val, b)
    assert np.max(np.abs(x - xt)) < 1e-10
    # adjoint: L^T y = g  <=>  <L^T y, z> == <y, L z>
    g = np.random.default_rng(1).standard_normal(m.n)
    y = oracle.solve_csr_transpose(m.rowptr, m.colidx, m.val, g)
    z = np.random.default_rng(2).standard_normal(m.n)
    assert abs(np.dot(g, z) - np.dot(y, cs.spmv(m, z))) < 1e-8 * np.linalg.norm(g) * np.linalg.norm(z) * 10


def test_oracle_rejects_malformed_instead_of_hanging():
    # row 1 references column 2 (> row): the serial in-degree check fails; the
    # reference would spin forever, the oracle returns an error
    rp = np.array([0, 1, 3, 4], np.int32)
    ci = np.array([0, 2, 1, 2], np.int32)
    v = np.ones(4)
    with pytest.raises(ValueError):
        oracle.solve_csr_lower(rp, ci, v, np.ones(3))


def test_oracle_grad_val_definition():
    m = cs.generate(n=200, kmin=1, kmax=4, band=20, seed=9)
    y = np.random.default_rng(0).standard_normal((m.n, 3))
    x = np.random.default_rng(1).standard_normal((m.n, 3))
    got = oracle.grad_val(m.rowptr, m.colidx, y, x)
    rows = np.repeat(np.arange(m.n), np.diff(m.rowptr))
    want = -np.sum(y[rows] * x[m.colidx], axis=1)
    assert np.allclose(got, want, rtol=1e-14, atol=1e-14)


def test_oracle_generator_matches_library_and_golden(golden):
    """The CPU legs generate their own inputs with liboracle's copy of the
    generator: same digest as the solver library's, and as the fixture."""
    n, rp, ci, v = oracle.generate("plain_20k", seed=0)
    assert int(rp[-1]) == int(golden["plain_20k_nnz"][0])
    assert oracle.digest(n, rp, ci, v) == int(golden["plain_20k_digest"][0])
    for name, kw in [("wide_4m", dict(n=50_000)), ("zipf_1m", dict(n=30_000)), ("grad_1m", dict(n=40_000)),
                     ("zipf40_1m", dict(n=5_000))]:
        on, orp, oci, ov = oracle.generate(name, seed=0, **kw)
        m = cs.generate(name, seed=0, **kw)
        assert on == m.n and oracle.digest(on, orp, oci, ov) == m.digest(), name
        assert np.array_equal(orp, m.rowptr) and np.array_equal(oci, m.colidx) and np.array_equal(ov, m.val)
    assert np.array_equal(oracle.normal(1000, seed=0, stream=7), cs.normal(1000, seed=0, stream=7))


def test_oracle_batched_generator_matches_library():
    n, rp, ci, v, so = oracle.generate_batched(24, seed=0)
    m = cs.generate_batched(24, seed=0)
    assert n == m.n
    for a, b in [(rp, m.rowptr), (ci, m.colidx), (v, m.val), (so, m.sys_rowoff)]:
        assert np.array_equal(a, b)


@pytest.mark.parametrize("t,dt", [("f64", np.float64), ("f32", np.float32)])
def test_oracle_get_x_b_matches_reference(golden, t, dt):
    m = cs.generate("plain_20k", seed=0)
    val = m.val.astype(dt)
    b = oracle.get_x_b(m.rowptr, val)
    assert np.array_equal(sha(b), golden[f"plain_20k_b_{t}_sha"])
    assert np.array_equal(b, cs.get_x_b(m.n, m.n, m.rowptr, m.colidx, val)[1])
