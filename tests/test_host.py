"""CPU tests of libcapsp's host side: the library loads and exports every
declared symbol, the generators and host preprocessing match the reference's
contracts (golden vectors from the reference itself), structure checks."""
from __future__ import annotations

import ctypes as C
import os
import re
from pathlib import Path

import numpy as np
import pytest

import capellinisptrsv_gb300 as cs
from capellinisptrsv_gb300 import _native as N

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    """Functions declared by the library headers (capsp_compat.h only holds inline
    wrappers over these and is checked by compiling against it)."""
    names = []
    for hdr in sorted((ROOT / "include").glob("*.h")):
        if hdr.name == "capsp_compat.h":
            continue
        text = re.sub(r"/\*.*?\*/", "", hdr.read_text(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M):
            name = m.group(1)
            if name not in ("if", "defined", "sizeof", "return"):
                names.append(name)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(N.lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert not [n for n in names if n not in N.EXPORTED]


COMPAT_C = r"""
#define CAPSP_COMPAT_HOST
#include "capsp_compat.h"
int use(const int *rp, const int *ci, const VT *v, int n, int nnz) {
    double t, g, bw, pre, wo, eo; int layer; double par;
    int *lrp, *lci; VT *lv; int nnzL; VT *x, *b;
    matrix_layer(n, n, nnz, rp, ci, v, &layer, &par);
    get_x_b(n, n, rp, ci, v, &x, &b);
    change2tran(n, nnz, (int *)rp, (int *)ci, (VT *)v, &nnzL, &lrp, &lci, &lv);
    sptrsv_syncfree_cuda(rp, ci, v, n, n, nnz, x, b, x, &pre, &t, &g, &bw);
    return spts_syncfree_cuda_csr_wrt(rp, ci, v, n, n, nnz, &t, &g, &bw) +
           spts_syncfree_cuda_csr(rp, ci, v, n, n, nnz, &t, &g, &bw) + (int)(pre + wo + eo);
}
"""


@pytest.mark.parametrize("lang,vt", [("c", "double"), ("c", "float"), ("c++", "double"), ("c++", "float")])
def test_compat_header_compiles_and_links(tmp_path, lang, vt):
    """Reference-style code (unsuffixed names, VALUE_TYPE chosen by the caller)
    compiles against capsp_compat.h and links against libcapsp.so."""
    import subprocess
    src = tmp_path / ("use.c" if lang == "c" else "use.cpp")
    src.write_text(COMPAT_C.replace("VT", vt))
    out = tmp_path / "libuse.so"
    cc = ["gcc", "-std=c11"] if lang == "c" else ["g++", "-std=c++17"]
    lib = ROOT / "capellinisptrsv_gb300" / "_build"
    r = subprocess.run([*cc, "-shared", "-fPIC", "-Werror", "-Wall", "-Wno-unused-variable",
                        "-Wno-uninitialized", "-Wno-maybe-uninitialized", "-I", str(ROOT / "include"),
                        str(src), "-L", str(lib), "-lcapsp", "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_generator_is_deterministic_and_follows_the_rules():
    a = cs.generate(n=7000, kmin=1, kmax=7, band=600, seed=3)
    b = cs.generate(n=7000, kmin=1, kmax=7, band=600, seed=3)
    assert a.digest() == b.digest()
    assert cs.generate(n=7000, kmin=1, kmax=7, band=600, seed=4).digest() != a.digest()
    rp, ci, v = a.rowptr, a.colidx, a.val
    for i in range(a.n):
        cols, vals = ci[rp[i]:rp[i + 1]], v[rp[i]:rp[i + 1]]
        k = len(cols) - 1
        assert cols[-1] == i
        assert k <= 7 and (k >= 1 or i == 0)
        assert np.all(np.diff(cols) > 0)
        assert np.all(cols[:-1] >= max(0, i - 600))
        assert np.all(np.abs(vals[:-1]) <= 1.0)
        assert vals[-1] == 1.0 + np.sum(np.abs(vals[:-1]))


def test_zipf_generator_near_far_rule():
    m = cs.generate(n=20_000, kind=N.GEN_ZIPF_NEAR_FAR, zipf_s=1.8, zipf_cap=512, near_window=32, seed=1)
    ks = np.diff(m.rowptr) - 1
    assert ks.max() <= 512 and ks[100:].min() >= 1
    i = 10_000
    cols = m.colidx[m.rowptr[i]:m.rowptr[i + 1] - 1]
    k = len(cols)
    assert np.sum(cols >= i - 32) >= (k + 1) // 2


def test_zipf_generator_count_floor():
    """kmin floors the Zipf count (zipf40_1m: mean ~40 off-diagonals per row); the
    default floor of 1 leaves the literal draw unchanged."""
    kw = dict(n=20_000, kind=N.GEN_ZIPF_NEAR_FAR, zipf_s=1.8, zipf_cap=512, near_window=32, seed=1)
    lit = cs.generate(**kw)
    assert cs.generate(kmin=1, **kw).digest() == lit.digest()
    m = cs.generate(kmin=38, **kw)
    ks = np.diff(m.rowptr) - 1
    rows = np.arange(m.n)
    assert np.all(ks == np.minimum(np.maximum(np.diff(lit.rowptr) - 1, 38), rows))
    assert 38 < ks[1000:].mean() < 43
    i = 10_000
    cols = m.colidx[m.rowptr[i]:m.rowptr[i + 1] - 1]
    assert np.sum(cols >= i - 32) >= min((len(cols) + 1) // 2, 32)


def test_normal_generator_moments():
    z = cs.normal(200_000, seed=5)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    assert np.array_equal(z, cs.normal(200_000, seed=5))


def test_change2tran_matches_reference(golden):
    rp, ci, va = golden["pre_A_rowptr"].copy(), golden["pre_A_colidx"].copy(), golden["pre_A_val"].copy()
    nnzL, lrp, lci, lv = cs.change2tran(len(rp) - 1, rp, ci, va)
    assert nnzL == len(golden["pre_L_colidx"])
    assert np.array_equal(lrp, golden["pre_L_rowptr"])
    assert np.array_equal(lci, golden["pre_L_colidx"])
    assert np.array_equal(lv, golden["pre_L_val"])


def test_layer_transposition_warp4_match_reference(golden):
    lrp, lci, lv = golden["pre_L_rowptr"], golden["pre_L_colidx"], golden["pre_L_val"]
    n = len(lrp) - 1
    lay, par = cs.matrix_layer(n, n, len(lci), lrp, lci, lv)
    assert lay == int(golden["pre_L_layer"][0]) and par == float(golden["pre_L_parallelism"][0])
    cp, ri, cv = cs.matrix_transposition(n, n, len(lci), lrp, lci, lv)
    assert np.array_equal(cp, golden["pre_L_csc_colptr"])
    assert np.array_equal(ri, golden["pre_L_csc_rowidx"])
    assert np.array_equal(cv, golden["pre_L_csc_val"])
    for border in (0, 2, 3, 10):
        ln, table, wo, eo = cs.matrix_warp4(n, n, len(lci), lrp, lci, lv, border=border)
        assert np.array_equal(table, golden[f"pre_warp4_{border}_table"])
        assert [wo, eo] == list(golden[f"pre_warp4_{border}_occ"])


def test_workload_stats_match_reference(golden):
    import hashlib
    m = cs.generate("plain_20k", seed=0)
    lay, par = cs.matrix_layer(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)
    assert lay == int(golden["plain_20k_layer"][0])
    assert par == float(golden["plain_20k_parallelism"][0])
    ln, table, wo, eo = cs.matrix_warp4(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val, border=10)
    assert ln == int(golden["plain_20k_warp4_len"][0])
    assert [wo, eo] == list(golden["plain_20k_warp4_occ"])
    assert np.array_equal(np.frombuffer(hashlib.sha256(table.tobytes()).digest(), np.uint8),
                          golden["plain_20k_warp4_sha"])


@pytest.mark.parametrize("name", ["general", "sym_pattern", "integer"])
def test_read_mtx_matches_reference(golden, tmp_path, name):
    p = tmp_path / f"{name}.mtx"
    p.write_bytes(golden[f"mtx_{name}_text"].tobytes())
    m, n, nnz, rp, ci, v = cs.read_mtx(str(p))
    assert (m, n, nnz) == tuple(int(golden[f"mtx_{name}_{k}"]) for k in ("m", "n", "nnz"))
    assert np.array_equal(rp, golden[f"mtx_{name}_rowptr"])
    assert np.array_equal(ci, golden[f"mtx_{name}_colidx"])
    assert np.array_equal(v, golden[f"mtx_{name}_val"])


def test_read_mtx_rejects_complex_and_missing(tmp_path):
    p = tmp_path / "c.mtx"
    p.write_text("%%MatrixMarket matrix coordinate complex general\n1 1 1\n1 1 1 0\n")
    with pytest.raises(ValueError):
        cs.read_mtx(str(p))
    with pytest.raises(ValueError):
        cs.read_mtx(str(tmp_path / "nope.mtx"))


def test_row_levels_histogram():
    m = cs.generate(n=3000, kmin=1, kmax=3, band=50, seed=2)
    levels, level, counts = cs.row_levels(m.n, m.rowptr, m.colidx)
    assert levels == cs.matrix_layer(m.n, m.n, m.nnz, m.rowptr, m.colidx)[0]
    assert counts[1:].sum() == m.n and counts[0] == 0
    for i in (0, 17, 2999):
        deps = m.colidx[m.rowptr[i]:m.rowptr[i + 1] - 1]
        assert level[i] == 1 + (level[deps].max() if len(deps) else 0)


@pytest.mark.parametrize("upper", [False, True])
def test_level_schedule_is_a_topological_level_order(upper):
    from capellinisptrsv_gb300.solver import level_layout, level_schedule
    m = cs.generate(n=4000, kmin=0, kmax=12, band=300, seed=6)
    rp, ci, v = m.rowptr, m.colidx, m.val
    if upper:  # the CSC of L is the CSR of U = L^T (diagonal first)
        rp, ci, v = cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)
    levels, order, pos, start = level_schedule(m.n, rp, ci, upper)
    assert levels == cs.matrix_layer(m.n, m.n, m.nnz, m.rowptr, m.colidx)[0]
    assert sorted(order) == list(range(m.n)) and np.array_equal(pos[order], np.arange(m.n))
    assert start[1] == 0 and start[levels + 1] == m.n
    dep_ptr, dep_idx, dep_src, diag_src = level_layout(m.n, rp, ci, order, pos, upper)
    for k in (0, 1, 777, m.n - 1):
        i = order[k]
        deps = dep_idx[dep_ptr[k]:dep_ptr[k + 1]]
        assert np.all(deps < k) and np.all(np.diff(deps) > 0)         # dependencies come first
        assert ci[diag_src[k]] == i
        assert sorted(order[deps]) == sorted(ci[dep_src[dep_ptr[k]:dep_ptr[k + 1]]])
        row = set(ci[rp[i]:rp[i + 1]]) - {i}
        assert set(order[deps]) == row
    # levels are contiguous blocks of positions
    lev_of_pos = np.repeat(np.arange(1, levels + 1), np.diff(start[1:levels + 2]))
    assert np.all(np.diff(lev_of_pos) >= 0)
    # inside a level (all narrower than 32k rows here): the rows of more than 8
    # dependencies (one pass of the row kernel) first, dependency count
    # non-increasing (63+ in one bucket), then solve order; then the other
    # rows by the position of their newest dependency, then solve order
    _check_level_order(rp, order, dep_ptr, dep_idx, start, levels, upper, wide=32768)
    ndep = np.diff(rp)[order] - 1
    assert np.any(ndep > 8)


def _check_level_order(rp, order, dep_ptr, dep_idx, start, levels, upper, wide):
    n = len(order)
    ndep = np.minimum(np.diff(rp)[order] - 1, 63)
    solve_rank = (n - 1 - order) if upper else order
    newest = np.array([dep_idx[dep_ptr[k]:dep_ptr[k + 1]].max() if dep_ptr[k + 1] > dep_ptr[k] else -1
                       for k in range(n)])
    for l in range(1, levels + 1):
        a, b = start[l], start[l + 1]
        d, key, r = ndep[a:b], newest[a:b], solve_rank[a:b]
        by_count = bool(d.size and d.max() > 8) and b - a >= wide
        multi = (d > 8) | by_count
        group = np.where(multi, 0, 1)
        bucket = np.where(multi, -d, 0)
        key = np.where(multi, 0, key)
        rows = list(zip(group.tolist(), bucket.tolist(), key.tolist(), r.tolist()))
        assert rows == sorted(rows), l


def test_level_order_of_a_wide_level():
    """A level of 32k rows or more that holds a multi-pass row is ordered by
    dependency count alone (then solve order)."""
    from capellinisptrsv_gb300.solver import level_layout, level_schedule
    rng = np.random.default_rng(3)
    n0, n1 = 100, 40_000  # level 1: rows 0..99; level 2: 40,000 rows on them
    counts = np.concatenate([np.zeros(n0, np.int64), rng.integers(1, 13, n1)])
    rp = np.concatenate([[0], np.cumsum(counts + 1)]).astype(np.int32)
    ci = np.empty(rp[-1], np.int32)
    for i in range(n0 + n1):
        ci[rp[i]:rp[i + 1] - 1] = np.sort(rng.choice(n0, counts[i], replace=False)) if counts[i] else []
        ci[rp[i + 1] - 1] = i
    levels, order, pos, start = level_schedule(n0 + n1, rp, ci, False)
    assert levels == 2 and start[3] - start[2] == n1
    dep_ptr, dep_idx, _, _ = level_layout(n0 + n1, rp, ci, order, pos, False)
    _check_level_order(rp, order, dep_ptr, dep_idx, start, levels, False, wide=32768)


def _validate(rp, ci, fmt=N.FMT_CSR, uplo=N.LOWER):
    rp, ci = np.asarray(rp, np.int32), np.asarray(ci, np.int32)
    msg = C.create_string_buffer(256)
    rc = N.lib.capsp_validate(len(rp) - 1, len(ci), rp.ctypes.data_as(C.c_void_p), ci.ctypes.data_as(C.c_void_p),
                              fmt, uplo, msg, 256)
    return rc, msg.value.decode()


def test_validation_catches_malformed_structures():
    assert _validate([0, 1, 3], [0, 0, 1])[0] == 0
    assert _validate([0, 1, 3], [0, 1, 0])[0] != 0          # diagonal not last
    assert _validate([0, 1, 2], [0, 0])[0] != 0             # row 1 lacks its diagonal
    assert _validate([0, 2, 3], [1, 0, 1])[0] != 0          # upper entry in a lower matrix
    assert _validate([0, 1, 1], [0])[0] != 0                # empty row
    assert _validate([0, 1, 3], [0, 1, 0], uplo=N.UPPER)[0] != 0
    assert _validate([0, 2, 3], [0, 1, 1], uplo=N.UPPER)[0] == 0   # CSR upper: diagonal first
    assert _validate([0, 2, 3], [0, 1, 1], fmt=N.FMT_CSC)[0] == 0  # CSC lower: diagonal first
    rc, msg = _validate([0, 1, 2], [0, 0])
    assert "row/column 1" in msg


def test_exclusive_scan_and_indegree():
    a = np.array([3, 0, 2, 5, 1], np.int32)
    N.lib.capsp_exclusive_scan(a.ctypes.data_as(C.c_void_p), len(a))
    assert list(a) == [0, 3, 3, 5, 10]
    idx = np.array([0, 2, 2, 1, 2], np.int32)
    deg = np.empty(3, np.int32)
    N.lib.capsp_indegree(3, 5, idx.ctypes.data_as(C.c_void_p), deg.ctypes.data_as(C.c_void_p))
    assert list(deg) == [1, 1, 3]


def test_batched_generator_is_block_diagonal():
    m = cs.generate_batched(nsys=12, seed=1, nmin=50, nmax=400)
    so = m.sys_rowoff
    assert so[0] == 0 and so[-1] == m.n and len(so) == 13
    sys_of_row = np.searchsorted(so, np.arange(m.n), side="right") - 1
    rows = np.repeat(np.arange(m.n), np.diff(m.rowptr))
    assert np.all(m.colidx >= so[sys_of_row[rows]])
    assert np.all(m.colidx <= rows)


def test_cli_usage_and_degenerate_matrix(tmp_path):
    """capsp_run: bad arguments print usage (exit 2); a 1x1 matrix exits 0 and
    writes nothing, as the reference's main.cu does for m <= 1 (no GPU needed)."""
    import subprocess
    from capellinisptrsv_gb300 import build as B
    r = subprocess.run([str(B.CLI)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([str(B.CLI), "--alg", "nope", "x.mtx"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
    p = tmp_path / "one.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n1 1 1\n1 1 2.0\n")
    out = tmp_path / "result.csv"
    r = subprocess.run([str(B.CLI), "--out", str(out), str(p)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0
    assert out.exists() and out.read_text() == ""


def test_level_schedule_same_on_one_thread():
    """The parallel per-level passes give the order and positions of a
    single-threaded build (levels of 2k rows and more run in parallel), and the
    threaded transpose its serial result."""
    import hashlib, subprocess, sys, textwrap
    code = textwrap.dedent("""
        import hashlib, numpy as np, capellinisptrsv_gb300 as cs
        from capellinisptrsv_gb300.solver import level_schedule, transpose_structure
        m = cs.generate(n=400_000, kmin=1, kmax=12, band=200_000, seed=21)  # 53 levels of 2k+ rows
        for upper in (False, True):
            rp, ci = m.rowptr, m.colidx
            if upper:
                rp, ci, _ = cs.matrix_transposition(m.n, m.n, m.nnz, m.rowptr, m.colidx, m.val)
            _, order, pos, _ = level_schedule(m.n, rp, ci, upper)
            print(hashlib.sha1(order.tobytes() + pos.tobytes()).hexdigest())
        t = transpose_structure(m.n, m.rowptr, m.colidx)
        print(hashlib.sha1(b"".join(a.tobytes() for a in t)).hexdigest())
    """)
    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, PYTHONPATH=str(root))
    outs = []
    for threads in ("1", "8"):
        env["OMP_NUM_THREADS"] = threads
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        outs.append(r.stdout.split())
    assert outs[0] == outs[1] and len(outs[0]) == 3


def test_transpose_structure_against_scipy():
    """The host transpose behind the transposed view: new rows in stored-row
    order, src mapping back to the stored entries, on a band matrix and on one
    where every row references row 0 (a 50,000-entry new row)."""
    sp = pytest.importorskip("scipy.sparse")
    from capellinisptrsv_gb300.solver import transpose_structure
    m = cs.generate(n=50_000, kmin=1, kmax=9, band=2_000, seed=31)
    rp, ci = m.rowptr.astype(np.int64), m.colidx.astype(np.int64)
    heavy_ci = ci.copy()
    first = rp[:-1][np.diff(rp) > 1]  # first stored entry of every row with an off-diagonal
    heavy_ci[first] = 0
    heavy = sp.csr_matrix((np.ones(len(ci)), heavy_ci, rp), shape=(m.n, m.n))
    heavy.sum_duplicates()
    heavy.sort_indices()
    for rows, cols in ((rp, ci), (heavy.indptr.astype(np.int64), heavy.indices.astype(np.int64))):
        n = len(rows) - 1
        tptr, tidx, src = transpose_structure(n, rows, cols)
        ref = sp.csr_matrix((np.arange(len(cols), dtype=np.float64), cols, rows), shape=(n, n)).T.tocsr()
        ref.sort_indices()
        assert np.array_equal(tptr, ref.indptr) and np.array_equal(tidx, ref.indices)
        assert np.array_equal(src, ref.data.astype(np.int64))
        assert np.array_equal(np.asarray(cols)[src], np.repeat(np.arange(n), np.diff(tptr)))
    assert np.diff(tptr).max() > 30_000


def test_transpose_structure_rejects_bad_index():
    from capellinisptrsv_gb300.solver import transpose_structure
    with pytest.raises(ValueError):
        transpose_structure(3, np.array([0, 1, 3, 5]), np.array([0, 0, 1, 7, 2]))
