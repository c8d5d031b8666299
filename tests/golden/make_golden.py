"""Regenerate tests/golden/golden.npz from the reference itself.

Every expected output in the fixture is produced by the reference's own code,
compiled from its headers into oracle/_ref (``make -C oracle ref``): the serial
sync-free executor (openCL/SynFree_csc/sptrsv_syncfree_serialref.h) and the
host helpers change2tran / get_x_b / matrix_layer / matrix_transposition /
matrix_warp4 / read_mtx (CUDA/mix/{read_mtx.h,tranpose.h}).  Inputs are
seeded: the 20k-row workload from the library's generator (pinned by its
digest) and small hand-built edge cases.  Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
import tempfile
from pathlib import Path

import hashlib

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import capellinisptrsv_gb300 as cs  # noqa: E402
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.npz"


def sha(a) -> np.ndarray:
    """SHA-256 of an array's bytes: bit-exact pins of large outputs stay small."""
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), dtype=np.uint8)


def rhs3(n: int) -> np.ndarray:
    """Seeded 3-column right-hand side (numpy PCG64, identical on every platform)."""
    return np.random.default_rng(3).standard_normal((n, 3))


def edge_rhs(n: int):
    """Seeded right-hand sides of the edge cases (1 and 4 columns)."""
    return (np.random.default_rng(11).standard_normal(n), np.random.default_rng(12).standard_normal((n, 4)))


def edge_cases():
    """Small lower-triangular CSR matrices covering the shapes the solver must handle."""
    cases = {}
    rng = np.random.default_rng(7)

    def build(n, rows):
        rowptr = [0]
        colidx, val = [], []
        for i in range(n):
            cols = sorted(rows(i))
            vals = list(rng.uniform(-1, 1, len(cols)))
            colidx += cols + [i]
            val += vals + [1.0 + float(np.sum(np.abs(vals)))]
            rowptr.append(len(colidx))
        return (np.array(rowptr, np.int32), np.array(colidx, np.int32), np.array(val, np.float64))

    cases["single"] = build(1, lambda i: [])
    cases["diagonal_only"] = build(100, lambda i: [])
    cases["bidiagonal_chain"] = build(400, lambda i: [i - 1] if i else [])
    cases["stride64_chain"] = build(640, lambda i: [i - 64] if i >= 64 else [])
    cases["dense_band_40"] = build(160, lambda i: list(range(max(0, i - 40), i)))
    cases["row_512"] = build(600, lambda i: list(range(i - 512, i)) if i == 599 else ([i - 1] if i else []))
    cases["ragged_33"] = build(33, lambda i: list(rng.choice(i, size=min(i, int(rng.integers(0, 6))), replace=False)) if i else [])
    cases["full_lower_64"] = build(64, lambda i: list(range(i)))
    return cases


def main() -> None:
    oracle.build(ref=True)
    ref = oracle.ref()
    if ref is None:
        raise SystemExit("oracle/_ref is not built: the reference sources are required")
    g = {}

    # 1. the 20k-row workload (FP64 and FP32), b = L*ones from the reference's get_x_b
    m = cs.generate("plain_20k", seed=0)
    g["plain_20k_digest"] = np.array([m.digest()], dtype=np.uint64)
    g["plain_20k_nnz"] = np.array([m.nnz])
    for t, dt in (("f64", np.float64), ("f32", np.float32)):
        val = m.val.astype(dt)
        xr, b = _ref_get_x_b(ref, t, m.n, m.rowptr, m.colidx, val)
        x = ref.solve_csr_lower(m.rowptr, m.colidx, val, b)
        g[f"plain_20k_b_{t}_sha"] = sha(b)
        g[f"plain_20k_x_{t}_sha"] = sha(x)
        g[f"plain_20k_x_{t}_head"] = x[:64]
    rhs = rhs3(m.n)
    g["plain_20k_x_rhs3_sha"] = sha(ref.solve_csr_lower(m.rowptr, m.colidx, m.val, rhs))
    g["plain_20k_y_rhs3_sha"] = sha(ref.solve_csr_transpose(m.rowptr, m.colidx, m.val, rhs))
    lv, par = _ref_layer(ref, m.n, m.rowptr, m.colidx, m.val)
    g["plain_20k_layer"] = np.array([lv])
    g["plain_20k_parallelism"] = np.array([par])

    # 2. edge cases: forward and backward (adjoint) solves, single and 4 RHS
    for name, (rp, ci, v) in edge_cases().items():
        n = len(rp) - 1
        b1, b4 = edge_rhs(n)
        g[f"edge_{name}_rowptr"], g[f"edge_{name}_colidx"], g[f"edge_{name}_val"] = rp, ci, v
        g[f"edge_{name}_x1"] = ref.solve_csr_lower(rp, ci, v, b1)
        g[f"edge_{name}_x4"] = ref.solve_csr_lower(rp, ci, v, b4)
        g[f"edge_{name}_y1"] = ref.solve_csr_transpose(rp, ci, v, b1)
        g[f"edge_{name}_y4"] = ref.solve_csr_transpose(rp, ci, v, b4)

    # 3. host preprocessing on a general sparse A (unsorted rows, upper entries, gaps)
    rng = np.random.default_rng(5)
    n = 500
    rows = [rng.choice(n, size=int(rng.integers(0, 12)), replace=False) for _ in range(n)]
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    ci = np.concatenate(rows).astype(np.int32)
    va = rng.uniform(-2, 2, len(ci))
    g["pre_A_rowptr"], g["pre_A_colidx"], g["pre_A_val"] = rp, ci, va
    nnzL, lrp, lci, lv_ = _ref_change2tran(ref, n, rp.copy(), ci.copy(), va.copy())
    g["pre_L_rowptr"], g["pre_L_colidx"], g["pre_L_val"] = lrp, lci, lv_
    lay, par = _ref_layer(ref, n, lrp, lci, lv_)
    g["pre_L_layer"] = np.array([lay])
    g["pre_L_parallelism"] = np.array([par])
    cp, ri, cv = _ref_transpose(ref, n, lrp, lci, lv_)
    g["pre_L_csc_colptr"], g["pre_L_csc_rowidx"], g["pre_L_csc_val"] = cp, ri, cv
    for border in (0, 2, 3, 10):
        ln, table, wo, eo = _ref_warp4(ref, n, lrp, lci, lv_, border)
        g[f"pre_warp4_{border}_table"] = table[:ln]
        g[f"pre_warp4_{border}_occ"] = np.array([wo, eo])
    # warp4 on the workload matrix with the reference's border 10
    ln, table, wo, eo = _ref_warp4(ref, m.n, m.rowptr, m.colidx, m.val, 10)
    g["plain_20k_warp4_len"] = np.array([ln])
    g["plain_20k_warp4_sha"] = sha(table[:ln])
    g["plain_20k_warp4_occ"] = np.array([wo, eo])

    # 4. Matrix Market reading (general real, symmetric pattern, integer)
    mtx = {
        "general": "%%MatrixMarket matrix coordinate real general\n% c\n4 4 6\n1 1 2.5\n2 1 -1\n3 3 4\n4 2 0.5\n2 2 3\n4 4 1e-3\n",
        "sym_pattern": "%%MatrixMarket matrix coordinate pattern symmetric\n3 3 4\n1 1\n2 1\n3 2\n3 3\n",
        "integer": "%%MatrixMarket matrix coordinate integer general\n3 3 3\n1 1 7\n3 1 -2\n2 3 5\n",
    }
    with tempfile.TemporaryDirectory() as d:
        for name, text in mtx.items():
            p = Path(d) / f"{name}.mtx"
            p.write_text(text)
            g[f"mtx_{name}_text"] = np.frombuffer(text.encode(), dtype=np.uint8)
            res = _ref_read_mtx(ref, str(p))
            for k, v in zip(("m", "n", "nnz", "rowptr", "colidx", "val"), res):
                g[f"mtx_{name}_{k}"] = np.asarray(v)

    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(g)} arrays)")


# -- thin ctypes helpers over oracle/_ref's preprocessing wrappers ----------

def _pre(ref, t):
    lib = ref.pre[t]
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _take(lib, t, ptr, count, dtype):
    arr = np.ctypeslib.as_array(C.cast(ptr, C.POINTER({np.int32: C.c_int, np.float64: C.c_double,
                                                       np.float32: C.c_float}[dtype])), shape=(count,)).copy()
    getattr(lib, f"ref_free_{t}")(ptr)
    return arr


def _ref_get_x_b(ref, t, n, rp, ci, val):
    lib = _pre(ref, t)
    px, pb = C.c_void_p(), C.c_void_p()
    getattr(lib, f"ref_get_x_b_{t}")(n, n, _p(rp), _p(ci), _p(val), C.byref(px), C.byref(pb))
    dt = np.float64 if t == "f64" else np.float32
    return _take(lib, t, px, n, dt), _take(lib, t, pb, n, dt)


def _ref_layer(ref, n, rp, ci, val):
    lib = _pre(ref, "f64")
    layer, par = C.c_int(), C.c_double()
    getattr(lib, "ref_matrix_layer_f64")(n, n, int(rp[-1]), _p(rp), _p(ci), _p(np.ascontiguousarray(val, np.float64)),
                                         C.byref(layer), C.byref(par))
    return layer.value, par.value


def _ref_change2tran(ref, n, rp, ci, va):
    lib = _pre(ref, "f64")
    nnzL = C.c_int()
    pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
    getattr(lib, "ref_change2tran_f64")(n, len(ci), _p(rp), _p(ci), _p(va), C.byref(nnzL),
                                        C.byref(pr), C.byref(pc), C.byref(pv))
    return (nnzL.value, _take(lib, "f64", pr, n + 1, np.int32), _take(lib, "f64", pc, nnzL.value, np.int32),
            _take(lib, "f64", pv, nnzL.value, np.float64))


def _ref_transpose(ref, n, rp, ci, v):
    lib = _pre(ref, "f64")
    cp = np.empty(n + 1, np.int32)
    ri = np.empty(len(ci), np.int32)
    cv = np.empty(len(ci), np.float64)
    fn = getattr(lib, "ref_matrix_transposition_f64")
    fn.restype = None
    fn(n, n, len(ci), _p(rp), _p(ci), _p(v), _p(ri), _p(cp), _p(cv))
    return cp, ri, cv


def _ref_warp4(ref, n, rp, ci, v, border):
    lib = _pre(ref, "f64")
    table = np.zeros(n + 1, np.int32)
    ln, wo, eo = C.c_int(), C.c_double(), C.c_double()
    fn = getattr(lib, "ref_matrix_warp4_f64")
    fn.restype = None
    fn(n, n, int(rp[-1]), _p(rp), _p(ci), _p(np.ascontiguousarray(v, np.float64)), border, C.byref(ln), _p(table),
       C.byref(wo), C.byref(eo))
    return ln.value, table, wo.value, eo.value


def _ref_read_mtx(ref, path):
    lib = _pre(ref, "f64")
    m, n, nnz = C.c_int(), C.c_int(), C.c_int()
    pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
    rc = getattr(lib, "ref_read_mtx_f64")(path.encode(), C.byref(m), C.byref(n), C.byref(nnz),
                                          C.byref(pr), C.byref(pc), C.byref(pv))
    assert rc == 0, rc
    return (m.value, n.value, nnz.value, _take(lib, "f64", pr, m.value + 1, np.int32),
            _take(lib, "f64", pc, nnz.value, np.int32), _take(lib, "f64", pv, nnz.value, np.float64))


if __name__ == "__main__":
    main()
