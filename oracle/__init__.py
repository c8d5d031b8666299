"""ORACLE -- test infrastructure, not product code.

ctypes access to (1) liboracle.so, the C restatement of the reference's serial
sync-free solve (oracle.c), and (2) when it has been built, oracle/_ref/, the
reference's own serial executor and host helpers compiled from its headers.
Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module,
and only as the checker or the timed CPU baseline.

liboracle.so also carries the workloads' seeded generator (compiled from the
solver library's generator source) and b = A*ones, so the CPU legs make their
inputs without loading the solver library; tests pin both to the solver
library's output and to the reference's.
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_DIR = HERE / "_ref"
REFERENCE = Path("/root/reference")

FORWARD, BACKWARD = 0, 1
P = C.c_void_p
GEN_SRC = HERE.parent / "capellinisptrsv_gb300" / "csrc" / "host" / "generate.c"
WORKLOADS_PY = HERE.parent / "capellinisptrsv_gb300" / "workloads.py"


class GenParams(C.Structure):
    """capsp_gen_params_t (include/capsp.h)."""
    _fields_ = [("n", C.c_int64), ("seed", C.c_uint64), ("stream", C.c_uint64), ("kind", C.c_int),
                ("kmin", C.c_int), ("kmax", C.c_int), ("band", C.c_int64), ("zipf_s", C.c_double),
                ("zipf_cap", C.c_int), ("near_window", C.c_int)]


_W = None


def workloads():
    """The workload table (capellinisptrsv_gb300/workloads.py), loaded by path
    so that the solver package, and with it its library, is not imported."""
    global _W
    if _W is None:
        sp = importlib.util.spec_from_file_location("_capsp_workloads", WORKLOADS_PY)
        _W = importlib.util.module_from_spec(sp)
        sp.loader.exec_module(_W)
    return _W


def build(ref: bool | None = None) -> None:
    """make -C oracle (and `make ref` when the reference sources are present)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True, capture_output=True)
    if ref is None:
        ref = REFERENCE.exists()
    if ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REFERENCE={REFERENCE}"], check=True,
                       capture_output=True)


def _p(a) -> C.c_void_p:
    return a.ctypes.data_as(C.c_void_p)


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        src = [HERE / "oracle.c", HERE / "oracle_impl.h", HERE / "oracle.h", GEN_SRC]
        if not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in src):
            build(ref=False)
        _lib = C.CDLL(str(LIB))
        for t in ("f64", "f32"):
            getattr(_lib, f"oracle_executor_{t}").argtypes = [P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, P]
            getattr(_lib, f"oracle_solve_csr_lower_{t}").argtypes = [C.c_int, C.c_int, P, P, P, C.c_int, P, P]
            getattr(_lib, f"oracle_solve_csr_transpose_{t}").argtypes = [C.c_int, C.c_int, P, P, P, C.c_int, P, P]
            getattr(_lib, f"oracle_grad_val_{t}").argtypes = [C.c_int, P, P, C.c_int, P, P, P]
            getattr(_lib, f"oracle_grad_val_{t}").restype = None
            getattr(_lib, f"oracle_transpose_{t}").argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, P, P, P]
            getattr(_lib, f"oracle_transpose_{t}").restype = None
            getattr(_lib, f"oracle_get_x_b_{t}").argtypes = [C.c_int, P, P, P]
            getattr(_lib, f"oracle_get_x_b_{t}").restype = None
        _lib.oracle_analyser.argtypes = [P, C.c_int, C.c_int, P]
        _lib.oracle_analyser.restype = None
        _lib.capsp_gen_rowptr.argtypes = [C.POINTER(GenParams), P]
        _lib.capsp_gen_fill_f64.argtypes = [C.POINTER(GenParams), P, P, P]
        _lib.capsp_gen_normal_f64.argtypes = [C.c_uint64, C.c_uint64, C.c_int64, P]
        _lib.capsp_digest.argtypes = [C.c_int, C.c_int, P, P, P, C.c_int]
        _lib.capsp_digest.restype = C.c_uint64
    return _lib


def _t(val) -> str:
    return "f64" if np.asarray(val).dtype == np.float64 else "f32"


def _prep(rowptr, colidx, val):
    return (np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(colidx, np.int32),
            np.ascontiguousarray(val))


def solve_csr_lower(rowptr, colidx, val, b) -> np.ndarray:
    """x = L^{-1} b through transpose + analyser + FORWARD executor (b: (n,) or (n, k))."""
    rowptr, colidx, val = _prep(rowptr, colidx, val)
    b = np.ascontiguousarray(b, dtype=val.dtype)
    n = len(rowptr) - 1
    k = 1 if b.ndim == 1 else b.shape[1]
    x = np.empty_like(b)
    rc = getattr(lib(), f"oracle_solve_csr_lower_{_t(val)}")(n, len(colidx), _p(rowptr), _p(colidx), _p(val),
                                                              k, _p(b), _p(x))
    if rc != 0:
        raise ValueError(f"oracle solve failed ({rc}): malformed matrix")
    return x


def solve_csr_transpose(rowptr, colidx, val, g) -> np.ndarray:
    """y = L^{-T} g through the BACKWARD executor on L's CSR arrays."""
    rowptr, colidx, val = _prep(rowptr, colidx, val)
    g = np.ascontiguousarray(g, dtype=val.dtype)
    n = len(rowptr) - 1
    k = 1 if g.ndim == 1 else g.shape[1]
    y = np.empty_like(g)
    rc = getattr(lib(), f"oracle_solve_csr_transpose_{_t(val)}")(n, len(colidx), _p(rowptr), _p(colidx),
                                                                  _p(val), k, _p(g), _p(y))
    if rc != 0:
        raise ValueError(f"oracle transpose solve failed ({rc})")
    return y


def executor(colptr, rowidx, val, indeg, substitution, b) -> np.ndarray:
    """The serial executor on explicit column arrays (FORWARD or BACKWARD)."""
    colptr, rowidx, val = _prep(colptr, rowidx, val)
    indeg = np.ascontiguousarray(indeg, np.int32)
    b = np.ascontiguousarray(b, dtype=val.dtype)
    n = len(colptr) - 1
    k = 1 if b.ndim == 1 else b.shape[1]
    x = np.empty_like(b)
    rc = getattr(lib(), f"oracle_executor_{_t(val)}")(_p(colptr), _p(rowidx), _p(val), _p(indeg), n, n,
                                                      substitution, k, _p(b), _p(x))
    if rc != 0:
        raise ValueError(f"oracle executor failed ({rc})")
    return x


def analyser(idx, n) -> np.ndarray:
    idx = np.ascontiguousarray(idx, np.int32)
    out = np.empty(n, np.int32)
    lib().oracle_analyser(_p(idx), n, len(idx), _p(out))
    return out


def transpose(rowptr, colidx, val):
    rowptr, colidx, val = _prep(rowptr, colidx, val)
    n = len(rowptr) - 1
    cp = np.empty(n + 1, np.int32)
    ri = np.empty(len(colidx), np.int32)
    cv = np.empty(len(colidx), val.dtype)
    getattr(lib(), f"oracle_transpose_{_t(val)}")(n, n, len(colidx), _p(rowptr), _p(colidx), _p(val),
                                                  _p(ri), _p(cp), _p(cv))
    return cp, ri, cv


def grad_val(rowptr, colidx, y, x) -> np.ndarray:
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colidx = np.ascontiguousarray(colidx, np.int32)
    y = np.ascontiguousarray(y)
    x = np.ascontiguousarray(x, dtype=y.dtype)
    k = 1 if y.ndim == 1 else y.shape[1]
    out = np.empty(len(colidx), dtype=y.dtype)
    getattr(lib(), f"oracle_grad_val_{_t(y)}")(len(rowptr) - 1, _p(rowptr), _p(colidx), k, _p(y), _p(x), _p(out))
    return out


def get_x_b(rowptr, val) -> np.ndarray:
    """b = A * ones in the value type, row order (the reference's get_x_b)."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    val = np.ascontiguousarray(val)
    b = np.empty(len(rowptr) - 1, dtype=val.dtype)
    getattr(lib(), f"oracle_get_x_b_{_t(val)}")(len(b), _p(rowptr), _p(val), _p(b))
    return b


# ---------------------------------------------------------------------------
# seeded inputs (the workloads' generator, built into liboracle.so)
# ---------------------------------------------------------------------------

def generate(workload=None, *, seed=0, stream=0, **params):
    """(n, rowptr, colidx, val) of a workload, from the same seeded generator as
    the solver library's ``generate``."""
    sp = workloads().spec(workload, **params)
    p = GenParams(int(sp["n"]), int(seed), int(stream), int(sp["kind"]), int(sp["kmin"]), int(sp["kmax"]),
                  int(sp["band"]), float(sp["zipf_s"]), int(sp["zipf_cap"]), int(sp["near_window"]))
    n = int(sp["n"])
    rowptr = np.empty(n + 1, dtype=np.int32)
    if lib().capsp_gen_rowptr(C.byref(p), _p(rowptr)) != 0:
        raise ValueError("generator rejected the parameters")
    colidx = np.empty(int(rowptr[-1]), dtype=np.int32)
    val = np.empty(int(rowptr[-1]), dtype=np.float64)
    if lib().capsp_gen_fill_f64(C.byref(p), _p(rowptr), _p(colidx), _p(val)) != 0:
        raise ValueError("generator fill failed")
    return n, rowptr, colidx, val


def generate_batched(nsys=None, *, seed=0):
    """(n, rowptr, colidx, val, sys_rowoff) of the batched workload."""
    W = workloads()
    d = dict(W.BATCH_DEFAULTS)
    nsys = nsys or d["nsys"]
    sizes = W.batched_sizes(nsys, seed, d["nmin"], d["nmax"])
    parts = [generate(seed=seed, stream=s + 1, **W.batched_system_spec(sizes[s], d["kmin"], d["kmax"],
                                                                       d["band_div"]))[1:]
             for s in range(nsys)]
    return W.assemble_batched(parts, sizes)


def normal(count, *, seed=0, stream=0) -> np.ndarray:
    out = np.empty(int(count), dtype=np.float64)
    lib().capsp_gen_normal_f64(int(seed), int(stream), int(count), _p(out))
    return out


def digest(n, rowptr, colidx, val) -> int:
    val = np.ascontiguousarray(val)
    return int(lib().capsp_digest(int(n), len(colidx), _p(np.ascontiguousarray(rowptr, np.int32)),
                                  _p(np.ascontiguousarray(colidx, np.int32)), _p(val), val.dtype.itemsize))


# ---------------------------------------------------------------------------
# the reference itself (oracle/_ref), when built
# ---------------------------------------------------------------------------

class _Ref:
    def __init__(self):
        self.serial = {t: C.CDLL(str(REF_DIR / f"libref_serial_{t}.so")) for t in ("f64", "f32")}
        self.pre = {t: C.CDLL(str(REF_DIR / f"libref_pre_{t}.so")) for t in ("f64", "f32")}
        for t in ("f64", "f32"):
            s = self.serial[t]
            getattr(s, f"ref_executor_{t}").argtypes = [P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, P, P]
            getattr(s, f"ref_analyser_{t}").argtypes = [P, C.c_int, C.c_int, C.c_int, P]
            getattr(s, f"ref_transposition_{t}").argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, P, P, P]
            getattr(s, f"ref_transposition_{t}").restype = None

    def solve_csr_lower(self, rowptr, colidx, val, b) -> np.ndarray:
        """The reference pipeline: matrix_transposition, analyser, FORWARD executor."""
        rowptr, colidx, val = _prep(rowptr, colidx, val)
        t = _t(val)
        b = np.ascontiguousarray(b, dtype=val.dtype)
        n, nnz = len(rowptr) - 1, len(colidx)
        k = 1 if b.ndim == 1 else b.shape[1]
        cp = np.empty(n + 1, np.int32)
        ri = np.empty(nnz, np.int32)
        cv = np.empty(nnz, val.dtype)
        s = self.serial[t]
        getattr(s, f"ref_transposition_{t}")(n, n, nnz, _p(rowptr), _p(colidx), _p(val), _p(ri), _p(cp), _p(cv))
        deg = np.empty(n, np.int32)
        getattr(s, f"ref_analyser_{t}")(_p(ri), n, n, nnz, _p(deg))
        x = np.empty_like(b)
        getattr(s, f"ref_executor_{t}")(_p(cp), _p(ri), _p(cv), _p(deg), n, n, FORWARD, k, _p(b), _p(x))
        return x

    def prepared_forward(self, rowptr, colidx, val):
        """Transpose + analyse once; returns a callable running only the executor."""
        rowptr, colidx, val = _prep(rowptr, colidx, val)
        t = _t(val)
        n, nnz = len(rowptr) - 1, len(colidx)
        cp = np.empty(n + 1, np.int32)
        ri = np.empty(nnz, np.int32)
        cv = np.empty(nnz, val.dtype)
        s = self.serial[t]
        getattr(s, f"ref_transposition_{t}")(n, n, nnz, _p(rowptr), _p(colidx), _p(val), _p(ri), _p(cp), _p(cv))
        deg = np.empty(n, np.int32)
        getattr(s, f"ref_analyser_{t}")(_p(ri), n, n, nnz, _p(deg))
        ex = getattr(s, f"ref_executor_{t}")

        def run(b, x):
            k = 1 if b.ndim == 1 else b.shape[1]
            ex(_p(cp), _p(ri), _p(cv), _p(deg), n, n, FORWARD, k, _p(b), _p(x))
            return x
        return run

    def solve_csr_transpose(self, rowptr, colidx, val, g) -> np.ndarray:
        rowptr, colidx, val = _prep(rowptr, colidx, val)
        t = _t(val)
        g = np.ascontiguousarray(g, dtype=val.dtype)
        n, nnz = len(rowptr) - 1, len(colidx)
        k = 1 if g.ndim == 1 else g.shape[1]
        s = self.serial[t]
        deg = np.empty(n, np.int32)
        getattr(s, f"ref_analyser_{t}")(_p(colidx), n, n, nnz, _p(deg))
        y = np.empty_like(g)
        getattr(s, f"ref_executor_{t}")(_p(rowptr), _p(colidx), _p(val), _p(deg), n, n, BACKWARD, k, _p(g), _p(y))
        return y


_ref = False


def ref():
    """The compiled reference (oracle/_ref) or None when it is not built here."""
    global _ref
    if _ref is False:
        try:
            _ref = _Ref()
        except OSError:
            _ref = None
    return _ref


def prepared_forward(rowptr, colidx, val):
    """Oracle-port equivalent of _Ref.prepared_forward (transpose + analyse once)."""
    cp, ri, cv = transpose(rowptr, colidx, val)
    deg = analyser(ri, len(rowptr) - 1)
    t = _t(cv)
    n = len(rowptr) - 1
    ex = getattr(lib(), f"oracle_executor_{t}")

    def run(b, x):
        k = 1 if b.ndim == 1 else b.shape[1]
        rc = ex(_p(cp), _p(ri), _p(cv), _p(deg), n, n, FORWARD, k, _p(b), _p(x))
        if rc != 0:
            raise ValueError("oracle executor failed")
        return x
    return run
