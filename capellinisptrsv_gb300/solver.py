"""Host-side mirror of the reference interface over the libcapsp C-ABI.

* ``TriangularSolver`` -- the native analyse/solve split: a triangular CSR
  (or CSC) matrix analysed once, then solved, transposed-solved and
  differentiated on the current CUDA stream with torch tensors as buffers.
* ``spts_syncfree_cuda_csr_wrt``, ``spts_syncfree_cuda_csr``,
  ``spts_syncfree_cuda_csr_wrt_mix``, ``sptrsv_syncfree_cuda`` -- the
  reference's benchmark drivers with their argument lists (numpy arrays in,
  the reference's out-parameters returned as a tuple), dispatched on dtype.
* Host preprocessing with the reference's contracts (``change2tran``,
  ``get_x_b``, ``matrix_layer``, ``matrix_transposition``, ``matrix_warp4``,
  ``read_mtx``).
* Seeded synthetic workloads (``generate``, ``generate_batched``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _native as N
from . import workloads as W

try:  # torch is plumbing for device memory and streams
    import torch
except ImportError:  # pragma: no cover - torch is present in every supported setup
    torch = None

__all__ = [
    "CSRMatrix", "TriangularSolver", "generate", "generate_batched", "WORKLOADS",
    "spts_syncfree_cuda_csr_wrt", "spts_syncfree_cuda_csr", "spts_syncfree_cuda_csr_wrt_mix",
    "sptrsv_syncfree_cuda", "change2tran", "get_x_b", "matrix_layer", "row_levels",
    "matrix_transposition", "matrix_warp4", "read_mtx", "hop_latency", "set_compat_repeat",
    "spmv", "normal", "digest",
]


def _ptr(a) -> C.c_void_p:
    if a is None:
        return C.c_void_p(0)
    if torch is not None and isinstance(a, torch.Tensor):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


def _dtype_code(dt) -> int:
    if dt in (np.float64, "float64") or (torch is not None and dt == torch.float64):
        return N.R_64F
    if dt in (np.float32, "float32") or (torch is not None and dt == torch.float32):
        return N.R_32F
    raise TypeError(f"unsupported value type {dt}; use float64 or float32")


# ---------------------------------------------------------------------------
# matrices and synthetic workloads
# ---------------------------------------------------------------------------

@dataclass
class CSRMatrix:
    """Plain CSR arrays (int32 indices, float values) of an n-by-n matrix."""
    n: int
    rowptr: np.ndarray
    colidx: np.ndarray
    val: np.ndarray
    sys_rowoff: Optional[np.ndarray] = None  # block-diagonal batches only

    @property
    def nnz(self) -> int:
        return int(self.rowptr[-1])

    def astype(self, dtype) -> "CSRMatrix":
        return CSRMatrix(self.n, self.rowptr, self.colidx, self.val.astype(dtype), self.sys_rowoff)

    def digest(self) -> int:
        return digest(self.n, self.rowptr, self.colidx, self.val)


# The seeded workloads of the benchmark definition (generator parameters in
# workloads.py, shared with the oracle's copy of the generator).
WORKLOADS = W.WORKLOADS


def _gen_params(n, seed=0, stream=0, kind=N.GEN_UNIFORM_BAND, kmin=1, kmax=5, band=0,
                zipf_s=1.8, zipf_cap=512, near_window=32) -> N.GenParams:
    return N.GenParams(int(n), int(seed), int(stream), int(kind), int(kmin), int(kmax), int(band),
                       float(zipf_s), int(zipf_cap), int(near_window))


def generate(workload: str | None = None, *, seed: int = 0, stream: int = 0, **params) -> CSRMatrix:
    """Generate a seeded lower-triangular CSR matrix (FP64 values).

    ``workload`` names an entry of WORKLOADS; keyword arguments override it or,
    without a workload, describe the matrix (n, kind, kmin, kmax, band, zipf_s,
    zipf_cap, near_window).
    """
    sp = W.spec(workload, **params)
    p = _gen_params(seed=seed, stream=stream, **sp)
    n = int(sp["n"])
    rowptr = np.empty(n + 1, dtype=np.int32)
    N.check(N.lib.capsp_gen_rowptr(C.byref(p), _ptr(rowptr)))
    nnz = int(rowptr[-1])
    colidx = np.empty(nnz, dtype=np.int32)
    val = np.empty(nnz, dtype=np.float64)
    N.check(N.lib.capsp_gen_fill_f64(C.byref(p), _ptr(rowptr), _ptr(colidx), _ptr(val)))
    return CSRMatrix(n, rowptr, colidx, val)


def generate_batched(nsys: int = 2048, *, seed: int = 0, nmin: int = 500, nmax: int = 50_000,
                     kmin: int = 3, kmax: int = 12, band_div: int = 8) -> CSRMatrix:
    """Block-diagonal batch of independent systems.

    System s has n_s = round(exp(U(ln nmin, ln nmax))) rows (log-uniform, drawn
    from a seeded numpy Generator), k~U{kmin..kmax} off-diagonals per row in a
    band of n_s // band_div; its rows come from generator stream s + 1.
    Column indices are global; ``sys_rowoff`` holds the first row of each system.
    """
    sizes = W.batched_sizes(nsys, seed, nmin, nmax)
    parts = []
    for s in range(nsys):
        m = generate(seed=seed, stream=s + 1, **W.batched_system_spec(sizes[s], kmin, kmax, band_div))
        parts.append((m.rowptr, m.colidx, m.val))
    n, rowptr, colidx, val, rowoff = W.assemble_batched(parts, sizes)
    return CSRMatrix(n, rowptr, colidx, val, rowoff)


def normal(count: int, *, seed: int = 0, stream: int = 0) -> np.ndarray:
    """count N(0,1) values from the library's hashed streams."""
    out = np.empty(int(count), dtype=np.float64)
    N.check(N.lib.capsp_gen_normal_f64(int(seed), int(stream), int(count), _ptr(out)))
    return out


def spmv(m: CSRMatrix, x: np.ndarray) -> np.ndarray:
    """y = A x in float64 (x of shape (n,) or (n, k))."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    k = 1 if x.ndim == 1 else x.shape[1]
    y = np.empty_like(x)
    val = np.ascontiguousarray(m.val, dtype=np.float64)
    N.check(N.lib.capsp_spmv_f64(m.n, _ptr(m.rowptr), _ptr(m.colidx), _ptr(val), k, _ptr(x), _ptr(y)))
    return y


def digest(n, rowptr, colidx, val) -> int:
    val = np.ascontiguousarray(val)
    return int(N.lib.capsp_digest(int(n), int(len(colidx)), _ptr(rowptr), _ptr(colidx), _ptr(val),
                                  val.dtype.itemsize))


# ---------------------------------------------------------------------------
# native solver
# ---------------------------------------------------------------------------

def _current_stream(stream):
    if stream is not None:
        return int(getattr(stream, "cuda_stream", stream))
    if torch is not None and torch.cuda.is_available():
        return int(torch.cuda.current_stream().cuda_stream)
    return 0


class TriangularSolver:
    """Analysed triangular matrix on the current CUDA device.

    Arrays given as CUDA tensors are borrowed (the solver keeps references);
    numpy arrays or CPU tensors are uploaded once.  Vectors passed to the solve
    methods are CUDA tensors of shape (n,) or (n, k) with unit stride along k.
    """

    def __init__(self, rowptr, colidx, val, *, n: Optional[int] = None, fmt: str = "csr",
                 uplo: str = "lower", algorithm: str = "auto", validate: bool = True,
                 sys_rowoff=None, schedule: Optional[str] = None):
        fmt_code = {"csr": N.FMT_CSR, "csc": N.FMT_CSC}[fmt]
        uplo_code = {"lower": N.LOWER, "upper": N.UPPER}[uplo]
        n = int(n if n is not None else len(rowptr) - 1)
        nnz = int(len(colidx))
        on_device = torch is not None and isinstance(val, torch.Tensor) and val.is_cuda
        flags = (N.DEVICE_POINTERS if on_device else 0) | (0 if validate else N.SKIP_VALIDATION)
        if on_device:
            rowptr = rowptr.to(device=val.device, dtype=torch.int32).contiguous()
            colidx = colidx.to(device=val.device, dtype=torch.int32).contiguous()
            val = val.contiguous()
            self._keep = [rowptr, colidx, val]
        else:
            if torch is not None and isinstance(val, torch.Tensor):
                rowptr, colidx, val = rowptr.numpy(), colidx.numpy(), val.numpy()
            rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
            colidx = np.ascontiguousarray(colidx, dtype=np.int32)
            val = np.ascontiguousarray(val)
            self._keep = []
        self.n, self.nnz, self.fmt, self.uplo = n, nnz, fmt, uplo
        self.dtype_code = _dtype_code(val.dtype)
        self.on_device = on_device
        self.rowptr, self.colidx = rowptr, colidx
        self._val_key = (val.data_ptr(), val._version) if on_device else None
        h = C.c_void_p()
        if sys_rowoff is not None:
            so = np.ascontiguousarray(sys_rowoff, dtype=np.int32)
            st = N.lib.capsp_batched_create(len(so) - 1, _ptr(so), n, nnz, _ptr(rowptr), _ptr(colidx),
                                            _ptr(val), self.dtype_code, flags, C.byref(h))
        else:
            st = N.lib.capsp_analyse(n, nnz, _ptr(rowptr), _ptr(colidx), _ptr(val), self.dtype_code,
                                     fmt_code, uplo_code, flags, C.byref(h))
        N.check(st)
        self._h = h
        if schedule is not None:
            self.set_schedule(schedule)
        if algorithm != "auto":
            self.set_algorithm(algorithm)

    # -- lifetime -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib.capsp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- configuration ------------------------------------------------------
    _ALGS = {"auto": N.ALG_AUTO, "wrtfst": N.ALG_WRTFST, "twopart": N.ALG_TWOPART, "mix": N.ALG_MIX,
             "syncfree_csc": N.ALG_SYNCFREE_CSC}

    def set_algorithm(self, algorithm: str) -> None:
        N.check(N.lib.capsp_set_algorithm(self._h, self._ALGS[algorithm]))

    def set_schedule(self, schedule: str) -> None:
        """'level' (rows sorted by dependency level, the default) or 'natural' (row order)."""
        N.check(N.lib.capsp_set_schedule(self._h, {"natural": N.SCHED_NATURAL, "level": N.SCHED_LEVEL}[schedule]))

    def set_l2_policy(self, mode: str) -> None:
        """'hints' (default), 'window+hints' or 'window': L2 treatment of the
        publication vector the dependency polls read (capsp_set_l2_policy)."""
        code = {"hints": N.L2_HINTS, "window+hints": N.L2_WINDOW_AND_HINTS, "window": N.L2_WINDOW}[mode]
        N.check(N.lib.capsp_set_l2_policy(self._h, code))

    def set_mix_border(self, border: int) -> None:
        N.check(N.lib.capsp_set_mix_border(self._h, int(border)))

    def set_tuning(self, rows_per_thread: int = 2, block: int = 256, blocks_per_sm: int = 0) -> None:
        N.check(N.lib.capsp_set_tuning(self._h, rows_per_thread, block, blocks_per_sm))

    def set_backoff(self, sleep_max_ns: int) -> None:
        N.check(N.lib.capsp_set_backoff(self._h, int(sleep_max_ns)))

    def set_timeout(self, seconds: float) -> None:
        N.check(N.lib.capsp_set_timeout(self._h, int(seconds * 1e9)))

    def debug_stuck_row(self, row: int, timeout_s: float = 0.0) -> None:
        N.check(N.lib.capsp_debug_set_stuck_row(self._h, int(row), int(timeout_s * 1e9)))

    def trace(self, buf=None) -> None:
        """Per-row timing trace into a CUDA int64 tensor of 4*n entries (None: off)."""
        N.check(N.lib.capsp_debug_trace(self._h, _ptr(buf)))
        self._trace_buf = buf

    def reserve(self, max_nrhs: int) -> None:
        N.check(N.lib.capsp_reserve(self._h, int(max_nrhs)))

    def info(self) -> dict:
        inf = N.Info()
        N.check(N.lib.capsp_get_info(self._h, C.byref(inf)))
        return {f: getattr(inf, f) for f, _ in N.Info._fields_}

    def set_values(self, val) -> None:
        """Replace the values (same structure); refreshes 1/diag."""
        if self.on_device:
            val = val.contiguous()
            self._keep[2] = val
            self._val_key = (val.data_ptr(), val._version)
        else:
            val = np.ascontiguousarray(val)
        N.check(N.lib.capsp_set_values(self._h, _ptr(val)))

    def bind_values(self, val) -> None:
        """set_values only if `val` is not the tensor (and version) already bound."""
        if (val.data_ptr(), val._version) != self._val_key:
            self.set_values(val)

    def refresh_values(self, val=None, stream=None) -> None:
        """Stream-ordered: borrow `val` (device handles) and recompute 1/diag, no sync.

        Catches in-place changes that bypass the version counter (``.data`` writes)."""
        if not self.on_device:
            raise ValueError("refresh_values needs a solver built from CUDA tensors; use set_values")
        if val is not None:
            val = val.contiguous()
            self._keep[2] = val
            self._val_key = (val.data_ptr(), val._version)
        N.check(N.lib.capsp_refresh_values(self._h, _ptr(val), C.c_void_p(_current_stream(stream))))

    def refresh_values_if_rebound(self, val, stream=None) -> None:
        """refresh_values(val) unless `val` is the tensor, at the version, that the
        solver's latest refresh or set_values bound."""
        if (val.data_ptr(), val._version) != self._val_key:
            self.refresh_values(val, stream)

    # -- vectors --------------------------------------------------------------
    def _vec(self, t, name):
        if not (torch is not None and isinstance(t, torch.Tensor) and t.is_cuda):
            raise TypeError(f"{name} must be a CUDA tensor")
        if t.shape[0] != self.n:
            raise ValueError(f"{name} has {t.shape[0]} rows, expected {self.n}")
        if t.dim() == 1:
            if t.stride(0) != 1:
                t = t.contiguous()
            return t, 1, 1
        if t.dim() != 2:
            raise ValueError(f"{name} must be 1-D or 2-D")
        if t.stride(1) != 1:
            t = t.contiguous()
        return t, t.shape[1], t.stride(0)

    def _out_like(self, b, out):
        if out is None:
            return torch.empty_like(b, memory_format=torch.contiguous_format)
        return out

    # -- operations -----------------------------------------------------------
    def solve(self, b, x=None, stream=None):
        """x = A^{-1} b (stream-ordered; no host synchronisation)."""
        b, k, ld = self._vec(b, "b")
        x = self._out_like(b, x)
        x2, k2, ld2 = self._vec(x, "x")
        if k2 != k or ld2 != ld:
            raise ValueError("x must have the shape and row stride of b")
        N.check(N.lib.capsp_solve(self._h, _ptr(b), _ptr(x2), k, ld, C.c_void_p(_current_stream(stream))))
        return x2

    def solve_transpose(self, g, y=None, stream=None):
        """y = A^{-T} g: over the handle's transposed copy, or column-driven on the
        stored arrays under algorithm "syncfree_csc" (CSR handles)."""
        g, k, ld = self._vec(g, "g")
        y = self._out_like(g, y)
        N.check(N.lib.capsp_solve_transpose(self._h, _ptr(g), _ptr(y), k, ld,
                                            C.c_void_p(_current_stream(stream))))
        return y

    def solve_transpose_grad(self, g, x, y=None, grad_val=None, stream=None):
        """Backward: y = A^{-T} g and grad_val[k] = -sum_r y[row_k, r] x[col_k, r]
        (fused into the column-driven sweep under "syncfree_csc")."""
        g, k, ld = self._vec(g, "g")
        x, kx, ldx = self._vec(x, "x")
        if (kx, ldx) != (k, ld):
            raise ValueError("x must match g's shape and row stride")
        y = self._out_like(g, y)
        if grad_val is None:
            grad_val = torch.empty(self.nnz, dtype=g.dtype, device=g.device)
        N.check(N.lib.capsp_solve_transpose_grad(self._h, _ptr(g), _ptr(x), _ptr(y), _ptr(grad_val), k, ld,
                                                 C.c_void_p(_current_stream(stream))))
        return y, grad_val

    def grad_val(self, y, x, out=None, stream=None):
        y, k, ld = self._vec(y, "y")
        x, _, _ = self._vec(x, "x")
        if out is None:
            out = torch.empty(self.nnz, dtype=y.dtype, device=y.device)
        N.check(N.lib.capsp_grad_val(self._h, _ptr(y), _ptr(x), _ptr(out), k, ld,
                                     C.c_void_p(_current_stream(stream))))
        return out

    def graph_solve(self, b, x, stream):
        b, k, ld = self._vec(b, "b")
        N.check(N.lib.capsp_graph_solve(self._h, _ptr(b), _ptr(x), k, ld, C.c_void_p(_current_stream(stream))))
        return x

    def autotune(self, b, x, stream=None) -> float:
        b, k, ld = self._vec(b, "b")
        ms = C.c_float()
        N.check(N.lib.capsp_autotune(self._h, _ptr(b), _ptr(x), k, ld, C.c_void_p(_current_stream(stream)),
                                     C.byref(ms)))
        return float(ms.value)

    def set_profiling(self, enable: bool = True) -> None:
        N.check(N.lib.capsp_set_profiling(self._h, int(bool(enable))))

    def last_kernel_ms(self) -> float:
        """Duration of the main solve kernel of the latest solve (profiling on)."""
        ms = C.c_float()
        N.check(N.lib.capsp_last_kernel_ms(self._h, C.byref(ms)))
        return float(ms.value)

    def status(self, stream=None) -> None:
        """Synchronise the stream and raise CapspError if the last solve timed out."""
        N.check(N.lib.capsp_status_sync(self._h, C.c_void_p(_current_stream(stream))))

    def solve_host(self, b: np.ndarray, x: Optional[np.ndarray] = None) -> np.ndarray:
        """Synchronous host-buffer solve (copies in, solves, copies out)."""
        b = np.ascontiguousarray(b)
        k = 1 if b.ndim == 1 else b.shape[1]
        if x is None:
            x = np.empty_like(b)
        N.check(N.lib.capsp_solve_host(self._h, _ptr(b), _ptr(x), k))
        return x


def hop_latency(n: int = 200_000, stride: int = 64, dtype=np.float64) -> float:
    """Per-hop dependency latency (ns) of a chain matrix solve; see capsp_hop_latency."""
    out = C.c_float()
    N.check(N.lib.capsp_hop_latency(int(n), int(stride), _dtype_code(np.dtype(dtype).type), C.byref(out)))
    return float(out.value)


# ---------------------------------------------------------------------------
# reference-compatible drivers
# ---------------------------------------------------------------------------

def set_compat_repeat(repeat: int) -> int:
    """Set BENCH_REPEAT for the reference-compatible drivers; returns the old value."""
    return int(N.lib.capsp_compat_set_repeat(int(repeat)))


def _sfx(val) -> str:
    return "_f64" if np.asarray(val).dtype == np.float64 else "_f32"


def _csr_driver(name, rowptr, colidx, val, m, n, nnz, extra=0):
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    colidx = np.ascontiguousarray(colidx, dtype=np.int32)
    val = np.ascontiguousarray(val)
    outs = [C.c_double() for _ in range(3 + extra)]
    fn = getattr(N.lib, name + _sfx(val))
    ret = fn(_ptr(rowptr), _ptr(colidx), _ptr(val), int(m), int(n), int(nnz), *[C.byref(o) for o in outs])
    return (int(ret), *[o.value for o in outs])


def spts_syncfree_cuda_csr_wrt(csrRowPtrL, csrColIdxL, csrValL, m, n, nnzL):
    """ourWrtFst driver -> (ret, solve_time_ms, gflops, bandwidth)."""
    return _csr_driver("spts_syncfree_cuda_csr_wrt", csrRowPtrL, csrColIdxL, csrValL, m, n, nnzL)


def spts_syncfree_cuda_csr(csrRowPtrL, csrColIdxL, csrValL, m, n, nnzL):
    """our2Part driver -> (ret, solve_time_ms, gflops, bandwidth)."""
    return _csr_driver("spts_syncfree_cuda_csr", csrRowPtrL, csrColIdxL, csrValL, m, n, nnzL)


def spts_syncfree_cuda_csr_wrt_mix(csrRowPtrL, csrColIdxL, csrValL, m, n, nnzL):
    """mix driver -> (ret, solve_time_ms, gflops, bandwidth, pre_time_ms, warp_occupy, element_occupy)."""
    return _csr_driver("spts_syncfree_cuda_csr_wrt_mix", csrRowPtrL, csrColIdxL, csrValL, m, n, nnzL, 3)


def sptrsv_syncfree_cuda(cscColPtr, cscRowIdx, cscVal, m, n, nnz, x, b, x_ref):
    """SyncFree_csc driver; fills x -> (ret, pre_time_ms, solve_time_ms, gflops, bandwidth)."""
    cp = np.ascontiguousarray(cscColPtr, dtype=np.int32)
    ri = np.ascontiguousarray(cscRowIdx, dtype=np.int32)
    cv = np.ascontiguousarray(cscVal)
    b = np.ascontiguousarray(b, dtype=cv.dtype)
    x_ref = np.ascontiguousarray(x_ref, dtype=cv.dtype)
    outs = [C.c_double() for _ in range(4)]
    fn = getattr(N.lib, "sptrsv_syncfree_cuda" + _sfx(cv))
    ret = fn(_ptr(cp), _ptr(ri), _ptr(cv), int(m), int(n), int(nnz), _ptr(x), _ptr(b), _ptr(x_ref),
             *[C.byref(o) for o in outs])
    return (int(ret), *[o.value for o in outs])


# ---------------------------------------------------------------------------
# host preprocessing
# ---------------------------------------------------------------------------

def _take(ptr, count, dtype) -> np.ndarray:
    """Copy a malloc'ed C array into numpy and free it."""
    if not ptr.value:
        raise MemoryError("host allocation failed")
    ctype = {np.int32: C.c_int, np.float64: C.c_double, np.float32: C.c_float}[dtype]
    arr = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(count,)).copy()
    N.libc.free(ptr)
    return arr


def change2tran(m, rowptrA, colidxA, valA):
    """Lower-triangular part with unit values + unit diagonal (rows of A sorted in place).

    Returns (nnzL, rowptrL, colidxL, valL)."""
    valA_arr = np.asarray(valA)
    if not (valA_arr.flags.c_contiguous and valA_arr.dtype in (np.float64, np.float32)):
        raise TypeError("valA must be a contiguous float64/float32 array (sorted in place)")
    nnzL = C.c_int()
    pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
    fn = getattr(N.lib, "change2tran" + _sfx(valA_arr))
    if fn(int(m), int(len(colidxA)), _ptr(rowptrA), _ptr(colidxA), _ptr(valA_arr), C.byref(nnzL),
          C.byref(pr), C.byref(pc), C.byref(pv)) != 0:
        raise MemoryError("change2tran allocation failed")
    dt = valA_arr.dtype.type
    return (nnzL.value, _take(pr, m + 1, np.int32), _take(pc, nnzL.value, np.int32), _take(pv, nnzL.value, dt))


def get_x_b(m, n, rowptr, colidx, val):
    """x_ref = ones, b = A x_ref in the value type -> (x_ref, b)."""
    val = np.ascontiguousarray(val)
    px, pb = C.c_void_p(), C.c_void_p()
    getattr(N.lib, "get_x_b" + _sfx(val))(int(m), int(n), _ptr(np.ascontiguousarray(rowptr, np.int32)),
                                          _ptr(np.ascontiguousarray(colidx, np.int32)), _ptr(val),
                                          C.byref(px), C.byref(pb))
    dt = val.dtype.type
    return _take(px, n, dt), _take(pb, m, dt)


def matrix_layer(m, n, nnz, rowptr, colidx, val=None):
    """-> (levels, rows per level)."""
    val = np.zeros(1) if val is None else np.ascontiguousarray(val)
    layer, par = C.c_int(), C.c_double()
    getattr(N.lib, "matrix_layer" + _sfx(val))(int(m), int(n), int(nnz), _ptr(rowptr), _ptr(colidx), _ptr(val),
                                               C.byref(layer), C.byref(par))
    return layer.value, par.value


def row_levels(n, rowptr, colidx):
    """-> (levels, level of each row, rows per level histogram)."""
    level = np.empty(n, dtype=np.int32)
    counts = np.empty(n + 1, dtype=np.int32)
    deepest = N.lib.capsp_row_levels(int(n), _ptr(rowptr), _ptr(colidx), _ptr(level), _ptr(counts))
    return int(deepest), level, counts[: deepest + 1]


def level_schedule(n, rowptr, colidx, upper: bool = False):
    """Level order of the solve -> (levels, order, position, level_start)."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colidx = np.ascontiguousarray(colidx, np.int32)
    order = np.empty(n, np.int32)
    position = np.empty(n, np.int32)
    start = np.empty(n + 2, np.int32)
    levels = N.lib.capsp_level_schedule(int(n), _ptr(rowptr), _ptr(colidx), int(bool(upper)), _ptr(order),
                                        _ptr(position), _ptr(start))
    if levels < 0:
        raise MemoryError("level schedule allocation failed")
    return int(levels), order, position, start[: levels + 2].copy()


def level_layout(n, rowptr, colidx, order, position, upper: bool = False):
    """Dependencies in schedule-position space -> (dep_ptr, dep_idx, dep_src, diag_src)."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colidx = np.ascontiguousarray(colidx, np.int32)
    nd = len(colidx) - n
    dep_ptr = np.empty(n + 1, np.int32)
    dep_idx = np.empty(max(nd, 1), np.int32)
    dep_src = np.empty(max(nd, 1), np.int32)
    diag_src = np.empty(n, np.int32)
    rc = N.lib.capsp_level_layout(int(n), _ptr(rowptr), _ptr(colidx), int(bool(upper)), _ptr(order), _ptr(position),
                                  _ptr(dep_ptr), _ptr(dep_idx), _ptr(dep_src), _ptr(diag_src))
    if rc != 0:
        raise ValueError("misplaced diagonal")
    return dep_ptr, dep_idx[:nd], dep_src[:nd], diag_src


def transpose_structure(n, rowptr, colidx):
    """The structure transposed -> (tptr, tidx, src): new row j lists the stored
    rows holding index j, ascending; src maps new entries to stored ones."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    colidx = np.ascontiguousarray(colidx, np.int32)
    nnz = len(colidx)
    tptr = np.empty(n + 1, np.int32)
    tidx = np.empty(max(nnz, 1), np.int32)
    src = np.empty(max(nnz, 1), np.int32)
    if N.lib.capsp_transpose_structure(int(n), nnz, _ptr(rowptr), _ptr(colidx), _ptr(tptr), _ptr(tidx), _ptr(src)) != 0:
        raise ValueError("an index is outside [0, n), or host memory ran out")
    return tptr, tidx[:nnz], src[:nnz]


def matrix_transposition(m, n, nnz, rowptr, colidx, val):
    """CSR -> CSC -> (cscColPtr, cscRowIdx, cscVal)."""
    val = np.ascontiguousarray(val)
    cp = np.empty(n + 1, dtype=np.int32)
    ri = np.empty(nnz, dtype=np.int32)
    cv = np.empty(nnz, dtype=val.dtype)
    getattr(N.lib, "matrix_transposition" + _sfx(val))(int(m), int(n), int(nnz), _ptr(rowptr), _ptr(colidx),
                                                       _ptr(val), _ptr(ri), _ptr(cp), _ptr(cv))
    return cp, ri, cv


def matrix_warp4(m, n, nnz, rowptr, colidx, val=None, border=10):
    """Mix selector -> (Len, warp_num[:Len], warp_occupy, element_occupy)."""
    val = np.zeros(1) if val is None else np.ascontiguousarray(val)
    table = np.zeros(m + 1, dtype=np.int32)
    ln, wo, eo = C.c_int(), C.c_double(), C.c_double()
    getattr(N.lib, "matrix_warp4" + _sfx(val))(int(m), int(n), int(nnz), _ptr(rowptr), _ptr(colidx), _ptr(val),
                                               int(border), C.byref(ln), _ptr(table), C.byref(wo), C.byref(eo))
    return ln.value, table[: ln.value].copy(), wo.value, eo.value


def read_mtx(filename: str, dtype=np.float64):
    """Matrix Market -> (m, n, nnz, rowptr, colidx, val); raises on a negative reader code."""
    m, n, nnz = C.c_int(), C.c_int(), C.c_int()
    pr, pc, pv = C.c_void_p(), C.c_void_p(), C.c_void_p()
    sfx = "_f64" if np.dtype(dtype) == np.float64 else "_f32"
    rc = getattr(N.lib, "read_mtx" + sfx)(str(filename).encode(), C.byref(m), C.byref(n), C.byref(nnz),
                                          C.byref(pr), C.byref(pc), C.byref(pv))
    if rc != 0:
        raise ValueError(f"read_mtx({filename}) failed with code {rc}")
    return (m.value, n.value, nnz.value, _take(pr, m.value + 1, np.int32), _take(pc, nnz.value, np.int32),
            _take(pv, nnz.value, np.dtype(dtype).type))
