"""ctypes binding of libcapsp.so (the C-ABI declared in include/capsp.h).

The library is loaded from the package's in-tree ``_build`` directory.  There
is no fallback: if the library is missing, importing this module raises with
the build command to run.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libcapsp.so"

# status codes (capsp_status_t)
OK, ERR_INVALID, ERR_TIMEOUT, ERR_CUDA, ERR_OOM, ERR_UNSUPPORTED = range(6)
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "TIMEOUT", 3: "CUDA", 4: "OOM", 5: "UNSUPPORTED"}
# enums
R_64F, R_32F = 0, 1
FMT_CSR, FMT_CSC = 0, 1
LOWER, UPPER = 0, 1
ALG_AUTO, ALG_WRTFST, ALG_TWOPART, ALG_MIX, ALG_SYNCFREE_CSC = range(5)
SCHED_NATURAL, SCHED_LEVEL = 0, 1
L2_HINTS, L2_WINDOW_AND_HINTS, L2_WINDOW = 0, 1, 2
DEVICE_POINTERS, SKIP_VALIDATION = 0x1, 0x2
GEN_UNIFORM_BAND, GEN_ZIPF_NEAR_FAR = 0, 1


class CapspError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"capsp {STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Info(C.Structure):
    _fields_ = [("n", C.c_int), ("nnz", C.c_int), ("dtype", C.c_int), ("format", C.c_int),
                ("uplo", C.c_int), ("algorithm", C.c_int), ("mix_len", C.c_int),
                ("warp_occupy", C.c_double), ("element_occupy", C.c_double),
                ("analyse_ms", C.c_double), ("rows_per_thread", C.c_int),
                ("block_threads", C.c_int), ("blocks_per_sm", C.c_int), ("num_sms", C.c_int),
                ("schedule", C.c_int), ("levels", C.c_int), ("cached_graphs", C.c_int)]


class GenParams(C.Structure):
    _fields_ = [("n", C.c_int64), ("seed", C.c_uint64), ("stream", C.c_uint64), ("kind", C.c_int),
                ("kmin", C.c_int), ("kmax", C.c_int), ("band", C.c_int64), ("zipf_s", C.c_double),
                ("zipf_cap", C.c_int), ("near_window", C.c_int)]


def _load() -> C.CDLL:
    if not _LIB_PATH.exists():
        raise ImportError(
            f"libcapsp.so not found at {_LIB_PATH}; build it first with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc)")
    return C.CDLL(str(_LIB_PATH), mode=os.RTLD_NOW | getattr(os, "RTLD_LOCAL", 0))


lib = _load()

P = C.c_void_p
I = C.c_int
IP = C.POINTER(C.c_int)
DP = C.POINTER(C.c_double)
H = C.c_void_p  # capsp_handle_t

_SIGS = {
    # native API
    "capsp_last_error": (C.c_char_p, []),
    "capsp_analyse": (I, [I, I, P, P, P, I, I, I, C.c_uint, C.POINTER(H)]),
    "capsp_batched_create": (I, [I, P, I, I, P, P, P, I, C.c_uint, C.POINTER(H)]),
    "capsp_set_values": (I, [H, P]),
    "capsp_refresh_values": (I, [H, P, P]),
    "capsp_set_backoff": (I, [H, C.c_uint]),
    "capsp_destroy": (I, [H]),
    "capsp_get_info": (I, [H, C.POINTER(Info)]),
    "capsp_set_algorithm": (I, [H, I]),
    "capsp_set_l2_policy": (I, [H, I]),
    "capsp_set_mix_border": (I, [H, I]),
    "capsp_set_schedule": (I, [H, I]),
    "capsp_set_tuning": (I, [H, I, I, I]),
    "capsp_set_timeout": (I, [H, C.c_uint64]),
    "capsp_solve": (I, [H, P, P, I, C.c_int64, P]),
    "capsp_solve_transpose": (I, [H, P, P, I, C.c_int64, P]),
    "capsp_grad_val": (I, [H, P, P, P, I, C.c_int64, P]),
    "capsp_solve_transpose_grad": (I, [H, P, P, P, P, I, C.c_int64, P]),
    "capsp_reserve": (I, [H, I]),
    "capsp_status_sync": (I, [H, P]),
    "capsp_solve_host": (I, [H, P, P, I]),
    "capsp_autotune": (I, [H, P, P, I, C.c_int64, P, C.POINTER(C.c_float)]),
    "capsp_graph_solve": (I, [H, P, P, I, C.c_int64, P]),
    "capsp_set_profiling": (I, [H, I]),
    "capsp_last_kernel_ms": (I, [H, C.POINTER(C.c_float)]),
    "capsp_device_sms": (I, [IP]),
    "capsp_debug_set_stuck_row": (I, [H, I, C.c_uint64]),
    "capsp_debug_trace": (I, [H, P]),
    "capsp_hop_latency": (I, [I, I, I, C.POINTER(C.c_float)]),
    "capsp_csc_solve_noalloc_f64": (I, [P, P, P, I, I, P, P, P]),
    # reference-compatible drivers
    "spts_syncfree_cuda_csr_wrt_f64": (I, [P, P, P, I, I, I, DP, DP, DP]),
    "spts_syncfree_cuda_csr_wrt_f32": (I, [P, P, P, I, I, I, DP, DP, DP]),
    "spts_syncfree_cuda_csr_f64": (I, [P, P, P, I, I, I, DP, DP, DP]),
    "spts_syncfree_cuda_csr_f32": (I, [P, P, P, I, I, I, DP, DP, DP]),
    "spts_syncfree_cuda_csr_wrt_mix_f64": (I, [P, P, P, I, I, I, DP, DP, DP, DP, DP, DP]),
    "spts_syncfree_cuda_csr_wrt_mix_f32": (I, [P, P, P, I, I, I, DP, DP, DP, DP, DP, DP]),
    "sptrsv_syncfree_cuda_f64": (I, [P, P, P, I, I, I, P, P, P, DP, DP, DP, DP]),
    "sptrsv_syncfree_cuda_f32": (I, [P, P, P, I, I, I, P, P, P, DP, DP, DP, DP]),
    "capsp_compat_set_repeat": (I, [I]),
    "capsp_compat_repeat": (I, []),
    # host preprocessing
    "capsp_exclusive_scan": (None, [P, I]),
    "change2tran_f64": (I, [I, I, P, P, P, IP, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "change2tran_f32": (I, [I, I, P, P, P, IP, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "get_x_b_f64": (None, [I, I, P, P, P, C.POINTER(P), C.POINTER(P)]),
    "get_x_b_f32": (None, [I, I, P, P, P, C.POINTER(P), C.POINTER(P)]),
    "matrix_layer_f64": (I, [I, I, I, P, P, P, IP, DP]),
    "matrix_layer_f32": (I, [I, I, I, P, P, P, IP, DP]),
    "capsp_row_levels": (I, [I, P, P, P, P]),
    "matrix_transposition_f64": (None, [I, I, I, P, P, P, P, P, P]),
    "matrix_transposition_f32": (None, [I, I, I, P, P, P, P, P, P]),
    "matrix_warp4_f64": (None, [I, I, I, P, P, P, I, IP, P, DP, DP]),
    "matrix_warp4_f32": (None, [I, I, I, P, P, P, I, IP, P, DP, DP]),
    "capsp_mix_table": (I, [I, P, I, I, I, P, DP, DP]),
    "capsp_indegree": (None, [I, I, P, P]),
    "capsp_level_schedule": (I, [I, P, P, I, P, P, P]),
    "capsp_level_layout": (I, [I, P, P, I, P, P, P, P, P, P]),
    "capsp_transpose_structure": (I, [I, I, P, P, P, P, P]),
    "capsp_validate": (I, [I, I, P, P, I, I, C.c_char_p, I]),
    "read_mtx_f64": (I, [C.c_char_p, IP, IP, IP, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "read_mtx_f32": (I, [C.c_char_p, IP, IP, IP, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "capsp_gen_rowptr": (I, [C.POINTER(GenParams), P]),
    "capsp_gen_fill_f64": (I, [C.POINTER(GenParams), P, P, P]),
    "capsp_gen_normal_f64": (I, [C.c_uint64, C.c_uint64, C.c_int64, P]),
    "capsp_spmv_f64": (I, [I, P, P, P, I, P, P]),
    "capsp_digest": (C.c_uint64, [I, I, P, P, P, I]),
}

for _name, (_res, _args) in _SIGS.items():
    _fn = getattr(lib, _name)
    _fn.restype = _res
    _fn.argtypes = _args

EXPORTED = tuple(_SIGS)

libc = C.CDLL(None)
libc.free.argtypes = [P]
libc.free.restype = None


def last_error() -> str:
    return (lib.capsp_last_error() or b"").decode(errors="replace")


def check(status: int) -> None:
    if status != OK:
        raise CapspError(status, last_error())
