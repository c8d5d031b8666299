"""capellinisptrsv_gb300 -- GB300-native synchronization-free sparse triangular solve.

Python surface over libcapsp.so (include/capsp.h).  The compute path is the
hand-written sm_103a CUDA in ``csrc/``; importing this package without the
built library raises ImportError (there is no CPU fallback).
"""
from . import _native
from ._native import CapspError
from .solver import (WORKLOADS, CSRMatrix, TriangularSolver, change2tran, digest, generate,
                     generate_batched, get_x_b, hop_latency, matrix_layer, matrix_transposition,
                     matrix_warp4, normal, read_mtx, row_levels, set_compat_repeat, spmv,
                     spts_syncfree_cuda_csr, spts_syncfree_cuda_csr_wrt,
                     spts_syncfree_cuda_csr_wrt_mix, sptrsv_syncfree_cuda)

__all__ = [
    "CapspError", "CSRMatrix", "TriangularSolver", "WORKLOADS", "generate", "generate_batched",
    "normal", "spmv", "digest", "hop_latency", "set_compat_repeat",
    "spts_syncfree_cuda_csr_wrt", "spts_syncfree_cuda_csr", "spts_syncfree_cuda_csr_wrt_mix",
    "sptrsv_syncfree_cuda", "change2tran", "get_x_b", "matrix_layer", "row_levels",
    "matrix_transposition", "matrix_warp4", "read_mtx", "sptrsv", "SparseTriangularSolve",
]


def __getattr__(name):  # autograd pieces import torch lazily
    if name in ("sptrsv", "SparseTriangularSolve", "DifferentiableTriangular"):
        from . import autograd
        return getattr(autograd, name)
    raise AttributeError(name)
