"""The benchmark workloads: generator parameters and the batched assembly.

Pure Python + numpy, with no library loaded: the solver package generates
matrices with libcapsp's generator, and the CPU-side checker (the oracle) with
the same generator built into its own library, from the same table.

Shared value rule: off-diagonals U[-1,1], diagonal 1 + sum|off-diagonals|
(last in its row).
"""
from __future__ import annotations

import numpy as np

# generator kinds (capsp_gen_params_t.kind)
GEN_UNIFORM_BAND, GEN_ZIPF_NEAR_FAR = 0, 1

WORKLOADS = {
    # n=20,000; k~U{1..5} distinct columns in [max(0,i-2000), i-1]; b = L*ones
    "plain_20k": dict(n=20_000, kind=GEN_UNIFORM_BAND, kmin=1, kmax=5, band=2000),
    # n=4,194,304; k~U{1..7} (mean 4) in [max(0,i-65536), i-1]; b = L*ones
    "wide_4m": dict(n=4_194_304, kind=GEN_UNIFORM_BAND, kmin=1, kmax=7, band=65536),
    # n=1,048,576; k~Zipf(1.8) on 1..512; ceil(k/2) cols in [i-32, i-1], the rest in [0, i-1]
    # (a literal Zipf(1.8): 6.96 off-diagonals per row on average, ~126k levels)
    "zipf_1m": dict(n=1_048_576, kind=GEN_ZIPF_NEAR_FAR, zipf_s=1.8, zipf_cap=512, near_window=32),
    # the same with the count floored at 38, which brings the mean to ~40 off-diagonals
    # per row; 19 of the previous 32 rows per row make it a near-serial chain
    "zipf40_1m": dict(n=1_048_576, kind=GEN_ZIPF_NEAR_FAR, kmin=38, zipf_s=1.8, zipf_cap=512,
                      near_window=32),
    # n=1,048,576; k~U{2..10} (mean 6) in a band of 16,384 (differentiation workload)
    "grad_1m": dict(n=1_048_576, kind=GEN_UNIFORM_BAND, kmin=2, kmax=10, band=16384),
}

GEN_DEFAULTS = dict(kind=GEN_UNIFORM_BAND, kmin=1, kmax=5, band=0, zipf_s=1.8, zipf_cap=512, near_window=32)

# batched workload: 2,048 systems, n log-uniform in [500, 50,000], 3-12
# off-diagonals per row in a band of n/8
BATCH_DEFAULTS = dict(nsys=2048, nmin=500, nmax=50_000, kmin=3, kmax=12, band_div=8)


def spec(workload: str | None = None, **params) -> dict:
    """Full generator parameters of a named workload, with overrides."""
    out = dict(GEN_DEFAULTS)
    if workload:
        out.update(WORKLOADS[workload])
    out.update(params)
    return out


def batched_sizes(nsys: int, seed: int, nmin: int, nmax: int) -> np.ndarray:
    """Rows per system: round(exp(U(ln nmin, ln nmax))) from a seeded numpy Generator."""
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=nsys))).astype(np.int64)


def batched_system_spec(n_s: int, kmin: int, kmax: int, band_div: int) -> dict:
    """Generator parameters of one system (its rows come from stream s + 1)."""
    return spec(n=int(n_s), kind=GEN_UNIFORM_BAND, kmin=kmin, kmax=kmax, band=max(1, int(n_s) // band_div))


def assemble_batched(parts, sizes):
    """Concatenate per-system CSR parts (rowptr, colidx, val) into one
    block-diagonal CSR with global indices -> (n, rowptr, colidx, val, sys_rowoff)."""
    nsys = len(parts)
    rowoff = np.zeros(nsys + 1, dtype=np.int64)
    np.cumsum(sizes, out=rowoff[1:])
    nnz_off = np.zeros(nsys + 1, dtype=np.int64)
    np.cumsum([int(p[0][-1]) for p in parts], out=nnz_off[1:])
    if nnz_off[-1] >= 2**31 or rowoff[-1] >= 2**31:
        raise ValueError("batch exceeds 32-bit indices")
    n = int(rowoff[-1])
    rowptr = np.empty(n + 1, dtype=np.int32)
    colidx = np.empty(int(nnz_off[-1]), dtype=np.int32)
    val = np.empty(int(nnz_off[-1]), dtype=np.float64)
    for s, (rp, ci, v) in enumerate(parts):
        r0, r1, k0 = int(rowoff[s]), int(rowoff[s + 1]), int(nnz_off[s])
        nnz = int(rp[-1])
        rowptr[r0:r1] = rp[:-1] + k0
        colidx[k0:k0 + nnz] = ci + r0
        val[k0:k0 + nnz] = v
    rowptr[n] = int(nnz_off[-1])
    return n, rowptr, colidx, val, rowoff.astype(np.int32)


def sub_system(rowptr, colidx, val, sys_rowoff, s):
    """Rows [r0, r1) of system s as a standalone CSR (indices rebased) -> (r0, r1, rowptr, colidx, val)."""
    r0, r1 = int(sys_rowoff[s]), int(sys_rowoff[s + 1])
    k0, k1 = int(rowptr[r0]), int(rowptr[r1])
    return (r0, r1, np.ascontiguousarray(rowptr[r0:r1 + 1] - k0, dtype=np.int32),
            np.ascontiguousarray(colidx[k0:k1] - r0, dtype=np.int32), np.ascontiguousarray(val[k0:k1]))
