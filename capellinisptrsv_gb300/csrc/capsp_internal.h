// Internal interface between the C-ABI layer (capsp_api.cu, capsp_compat.cu)
// and the kernel translation units.  Not installed; no C-ABI types here.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "capsp_device.cuh"

namespace capsp {

// Arguments of the row-driven solve (thread / two-phase / mix kernels).
// Logical ("solve order") row p maps to physical row i = p for lower and
// i = n-1-p for upper matrices; the diagonal is the last entry of a lower
// row and the first entry of an upper row.
template <typename T>
struct RowArgs {
    // natural solve order: the matrix arrays themselves
    const int *ptr;
    const int *idx;
    const T *val;
    const T *inv_diag;
    // level schedule (perm != nullptr): everything indexed by schedule
    // position k; row perm[k] has dependencies at positions
    // lidx[lptr[k] .. lptr[k+1]) (ascending) with values lval[...], and
    // publishes into the position-ordered scratch xp (element (k, r) at
    // k*ldp + r) as well as into the caller's x.
    const int *perm;
    const int *lptr;
    const int *lidx;
    const T *lval;
    const T *linv;
    T *xp;
    long long ldp;
    const T *b;
    T *x;
    long long ld;  // element (i, r) at i*ld + r
    int n;
    int nrhs;      // right-hand sides handled by this launch (<= 32)
    int upper;
    const int *table;  // mix virtual-warp table in solve order (MIX only)
    int table_len;
    unsigned *ticket;
    int *err;
    WaitCfg wait;
    int stuck_row;  // debug: this row never publishes (-1: none)
    unsigned long long *trace;  // tracing, per row i: [4i] chunk taken, [4i+1] first poll, [4i+2] last dependency received, [4i+3] published (ns)
    int keep_hint;  // publication vector polled and stored with evict_last (1) or evict_normal (0)
    // host side: an access-policy window (persisting) over the publication
    // vector for this launch; win_bytes == 0: none
    void *win_base;
    size_t win_bytes;
    float win_hit;
    // level schedule: completion counters of the row segments of x, rows
    // [s*seg_rows, (s+1)*seg_rows) counted into seg_count[s] as they finish
    // (a copy stream waits on them); seg_count == nullptr: not counted
    int *seg_count;
    int seg_rows;
    // level schedule: b_ready[k] != 0 once a copy stream has put b's rows of
    // segment k in place; nullptr: b is resident.  Segments double: k covers
    // rows [b0 (2^k - 1), b0 (2^(k+1) - 1)).  b_group_seg[q] is the highest
    // segment of the rows at positions [32q, 32q + 32): a warp waits for that
    // flag before it starts a chunk there (flags are set in segment order).
    const int *b_ready;
    const unsigned char *b_group_seg;
};

// Arguments of the column-driven solve (SyncFree CSC kernel, and the
// transpose solve that walks CSR rows as columns of the transpose).
template <typename T>
struct ColArgs {
    const int *ptr;
    const int *idx;
    const T *val;
    const T *inv_diag;
    const int *indeg;  // entries targeting each row, diagonal included
    const int *order;  // visiting order of the columns (nullptr: index order)
    int *arrived;      // zeroed before the launch
    T *left_sum;       // zeroed before the launch, element (i, r) at i*lsld + r
    void *slots;       // sum-and-count words instead of left_sum + arrived (nullptr: those),
                       // zeroed before the launch; FP64 16 bytes, FP32 8 bytes per (i, r)
    long long lsld;
    const T *b;
    T *x;
    long long ld;
    int n;
    int nrhs;  // <= 32
    int backward;  // columns visited n-1..0, diagonal last in each column
    const T *xf;   // forward solution for the fused grad_val (nullptr: no grad)
    T *grad_val;
    int grad_accumulate;  // add into grad_val instead of overwriting
    unsigned *ticket;
    int *err;
    WaitCfg wait;
    int stuck_row;
};

enum RowKernelKind { kRowWrtFst = 1, kRowTwoPart = 2, kRowMix = 3 };

// lanes per row for a launch with nrhs right-hand sides (next power of two, <= 32)
inline int lanes_for_rhs(int nrhs)
{
    int g = 1;
    while (g < nrhs && g < 32)
        g <<= 1;
    return g;
}

// Launches that capsp_solve_host can overlap with its copies (a b_ready /
// seg_count launch): one right-hand side, one row per lane, write-first or
// mixed, level schedule, without the register cap
inline bool row_hostio_supported(int kind, int rows_per_thread, int nrhs)
{
    return nrhs == 1 && rows_per_thread == 1 && (kind == kRowWrtFst || kind == kRowMix);
}

// regcap: the 64-register build of the multi-RHS write-first level kernel;
// stage: one lane per row on the level schedule with each 32-row sub-chunk's
// entries staged in shared memory (FP64 only; ignored for other launches)
template <typename T>
cudaError_t launch_row_solve(const RowArgs<T> &a, int kind, int rows_per_thread, int block,
                             int blocks_per_sm, int num_sms, bool regcap, bool stage, cudaStream_t st);

template <typename T>
cudaError_t launch_col_solve(const ColArgs<T> &a, int block, int blocks_per_sm, int num_sms,
                             cudaStream_t st);

// x[i*ld + r] = pending pattern for i < n, r < nrhs; ticket[0..nticket) = 0; err[0..3] = 0
template <typename T>
cudaError_t launch_fill_pending(T *x, int n, int nrhs, long long ld, unsigned *ticket, int nticket,
                                int *err, cudaStream_t st);

// inv[i] = 1/val[diag(i)]; records the first row with a zero or non-finite diagonal in *bad
template <typename T>
cudaError_t launch_inv_diag(const int *ptr, const T *val, T *inv, int n, int diag_last, int *bad,
                            cudaStream_t st);

// level-schedule values: linv[p] = 1/val[diag_src[p]] and the pre-scaled
// dependency values lval[k] = -val[dep_src[k]] * linv[p] for k in lptr[p]..lptr[p+1]
// (records the first position with a zero or non-finite diagonal in *bad)
template <typename T>
cudaError_t launch_level_values(const int *lptr, const int *dep_src, const int *diag_src, int n,
                                const T *val, T *lval, T *linv, int *bad, cudaStream_t st);

template <typename T>
cudaError_t launch_grad_val(const int *rowptr, const int *colidx, const T *y, const T *x,
                            T *grad_val, int n, int nrhs, long long ld, int accumulate,
                            cudaStream_t st);

// structure check on device arrays; *bad = first bad row (must be preset to INT_MAX)
cudaError_t launch_validate(const int *ptr, const int *idx, int n, int nnz, int diag_last,
                            int *bad, cudaStream_t st);

// out[idx[k]] += 1 (out must be zeroed)
cudaError_t launch_histogram(const int *idx, int nnz, int *out, cudaStream_t st);

}  // namespace capsp
