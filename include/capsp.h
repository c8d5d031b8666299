/*
 * capsp.h -- C-ABI of the GB300-native synchronization-free sparse triangular
 * solve library (libcapsp.so).
 *
 * Three groups of entry points live here:
 *
 *  1. The native, stream-ordered API (capsp_*): analyse a triangular matrix
 *     once into an opaque handle, then solve L x = b (or the transpose) as many
 *     times as wanted on a caller-supplied cudaStream_t.  Plain pointers and
 *     sizes only; no C++ or torch types cross this boundary.
 *
 *  2. Reference-compatible drivers with the exact argument lists of the
 *     CapelliniSpTRSV benchmark drivers (spts_syncfree_cuda_csr_wrt,
 *     spts_syncfree_cuda_csr, the mix driver and sptrsv_syncfree_cuda).  The
 *     reference compiles one VALUE_TYPE per binary; C has no overloading, so
 *     each driver is exported twice with an _f64 / _f32 suffix.
 *     capsp_compat.h maps the unsuffixed reference names onto them.
 *
 *  3. Host preprocessing with the reference's contracts (lower-triangular
 *     extraction, b = L*ones, level statistics, CSR->CSC transposition, the
 *     mix selector table) and seeded synthetic matrix generators.
 *
 * Conventions
 *  - Indices are 32-bit signed ints (n < 2^31, nnz < 2^31), as in the reference.
 *  - Multi-RHS vectors are row-major: element (row i, rhs r) at i*ld + r,
 *    the layout of sptrsv_syncfree_executor's "rhs" argument
 *    (openCL/SynFree_csc/sptrsv_syncfree_serialref.h:59-61).
 *  - Every native entry point returns a capsp_status_t; capsp_last_error()
 *    gives a human-readable message for the calling thread.
 *  - Solve entry points are asynchronous with respect to the host; a dependency
 *    wait that runs out of its time budget on the device is reported by
 *    capsp_status_sync() as CAPSP_ERR_TIMEOUT.
 */
#ifndef CAPSP_H
#define CAPSP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CAPSP_VERSION_MAJOR 0
#define CAPSP_VERSION_MINOR 1

/* ------------------------------------------------------------------------ */
/* Status codes, enums                                                       */
/* ------------------------------------------------------------------------ */

typedef enum capsp_status {
    CAPSP_OK = 0,
    CAPSP_ERR_INVALID = 1,     /* malformed matrix or bad argument (checked before any launch) */
    CAPSP_ERR_TIMEOUT = 2,     /* a device dependency wait exceeded its budget */
    CAPSP_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    CAPSP_ERR_OOM = 4,         /* device or host allocation failed */
    CAPSP_ERR_UNSUPPORTED = 5  /* valid request this build does not implement */
} capsp_status_t;

typedef enum capsp_dtype {
    CAPSP_R_64F = 0,   /* double: VALUE_TYPE double in the reference's common.h */
    CAPSP_R_32F = 1    /* float */
} capsp_dtype_t;

typedef enum capsp_format {
    CAPSP_FMT_CSR = 0, /* ptr = row pointer, idx = column indices */
    CAPSP_FMT_CSC = 1  /* ptr = column pointer, idx = row indices */
} capsp_format_t;

typedef enum capsp_uplo {
    CAPSP_LOWER = 0,   /* CSR: diagonal last in each row;  CSC: diagonal first in each column */
    CAPSP_UPPER = 1    /* CSR: diagonal first in each row; CSC: diagonal last in each column  */
} capsp_uplo_t;

/* Solve algorithms.  A handle solves the orientation it stores (CSR rows, or
 * the transpose of a CSC matrix) by walking its rows; the other orientation
 * (the plain solve of a CSC handle, the transpose of a CSR handle) walks the
 * rows of a transposed copy of the structure that the handle builds once on
 * the host, whose entries point back into the stored values.  The row-driven
 * algorithms below apply to both; CAPSP_ALG_SYNCFREE_CSC instead solves the
 * other orientation column by column on the stored arrays. */
typedef enum capsp_algorithm {
    CAPSP_ALG_AUTO = 0,        /* mix when the selector finds heavy row groups, else WRTFST */
    CAPSP_ALG_WRTFST = 1,      /* thread per row, write-first (CUDA/ourWrtFst) */
    CAPSP_ALG_TWOPART = 2,     /* thread per row, out-of-warp then in-warp phases (CUDA/our2Part) */
    CAPSP_ALG_MIX = 3,         /* thread or warp per row by nnz/row of 32-row groups (CUDA/mix) */
    CAPSP_ALG_SYNCFREE_CSC = 4 /* warp per column, atomic partial sums + arrival counts (CUDA/SyncFree_csc),
                                  for the orientation a handle does not store; rows as AUTO */
} capsp_algorithm_t;

/* Order in which the row-driven kernels start rows.  Any order that lists a
 * row after its dependencies keeps the solve synchronization-free. */
typedef enum capsp_schedule {
    CAPSP_SCHED_NATURAL = 0, /* row index order, no preprocessing (the reference's order) */
    CAPSP_SCHED_LEVEL = 1    /* rows sorted by dependency level, built at analysis (default) */
} capsp_schedule_t;

/* L2 treatment of the position-ordered publication vector that every
 * dependency poll reads (capsp_set_l2_policy). */
typedef enum capsp_l2_policy {
    CAPSP_L2_HINTS = 0,            /* polls and publications carry evict_last hints (default) */
    CAPSP_L2_WINDOW_AND_HINTS = 1, /* plus a persisting access-policy window over the vector */
    CAPSP_L2_WINDOW = 2            /* the window alone (evict_normal polls) */
} capsp_l2_policy_t;

/* capsp_analyse flags */
#define CAPSP_DEVICE_POINTERS 0x1u /* ptr/idx/val are device pointers; the handle borrows them */
#define CAPSP_SKIP_VALIDATION 0x2u /* trust the structure (no host/device structure check) */

typedef struct capsp_handle_s *capsp_handle_t;

/* Per-handle statistics filled by capsp_get_info. */
typedef struct capsp_info {
    int n;
    int nnz;
    int dtype;
    int format;
    int uplo;
    int algorithm;          /* algorithm the next plain solve will use (AUTO resolved once
                               its selector table exists) */
    int mix_len;            /* entries of the mix virtual-warp table (0 until built) */
    double warp_occupy;     /* rows handled warp-per-row / n   (mix/spts_..._wrt.h:152-156) */
    double element_occupy;  /* nnz in warp-per-row rows / nnz */
    double analyse_ms;      /* wall time of capsp_analyse */
    int rows_per_thread;    /* launch tuning currently in force */
    int block_threads;
    int blocks_per_sm;
    int num_sms;
    int schedule;           /* capsp_schedule_t of the plain solve's rows */
    int levels;             /* dependency levels of the plain solve's rows (0 until built) */
    int cached_graphs;      /* instantiated graphs held for capsp_graph_solve; every change that a
                               captured solve depends on (scratch growth, new value pointer,
                               schedule, tuning, wait budget, debug hooks) drops them all */
} capsp_info_t;

/* ------------------------------------------------------------------------ */
/* 1. Native API                                                             */
/* ------------------------------------------------------------------------ */

/* Message describing the last failing capsp_* call on this host thread. */
const char *capsp_last_error(void);

/* Analyse an n-by-n triangular matrix.  Checks the structure (diagonal
 * present at the documented end of every row/column, all other indices on the
 * triangular side, nonzero diagonal), uploads host arrays (or borrows device
 * arrays with CAPSP_DEVICE_POINTERS), precomputes 1/diag and builds the level
 * schedule of the plain solve (of the transposed structure for CSC).
 * Replaces the upload + analysis half of spts_syncfree_cuda_csr_wrt
 * (CUDA/ourWrtFst/spts_syncfree_cuda_csr_wrt.h:66-124) and the in-degree
 * analyser of sptrsv_syncfree_cuda (CUDA/SyncFree_csc/spts_syncfree_cuda2.h:139-160). */
capsp_status_t capsp_analyse(int n, int nnz, const int *ptr, const int *idx,
                             const void *val, int dtype, int format, int uplo,
                             unsigned flags, capsp_handle_t *out);

/* Block-diagonal batch of independent systems.  ptr/idx/val describe the
 * concatenated matrix with GLOBAL indices; sys_rowoff[nsys+1] gives the first
 * row of every system (sys_rowoff[0] = 0, sys_rowoff[nsys] = n).  The result
 * is an ordinary handle: capsp_solve solves every system in one launch.
 * No reference counterpart (the reference solves one system per process). */
capsp_status_t capsp_batched_create(int nsys, const int *sys_rowoff, int n, int nnz,
                                    const int *ptr, const int *idx, const void *val,
                                    int dtype, unsigned flags, capsp_handle_t *out);

/* Replace the numerical values (same structure) and refresh 1/diag.  val is a
 * device pointer for CAPSP_DEVICE_POINTERS handles (borrowed), else host. */
capsp_status_t capsp_set_values(capsp_handle_t h, const void *val);

/* Stream-ordered variant for CAPSP_DEVICE_POINTERS handles: borrow val (or,
 * with val = NULL, keep the current pointer) and recompute 1/diag on `stream`
 * without synchronising.  Meant for values that change between solves, e.g.
 * parameters updated in place by an optimiser; a zero diagonal then shows up
 * as inf/NaN in the results instead of an error code. */
capsp_status_t capsp_refresh_values(capsp_handle_t h, const void *val, void *stream);

capsp_status_t capsp_destroy(capsp_handle_t h);

capsp_status_t capsp_get_info(capsp_handle_t h, capsp_info_t *info);

/* L2 treatment of the publication vector of level-schedule row solves
 * (capsp_l2_policy_t).  The window modes reserve a persisting L2 carve-out of
 * up to the vector's size (cudaLimitPersistingL2CacheSize, a setting of the
 * calling process's context) and attach an access-policy window to each solve
 * launch; returning to CAPSP_L2_HINTS or destroying the handle restores the
 * carve-out value this handle found when it first changed it (handles that
 * change it concurrently restore in their own order).  The default needs
 * neither. */
capsp_status_t capsp_set_l2_policy(capsp_handle_t h, int mode);

/* Choose the solve algorithm (capsp_algorithm_t). */
capsp_status_t capsp_set_algorithm(capsp_handle_t h, int algorithm);

/* Schedule of the rows of the stored orientation (capsp_schedule_t).
 * CAPSP_SCHED_LEVEL builds the level order on first use if capsp_analyse did
 * not; the build is host work proportional to nnz.  The transposed copy is
 * always level-ordered. */
capsp_status_t capsp_set_schedule(capsp_handle_t h, int schedule);

/* Mix selector threshold: 32-row groups whose mean nnz/row is >= border go
 * warp-per-row (the reference hard-codes 10, mix/spts_syncfree_cuda_csr_wrt.h:188). */
capsp_status_t capsp_set_mix_border(capsp_handle_t h, int border);

/* Launch tuning: rows per thread (1, 2 or 4), threads per block (64..1024,
 * multiple of 32) and resident blocks per SM (0 = occupancy maximum). */
capsp_status_t capsp_set_tuning(capsp_handle_t h, int rows_per_thread,
                                int block_threads, int blocks_per_sm);

/* Budget for any single device dependency wait (default 10 s). */
capsp_status_t capsp_set_timeout(capsp_handle_t h, uint64_t timeout_ns);

/* Ceiling of the exponential __nanosleep backoff between polls of a pending
 * dependency (default 0 = never sleep: on GB300 sleeping only delays the
 * detection of a landed dependency; the wall-clock timeout still bounds it). */
capsp_status_t capsp_set_backoff(capsp_handle_t h, unsigned sleep_max_ns);

/* Solve op(A) X = B for nrhs right-hand sides (device pointers, element
 * (i,r) at i*ld + r, ld >= nrhs).  x must not alias b.  Stream-ordered,
 * no host synchronisation, no allocation once capsp_reserve covered nrhs.
 * Replaces the timed launch of spts_syncfree_cuda_executor_csr_wrt
 * (CUDA/ourWrtFst/spts_syncfree_cuda_csr_wrt.h:10-57,160), of
 * spts_syncfree_cuda_executor_csr (CUDA/our2Part/spts_syncfree_cuda_csr.h:10-124),
 * of the mix executor (CUDA/mix/spts_syncfree_cuda_csr_wrt.h:15-137) and of
 * sptrsv_syncfree_cuda_executor_update (CUDA/SyncFree_csc/spts_syncfree_cuda2.h:24-86). */
capsp_status_t capsp_solve(capsp_handle_t h, const void *b, void *x, int nrhs,
                           int64_t ld, void *stream);

/* Solve A^T Y = G.  A CSR handle walks the rows of its transposed copy (built
 * on first use), or under CAPSP_ALG_SYNCFREE_CSC its own rows as columns of
 * A^T with the column-driven kernel, the BACKWARD mode of
 * sptrsv_syncfree_cuda_executor_update (CUDA/SyncFree_csc/spts_syncfree_cuda2.h:50-82)
 * and of the serial executor (openCL/SynFree_csc/sptrsv_syncfree_serialref.h:73-102).
 * A CSC handle walks its stored columns as rows of A^T. */
capsp_status_t capsp_solve_transpose(capsp_handle_t h, const void *g, void *y,
                                     int nrhs, int64_t ld, void *stream);

/* grad_val[k] = -sum_r y[row(k), r] * x[col(k), r] over the stored nonzeros
 * (CSR or CSC).  No reference counterpart: the gradient of L x = b with
 * respect to the values of L, given y = L^{-T} g. */
capsp_status_t capsp_grad_val(capsp_handle_t h, const void *y, const void *x,
                              void *grad_val, int nrhs, int64_t ld, void *stream);

/* Backward of x = L^{-1} b: y = L^{-T} g (as capsp_solve_transpose), then
 * grad_val as capsp_grad_val; under CAPSP_ALG_SYNCFREE_CSC a CSR handle fuses
 * grad_val into its column-driven sweep.  No reference counterpart. */
capsp_status_t capsp_solve_transpose_grad(capsp_handle_t h, const void *g,
                                          const void *x, void *y, void *grad_val,
                                          int nrhs, int64_t ld, void *stream);

/* Pre-allocate per-handle scratch for up to max_nrhs right-hand sides so later
 * solves (and CUDA-graph captures of them) allocate nothing. */
capsp_status_t capsp_reserve(capsp_handle_t h, int max_nrhs);

/* Synchronise `stream` and report the device-side status of the latest
 * solve on this handle (CAPSP_OK or CAPSP_ERR_TIMEOUT). */
capsp_status_t capsp_status_sync(capsp_handle_t h, void *stream);

/* Host-buffer solve: b (host) in, solve, x (host) out, synchronously, through
 * handle-owned device staging buffers.  With page-locked b and x, one
 * right-hand side and more than 64k rows on the level schedule, the copies
 * overlap the solve: b goes up in doubling row segments on a second stream
 * (each chunk of rows waits for its segment), and x comes back in up to 32
 * segments, each as soon as the kernel has counted all its rows finished
 * (stream memory operations, cuStreamWaitValue32 / cuStreamWriteValue32).
 * Otherwise b is copied (or, up to 64k rows, read in place when page-locked)
 * before the solve and x after it. */
capsp_status_t capsp_solve_host(capsp_handle_t h, const void *b_host, void *x_host,
                                int nrhs);

/* Time the candidate launch configurations (rows per thread x block size x
 * mix border) on this handle with the given device buffers (x is
 * overwritten), keep the fastest for this nrhs, and report its time. */
capsp_status_t capsp_autotune(capsp_handle_t h, const void *b, void *x, int nrhs,
                              int64_t ld, void *stream, float *best_ms);

/* Solve through a CUDA graph: the first call for a given (b, x, nrhs, ld,
 * stream) captures the whole solve sequence, later calls replay it. */
capsp_status_t capsp_graph_solve(capsp_handle_t h, const void *b, void *x, int nrhs,
                                 int64_t ld, void *stream);

/* Kernel timing: while enabled, every solve records two handle-owned CUDA
 * events around its main solve kernel (the first right-hand-side block);
 * capsp_last_kernel_ms waits for the second and returns the elapsed time, so
 * the fill of x and the scratch resets are excluded. */
capsp_status_t capsp_set_profiling(capsp_handle_t h, int enable);
capsp_status_t capsp_last_kernel_ms(capsp_handle_t h, float *ms);

/* Tracing: with a device buffer of 4*n uint64 (NULL switches it off), every
 * row-driven solve records per row i the global-timer nanoseconds at which its
 * warp took the row ([4i]), first polled its dependencies ([4i+1]), had
 * received the last of them ([4i+2]) and published its value ([4i+3]).
 * A row's receipt minus its last dependency's publication is the
 * dependency-hop latency. */
capsp_status_t capsp_debug_trace(capsp_handle_t h, void *row_times_ns);

/* Device properties used for launch sizing (SM count of the current device). */
capsp_status_t capsp_device_sms(int *num_sms);

/* Debug/testing: the owner of `row` computes but never publishes its value,
 * so its dependants' waits run out after `timeout_ns` and the solve reports
 * CAPSP_ERR_TIMEOUT.  row = -1 restores normal operation. */
capsp_status_t capsp_debug_set_stuck_row(capsp_handle_t h, int row, uint64_t timeout_ns);

/* Measure the per-hop dependency latency: solves a chain matrix where row i
 * depends on row i - stride (stride 1: neighbouring lanes of one warp;
 * stride 32*k: different warps) and returns the solve time divided by the
 * number of hops.  Allocates and frees its own matrix. */
capsp_status_t capsp_hop_latency(int n, int stride, int dtype, float *ns_per_hop);

/* No counterpart in the reference.  Lower-triangular CSC solve Lx = b in FP64
 * (the column-driven solve, one right-hand side) that allocates nothing, for
 * callers that must not call cudaMalloc: code whose host framework owns all
 * device memory through its own pool (so a private allocation could fail or
 * break its budget), and code on a latency-critical path, where cudaMalloc /
 * cudaFree can synchronise the device and stall other streams.  Its scratch
 * (1/diag, left_sum, in-degree and arrival counters, ticket, error word) is
 * one static device array of 1.5 MiB, sized for at most 65,536 rows, that
 * every GPU which loads the library holds until the process exits; a larger
 * n is rejected with CAPSP_ERR_INVALID.  All pointers are device pointers;
 * colptr/rowidx must hold the diagonal first in each column and every other
 * row index below it and below n (checked on the device before the solve).  The call resets every scratch part that must
 * start at zero itself, then synchronises `stream` and returns the solve's
 * status: it is synchronous.  Every call resolves the scratch's device address
 * (cudaGetSymbolAddress, with the caller's device current), so a device reset
 * by the caller is picked up.  All calls share the scratch, so overlapping
 * calls would race on it: a process-wide lock serialises them. */
capsp_status_t capsp_csc_solve_noalloc_f64(const int *colptr, const int *rowidx, const double *val,
                                           int n, int nnz, const double *b, double *x, void *stream);

/* ------------------------------------------------------------------------ */
/* 2. Reference-compatible drivers (exact reference argument lists)          */
/*    Each allocates device memory, builds b = L*ones (get_x_b), runs        */
/*    capsp_compat_repeat() timed solves, validates |x-1| <= 0.01 per        */
/*    element (or L1-relative < 1e-4 for the CSC driver) and frees.          */
/*    Return -1 on a non-square matrix, as the reference does.               */
/* ------------------------------------------------------------------------ */

/* CUDA/ourWrtFst/spts_syncfree_cuda_csr_wrt.h:66-75 */
int spts_syncfree_cuda_csr_wrt_f64(const int *csrRowPtrL_tmp, const int *csrColIdxL_tmp,
                                   const double *csrValL_tmp, const int m, const int n,
                                   const int nnzL, double *solve_time_add,
                                   double *gflops_add, double *bandwith_add);
int spts_syncfree_cuda_csr_wrt_f32(const int *csrRowPtrL_tmp, const int *csrColIdxL_tmp,
                                   const float *csrValL_tmp, const int m, const int n,
                                   const int nnzL, double *solve_time_add,
                                   double *gflops_add, double *bandwith_add);

/* CUDA/our2Part/spts_syncfree_cuda_csr.h:133-142 */
int spts_syncfree_cuda_csr_f64(const int *csrRowPtrL_tmp, const int *csrColIdxL_tmp,
                               const double *csrValL_tmp, const int m, const int n,
                               const int nnzL, double *solve_time_add,
                               double *gflops_add, double *bandwith_add);
int spts_syncfree_cuda_csr_f32(const int *csrRowPtrL_tmp, const int *csrColIdxL_tmp,
                               const float *csrValL_tmp, const int m, const int n,
                               const int nnzL, double *solve_time_add,
                               double *gflops_add, double *bandwith_add);

/* CUDA/mix/spts_syncfree_cuda_csr_wrt.h:146-158 (same name as the ourWrtFst
 * driver in the reference, distinguished here by the _mix infix). */
int spts_syncfree_cuda_csr_wrt_mix_f64(const int *csrRowPtrL_tmp, const int *csrColIdxL_tmp,
                                       const double *csrValL_tmp, const int m, const int n,
                                       const int nnzL, double *solve_time_add,
                                       double *gflops_add, double *bandwith_add,
                                       double *pre_time_add, double *warp_occupy_add,
                                       double *element_occupy_add);
int spts_syncfree_cuda_csr_wrt_mix_f32(const int *csrRowPtrL_tmp, const int *csrColIdxL_tmp,
                                       const float *csrValL_tmp, const int m, const int n,
                                       const int nnzL, double *solve_time_add,
                                       double *gflops_add, double *bandwith_add,
                                       double *pre_time_add, double *warp_occupy_add,
                                       double *element_occupy_add);

/* CUDA/SyncFree_csc/spts_syncfree_cuda2.h:89-102 */
int sptrsv_syncfree_cuda_f64(const int *cscColPtrTR, const int *cscRowIdxTR,
                             const double *cscValTR, const int m, const int n,
                             const int nnzTR, double *x, const double *b,
                             const double *x_ref, double *pre_time_add,
                             double *solve_time_add, double *gflops_add,
                             double *bandwidth_add);
int sptrsv_syncfree_cuda_f32(const int *cscColPtrTR, const int *cscRowIdxTR,
                             const float *cscValTR, const int m, const int n,
                             const int nnzTR, float *x, const float *b,
                             const float *x_ref, double *pre_time_add,
                             double *solve_time_add, double *gflops_add,
                             double *bandwidth_add);

/* Number of timed solves the drivers above average over (BENCH_REPEAT, 100 in
 * CUDA/ourWrtFst/common.h:20-22).  Returns the previous value. */
int capsp_compat_set_repeat(int repeat);
int capsp_compat_repeat(void);

/* ------------------------------------------------------------------------ */
/* 3. Host preprocessing (reference contracts) and synthetic generators      */
/* ------------------------------------------------------------------------ */

/* In-place exclusive scan (CUDA/ourWrtFst/tranpose.h:16-32). */
void capsp_exclusive_scan(int *input, int length);

/* Lower-triangular extraction (CUDA/ourWrtFst/read_mtx.h:194-257): sorts every
 * row of A in place, keeps the entries with col < row, forces their values to
 * 1 and appends a unit diagonal.  The three output arrays are malloc'ed and
 * owned by the caller (free()).  Returns 0, or -1 on allocation failure. */
int change2tran_f64(int m, int nnzA, int *csrRowPtrA, int *csrColIdxA, double *csrValA,
                    int *nnzL_add, int **csrRowPtrL_tmp_add, int **csrColIdxL_tmp_add,
                    double **csrValL_tmp_add);
int change2tran_f32(int m, int nnzA, int *csrRowPtrA, int *csrColIdxA, float *csrValA,
                    int *nnzL_add, int **csrRowPtrL_tmp_add, int **csrColIdxL_tmp_add,
                    float **csrValL_tmp_add);

/* x_ref = ones, b = A*x_ref in VALUE_TYPE arithmetic (CUDA/ourWrtFst/read_mtx.h:260-278).
 * Both arrays are malloc'ed and owned by the caller. */
void get_x_b_f64(int m, int n, const int *csrRowPtrA, const int *csrColIdxA,
                 const double *csrValA, double **x_add, double **b_add);
void get_x_b_f32(int m, int n, const int *csrRowPtrA, const int *csrColIdxA,
                 const float *csrValA, float **x_add, float **b_add);

/* Level count and mean rows per level (CUDA/ourWrtFst/tranpose.h:78-142).
 * Returns the level count. */
int matrix_layer_f64(const int m, const int n, const int nnz, const int *csrRowPtr,
                     const int *csrColIdx, const double *csrVal, int *layer_add,
                     double *parallelism_add);
int matrix_layer_f32(const int m, const int n, const int nnz, const int *csrRowPtr,
                     const int *csrColIdx, const float *csrVal, int *layer_add,
                     double *parallelism_add);

/* Level of every row plus the level histogram (level_count[1..levels]);
 * level_count may be NULL.  Same recurrence as matrix_layer. */
int capsp_row_levels(int n, const int *rowptr, const int *colidx, int *level,
                     int *level_count);

/* CSR -> CSC by counting sort; rows ascend within each column
 * (CUDA/ourWrtFst/tranpose.h:36-75).  Caller allocates the outputs. */
void matrix_transposition_f64(const int m, const int n, const int nnz, const int *csrRowPtr,
                              const int *csrColIdx, const double *csrVal, int *cscRowIdx,
                              int *cscColPtr, double *cscVal);
void matrix_transposition_f32(const int m, const int n, const int nnz, const int *csrRowPtr,
                              const int *csrColIdx, const float *csrVal, int *cscRowIdx,
                              int *cscColPtr, float *cscVal);

/* Mix selector table (CUDA/mix/tranpose.h:1423-1483): warp_num (caller
 * allocates m+1 ints) lists the first row of every virtual warp; a 32-row
 * group whose mean nnz/row >= border contributes one virtual warp per row,
 * any other group one virtual warp for the whole group. */
void matrix_warp4_f64(const int m, const int n, const int nnz, const int *csrRowPtr,
                      const int *csrColIdx, const double *csrVal, const int border,
                      int *Len_add, int *warp_num, double *warp_occupy_add,
                      double *element_occupy_add);
void matrix_warp4_f32(const int m, const int n, const int nnz, const int *csrRowPtr,
                      const int *csrColIdx, const float *csrVal, const int border,
                      int *Len_add, int *warp_num, double *warp_occupy_add,
                      double *element_occupy_add);

/* Generalised selector over `group_rows`-row groups in solve order (reversed
 * for upper-triangular matrices).  Returns the table length. */
int capsp_mix_table(int n, const int *rowptr, int upper, int group_rows, int border,
                    int *table, double *warp_occupy, double *element_occupy);

/* Level schedule of a triangular matrix read row by row in solve order
 * (rows 0..n-1 with the diagonal last, or with upper != 0 rows n-1..0 with the
 * diagonal first): level = 1 + deepest dependency level (the recurrence of
 * matrix_layer); order[k] = k-th row of a sort by level and, inside a level,
 * the rows of more than 8 dependencies first by count (most first), then the
 * others by the position of their newest dependency (a level of 32k rows or
 * more that holds such a row: by count alone), ties in solve order;
 * position = its inverse; level_start (optional, n+2 ints) = first position
 * of each level.  Returns the level count or -1. */
int capsp_level_schedule(int n, const int *ptr, const int *idx, int upper, int *order,
                         int *position, int *level_start);

/* The structure transposed: new row j lists the stored rows i that hold index
 * j, ascending; src[p] is the stored index of new entry p.  tptr: n+1; tidx,
 * src: nnz.  Runs on all host threads; the result does not depend on their
 * number.  Returns 0, or -1 when an index is outside [0, n). */
int capsp_transpose_structure(int n, int nnz, const int *ptr, const int *idx, int *tptr, int *tidx,
                              int *src);

/* Dependencies of every schedule position as positions (ascending), with the
 * source index of each dependency value (dep_src) and of each diagonal
 * (diag_src) in the original arrays.  dep_ptr: n+1; dep_idx, dep_src: nnz-n;
 * diag_src: n.  Returns 0 or -1 when a diagonal is misplaced. */
int capsp_level_layout(int n, const int *ptr, const int *idx, int upper, const int *order,
                       const int *position, int *dep_ptr, int *dep_idx, int *dep_src,
                       int *diag_src);

/* In-degree analyser: histogram of idx (CUDA/SyncFree_csc/spts_syncfree_cuda2.h:10-21,
 * openCL/SynFree_csc/sptrsv_syncfree_serialref.h:6-23). */
void capsp_indegree(int n, int nnz, const int *idx, int *indeg);

/* Structure check used by capsp_analyse.  Returns 0 when valid, else the
 * first offending row/column (>= 0 encoded as -(row+2)) and writes a message. */
int capsp_validate(int n, int nnz, const int *ptr, const int *idx, int format,
                   int uplo, char *msg, int msg_len);

/* Matrix Market reader with the reference's contract (CUDA/ourWrtFst/read_mtx.h:6-191):
 * real / integer / pattern, general or symmetric, 1-based coordinates -> CSR.
 * Arrays are malloc'ed and owned by the caller.  Returns 0 or a negative code. */
int read_mtx_f64(const char *filename, int *m_add, int *n_add, int *nnzA_add,
                 int **csrRowPtrA_add, int **csrColIdxA_add, double **csrValA_add);
int read_mtx_f32(const char *filename, int *m_add, int *n_add, int *nnzA_add,
                 int **csrRowPtrA_add, int **csrColIdxA_add, float **csrValA_add);

/* Seeded synthetic lower-triangular generators (stand-ins for SuiteSparse
 * matrices).  Every row draws from its own splitmix64 stream keyed by
 * (seed, stream, row), so the result is independent of thread count. */
typedef enum capsp_gen_kind {
    CAPSP_GEN_UNIFORM_BAND = 0, /* k ~ U{kmin..kmax}, distinct cols uniform in [max(0,i-band), i-1] */
    CAPSP_GEN_ZIPF_NEAR_FAR = 1 /* k ~ max(kmin, Zipf(s) on 1..cap); ceil(k/2) cols in [i-near, i-1]
                                   (at most near of them), the rest uniform in [0, i-1] */
} capsp_gen_kind_t;

typedef struct capsp_gen_params {
    int64_t n;
    uint64_t seed;
    uint64_t stream;
    int kind;
    int kmin;
    int kmax;
    int64_t band;       /* <= 0: whole prefix [0, i-1] */
    double zipf_s;
    int zipf_cap;
    int near_window;
} capsp_gen_params_t;

/* Pass 1: rowptr[0..n] of the generated matrix (off-diagonals + diagonal). */
capsp_status_t capsp_gen_rowptr(const capsp_gen_params_t *p, int *rowptr);
/* Pass 2: columns ascending, values U[-1,1], diagonal 1 + sum|offdiag| last. */
capsp_status_t capsp_gen_fill_f64(const capsp_gen_params_t *p, const int *rowptr,
                                  int *colidx, double *val);
/* count values ~ N(0,1) (Box-Muller over the same hashed streams). */
capsp_status_t capsp_gen_normal_f64(uint64_t seed, uint64_t stream, int64_t count,
                                    double *out);
/* y[i*nrhs + r] = sum_j val[j] * x[col_j*nrhs + r] in double (lower or upper CSR). */
capsp_status_t capsp_spmv_f64(int n, const int *rowptr, const int *colidx,
                              const double *val, int nrhs, const double *x, double *y);
/* 64-bit FNV-1a digest of the structure and value bits (fixture pinning). */
uint64_t capsp_digest(int n, int nnz, const int *rowptr, const int *colidx,
                      const void *val, int val_bytes);

#ifdef __cplusplus
}
#endif

#endif /* CAPSP_H */
