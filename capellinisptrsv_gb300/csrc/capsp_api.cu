// Native C-ABI of libcapsp: handle lifetime, analysis, solve dispatch,
// autotuning and CUDA-graph replay.  All device work is stream-ordered on the
// caller's stream; the only synchronising calls are capsp_analyse,
// capsp_set_values, capsp_status_sync, capsp_solve_host and capsp_autotune.
#include "capsp.h"
#include "capsp_internal.h"
#include "graph_cache.h"

#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

using namespace capsp;

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------

static thread_local std::string g_last_error;

static capsp_status_t fail(capsp_status_t st, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

#define CAPSP_CUDA(call)                                                                       \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? CAPSP_ERR_OOM : CAPSP_ERR_CUDA,      \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                       \
    } while (0)

#define CAPSP_TRY(expr)                                                                        \
    do {                                                                                       \
        capsp_status_t s_ = (expr);                                                            \
        if (s_ != CAPSP_OK)                                                                    \
            return s_;                                                                         \
    } while (0)

extern "C" const char *capsp_last_error(void) { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------

namespace {

struct Tuning {
    int kind;   // kRowWrtFst / kRowTwoPart / kRowMix (row path); ignored on the column path
    int R;      // rows per thread
    int block;  // threads per block
    int bps;    // blocks per SM (0: occupancy maximum)
    int border; // mix border
    bool dflt;  // the handle's defaults (no explicit or autotuned choice)
};

struct MixTable {
    int *d = nullptr;
    int len = 0;
    int border = INT_MIN;
    double wo = 0.0, eo = 0.0;
};

void destroy_graph_exec(cudaGraphExec_t e) { cudaGraphExecDestroy(e); }
typedef GraphCache<cudaGraphExec_t, destroy_graph_exec> Graphs;

// Level schedule of one row-driven view of the matrix (capsp_level_layout):
// view 0 reads the stored arrays as rows (CSR rows; CSC columns, i.e. rows of
// the transpose), view 1 their transpose, built on the host from the stored
// structure.  Entries and diagonals keep their index into the stored values
// (d_lsrc, d_dsrc), so one value array serves both views.
struct RowView {
    bool built = false;
    int upper = 0;        // its rows are upper-triangular (diagonal first)
    int levels = 0;
    bool narrow = false;  // levels narrower than ~4k rows on average
    int *d_perm = nullptr, *d_lptr = nullptr, *d_lidx = nullptr, *d_lsrc = nullptr, *d_dsrc = nullptr;
    void *d_lval = nullptr, *d_linv = nullptr;
    std::vector<int> h_lcum;  // lptr[k] + k: row-count prefix in position space (mix tables)
    // capsp_solve_host's b upload: highest b segment per 32 positions (kernel: b_group_seg)
    unsigned char *d_group_seg = nullptr;
    long long group_seg_b0 = 0;  // first segment's rows the table was built for
};

// Which operations a handle solves through which view: the plain solve of a
// CSR handle and the transpose of a CSC handle walk the stored arrays as rows
// (view 0); the other two walk the transposed view (view 1), or, under
// CAPSP_ALG_SYNCFREE_CSC, the stored arrays column by column.
enum Op { kOpSolve, kOpTranspose, kOpTransposeGrad };

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev)
            cudaSetDevice(dev);
        else
            prev = -1;
    }
    ~DeviceGuard()
    {
        if (prev >= 0)
            cudaSetDevice(prev);
    }
};

}  // namespace

struct capsp_handle_s {
    int device = 0;
    int num_sms = 1;
    int n = 0, nnz = 0, dtype = 0, format = 0, uplo = 0;
    unsigned flags = 0;
    size_t vbytes = 8;
    int *d_ptr = nullptr;
    int *d_idx = nullptr;
    void *d_val = nullptr;
    bool own_struct = false;  // d_ptr / d_idx allocated here
    bool own_val = false;     // d_val allocated here
    std::vector<int> h_ptr;
    void *d_inv = nullptr;
    unsigned *d_ticket = nullptr;  // [64] ticket counters followed by the error word
    int *d_err = nullptr;          // [4]
    int *d_indeg = nullptr;
    int *d_arrived = nullptr;
    int *d_corder[2] = {nullptr, nullptr};  // column-path visiting order: [forward, backward]
    bool col_narrow[2] = {false, false};     // ... and whether its levels are narrower than ~4k
    void *d_left = nullptr;
    int left_cap = 0;  // right-hand sides the left_sum scratch holds
    std::map<int, MixTable> mix;
    int alg = CAPSP_ALG_AUTO;
    int border = 10;
    bool border_explicit = false;
    // measured on GB300 (wide-level solves): one chunk per lane, 8 resident
    // warps per SM; more resident warps only add pollers
    Tuning tune = {kRowWrtFst, 1, 256, 1, 10};
    bool tune_explicit = false;
    std::map<int, Tuning> tuned;  // autotuned plain solves, by nrhs
    // no nanosleep backoff by default: measured neutral on wide levels and
    // 7 % faster on deep chains (zipf_1m), where it delays each detection
    WaitCfg wait = {10000000000ull, 1u << 30, 0u};
    int stuck_row = -1;
    Graphs graphs;  // capsp_graph_solve; invalidated by every change a capture bakes in
    void *d_stage = nullptr;
    size_t stage_bytes = 0;
    cudaStream_t stage_stream = nullptr;
    // capsp_solve_host uploads b and copies finished row segments of x back
    // while the solve runs
    cudaStream_t copy_stream = nullptr, upload_stream = nullptr;
    cudaEvent_t ev_seg0 = nullptr, ev_seg1 = nullptr, ev_up = nullptr;
    int *d_seg = nullptr;            // kMaxSegments completion counters, then kMaxSegments b flags
    int *seg_req = nullptr;          // counters the next level launch counts into (nullptr: none)
    const int *bready_req = nullptr; // b flags the next level launch waits on (nullptr: none)
    int seg_req_rows = 0;            // ... rows per segment of x
    double analyse_ms = 0.0;
    bool profiling = false;
    cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;
    unsigned long long *trace = nullptr;  // borrowed tracing buffer (2n entries)
    // L2 treatment of the publication vector (capsp_set_l2_policy)
    int l2_mode = CAPSP_L2_HINTS;
    bool l2_limit_set = false;
    size_t l2_prev_limit = 0;  // persisting carve-out before this handle changed it
    size_t l2_window = 0;      // largest window the device accepts
    size_t l2_persist = 0;     // persisting carve-out this handle asked for
    int sched = CAPSP_SCHED_LEVEL;  // schedule of view 0; view 1 is always level-ordered
    RowView view[2];
    void *d_xp = nullptr;     // position-ordered publication scratch (both views)
    int xp_cap = 0;           // right-hand sides it holds
    int nsys = 0;
    std::vector<int> sys_rowoff;
    std::recursive_mutex mu;
};

static bool diag_last_of(int format, int uplo) { return (format == CAPSP_FMT_CSR) == (uplo == CAPSP_LOWER); }

static void free_handle(capsp_handle_t h)
{
    if (!h)
        return;
    DeviceGuard g(h->device);
    h->graphs.clear();
    if (h->l2_limit_set)
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, h->l2_prev_limit);
    for (auto &kv : h->mix)
        cudaFree(kv.second.d);
    if (h->own_struct) {
        cudaFree(h->d_ptr);
        cudaFree(h->d_idx);
    }
    if (h->own_val)
        cudaFree(h->d_val);
    cudaFree(h->d_inv);
    cudaFree(h->d_ticket);
    cudaFree(h->d_indeg);
    cudaFree(h->d_arrived);
    cudaFree(h->d_corder[0]);
    cudaFree(h->d_corder[1]);
    cudaFree(h->d_left);
    cudaFree(h->d_stage);
    for (RowView &rv : h->view) {
        cudaFree(rv.d_perm);
        cudaFree(rv.d_lptr);
        cudaFree(rv.d_lidx);
        cudaFree(rv.d_lsrc);
        cudaFree(rv.d_dsrc);
        cudaFree(rv.d_lval);
        cudaFree(rv.d_linv);
        cudaFree(rv.d_group_seg);
    }
    cudaFree(h->d_xp);
    if (h->stage_stream)
        cudaStreamDestroy(h->stage_stream);
    if (h->copy_stream)
        cudaStreamDestroy(h->copy_stream);
    if (h->upload_stream)
        cudaStreamDestroy(h->upload_stream);
    if (h->ev_seg0)
        cudaEventDestroy(h->ev_seg0);
    if (h->ev_seg1)
        cudaEventDestroy(h->ev_seg1);
    if (h->ev_up)
        cudaEventDestroy(h->ev_up);
    cudaFree(h->d_seg);
    if (h->ev_k0)
        cudaEventDestroy(h->ev_k0);
    if (h->ev_k1)
        cudaEventDestroy(h->ev_k1);
    delete h;
}

// refresh 1/diag from the handle's current values; synchronous
static capsp_status_t refresh_inv_diag(capsp_handle_t h)
{
    int *d_bad = nullptr;
    CAPSP_CUDA(cudaMalloc(&d_bad, sizeof(int)));
    const int big = INT_MAX;
    cudaError_t e = cudaMemcpy(d_bad, &big, sizeof(int), cudaMemcpyHostToDevice);
    const int dl = diag_last_of(h->format, h->uplo);
    if (e == cudaSuccess) {
        if (h->dtype == CAPSP_R_64F)
            e = launch_inv_diag<double>(h->d_ptr, (const double *)h->d_val, (double *)h->d_inv, h->n,
                                        dl, d_bad, 0);
        else
            e = launch_inv_diag<float>(h->d_ptr, (const float *)h->d_val, (float *)h->d_inv, h->n, dl,
                                       d_bad, 0);
    }
    int bad = INT_MAX;
    if (e == cudaSuccess)
        e = cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d_bad);
    if (e != cudaSuccess)
        return fail(CAPSP_ERR_CUDA, "computing 1/diag failed: %s", cudaGetErrorString(e));
    if (bad != INT_MAX)
        return fail(CAPSP_ERR_INVALID, "diagonal entry of row/column %d is zero or not finite", bad);
    return CAPSP_OK;
}

// level-schedule values of one built view from the handle's current values, on `st`
static capsp_status_t launch_view_refresh(capsp_handle_t h, const RowView &rv, int *bad, cudaStream_t st)
{
    if (!rv.built)
        return CAPSP_OK;
    if (h->dtype == CAPSP_R_64F)
        CAPSP_CUDA(launch_level_values<double>(rv.d_lptr, rv.d_lsrc, rv.d_dsrc, h->n, (const double *)h->d_val,
                                               (double *)rv.d_lval, (double *)rv.d_linv, bad, st));
    else
        CAPSP_CUDA(launch_level_values<float>(rv.d_lptr, rv.d_lsrc, rv.d_dsrc, h->n, (const float *)h->d_val,
                                              (float *)rv.d_lval, (float *)rv.d_linv, bad, st));
    return CAPSP_OK;
}

// ... of every built view
static capsp_status_t launch_level_refresh(capsp_handle_t h, int *bad, cudaStream_t st)
{
    // Eager, for every built view: a solve captured in a caller's CUDA graph
    // replays with whatever values the views hold, so a refresh outside the
    // graph must not be deferred to a later solve
    for (RowView &rv : h->view)
        CAPSP_TRY(launch_view_refresh(h, rv, bad, st));
    return CAPSP_OK;
}

// view 0: CSR rows in solve order, or CSC columns read as rows of the transpose
static int row_view_upper(capsp_handle_t h)
{
    return h->format == CAPSP_FMT_CSR ? (h->uplo == CAPSP_UPPER) : (h->uplo == CAPSP_LOWER);
}

// the view an operation walks (when it is row-driven)
static int view_of(capsp_handle_t h, Op op) { return (h->format == CAPSP_FMT_CSR) == (op == kOpSolve) ? 0 : 1; }

// whether an operation runs column-driven on the stored arrays
static bool column_driven(capsp_handle_t h, Op op) { return view_of(h, op) == 1 && h->alg == CAPSP_ALG_SYNCFREE_CSC; }

// whether a view's solves follow its level schedule (view 1 has no other)
static bool view_level(capsp_handle_t h, int v) { return v == 1 || h->sched == CAPSP_SCHED_LEVEL; }

// The stored structure transposed by a counting sort over idx.  Each new row
// lists its entries in stored-row order, so its diagonal comes first when the
// stored rows are lower-triangular and last when they are upper-triangular,
// as the transposed view needs; src[p] is the stored index of new entry p.
static capsp_status_t transpose_structure(int n, int nnz, const int *ptr, const int *idx, std::vector<int> &tptr,
                                          std::vector<int> &tidx, std::vector<int> &src)
{
    tptr.resize((size_t)n + 1);
    tidx.resize((size_t)nnz);
    src.resize((size_t)nnz);
    if (capsp_transpose_structure(n, nnz, ptr, idx, tptr.data(), tidx.data(), src.data()) != 0)
        return fail(CAPSP_ERR_INVALID, "an index is outside [0, %d), or host memory ran out", n);
    return CAPSP_OK;
}

// Build the level schedule of view v (host work O(nnz) plus one upload);
// synchronous.
static capsp_status_t build_view(capsp_handle_t h, int v)
{
    RowView &rv = h->view[v];
    if (rv.built)
        return CAPSP_OK;
    h->graphs.invalidate();
    const int n = h->n, nnz = h->nnz;
    int upper = row_view_upper(h);
    std::vector<int> idx((size_t)nnz);
    CAPSP_CUDA(cudaMemcpy(idx.data(), h->d_idx, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToHost));
    const int *vptr = h->h_ptr.data(), *vidx = idx.data();
    std::vector<int> tptr, tidx, tsrc;
    if (v == 1) {
        CAPSP_TRY(transpose_structure(n, nnz, vptr, vidx, tptr, tidx, tsrc));
        vptr = tptr.data();
        vidx = tidx.data();
        upper = !upper;
    }
    std::vector<int> order((size_t)n), position((size_t)n), lptr((size_t)n + 1), dsrc((size_t)n);
    const size_t ndeps = (size_t)nnz - (size_t)n;
    std::vector<int> lidx(ndeps > 0 ? ndeps : 1), lsrc(ndeps > 0 ? ndeps : 1);
    const int levels = capsp_level_schedule(n, vptr, vidx, upper, order.data(), position.data(), nullptr);
    if (levels < 0)
        return fail(CAPSP_ERR_OOM, "host allocation failed while building the level schedule");
    if (capsp_level_layout(n, vptr, vidx, upper, order.data(), position.data(), lptr.data(), lidx.data(),
                           lsrc.data(), dsrc.data()) != 0)
        return fail(CAPSP_ERR_INVALID, "misplaced diagonal while building the level schedule");
    if (v == 1) {
        for (size_t e = 0; e < ndeps; ++e)
            lsrc[e] = tsrc[(size_t)lsrc[e]];
        for (int q = 0; q < n; ++q)
            dsrc[(size_t)q] = tsrc[(size_t)dsrc[(size_t)q]];
    }
    const size_t vb = h->vbytes;
    for (int **p : {&rv.d_perm, &rv.d_lptr, &rv.d_lidx, &rv.d_lsrc, &rv.d_dsrc}) {  // an earlier failed build
        cudaFree(*p);
        *p = nullptr;
    }
    for (void **p : {&rv.d_lval, &rv.d_linv}) {
        cudaFree(*p);
        *p = nullptr;
    }
    CAPSP_CUDA(cudaMalloc(&rv.d_perm, sizeof(int) * (size_t)n));
    CAPSP_CUDA(cudaMalloc(&rv.d_lptr, sizeof(int) * ((size_t)n + 1)));
    // 4 entries of padding: the row kernels stage a chunk's entries in 16-byte
    // pieces from a 16-byte boundary, up to 3 entries past its last one
    CAPSP_CUDA(cudaMalloc(&rv.d_lidx, sizeof(int) * (lidx.size() + 4)));
    CAPSP_CUDA(cudaMalloc(&rv.d_lsrc, sizeof(int) * lsrc.size()));
    CAPSP_CUDA(cudaMalloc(&rv.d_dsrc, sizeof(int) * (size_t)n));
    CAPSP_CUDA(cudaMalloc(&rv.d_lval, vb * (lidx.size() + 4)));
    CAPSP_CUDA(cudaMemset(rv.d_lidx + lidx.size(), 0, sizeof(int) * 4));
    CAPSP_CUDA(cudaMemset((char *)rv.d_lval + vb * lidx.size(), 0, vb * 4));
    CAPSP_CUDA(cudaMalloc(&rv.d_linv, vb * (size_t)n));
    CAPSP_CUDA(cudaMemcpy(rv.d_perm, order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice));
    CAPSP_CUDA(cudaMemcpy(rv.d_lptr, lptr.data(), sizeof(int) * ((size_t)n + 1), cudaMemcpyHostToDevice));
    CAPSP_CUDA(cudaMemcpy(rv.d_lidx, lidx.data(), sizeof(int) * lidx.size(), cudaMemcpyHostToDevice));
    CAPSP_CUDA(cudaMemcpy(rv.d_lsrc, lsrc.data(), sizeof(int) * lsrc.size(), cudaMemcpyHostToDevice));
    CAPSP_CUDA(cudaMemcpy(rv.d_dsrc, dsrc.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice));
    rv.h_lcum.resize((size_t)n + 1);
    for (int k = 0; k <= n; ++k)
        rv.h_lcum[k] = lptr[k] + k;
    rv.upper = upper;
    rv.levels = levels;
    // levels narrower than ~4k rows: two resident warps per SM for the row
    // path by default (more rows in flight than a few levels only add pollers)
    rv.narrow = (long long)n < 4096LL * (long long)levels;
    rv.built = true;
    int *d_bad = nullptr;
    CAPSP_CUDA(cudaMalloc(&d_bad, sizeof(int)));
    const int big = INT_MAX;
    int bad = INT_MAX;
    cudaError_t e = cudaMemcpy(d_bad, &big, sizeof(int), cudaMemcpyHostToDevice);
    capsp_status_t s = e == cudaSuccess ? launch_view_refresh(h, rv, d_bad, 0) : CAPSP_ERR_CUDA;
    if (s == CAPSP_OK)
        e = cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d_bad);
    if (s != CAPSP_OK || e != cudaSuccess)
        return fail(CAPSP_ERR_CUDA, "level-schedule upload failed");
    if (bad != INT_MAX)
        return fail(CAPSP_ERR_INVALID, "zero or non-finite diagonal at schedule position %d", bad);
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_device_sms(int *num_sms)
{
    if (!num_sms)
        return fail(CAPSP_ERR_INVALID, "num_sms is NULL");
    int dev = 0;
    CAPSP_CUDA(cudaGetDevice(&dev));
    CAPSP_CUDA(cudaDeviceGetAttribute(num_sms, cudaDevAttrMultiProcessorCount, dev));
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_analyse(int n, int nnz, const int *ptr, const int *idx,
                                        const void *val, int dtype, int format, int uplo,
                                        unsigned flags, capsp_handle_t *out)
{
    const auto t0 = std::chrono::steady_clock::now();
    if (!out)
        return fail(CAPSP_ERR_INVALID, "out handle pointer is NULL");
    *out = nullptr;
    if (!ptr || !idx || !val)
        return fail(CAPSP_ERR_INVALID, "ptr, idx and val must be non-NULL");
    if (n < 1 || nnz < n)
        return fail(CAPSP_ERR_INVALID, "need n >= 1 and nnz >= n (got n=%d, nnz=%d)", n, nnz);
    if (dtype != CAPSP_R_64F && dtype != CAPSP_R_32F)
        return fail(CAPSP_ERR_INVALID, "unknown dtype %d", dtype);
    if (format != CAPSP_FMT_CSR && format != CAPSP_FMT_CSC)
        return fail(CAPSP_ERR_INVALID, "unknown format %d", format);
    if (uplo != CAPSP_LOWER && uplo != CAPSP_UPPER)
        return fail(CAPSP_ERR_INVALID, "unknown uplo %d", uplo);

    capsp_handle_t h = new (std::nothrow) capsp_handle_s();
    if (!h)
        return fail(CAPSP_ERR_OOM, "host allocation of the handle failed");
    h->n = n;
    h->nnz = nnz;
    h->dtype = dtype;
    h->format = format;
    h->uplo = uplo;
    h->flags = flags;
    h->vbytes = dtype == CAPSP_R_64F ? 8 : 4;
    capsp_status_t st = CAPSP_OK;
    cudaError_t e = cudaGetDevice(&h->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
    if (e != cudaSuccess) {
        free_handle(h);
        return fail(CAPSP_ERR_CUDA, "no usable CUDA device: %s", cudaGetErrorString(e));
    }
    const int dl = diag_last_of(format, uplo);
    h->h_ptr.resize((size_t)n + 1);

    if (!(flags & CAPSP_DEVICE_POINTERS)) {
        if (!(flags & CAPSP_SKIP_VALIDATION)) {
            char msg[256];
            if (capsp_validate(n, nnz, ptr, idx, format, uplo, msg, sizeof(msg)) != 0) {
                free_handle(h);
                return fail(CAPSP_ERR_INVALID, "invalid matrix: %s", msg);
            }
        }
        memcpy(h->h_ptr.data(), ptr, sizeof(int) * ((size_t)n + 1));
        h->own_struct = h->own_val = true;
        e = cudaMalloc(&h->d_ptr, sizeof(int) * ((size_t)n + 1));
        if (e == cudaSuccess)
            e = cudaMalloc(&h->d_idx, sizeof(int) * (size_t)nnz);
        if (e == cudaSuccess)
            e = cudaMalloc(&h->d_val, h->vbytes * (size_t)nnz);
        if (e == cudaSuccess)
            e = cudaMemcpy(h->d_ptr, ptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(h->d_idx, idx, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(h->d_val, val, h->vbytes * (size_t)nnz, cudaMemcpyHostToDevice);
    } else {
        h->d_ptr = const_cast<int *>(ptr);
        h->d_idx = const_cast<int *>(idx);
        h->d_val = const_cast<void *>(val);
        e = cudaMemcpy(h->h_ptr.data(), ptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && !(flags & CAPSP_SKIP_VALIDATION)) {
            int *d_bad = nullptr;
            e = cudaMalloc(&d_bad, sizeof(int));
            const int big = INT_MAX;
            int bad = INT_MAX;
            if (e == cudaSuccess)
                e = cudaMemcpy(d_bad, &big, sizeof(int), cudaMemcpyHostToDevice);
            if (e == cudaSuccess)
                e = launch_validate(h->d_ptr, h->d_idx, n, nnz, dl, d_bad, 0);
            if (e == cudaSuccess)
                e = cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost);
            cudaFree(d_bad);
            if (e == cudaSuccess && (bad != INT_MAX || h->h_ptr[0] != 0 || h->h_ptr[n] != nnz)) {
                free_handle(h);
                return fail(CAPSP_ERR_INVALID,
                            "invalid matrix: row/column %d has a missing or misplaced diagonal, an "
                            "index on the wrong side of it, or an out-of-order pointer",
                            bad == INT_MAX ? 0 : bad);
            }
        }
    }
    if (e == cudaSuccess)
        e = cudaMalloc(&h->d_inv, h->vbytes * (size_t)n);
    if (e == cudaSuccess)
        e = cudaMalloc(&h->d_ticket, sizeof(unsigned) * 64 + sizeof(int) * 4);
    if (e == cudaSuccess)
        e = cudaMemset(h->d_ticket, 0, sizeof(unsigned) * 64 + sizeof(int) * 4);
    if (e != cudaSuccess) {
        free_handle(h);
        return fail(e == cudaErrorMemoryAllocation ? CAPSP_ERR_OOM : CAPSP_ERR_CUDA,
                    "analysis failed: %s", cudaGetErrorString(e));
    }
    h->d_err = reinterpret_cast<int *>(h->d_ticket + 64);
    st = refresh_inv_diag(h);
    if (st == CAPSP_OK)
        st = build_view(h, view_of(h, kOpSolve));  // the default path of the plain solve
    if (st != CAPSP_OK) {
        free_handle(h);
        return st;
    }
    h->analyse_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    *out = h;
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_batched_create(int nsys, const int *sys_rowoff, int n, int nnz,
                                               const int *ptr, const int *idx, const void *val,
                                               int dtype, unsigned flags, capsp_handle_t *out)
{
    if (!out)
        return fail(CAPSP_ERR_INVALID, "out handle pointer is NULL");
    *out = nullptr;
    if (nsys < 1 || !sys_rowoff)
        return fail(CAPSP_ERR_INVALID, "need nsys >= 1 and a system row-offset table");
    if (sys_rowoff[0] != 0 || sys_rowoff[nsys] != n)
        return fail(CAPSP_ERR_INVALID, "sys_rowoff must start at 0 and end at n=%d", n);
    for (int s = 0; s < nsys; ++s)
        if (sys_rowoff[s + 1] <= sys_rowoff[s])
            return fail(CAPSP_ERR_INVALID, "system %d is empty or out of order", s);
    if (!(flags & CAPSP_DEVICE_POINTERS) && !(flags & CAPSP_SKIP_VALIDATION) && ptr && idx) {
        // every entry must stay inside its own system's diagonal block
        for (int s = 0; s < nsys; ++s)
            for (int i = sys_rowoff[s]; i < sys_rowoff[s + 1]; ++i)
                for (int j = ptr[i]; j < ptr[i + 1]; ++j)
                    if (idx[j] < sys_rowoff[s] || idx[j] > i)
                        return fail(CAPSP_ERR_INVALID,
                                    "row %d of system %d references column %d outside its block", i,
                                    s, idx[j]);
    }
    capsp_handle_t h = nullptr;
    CAPSP_TRY(capsp_analyse(n, nnz, ptr, idx, val, dtype, CAPSP_FMT_CSR, CAPSP_LOWER, flags, &h));
    h->nsys = nsys;
    h->sys_rowoff.assign(sys_rowoff, sys_rowoff + nsys + 1);
    *out = h;
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_destroy(capsp_handle_t h)
{
    free_handle(h);
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_set_values(capsp_handle_t h, const void *val)
{
    if (!h || !val)
        return fail(CAPSP_ERR_INVALID, "handle and val must be non-NULL");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    h->graphs.invalidate();  // captured natural-schedule solves read d_val directly
    if (h->flags & CAPSP_DEVICE_POINTERS) {
        h->d_val = const_cast<void *>(val);
    } else {
        CAPSP_CUDA(cudaMemcpy(h->d_val, val, h->vbytes * (size_t)h->nnz, cudaMemcpyHostToDevice));
    }
    CAPSP_TRY(refresh_inv_diag(h));
    CAPSP_TRY(launch_level_refresh(h, h->d_err + 3, 0));
    CAPSP_CUDA(cudaDeviceSynchronize());
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_refresh_values(capsp_handle_t h, const void *val, void *stream)
{
    if (!h)
        return fail(CAPSP_ERR_INVALID, "handle is NULL");
    if (!(h->flags & CAPSP_DEVICE_POINTERS))
        return fail(CAPSP_ERR_INVALID,
                    "capsp_refresh_values needs a CAPSP_DEVICE_POINTERS handle; use capsp_set_values");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    if (val && val != h->d_val) {
        h->graphs.invalidate();
        h->d_val = const_cast<void *>(val);
    }
    const int dl = diag_last_of(h->format, h->uplo);
    cudaStream_t st = (cudaStream_t)stream;
    int *bad = h->d_err + 3;  // sticky diagnostic slot: first row with a bad diagonal
    if (h->dtype == CAPSP_R_64F)
        CAPSP_CUDA(launch_inv_diag<double>(h->d_ptr, (const double *)h->d_val, (double *)h->d_inv, h->n, dl, bad, st));
    else
        CAPSP_CUDA(launch_inv_diag<float>(h->d_ptr, (const float *)h->d_val, (float *)h->d_inv, h->n, dl, bad, st));
    return launch_level_refresh(h, bad, st);
}

extern "C" capsp_status_t capsp_set_schedule(capsp_handle_t h, int schedule)
{
    if (!h)
        return fail(CAPSP_ERR_INVALID, "handle is NULL");
    if (schedule != CAPSP_SCHED_NATURAL && schedule != CAPSP_SCHED_LEVEL)
        return fail(CAPSP_ERR_INVALID, "unknown schedule %d", schedule);
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    h->sched = schedule;
    h->tuned.clear();
    h->graphs.invalidate();
    if (schedule == CAPSP_SCHED_LEVEL)
        return build_view(h, 0);
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_set_backoff(capsp_handle_t h, unsigned sleep_max_ns)
{
    if (!h)
        return fail(CAPSP_ERR_INVALID, "handle is NULL");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    h->wait.sleep_max_ns = sleep_max_ns;
    h->graphs.invalidate();
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_set_l2_policy(capsp_handle_t h, int mode)
{
    if (!h || (mode != CAPSP_L2_HINTS && mode != CAPSP_L2_WINDOW_AND_HINTS && mode != CAPSP_L2_WINDOW))
        return fail(CAPSP_ERR_INVALID, "need a handle and a capsp_l2_policy_t mode");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    if (mode != CAPSP_L2_HINTS && !h->l2_limit_set) {
        int max_win = 0, max_persist = 0;
        CAPSP_CUDA(cudaDeviceGetAttribute(&max_win, cudaDevAttrMaxAccessPolicyWindowSize, h->device));
        CAPSP_CUDA(cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, h->device));
        if (max_win <= 0 || max_persist <= 0)
            return fail(CAPSP_ERR_UNSUPPORTED, "this device has no persisting L2 carve-out");
        CAPSP_CUDA(cudaDeviceGetLimit(&h->l2_prev_limit, cudaLimitPersistingL2CacheSize));
        const size_t want = h->vbytes * (size_t)h->n;
        h->l2_persist = want < (size_t)max_persist ? want : (size_t)max_persist;
        CAPSP_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, h->l2_persist));
        h->l2_limit_set = true;
        h->l2_window = (size_t)max_win;
    } else if (mode == CAPSP_L2_HINTS && h->l2_limit_set) {
        CAPSP_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, h->l2_prev_limit));
        h->l2_limit_set = false;
    }
    h->l2_mode = mode;
    h->graphs.invalidate();
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_set_algorithm(capsp_handle_t h, int algorithm)
{
    if (!h)
        return fail(CAPSP_ERR_INVALID, "handle is NULL");
    if (algorithm < CAPSP_ALG_AUTO || algorithm > CAPSP_ALG_SYNCFREE_CSC)
        return fail(CAPSP_ERR_INVALID, "unknown algorithm %d", algorithm);
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    h->alg = algorithm;
    h->tuned.clear();
    h->graphs.invalidate();
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_set_mix_border(capsp_handle_t h, int border)
{
    if (!h)
        return fail(CAPSP_ERR_INVALID, "handle is NULL");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    h->border = border;
    h->tune.border = border;
    h->border_explicit = true;
    h->tuned.clear();
    h->graphs.invalidate();
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_set_tuning(capsp_handle_t h, int rows_per_thread, int block_threads,
                                           int blocks_per_sm)
{
    if (!h)
        return fail(CAPSP_ERR_INVALID, "handle is NULL");
    if (rows_per_thread != 1 && rows_per_thread != 2 && rows_per_thread != 4)
        return fail(CAPSP_ERR_INVALID, "rows_per_thread must be 1, 2 or 4");
    if (block_threads < 64 || block_threads > 512 || block_threads % 32)
        return fail(CAPSP_ERR_INVALID, "block_threads must be a multiple of 32 in [64, 512]");
    if (blocks_per_sm < 0)
        return fail(CAPSP_ERR_INVALID, "blocks_per_sm must be >= 0");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    h->tune.R = rows_per_thread;
    h->tune.block = block_threads;
    h->tune.bps = blocks_per_sm;
    h->tune_explicit = true;
    h->tuned.clear();
    h->graphs.invalidate();
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_set_timeout(capsp_handle_t h, uint64_t timeout_ns)
{
    if (!h || timeout_ns == 0)
        return fail(CAPSP_ERR_INVALID, "need a handle and a positive timeout");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    h->wait.timeout_ns = timeout_ns;
    h->graphs.invalidate();
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_debug_set_stuck_row(capsp_handle_t h, int row, uint64_t timeout_ns)
{
    if (!h || row < -1 || row >= h->n)
        return fail(CAPSP_ERR_INVALID, "need a handle and a row in [-1, n)");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    h->stuck_row = row;
    if (timeout_ns)
        h->wait.timeout_ns = timeout_ns;
    h->graphs.invalidate();
    return CAPSP_OK;
}

// ---------------------------------------------------------------------------
// lazily built analysis products (never called while a stream is captured
// for the first time: prepare() runs them before capture)
// ---------------------------------------------------------------------------

// rows per mix group for a launch with nrhs right-hand sides
static int group_rows_for(int nrhs) { return 32 / lanes_for_rhs(nrhs < 32 ? nrhs : 32); }

// Selector table over `group_rows` consecutive schedule positions of view v;
// its row counts come from the view's level layout (dependencies + diagonal
// per position) or, for view 0's natural schedule, from the stored row pointer.
static capsp_status_t ensure_mix(capsp_handle_t h, int v, int group_rows, int border, MixTable **out)
{
    const bool level = view_level(h, v);
    MixTable &mt = h->mix[(group_rows * 2 + (level ? 1 : 0)) * 2 + v];
    if (mt.d == nullptr || mt.border != border) {
        h->graphs.invalidate();  // a captured launch holds the old table's length
        std::vector<int> table((size_t)h->n + 2);
        double wo = 0.0, eo = 0.0;
        const int len = level ? capsp_mix_table(h->n, h->view[v].h_lcum.data(), 0, group_rows, border,
                                                table.data(), &wo, &eo)
                              : capsp_mix_table(h->n, h->h_ptr.data(), row_view_upper(h), group_rows, border,
                                                table.data(), &wo, &eo);
        if (mt.d == nullptr)
            CAPSP_CUDA(cudaMalloc(&mt.d, sizeof(int) * ((size_t)h->n + 2)));
        CAPSP_CUDA(cudaMemcpy(mt.d, table.data(), sizeof(int) * (size_t)len, cudaMemcpyHostToDevice));
        mt.len = len;
        mt.border = border;
        mt.wo = wo;
        mt.eo = eo;
    }
    *out = &mt;
    return CAPSP_OK;
}

// Column-driven solves keep each target's partial sum and arrival count in one
// atomic word (col_solve_packed_kernel) instead of a left_sum array, a counter
// array and a fence between them.
constexpr bool kPackedColumns = true;

static capsp_status_t ensure_column_scratch(capsp_handle_t h, int nrhs)
{
    if (!h->d_indeg) {
        CAPSP_CUDA(cudaMalloc(&h->d_indeg, sizeof(int) * (size_t)h->n));
        CAPSP_CUDA(cudaMemset(h->d_indeg, 0, sizeof(int) * (size_t)h->n));
        CAPSP_CUDA(launch_histogram(h->d_idx, h->nnz, h->d_indeg, 0));
        CAPSP_CUDA(cudaDeviceSynchronize());
    }
    if (!h->d_arrived)
        CAPSP_CUDA(cudaMalloc(&h->d_arrived, sizeof(int) * (size_t)h->n));
    const int want = nrhs < 32 ? nrhs : 32;
    if (h->left_cap < want) {
        h->graphs.invalidate();  // captured column solves point at the old words
        cudaFree(h->d_left);
        h->d_left = nullptr;
        h->left_cap = 0;
        // twice the left_sum size: the column kernels keep a sum-and-count
        // word (two values' width) per element
        CAPSP_CUDA(cudaMalloc(&h->d_left, 2 * h->vbytes * (size_t)h->n * (size_t)want));
        h->left_cap = want;
    }
    return CAPSP_OK;
}

// Visiting order of the column-driven solve: columns stable-sorted by their
// level in the column DAG (a column's level is one more than the deepest
// column that scatters into it).  Warps then take columns that become ready
// together instead of a window of consecutive indices that holds only a few
// columns of the current level.  Every producer of a column comes before it,
// so ticket order keeps forward progress independent of block scheduling.
// Forward: columns ascend and scatter into rows below the diagonal; backward:
// columns descend and scatter into smaller indices (the transpose solve on
// the CSR arrays of a lower-triangular matrix).
static capsp_status_t ensure_column_order(capsp_handle_t h, int backward)
{
    if (h->d_corder[backward])
        return CAPSP_OK;
    const int n = h->n, nnz = h->nnz;
    std::vector<int> idx((size_t)nnz);
    CAPSP_CUDA(cudaMemcpy(idx.data(), h->d_idx, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToHost));
    const int *ptr = h->h_ptr.data();
    std::vector<int> lev((size_t)n, 0);
    int deepest = 0;
    for (int s = 0; s < n; ++s) {
        const int j = backward ? n - 1 - s : s;
        const int next = lev[j] + 1;
        if (lev[j] > deepest)
            deepest = lev[j];
        for (int k = ptr[j]; k < ptr[j + 1]; ++k) {
            const int r = idx[k];
            if (r != j && lev[r] < next)
                lev[r] = next;
        }
    }
    std::vector<int> start((size_t)deepest + 2, 0), order((size_t)n);
    for (int j = 0; j < n; ++j)
        ++start[(size_t)lev[j] + 1];
    for (int l = 0; l <= deepest; ++l)
        start[(size_t)l + 1] += start[(size_t)l];
    for (int s = 0; s < n; ++s) {
        const int j = backward ? n - 1 - s : s;
        order[(size_t)start[(size_t)lev[j]]++] = j;
    }
    int *d = nullptr;
    CAPSP_CUDA(cudaMalloc(&d, sizeof(int) * (size_t)n));
    const cudaError_t e = cudaMemcpy(d, order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return fail(CAPSP_ERR_CUDA, "column order upload failed: %s", cudaGetErrorString(e));
    }
    h->d_corder[backward] = d;
    h->col_narrow[backward] = (long long)n < 4096LL * (long long)(deepest + 1);
    return CAPSP_OK;
}

// Launch shape of a row-path launch with nrhs right-hand sides.  Defaults
// measured on GB300: with one lane per row (32 rows per warp) four resident
// warps per SM suit narrow levels (more rows in flight than a few levels only
// add pollers; 4 against 2 warps: grad_1m 1.253 against 1.268 ms, its
// transpose 1.296 against 1.314 ms, zipf40_1m 510 against 527 ms, zipf_1m
// 100.7 against 100.3 ms), ten suit levels of 4k-32k rows (wide_4m, 5.8k rows per
// level, warps per SM 2/4/6/8/12/16: 1.708/1.091/0.877/0.765/0.748/0.782 ms;
// with the L2 prefetch of the next round's metadata, 10 against 12 warps:
// 0.718 against 0.727 ms, FP32 0.655 against 0.666 ms; the capsp_solve_host
// build, whose chunks also wait for b and count their rows, keeps 12: 0.742
// against 0.762 ms) and every warp the SM holds on levels of 32k rows and
// more, which are bound by throughput (2,048 banded systems, 93k rows per
// level: 2.95 ms at 8 warps, 1.77 ms at 16, 1.62 ms at 20 in 128-thread
// blocks); with G >= 4 lanes per row a warp holds few rows, so there too
// every warp the SM can hold in 128-thread blocks pays off.
// Wide levels with G >= 4 lanes per row also take the 64-register kernel build
// (*cap), whatever the shape.
// Levels of 32k rows and more on average keep the GPU busy without waiting on
// the dependency chain: the solve is then bound by throughput, not latency.
static bool wide_levels(capsp_handle_t h, int v)
{
    const RowView &rv = h->view[v];
    return rv.built && (long long)h->n >= 32768LL * (long long)rv.levels;
}

static void row_shape(capsp_handle_t h, int v, const Tuning &tn, int nrhs, int *block, int *bps,
                      bool *cap = nullptr, bool hostio = false)
{
    const int g = lanes_for_rhs(nrhs);
    const bool level = view_level(h, v);
    const bool narrow = h->view[v].narrow && level;
    if (cap)
        *cap = g >= 4 && !narrow && level;
    *block = tn.block;
    *bps = tn.bps;
    if (!tn.dflt)
        return;
    if (g == 1 && wide_levels(h, v)) {
        *block = 128;  // every warp the SM holds
        *bps = 0;
    } else if (g == 1) {
        *block = narrow ? 128 : (hostio ? 384 : 320);
        *bps = 1;
    } else if (g == 2) {
        *block = 256;
        *bps = narrow ? 1 : 0;
    } else {
        *block = 128;
        *bps = 0;
    }
}

// launch tuning of an operation with nrhs right-hand sides (autotuned choices
// cover the plain solve)
static Tuning current_tuning(capsp_handle_t h, Op op, int nrhs)
{
    if (op == kOpSolve) {
        auto it = h->tuned.find(nrhs);
        if (it != h->tuned.end())
            return it->second;
    }
    const int v = view_of(h, op);
    const RowView &rv = h->view[v];
    Tuning t = h->tune;
    t.border = h->border;
    t.dflt = !h->tune_explicit;
    // deep matrices, whose levels are narrower than a warp's 32 rows, have no
    // row parallelism to spread over lanes: AUTO gives every row a whole warp
    // (measured on GB300: zipf_1m, 8 rows per level, 177 -> 144 ms)
    // Otherwise AUTO gives a row group a warp per row only when its rows hold
    // a warp's worth of entries on average: shorter rows run faster one per
    // lane (measured on GB300: 2,048 banded systems with 4-13 entries per row,
    // mixed at the reference's border of 10: 2.98 ms; one lane per row:
    // 1.96 ms).
    if ((h->alg == CAPSP_ALG_AUTO || h->alg == CAPSP_ALG_SYNCFREE_CSC) && !h->border_explicit) {
        if (rv.built && view_level(h, v) && (long long)h->n < 32LL * (long long)rv.levels)
            t.border = 1;
        else if (t.border < 32)
            t.border = 32;
    }
    switch (h->alg) {
    case CAPSP_ALG_TWOPART: t.kind = kRowTwoPart; break;
    case CAPSP_ALG_MIX: t.kind = kRowMix; break;
    case CAPSP_ALG_WRTFST: t.kind = kRowWrtFst; break;
    default: t.kind = -1; break;  // AUTO: decided from the mix table
    }
    return t;
}

// ---------------------------------------------------------------------------
// enqueue paths
// ---------------------------------------------------------------------------

// position-ordered publication scratch for the level schedule
static capsp_status_t ensure_xp(capsp_handle_t h, int nrhs)
{
    const int want = nrhs < 32 ? nrhs : 32;
    if (h->xp_cap < want) {
        h->graphs.invalidate();  // captured row solves point at the old scratch
        cudaFree(h->d_xp);
        h->d_xp = nullptr;
        h->xp_cap = 0;
        CAPSP_CUDA(cudaMalloc(&h->d_xp, h->vbytes * (size_t)h->n * (size_t)want));
        h->xp_cap = want;
    }
    return CAPSP_OK;
}

// row-driven solve over view v
template <typename T>
static capsp_status_t enqueue_rows(capsp_handle_t h, int v, const T *b, T *x, int nrhs, int64_t ld,
                                   const Tuning &tn, cudaStream_t st)
{
    const bool level = view_level(h, v);
    const RowView &rv = h->view[v];
    if (level) {
        CAPSP_TRY(build_view(h, v));
        CAPSP_TRY(ensure_xp(h, nrhs));
    }
    for (int r0 = 0; r0 < nrhs; r0 += 32) {
        const int nb = nrhs - r0 < 32 ? nrhs - r0 : 32;
        int kind = tn.kind;
        MixTable *mt = nullptr;
        // AUTO with 8+ lanes per row: a heavy row would get only 32/G slices,
        // too few to pay for the warp's reduction (measured on GB300: grad_1m
        // 16 RHS 1.34 ms mixed, 1.13 ms thread-per-row)
        if (kind < 0 && lanes_for_rhs(nb) >= 8)
            kind = kRowWrtFst;
        if (kind == kRowMix || kind < 0) {
            CAPSP_TRY(ensure_mix(h, v, group_rows_for(nb), tn.border, &mt));
            if (kind < 0)
                kind = mt->wo > 0.0 ? kRowMix : kRowWrtFst;
        }
        // the publication vector starts all-pending: the caller's x (natural
        // schedule) or the position-ordered scratch (level schedule)
        if (level)
            CAPSP_CUDA(launch_fill_pending<T>((T *)h->d_xp, h->n, nb, nb, h->d_ticket, 1,
                                              r0 == 0 ? h->d_err : nullptr, st));
        else
            CAPSP_CUDA(launch_fill_pending<T>(x + r0, h->n, nb, ld, h->d_ticket, 1,
                                              r0 == 0 ? h->d_err : nullptr, st));
        RowArgs<T> a;
        a.ptr = h->d_ptr;
        a.idx = h->d_idx;
        a.val = (const T *)h->d_val;
        a.inv_diag = (const T *)h->d_inv;
        a.perm = level ? rv.d_perm : nullptr;
        a.lptr = rv.d_lptr;
        a.lidx = rv.d_lidx;
        a.lval = (const T *)rv.d_lval;
        a.linv = (const T *)rv.d_linv;
        a.xp = (T *)h->d_xp;
        a.ldp = nb;
        a.b = b + r0;
        a.x = x + r0;
        a.ld = ld;
        a.n = h->n;
        a.nrhs = nb;
        a.upper = row_view_upper(h);  // read by view 0's natural schedule only
        a.table = kind == kRowMix ? mt->d : nullptr;
        a.table_len = kind == kRowMix ? mt->len : 0;
        a.ticket = h->d_ticket;
        a.err = h->d_err;
        a.wait = h->wait;
        a.stuck_row = h->stuck_row;
        a.trace = r0 == 0 ? h->trace : nullptr;
        a.keep_hint = h->l2_mode != CAPSP_L2_WINDOW;
        a.win_base = nullptr;
        a.win_bytes = 0;
        a.win_hit = 0.f;
        // rows are complete once the launch of the last right-hand sides ends
        const bool count = level && h->seg_req != nullptr && r0 + nb == nrhs;
        a.seg_count = count ? h->seg_req : nullptr;
        a.b_ready = level && rv.d_group_seg ? h->bready_req : nullptr;
        a.b_group_seg = a.b_ready ? rv.d_group_seg : nullptr;
        a.seg_rows = count ? h->seg_req_rows : 1;
        if (level && h->l2_mode != CAPSP_L2_HINTS && h->l2_window > 0) {
            const size_t bytes = h->vbytes * (size_t)h->n * (size_t)nb;
            a.win_base = h->d_xp;
            a.win_bytes = bytes < h->l2_window ? bytes : h->l2_window;
            const double hit = (double)h->l2_persist / (double)a.win_bytes;
            a.win_hit = hit >= 1.0 ? 1.f : (float)hit;
        }
        const bool prof = h->profiling && r0 == 0;
        if (prof)
            CAPSP_CUDA(cudaEventRecord(h->ev_k0, st));
        int blk = 0, bps = 0;
        bool cap = false;
        row_shape(h, v, tn, nb, &blk, &bps, &cap, a.seg_count != nullptr || a.b_ready != nullptr);
        // One lane per row stages each sub-chunk's entries in shared memory
        // with coalesced copies, which shortens the dependency hops of
        // latency-bound FP64 solves (measured on GB300: wide_4m 0.792 -> 0.771
        // ms, grad_1m 1.324 -> 1.311 ms) but slows throughput-bound ones
        // (2,048 systems with 93k rows per level: 1.66 -> 2.34 ms).  FP32
        // entries are 8 bytes, and there it was mixed (wide_4m 0.715 -> 0.730
        // ms, grad_1m 1.242 -> 1.230 ms), so FP32 walks the rows directly.
        const bool stage = level && nb == 1 && !wide_levels(h, v) && sizeof(T) == 8;
        CAPSP_CUDA(launch_row_solve<T>(a, kind, tn.R, blk, bps, h->num_sms, cap, stage, st));
        if (prof)
            CAPSP_CUDA(cudaEventRecord(h->ev_k1, st));
    }
    return CAPSP_OK;
}

template <typename T>
static capsp_status_t enqueue_cols(capsp_handle_t h, const T *b, T *x, int nrhs, int64_t ld,
                                   int backward, const T *xf, T *grad, const Tuning &tn,
                                   cudaStream_t st)
{
    CAPSP_TRY(ensure_column_scratch(h, nrhs));
    CAPSP_TRY(ensure_column_order(h, backward));
    for (int r0 = 0; r0 < nrhs; r0 += 32) {
        const int nb = nrhs - r0 < 32 ? nrhs - r0 : 32;
        if (kPackedColumns) {
            CAPSP_CUDA(cudaMemsetAsync(h->d_left, 0, 2 * h->vbytes * (size_t)h->n * (size_t)nb, st));
        } else {
            CAPSP_CUDA(cudaMemsetAsync(h->d_arrived, 0, sizeof(int) * (size_t)h->n, st));
            CAPSP_CUDA(cudaMemsetAsync(h->d_left, 0, h->vbytes * (size_t)h->n * (size_t)nb, st));
        }
        CAPSP_CUDA(cudaMemsetAsync(h->d_ticket, 0, sizeof(unsigned), st));
        if (r0 == 0)
            CAPSP_CUDA(cudaMemsetAsync(h->d_err, 0, sizeof(int) * 4, st));
        ColArgs<T> a;
        a.ptr = h->d_ptr;
        a.idx = h->d_idx;
        a.val = (const T *)h->d_val;
        a.inv_diag = (const T *)h->d_inv;
        a.indeg = h->d_indeg;
        a.order = h->d_corder[backward];
        a.arrived = h->d_arrived;
        a.left_sum = (T *)h->d_left;
        a.slots = kPackedColumns ? h->d_left : nullptr;
        a.lsld = nb;
        a.b = b + r0;
        a.x = x + r0;
        a.ld = ld;
        a.n = h->n;
        a.nrhs = nb;
        a.backward = backward;
        a.xf = xf ? xf + r0 : nullptr;
        a.grad_val = grad;
        a.grad_accumulate = r0 > 0;
        a.ticket = h->d_ticket;
        a.err = h->d_err;
        a.wait = h->wait;
        a.stuck_row = h->stuck_row;
        const bool prof = h->profiling && r0 == 0;
        if (prof)
            CAPSP_CUDA(cudaEventRecord(h->ev_k0, st));
        // default launch shape of the column path (measured on GB300, one warp
        // per column): three blocks per SM.  Narrow levels take 128-thread
        // blocks, except a single right-hand side with the fused gradient,
        // whose longer per-column work wants 256 (grad_1m transpose + grad:
        // 1.69 -> 1.53 ms at 1 RHS, 4.26 -> 4.09 ms at 16 RHS, against two
        // blocks of 256; CSC forward 2.01 -> 1.87 ms).  Wide levels take
        // 256-thread blocks (wide_4m CSC forward 4.94 -> 4.11 ms, transpose
        // with 4 RHS 3.98 -> 3.59 ms, against every resident warp).
        const bool cnarrow = h->col_narrow[backward];
        const int cblock = tn.dflt ? (cnarrow && (nb > 1 || grad == nullptr) ? 128 : 256) : tn.block;
        const int cbps = tn.dflt ? 3 : tn.bps;
        CAPSP_CUDA(launch_col_solve<T>(a, cblock, cbps, h->num_sms, st));
        if (prof)
            CAPSP_CUDA(cudaEventRecord(h->ev_k1, st));
    }
    return CAPSP_OK;
}

// grad[k] = -sum_r y[row(k), r] * x[col(k), r] over the stored entries, in
// chunks of 32 right-hand sides (a CSC handle stores (col, row idx[k]), so y
// and x swap roles); the first chunk overwrites grad, later ones subtract
template <typename T>
static capsp_status_t enqueue_grad(capsp_handle_t h, const T *y, const T *x, T *grad, int nrhs, int64_t ld,
                                   cudaStream_t st)
{
    const bool csr = h->format == CAPSP_FMT_CSR;
    for (int r0 = 0; r0 < nrhs; r0 += 32) {
        const int nb = nrhs - r0 < 32 ? nrhs - r0 : 32;
        CAPSP_CUDA(launch_grad_val<T>(h->d_ptr, h->d_idx, csr ? y + r0 : x + r0, csr ? x + r0 : y + r0, grad, h->n,
                                      nb, ld, r0 > 0, st));
    }
    return CAPSP_OK;
}

template <typename T>
static capsp_status_t enqueue_op(capsp_handle_t h, Op op, const T *in, T *out, const T *xf, T *grad,
                                 int nrhs, int64_t ld, const Tuning &tn, cudaStream_t st)
{
    if (column_driven(h, op)) {
        // CSC solve (forward for lower) or CSR transpose (backward for lower),
        // with the gradient fused into the CSR transpose
        const int backward = op != kOpSolve ? (h->uplo == CAPSP_LOWER) : (h->uplo == CAPSP_UPPER);
        return enqueue_cols<T>(h, in, out, nrhs, ld, backward, xf, grad, tn, st);
    }
    CAPSP_TRY(enqueue_rows<T>(h, view_of(h, op), in, out, nrhs, ld, tn, st));
    if (op == kOpTransposeGrad)
        CAPSP_TRY(enqueue_grad<T>(h, out, xf, grad, nrhs, ld, st));
    return CAPSP_OK;
}

static capsp_status_t check_vec_args(capsp_handle_t h, const void *a, const void *b, int nrhs, int64_t ld)
{
    if (!h)
        return fail(CAPSP_ERR_INVALID, "handle is NULL");
    if (!a || !b)
        return fail(CAPSP_ERR_INVALID, "vector pointers must be non-NULL");
    if (nrhs < 1 || ld < nrhs)
        return fail(CAPSP_ERR_INVALID, "need nrhs >= 1 and ld >= nrhs (got %d, %lld)", nrhs, (long long)ld);
    if (a == b)
        return fail(CAPSP_ERR_INVALID, "input and output must not alias");
    return CAPSP_OK;
}

static capsp_status_t dispatch(capsp_handle_t h, Op op, const void *in, void *out, const void *xf,
                               void *grad, int nrhs, int64_t ld, cudaStream_t st)
{
    const Tuning tn = current_tuning(h, op, nrhs);
    if (h->dtype == CAPSP_R_64F)
        return enqueue_op<double>(h, op, (const double *)in, (double *)out, (const double *)xf,
                                  (double *)grad, nrhs, ld, tn, st);
    return enqueue_op<float>(h, op, (const float *)in, (float *)out, (const float *)xf, (float *)grad,
                             nrhs, ld, tn, st);
}

extern "C" capsp_status_t capsp_solve(capsp_handle_t h, const void *b, void *x, int nrhs, int64_t ld,
                                      void *stream)
{
    CAPSP_TRY(check_vec_args(h, b, x, nrhs, ld));
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    return dispatch(h, kOpSolve, b, x, nullptr, nullptr, nrhs, ld, (cudaStream_t)stream);
}

extern "C" capsp_status_t capsp_solve_transpose(capsp_handle_t h, const void *gv, void *y, int nrhs,
                                                int64_t ld, void *stream)
{
    CAPSP_TRY(check_vec_args(h, gv, y, nrhs, ld));
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    return dispatch(h, kOpTranspose, gv, y, nullptr, nullptr, nrhs, ld, (cudaStream_t)stream);
}

extern "C" capsp_status_t capsp_solve_transpose_grad(capsp_handle_t h, const void *gv, const void *x,
                                                     void *y, void *grad_val, int nrhs, int64_t ld,
                                                     void *stream)
{
    CAPSP_TRY(check_vec_args(h, gv, y, nrhs, ld));
    if (!x || !grad_val)
        return fail(CAPSP_ERR_INVALID, "x and grad_val must be non-NULL");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    return dispatch(h, kOpTransposeGrad, gv, y, x, grad_val, nrhs, ld, (cudaStream_t)stream);
}

extern "C" capsp_status_t capsp_grad_val(capsp_handle_t h, const void *y, const void *x, void *grad_val,
                                         int nrhs, int64_t ld, void *stream)
{
    CAPSP_TRY(check_vec_args(h, y, x, nrhs, ld));
    if (!grad_val)
        return fail(CAPSP_ERR_INVALID, "grad_val must be non-NULL");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    cudaStream_t st = (cudaStream_t)stream;
    if (h->dtype == CAPSP_R_64F)
        return enqueue_grad<double>(h, (const double *)y, (const double *)x, (double *)grad_val, nrhs, ld, st);
    return enqueue_grad<float>(h, (const float *)y, (const float *)x, (float *)grad_val, nrhs, ld, st);
}

// allocate every lazily-built product an operation with nrhs right-hand sides needs
static capsp_status_t prepare(capsp_handle_t h, int nrhs, Op op)
{
    if (column_driven(h, op)) {
        const int backward = op != kOpSolve ? (h->uplo == CAPSP_LOWER) : (h->uplo == CAPSP_UPPER);
        CAPSP_TRY(ensure_column_order(h, backward));
        return ensure_column_scratch(h, nrhs);
    }
    const int v = view_of(h, op);
    if (view_level(h, v)) {
        CAPSP_TRY(build_view(h, v));
        CAPSP_TRY(ensure_xp(h, nrhs));
    }
    const Tuning tn = current_tuning(h, op, nrhs);
    if (tn.kind == kRowMix || tn.kind < 0) {
        MixTable *mt = nullptr;
        for (int r0 = 0; r0 < nrhs; r0 += 32) {
            const int nb = nrhs - r0 < 32 ? nrhs - r0 : 32;
            CAPSP_TRY(ensure_mix(h, v, group_rows_for(nb), tn.border, &mt));
        }
    }
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_reserve(capsp_handle_t h, int max_nrhs)
{
    if (!h || max_nrhs < 1)
        return fail(CAPSP_ERR_INVALID, "need a handle and max_nrhs >= 1");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    CAPSP_TRY(prepare(h, max_nrhs, kOpSolve));
    CAPSP_TRY(prepare(h, max_nrhs, kOpTranspose));
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_status_sync(capsp_handle_t h, void *stream)
{
    if (!h)
        return fail(CAPSP_ERR_INVALID, "handle is NULL");
    DeviceGuard g(h->device);
    CAPSP_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    int err[4] = {0, 0, 0, 0};
    CAPSP_CUDA(cudaMemcpy(err, h->d_err, sizeof(err), cudaMemcpyDeviceToHost));
    if (err[kErrStatus] == kStatusTimeout)
        return fail(CAPSP_ERR_TIMEOUT,
                    "dependency wait ran out of its budget (row/column %d waiting on %d); the "
                    "affected results are NaN",
                    err[kErrRow], err[kErrWaitedOn]);
    if (err[kErrStatus] != 0)
        return fail(CAPSP_ERR_CUDA, "device reported status %d", err[kErrStatus]);
    return CAPSP_OK;
}

// Device address, on `device`, of page-locked host memory (nullptr for
// pageable or device memory, and for memory page-locked in another device's
// context, which need not be mapped for this one).
static void *pinned_alias(const void *p, int device)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || at.device != device)
        return nullptr;
    return at.devicePointer;
}

// cuStreamWaitValue32 / cuStreamWriteValue32 from the driver, or nullptr
// where the driver has no stream memory operations (then capsp_solve_host
// uploads b before the solve and copies x after it)
typedef int (*StreamValue32Fn)(cudaStream_t, unsigned long long, unsigned int, unsigned int);
static std::atomic<bool> g_stream_value_failed{false};
static StreamValue32Fn driver_stream_value32(const char *name)
{
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return reinterpret_cast<StreamValue32Fn>(p);
}
static StreamValue32Fn wait_value32()
{
    static const StreamValue32Fn fn = driver_stream_value32("cuStreamWaitValue32");
    return g_stream_value_failed.load() ? nullptr : fn;
}
static StreamValue32Fn write_value32()
{
    static const StreamValue32Fn fn = driver_stream_value32("cuStreamWriteValue32");
    return g_stream_value_failed.load() ? nullptr : fn;
}

// Highest b segment (segments of b0 (2^k - 1) .. b0 (2^(k+1) - 1) rows) among
// the rows of every 32 schedule positions of view v; built once per handle
static capsp_status_t ensure_b_groups(capsp_handle_t h, int v, long long b0)
{
    RowView &rv = h->view[v];
    if (rv.d_group_seg != nullptr && rv.group_seg_b0 == b0)
        return CAPSP_OK;
    const int n = h->n, ng = (n + 31) / 32;
    std::vector<int> perm((size_t)n);
    CAPSP_CUDA(cudaMemcpy(perm.data(), rv.d_perm, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
    std::vector<unsigned char> grp((size_t)ng, 0);
    for (int p = 0; p < n; ++p) {
        unsigned long long q = (unsigned long long)(perm[(size_t)p] / b0) + 1ull;
        unsigned char k = 0;
        while (q > 1ull) {
            q >>= 1;
            ++k;
        }
        if (k > grp[(size_t)p >> 5])
            grp[(size_t)p >> 5] = k;
    }
    if (rv.d_group_seg == nullptr)
        CAPSP_CUDA(cudaMalloc(&rv.d_group_seg, (size_t)ng));
    CAPSP_CUDA(cudaMemcpy(rv.d_group_seg, grp.data(), (size_t)ng, cudaMemcpyHostToDevice));
    rv.group_seg_b0 = b0;
    return CAPSP_OK;
}

// Copies of x that overlap the solve: rows finish roughly in index order on
// banded matrices (wide_4m: with 32 segments of rows, segment s is complete
// at about 0.1 + 0.9 s/32 of the level chain), so each segment goes to the
// host as soon as the kernel has counted all its rows.  Segments of at least
// 64k rows, at most 32 of them.
constexpr int kMaxSegments = 32;
constexpr int kSegmentRowsMin = 65536;
constexpr unsigned kWaitValueGeq = 0u;   // CU_STREAM_WAIT_VALUE_GEQ
constexpr unsigned kWriteValueFenced = 0u; // CU_STREAM_WRITE_VALUE_DEFAULT: prior copies visible first

extern "C" capsp_status_t capsp_solve_host(capsp_handle_t h, const void *b_host, void *x_host, int nrhs)
{
    CAPSP_TRY(check_vec_args(h, b_host, x_host, nrhs, nrhs));
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    if (!h->stage_stream)
        CAPSP_CUDA(cudaStreamCreateWithFlags(&h->stage_stream, cudaStreamNonBlocking));
    const size_t bytes = h->vbytes * (size_t)h->n * (size_t)nrhs;
    if (h->stage_bytes < 2 * bytes) {
        cudaFree(h->d_stage);
        h->d_stage = nullptr;
        h->stage_bytes = 0;
        CAPSP_CUDA(cudaMalloc(&h->d_stage, 2 * bytes));
        h->stage_bytes = 2 * bytes;
    }
    char *db = (char *)h->d_stage, *dx = db + bytes;
    cudaStream_t st = h->stage_stream;
    const int v = view_of(h, kOpSolve);
    const long long nseg_want = ((long long)h->n + kSegmentRowsMin - 1) / kSegmentRowsMin;
    const Tuning tn = current_tuning(h, kOpSolve, nrhs);
    const bool progressive = !column_driven(h, kOpSolve) && view_level(h, v) && nseg_want >= 2 &&
                             row_hostio_supported(tn.kind < 0 ? kRowWrtFst : tn.kind, tn.R, nrhs) &&
                             wait_value32() != nullptr && pinned_alias(x_host, h->device) != nullptr;
    if (!progressive) {
        // Copies before and after the solve.  A page-locked b is read in place
        // on the level schedule: the row kernel reads each b element once, at
        // row set-up, over the coherent CPU-GPU link, so the H2D copy
        // disappears.  x stays staged: the rows finish scattered over x, and
        // scattered stores to host memory were slower than one D2H copy
        // (wide_4m: 1.49 ms).  Levels of 32k rows and more keep the GPU busy
        // without waiting, and then a single right-hand side, 8 bytes per
        // scattered read over the link, costs more than the copy (2,048
        // systems with 93k rows per level: 5.66 ms in place, 4.80 ms copied;
        // with 4 right-hand sides, 32 bytes per read, 8.97 ms in place, 11.2
        // copied).
        void *b_in_place =
            (!column_driven(h, kOpSolve) && view_level(h, v) && !(wide_levels(h, v) && nrhs == 1))
                ? pinned_alias(b_host, h->device)
                : nullptr;
        if (b_in_place) {
            CAPSP_TRY(dispatch(h, kOpSolve, b_in_place, dx, nullptr, nullptr, nrhs, nrhs, st));
        } else {
            CAPSP_CUDA(cudaMemcpyAsync(db, b_host, bytes, cudaMemcpyHostToDevice, st));
            CAPSP_TRY(dispatch(h, kOpSolve, db, dx, nullptr, nullptr, nrhs, nrhs, st));
        }
        CAPSP_CUDA(cudaMemcpyAsync(x_host, dx, bytes, cudaMemcpyDeviceToHost, st));
        return capsp_status_sync(h, st);
    }
    if (!h->copy_stream) {
        CAPSP_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        CAPSP_CUDA(cudaStreamCreateWithFlags(&h->upload_stream, cudaStreamNonBlocking));
    }
    if (!h->ev_seg0) {
        CAPSP_CUDA(cudaEventCreateWithFlags(&h->ev_seg0, cudaEventDisableTiming));
        CAPSP_CUDA(cudaEventCreateWithFlags(&h->ev_seg1, cudaEventDisableTiming));
        CAPSP_CUDA(cudaEventCreateWithFlags(&h->ev_up, cudaEventDisableTiming));
    }
    if (!h->d_seg)
        CAPSP_CUDA(cudaMalloc(&h->d_seg, sizeof(int) * 2 * kMaxSegments));
    int *d_count = h->d_seg, *d_bready = h->d_seg + kMaxSegments;
    const int nseg0 = nseg_want < kMaxSegments ? (int)nseg_want : kMaxSegments;
    // a multiple of 16 rows: no 128-byte line of b or x spans two segments
    const int seg_rows = (int)((((long long)h->n + nseg0 - 1) / nseg0 + 15) / 16 * 16);
    const int nseg = (int)(((long long)h->n + seg_rows - 1) / seg_rows);
    const size_t row_bytes = h->vbytes * (size_t)nrhs;
    CAPSP_CUDA(cudaMemsetAsync(h->d_seg, 0, sizeof(int) * 2 * kMaxSegments, st));
    CAPSP_CUDA(cudaEventRecord(h->ev_seg0, st));
    // b: a page-locked b goes up segment by segment on its own stream, each
    // segment followed by its flag, and every row's set-up waits for its
    // segment's flag, so the upload overlaps the solve (reading b in place
    // over the link instead slowed the wide_4m kernel from 0.73 to 0.92 ms
    // when x was coming back at the same time).  The upload is enqueued
    // before the solve, so it never queues behind it; its segments double
    // from n/256 rows, so the first lands within a microsecond and the host
    // issues few calls before the launch.
    const StreamValue32Fn write_fn = write_value32(), wait_fn = wait_value32();
    const bool side_upload = pinned_alias(b_host, h->device) != nullptr && write_fn != nullptr;
    bool b_flags = side_upload;
    const long long b0 = ((h->n / 256 > 1024 ? h->n / 256 : 1024) + 15) / 16 * 16;
    if (side_upload) {
        CAPSP_TRY(ensure_b_groups(h, v, b0));
        CAPSP_CUDA(cudaStreamWaitEvent(h->upload_stream, h->ev_seg0, 0));
        for (int sg = 0; b0 * ((1LL << sg) - 1) < h->n; ++sg) {
            const long long r0 = b0 * ((1LL << sg) - 1);
            const long long r1 = b0 * ((1LL << (sg + 1)) - 1) < h->n ? b0 * ((1LL << (sg + 1)) - 1) : h->n;
            CAPSP_CUDA(cudaMemcpyAsync(db + (size_t)r0 * row_bytes, (const char *)b_host + (size_t)r0 * row_bytes,
                                       (size_t)(r1 - r0) * row_bytes, cudaMemcpyHostToDevice, h->upload_stream));
            if (b_flags && write_fn(h->upload_stream, (unsigned long long)(uintptr_t)(d_bready + sg), 1u,
                                    kWriteValueFenced) != 0) {
                g_stream_value_failed.store(true);
                b_flags = false;  // the solve waits for the whole upload instead
            }
        }
        CAPSP_CUDA(cudaEventRecord(h->ev_up, h->upload_stream));
        if (!b_flags)
            CAPSP_CUDA(cudaStreamWaitEvent(st, h->ev_up, 0));
    } else {
        CAPSP_CUDA(cudaMemcpyAsync(db, b_host, bytes, cudaMemcpyHostToDevice, st));
    }
    h->seg_req = d_count;
    h->bready_req = b_flags ? d_bready : nullptr;
    h->seg_req_rows = seg_rows;
    const capsp_status_t sd = dispatch(h, kOpSolve, db, dx, nullptr, nullptr, nrhs, nrhs, st);
    h->seg_req = nullptr;
    h->bready_req = nullptr;
    if (side_upload)
        CAPSP_CUDA(cudaStreamWaitEvent(st, h->ev_up, 0));  // db is free again once st is done
    CAPSP_TRY(sd);
    // once the solve has ended every counter is past its target, whatever it
    // counted: no wait below can outlive the kernel.  This is enqueued on the
    // solve's stream before any wait, so it cannot queue behind one.
    CAPSP_CUDA(cudaMemsetAsync(d_count, 0x3F, sizeof(int) * (size_t)nseg, st));
    CAPSP_CUDA(cudaStreamWaitEvent(h->copy_stream, h->ev_seg0, 0));
    bool waits = true;
    for (int sg = 0; sg < nseg; ++sg) {
        const long long r0 = (long long)sg * seg_rows;
        const long long r1 = r0 + seg_rows < h->n ? r0 + seg_rows : h->n;
        if (waits && (wait_fn == nullptr || wait_fn(h->copy_stream, (unsigned long long)(uintptr_t)(d_count + sg),
                                                    (unsigned)(r1 - r0), kWaitValueGeq) != 0)) {
            // no stream memory operations after all: the other copies follow the solve
            g_stream_value_failed.store(true);
            waits = false;
            CAPSP_CUDA(cudaEventRecord(h->ev_seg1, st));
            CAPSP_CUDA(cudaStreamWaitEvent(h->copy_stream, h->ev_seg1, 0));
        }
        CAPSP_CUDA(cudaMemcpyAsync((char *)x_host + (size_t)r0 * row_bytes, dx + (size_t)r0 * row_bytes,
                                   (size_t)(r1 - r0) * row_bytes, cudaMemcpyDeviceToHost, h->copy_stream));
    }
    CAPSP_CUDA(cudaEventRecord(h->ev_seg1, h->copy_stream));
    CAPSP_CUDA(cudaStreamWaitEvent(st, h->ev_seg1, 0));
    return capsp_status_sync(h, st);
}

// ---------------------------------------------------------------------------
// autotuner
// ---------------------------------------------------------------------------

extern "C" capsp_status_t capsp_autotune(capsp_handle_t h, const void *b, void *x, int nrhs, int64_t ld,
                                         void *stream, float *best_ms)
{
    CAPSP_TRY(check_vec_args(h, b, x, nrhs, ld));
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<Tuning> cands;
    const bool row_path = !column_driven(h, kOpSolve);
    const int v = view_of(h, kOpSolve);
    const int blocks[3] = {64, 128, 256};
    if (row_path) {
        const int rs[2] = {1, 2};
        // the row path of a CAPSP_ALG_SYNCFREE_CSC handle chooses as AUTO does
        const int alg = h->alg == CAPSP_ALG_SYNCFREE_CSC ? CAPSP_ALG_AUTO : h->alg;
        const bool allow_thread = alg == CAPSP_ALG_AUTO || alg == CAPSP_ALG_WRTFST;
        const bool allow_mix = alg == CAPSP_ALG_AUTO || alg == CAPSP_ALG_MIX;
        const int bpss[3] = {1, 2, 0};
        if (allow_thread) {
            // the default launch shape first: the search never ends worse
            cands.push_back({kRowWrtFst, 1, 256, 1, h->border, true});
        }
        if (allow_thread)
            for (int bl : blocks)
                for (int r : rs)
                    for (int bp : bpss)
                        cands.push_back({kRowWrtFst, r, bl, bp, h->border});
        if (h->alg == CAPSP_ALG_TWOPART)
            for (int bl : blocks)
                for (int r : rs)
                    for (int bp : bpss)
                        cands.push_back({kRowTwoPart, r, bl, bp, h->border});
        if (allow_mix) {
            const int borders[4] = {4, 8, 16, 32};
            for (int bl : blocks)
                for (int bo : borders)
                    cands.push_back({kRowMix, 1, bl, 0, bo});
        }
    } else {
        cands.push_back({kRowWrtFst, 1, 256, 0, h->border, true});  // the default shape
        for (int bl : blocks)
            for (int bp : {0, 2, 3, 4})
                cands.push_back({kRowWrtFst, 1, bl, bp, h->border});
    }
    cudaEvent_t e0, e1;
    CAPSP_CUDA(cudaEventCreate(&e0));
    CAPSP_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    Tuning best_t = cands[0];
    capsp_status_t st_all = CAPSP_OK;
    for (const Tuning &tn : cands) {
        // build tables / scratch outside the timed region
        if (row_path && tn.kind == kRowMix) {
            MixTable *mt = nullptr;
            for (int r0 = 0; r0 < nrhs && st_all == CAPSP_OK; r0 += 32) {
                const int nb = nrhs - r0 < 32 ? nrhs - r0 : 32;
                st_all = ensure_mix(h, v, group_rows_for(nb), tn.border, &mt);
            }
        }
        if (st_all != CAPSP_OK)
            break;
        float tot = 0.f;
        for (int rep = 0; rep < 4 && st_all == CAPSP_OK; ++rep) {
            cudaEventRecord(e0, st);
            if (h->dtype == CAPSP_R_64F)
                st_all = enqueue_op<double>(h, kOpSolve, (const double *)b, (double *)x, nullptr, nullptr,
                                            nrhs, ld, tn, st);
            else
                st_all = enqueue_op<float>(h, kOpSolve, (const float *)b, (float *)x, nullptr, nullptr,
                                           nrhs, ld, tn, st);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                st_all = fail(CAPSP_ERR_CUDA, "autotune launch failed");
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0)
                tot += ms;
        }
        if (st_all != CAPSP_OK)
            break;
        const float avg = tot / 3.f;
        if (avg < best) {
            best = avg;
            best_t = tn;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CAPSP_TRY(st_all);
    CAPSP_TRY(capsp_status_sync(h, stream));
    h->tuned[nrhs] = best_t;
    h->graphs.invalidate();
    if (best_ms)
        *best_ms = best;
    return CAPSP_OK;
}

// ---------------------------------------------------------------------------
// CUDA graph replay
// ---------------------------------------------------------------------------

extern "C" capsp_status_t capsp_graph_solve(capsp_handle_t h, const void *b, void *x, int nrhs, int64_t ld,
                                            void *stream)
{
    CAPSP_TRY(check_vec_args(h, b, x, nrhs, ld));
    if (!stream)
        return fail(CAPSP_ERR_INVALID,
                    "graph replay needs an explicit (non-default) stream to capture on");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    cudaStream_t st = (cudaStream_t)stream;
    // scratch first: a reallocation here invalidates the cache, so the key
    // below carries the generation the capture will be valid for
    CAPSP_TRY(prepare(h, nrhs, kOpSolve));
    const Tuning tn = current_tuning(h, kOpSolve, nrhs);
    const GraphKey key = {b, x, nrhs, ld, stream, tn.kind, tn.R, tn.block, tn.bps, tn.border, tn.dflt ? 1 : 0,
                          h->graphs.generation()};
    cudaGraphExec_t *exec_p = h->graphs.find(key);
    if (!exec_p) {
        CAPSP_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        capsp_status_t s = dispatch(h, kOpSolve, b, x, nullptr, nullptr, nrhs, ld, st);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(st, &graph);
        if (s != CAPSP_OK) {
            if (graph)
                cudaGraphDestroy(graph);
            return s;
        }
        if (e != cudaSuccess)
            return fail(CAPSP_ERR_CUDA, "stream capture failed: %s", cudaGetErrorString(e));
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess)
            return fail(CAPSP_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
        // the capture must not have changed what it depends on (prepare() ran first)
        if (!h->graphs.put(key, exec))
            return fail(CAPSP_ERR_CUDA, "scratch changed during graph capture");
        exec_p = h->graphs.find(key);
    }
    CAPSP_CUDA(cudaGraphLaunch(*exec_p, st));
    return CAPSP_OK;
}

// ---------------------------------------------------------------------------
// kernel timing
// ---------------------------------------------------------------------------

extern "C" capsp_status_t capsp_set_profiling(capsp_handle_t h, int enable)
{
    if (!h)
        return fail(CAPSP_ERR_INVALID, "handle is NULL");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    DeviceGuard g(h->device);
    if (enable && !h->ev_k0) {
        CAPSP_CUDA(cudaEventCreate(&h->ev_k0));
        CAPSP_CUDA(cudaEventCreate(&h->ev_k1));
    }
    if (h->profiling != (enable != 0))
        h->graphs.invalidate();  // captures record the timing events only while profiling
    h->profiling = enable != 0;
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_debug_trace(capsp_handle_t h, void *row_times_ns)
{
    if (!h)
        return fail(CAPSP_ERR_INVALID, "handle is NULL");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    h->trace = (unsigned long long *)row_times_ns;
    h->graphs.invalidate();
    return CAPSP_OK;
}

extern "C" capsp_status_t capsp_last_kernel_ms(capsp_handle_t h, float *ms)
{
    if (!h || !ms)
        return fail(CAPSP_ERR_INVALID, "handle and ms must be non-NULL");
    if (!h->ev_k0)
        return fail(CAPSP_ERR_INVALID, "profiling was never enabled on this handle");
    DeviceGuard g(h->device);
    CAPSP_CUDA(cudaEventSynchronize(h->ev_k1));
    CAPSP_CUDA(cudaEventElapsedTime(ms, h->ev_k0, h->ev_k1));
    return CAPSP_OK;
}

// ---------------------------------------------------------------------------
// info
// ---------------------------------------------------------------------------

extern "C" capsp_status_t capsp_get_info(capsp_handle_t h, capsp_info_t *info)
{
    if (!h || !info)
        return fail(CAPSP_ERR_INVALID, "handle and info must be non-NULL");
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    memset(info, 0, sizeof(*info));
    info->n = h->n;
    info->nnz = h->nnz;
    info->dtype = h->dtype;
    info->format = h->format;
    info->uplo = h->uplo;
    info->analyse_ms = h->analyse_ms;
    info->num_sms = h->num_sms;
    Tuning tn = current_tuning(h, kOpSolve, 1);
    info->rows_per_thread = tn.R;
    int blk = tn.block, bps = tn.bps;
    const int v = view_of(h, kOpSolve);
    if (!column_driven(h, kOpSolve))
        row_shape(h, v, tn, 1, &blk, &bps);
    info->block_threads = blk;
    info->blocks_per_sm = bps;
    info->schedule = view_level(h, v) ? CAPSP_SCHED_LEVEL : CAPSP_SCHED_NATURAL;
    info->levels = h->view[v].levels;
    info->cached_graphs = (int)h->graphs.size();
    if (column_driven(h, kOpSolve)) {
        info->algorithm = CAPSP_ALG_SYNCFREE_CSC;
    } else {
        int alg = h->alg == CAPSP_ALG_SYNCFREE_CSC ? CAPSP_ALG_AUTO : h->alg;
        auto mit = h->mix.find((32 * 2 + (view_level(h, v) ? 1 : 0)) * 2 + v);
        if (mit != h->mix.end() && mit->second.d) {
            info->mix_len = mit->second.len;
            info->warp_occupy = mit->second.wo;
            info->element_occupy = mit->second.eo;
            if (alg == CAPSP_ALG_AUTO)
                alg = mit->second.wo > 0.0 ? CAPSP_ALG_MIX : CAPSP_ALG_WRTFST;
        }
        info->algorithm = alg;
    }
    return CAPSP_OK;
}

// ---------------------------------------------------------------------------
// per-hop latency probe
// ---------------------------------------------------------------------------

extern "C" capsp_status_t capsp_hop_latency(int n, int stride, int dtype, float *ns_per_hop)
{
    if (n < 2 || stride < 1 || stride >= n || !ns_per_hop)
        return fail(CAPSP_ERR_INVALID, "need n >= 2, 1 <= stride < n and an output pointer");
    if (dtype != CAPSP_R_64F && dtype != CAPSP_R_32F)
        return fail(CAPSP_ERR_INVALID, "unknown dtype %d", dtype);
    // row i: x_i = (1 + 0.5 x_{i-stride}) / 1  ->  chain of n/stride hops
    std::vector<int> ptr((size_t)n + 1), idx;
    std::vector<double> v64;
    idx.reserve((size_t)2 * n);
    v64.reserve((size_t)2 * n);
    ptr[0] = 0;
    for (int i = 0; i < n; ++i) {
        if (i >= stride) {
            idx.push_back(i - stride);
            v64.push_back(-0.5);
        }
        idx.push_back(i);
        v64.push_back(1.0);
        ptr[i + 1] = (int)idx.size();
    }
    const int nnz = (int)idx.size();
    std::vector<float> v32(v64.begin(), v64.end());
    const void *val = dtype == CAPSP_R_64F ? (const void *)v64.data() : (const void *)v32.data();
    capsp_handle_t h = nullptr;
    CAPSP_TRY(capsp_analyse(n, nnz, ptr.data(), idx.data(), val, dtype, CAPSP_FMT_CSR, CAPSP_LOWER, 0, &h));
    const size_t vb = dtype == CAPSP_R_64F ? 8 : 4;
    void *d_b = nullptr, *d_x = nullptr;
    std::vector<double> ones64((size_t)n, 1.0);
    std::vector<float> ones32((size_t)n, 1.0f);
    cudaError_t e = cudaMalloc(&d_b, vb * n);
    if (e == cudaSuccess)
        e = cudaMalloc(&d_x, vb * n);
    if (e == cudaSuccess)
        e = cudaMemcpy(d_b, dtype == CAPSP_R_64F ? (const void *)ones64.data() : (const void *)ones32.data(),
                       vb * n, cudaMemcpyHostToDevice);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float best = 1e30f;
    capsp_status_t st = CAPSP_OK;
    if (e == cudaSuccess)
        e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    for (int rep = 0; rep < 5 && e == cudaSuccess && st == CAPSP_OK; ++rep) {
        cudaEventRecord(e0, 0);
        st = capsp_solve(h, d_b, d_x, 1, 1, 0);
        cudaEventRecord(e1, 0);
        e = cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best)
            best = ms;
    }
    if (st == CAPSP_OK && e == cudaSuccess)
        st = capsp_status_sync(h, 0);
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    cudaFree(d_b);
    cudaFree(d_x);
    capsp_destroy(h);
    if (e != cudaSuccess)
        return fail(CAPSP_ERR_CUDA, "hop latency probe failed: %s", cudaGetErrorString(e));
    CAPSP_TRY(st);
    const double hops = (double)(n - 1) / stride;
    *ns_per_hop = (float)(best * 1e6 / hops);
    return CAPSP_OK;
}

// ---------------------------------------------------------------------------
// no-allocation column solve (static device scratch)
// ---------------------------------------------------------------------------
//
// The scratch of the column-driven solve lives in one file-scope device array
// instead of handle allocations: a 256-byte header (ticket at byte 0, the
// four-int error word at byte 16, the first malformed column at byte 32),
// then 1/diag and left_sum (double[kNoallocMaxN] each) and the in-degree and
// arrival counters (int[kNoallocMaxN] each): 24 bytes per row, 1.5 MiB in all.
// Every part that must start at zero (ticket, error word, left_sum, both
// counter arrays) or at "no bad row" (0x7F7F7F7F) is reset on the stream at
// the start of every call, so the caller prepares nothing.

namespace {

constexpr int kNoallocMaxN = 65536;
constexpr size_t kNoallocHeader = 256;
constexpr size_t kNoallocInv = kNoallocHeader;
constexpr size_t kNoallocLeft = kNoallocInv + sizeof(double) * kNoallocMaxN;
constexpr size_t kNoallocIndeg = kNoallocLeft + sizeof(double) * kNoallocMaxN;
constexpr size_t kNoallocArrived = kNoallocIndeg + sizeof(int) * kNoallocMaxN;
constexpr size_t kNoallocBytes = kNoallocArrived + sizeof(int) * kNoallocMaxN;

std::mutex g_noalloc_mu;

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

extern "C" capsp_status_t capsp_csc_solve_noalloc_f64(const int *colptr, const int *rowidx,
                                                      const double *val, int n, int nnz,
                                                      const double *b, double *x, void *stream)
{
    if (!colptr || !rowidx || !val || !b || !x)
        return fail(CAPSP_ERR_INVALID, "all array pointers must be non-NULL");
    if (n < 1 || nnz < n)
        return fail(CAPSP_ERR_INVALID, "need n >= 1 and nnz >= n (got n=%d nnz=%d)", n, nnz);
    if (n > kNoallocMaxN)
        return fail(CAPSP_ERR_INVALID,
                    "n=%d exceeds the static scratch of capsp_csc_solve_noalloc_f64 (at most %d rows)", n,
                    kNoallocMaxN);
    if ((const void *)b == (const void *)x)
        return fail(CAPSP_ERR_INVALID, "b and x must not alias");
    // one call at a time in this process: every call uses the same scratch
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    int dev = 0, sms = 0;
    CAPSP_CUDA(cudaGetDevice(&dev));
    // The scratch's device address, resolved with the caller's device current
    // on every call: g_noalloc_scratch names a host-side stand-in in host
    // code, and the address can change when the caller resets the device
    // (the module is loaded again into the new context).  The lookup
    // allocates nothing and costs far less than the call's two synchronisations.
    void *scratch = nullptr;
    {
        const cudaError_t e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);
        if (e != cudaSuccess || !scratch)
            return fail(CAPSP_ERR_CUDA, "cudaGetSymbolAddress of the static scratch failed: %s",
                        cudaGetErrorString(e));
    }
    CAPSP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    unsigned char *base = static_cast<unsigned char *>(scratch);
    unsigned *ticket = reinterpret_cast<unsigned *>(base);
    int *err = reinterpret_cast<int *>(base + 16);
    int *bad = reinterpret_cast<int *>(base + 32);
    double *inv = reinterpret_cast<double *>(base + kNoallocInv);
    double *left = reinterpret_cast<double *>(base + kNoallocLeft);
    int *indeg = reinterpret_cast<int *>(base + kNoallocIndeg);
    int *arrived = reinterpret_cast<int *>(base + kNoallocArrived);
    cudaStream_t st = (cudaStream_t)stream;
    const size_t nn = (size_t)n;

    // structure first: a malformed column must not reach the solve
    CAPSP_CUDA(cudaMemsetAsync(base, 0, 32, st));        // ticket + error word
    CAPSP_CUDA(cudaMemsetAsync(err + 3, 0x7F, sizeof(int), st));
    CAPSP_CUDA(cudaMemsetAsync(bad, 0x7F, sizeof(int), st));
    CAPSP_CUDA(launch_validate(colptr, rowidx, n, nnz, 0, bad, st));
    int h_bad = 0;
    CAPSP_CUDA(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    CAPSP_CUDA(cudaStreamSynchronize(st));
    if (h_bad < n)
        return fail(CAPSP_ERR_INVALID, "column %d is malformed (lower CSC needs the diagonal first and "
                                       "every other row index below it and below n)", h_bad);

    CAPSP_CUDA(cudaMemsetAsync(left, 0, sizeof(double) * nn, st));
    CAPSP_CUDA(cudaMemsetAsync(indeg, 0, sizeof(int) * nn, st));
    CAPSP_CUDA(cudaMemsetAsync(arrived, 0, sizeof(int) * nn, st));
    CAPSP_CUDA(launch_inv_diag<double>(colptr, val, inv, n, 0, err + 3, st));
    CAPSP_CUDA(launch_histogram(rowidx, nnz, indeg, st));
    ColArgs<double> a;
    a.ptr = colptr;
    a.idx = rowidx;
    a.val = val;
    a.inv_diag = inv;
    a.indeg = indeg;
    a.order = nullptr;
    a.slots = nullptr;
    a.arrived = arrived;
    a.left_sum = left;
    a.lsld = 1;
    a.b = b;
    a.x = x;
    a.ld = 1;
    a.n = n;
    a.nrhs = 1;
    a.backward = 0;
    a.xf = nullptr;
    a.grad_val = nullptr;
    a.grad_accumulate = 0;
    a.ticket = ticket;
    a.err = err;
    a.wait = WaitCfg{10000000000ull, 1u << 30, 256u};
    a.stuck_row = -1;
    CAPSP_CUDA(launch_col_solve<double>(a, 256, 0, sms, st));
    int h_err[4] = {0, 0, 0, 0};
    CAPSP_CUDA(cudaMemcpyAsync(h_err, err, sizeof(h_err), cudaMemcpyDeviceToHost, st));
    CAPSP_CUDA(cudaStreamSynchronize(st));
    if (h_err[3] < n)
        return fail(CAPSP_ERR_INVALID, "column %d has a zero or non-finite diagonal", h_err[3]);
    if (h_err[kErrStatus] == kStatusTimeout)
        return fail(CAPSP_ERR_TIMEOUT, "column %d gave up waiting (dependency %d)", h_err[kErrRow],
                    h_err[kErrWaitedOn]);
    if (h_err[kErrStatus] != 0)
        return fail(CAPSP_ERR_CUDA, "device status %d", h_err[kErrStatus]);
    return CAPSP_OK;
}
