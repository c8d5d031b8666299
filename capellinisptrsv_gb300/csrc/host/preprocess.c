/*
 * Host preprocessing for the sync-free triangular solve: structure checks,
 * level statistics, the mix selector table, transposition, the in-degree
 * analyser, b = L*ones and a Matrix Market reader.  Written against the
 * contracts of the reference's host helpers (CUDA/ourWrtFst/read_mtx.h,
 * CUDA/ourWrtFst/tranpose.h, CUDA/mix/tranpose.h) -- see each function.
 */
#include "capsp.h"

#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* dependencies the thread-per-row kernel takes in one pass (kBatch in
 * kernels_row.cuh) */
#define CAPSP_ROW_PASS 8

/* a level this wide keeps the GPU busy without waiting on the dependency
 * chain (the launch-shape rule in capsp_api.cu uses the same width) */
#define CAPSP_WIDE_LEVEL 32768

/* ------------------------------------------------------------------ */
/* small helpers                                                        */
/* ------------------------------------------------------------------ */

/* Stable sort of (col, value) pairs of one row by col; values are opaque
 * blobs of vbytes bytes.  Insertion sort for short rows, merge sort above. */
static void sort_row_pairs_generic(int *col, unsigned char *val, size_t vbytes, int cnt)
{
    if (cnt < 2)
        return;
    if (cnt <= 64) {
        unsigned char tmp[16];
        for (int t = 1; t < cnt; ++t) {
            int c = col[t];
            memcpy(tmp, val + (size_t)t * vbytes, vbytes);
            int u = t - 1;
            while (u >= 0 && col[u] > c) {
                col[u + 1] = col[u];
                memcpy(val + (size_t)(u + 1) * vbytes, val + (size_t)u * vbytes, vbytes);
                --u;
            }
            col[u + 1] = c;
            memcpy(val + (size_t)(u + 1) * vbytes, tmp, vbytes);
        }
        return;
    }
    int *c2 = (int *)malloc(sizeof(int) * (size_t)cnt);
    unsigned char *v2 = (unsigned char *)malloc(vbytes * (size_t)cnt);
    if (!c2 || !v2) { /* fall back to the quadratic path */
        free(c2);
        free(v2);
        for (int t = 1; t < cnt; ++t) {
            unsigned char tmp[16];
            int c = col[t];
            memcpy(tmp, val + (size_t)t * vbytes, vbytes);
            int u = t - 1;
            while (u >= 0 && col[u] > c) {
                col[u + 1] = col[u];
                memcpy(val + (size_t)(u + 1) * vbytes, val + (size_t)u * vbytes, vbytes);
                --u;
            }
            col[u + 1] = c;
            memcpy(val + (size_t)(u + 1) * vbytes, tmp, vbytes);
        }
        return;
    }
    for (int width = 1; width < cnt; width *= 2) {
        for (int lo = 0; lo < cnt; lo += 2 * width) {
            int mid = lo + width < cnt ? lo + width : cnt;
            int hi = lo + 2 * width < cnt ? lo + 2 * width : cnt;
            int a = lo, b = mid, w = lo;
            while (a < mid || b < hi) {
                int take_a = (b >= hi) || (a < mid && col[a] <= col[b]);
                int src = take_a ? a++ : b++;
                c2[w] = col[src];
                memcpy(v2 + (size_t)w * vbytes, val + (size_t)src * vbytes, vbytes);
                ++w;
            }
        }
        memcpy(col, c2, sizeof(int) * (size_t)cnt);
        memcpy(val, v2, vbytes * (size_t)cnt);
    }
    free(c2);
    free(v2);
}

void capsp_exclusive_scan(int *input, int length)
{
    if (length <= 1) {
        if (length == 1)
            input[0] = 0;
        return;
    }
    int running = 0;
    for (int i = 0; i < length; ++i) {
        int v = input[i];
        input[i] = running;
        running += v;
    }
}

/* Selector over `group_rows`-row groups in solve order.  The table lists the
 * first solve-order row of every virtual warp plus a final end entry; its
 * length is returned.  Mirrors matrix_warp4 (CUDA/mix/tranpose.h:1423-1483). */
static int mix_table_impl(int n, const int *rowptr, int upper, int group_rows, int border,
                          int nnz, int *table, double *wo, double *eo)
{
    double row_warp = 0.0, elem_warp = 0.0;
    int k = 1, row = 0;
    table[0] = 0;
    for (int p0 = 0; p0 < n; p0 += group_rows) {
        int p1 = p0 + group_rows < n ? p0 + group_rows : n;
        int elems = upper ? rowptr[n - p0] - rowptr[n - p1] : rowptr[p1] - rowptr[p0];
        double avg = (double)elems / (double)(p1 - p0);
        if (avg >= (double)border) {
            elem_warp += (double)elems;
            row_warp += (double)(p1 - p0);
            for (int t = p0; t < p1; ++t)
                table[k++] = ++row;
        } else {
            row += p1 - p0;
            table[k++] = row;
        }
    }
    *wo = n > 0 ? row_warp / n : 0.0;
    *eo = nnz > 0 ? elem_warp / nnz : 0.0;
    return k;
}

int capsp_mix_table(int n, const int *rowptr, int upper, int group_rows, int border, int *table,
                    double *warp_occupy, double *element_occupy)
{
    double wo = 0.0, eo = 0.0;
    if (n < 0 || group_rows < 1 || !rowptr || !table)
        return 0;
    int len = mix_table_impl(n, rowptr, upper, group_rows, border, rowptr[n] - rowptr[0], table,
                             &wo, &eo);
    if (warp_occupy)
        *warp_occupy = wo;
    if (element_occupy)
        *element_occupy = eo;
    return len;
}

/* Level recurrence of matrix_layer (CUDA/ourWrtFst/tranpose.h:95-117): every
 * row's level is one more than the deepest level among its stored columns,
 * where columns not yet visited (the diagonal itself) count as level 0. */
int capsp_row_levels(int n, const int *rowptr, const int *colidx, int *level, int *level_count)
{
    memset(level, 0, sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (level_count)
        memset(level_count, 0, sizeof(int) * ((size_t)n + 1));
    int deepest = 0;
    for (int row = 0; row < n; ++row) {
        int lv = 0;
        for (int j = rowptr[row]; j < rowptr[row + 1]; ++j) {
            int c = level[colidx[j]] + 1;
            if (c > lv)
                lv = c;
        }
        level[row] = lv;
        if (level_count)
            level_count[lv]++;
        if (lv > deepest)
            deepest = lv;
    }
    return deepest;
}

/* Level schedule of a triangular matrix read row by row (rows of a CSR, or
 * columns of a CSC read as rows of the transpose).  Solve order visits rows
 * 0..n-1 (diagonal last, dependencies on smaller rows) or, with upper != 0,
 * rows n-1..0 (diagonal first, dependencies on larger rows).  Every row gets
 * level 1 + the deepest level among its dependencies, and the levels are laid
 * out one after another, giving order[k] (k-th row to solve) and
 * position[row] = k.  Any order that lists dependencies first keeps the
 * sync-free solve correct.  Inside a level (then solve order):
 *   - the rows of more than CAPSP_ROW_PASS dependencies (more than the row
 *     kernel takes in one pass) come first, by dependency count, most first
 *     (counts of 63 and more share a bucket): a warp's 32 consecutive rows then
 *     need the same number of passes instead of all waiting for the longest
 *     (measured on GB300: 2,048 banded systems with 3-12 dependencies per row,
 *     1.96 -> 1.64 ms; 1M rows with 2-10, 1.38 -> 1.35 ms);
 *   - the other rows follow by the position of their newest dependency (the
 *     last to be published, as a rule): a warp's 32 rows then wait on a few
 *     neighbouring rows of the previous level, published by one or two warps,
 *     so their polls share cache lines instead of reaching 32 unrelated
 *     producers (measured on GB300: wide_4m 0.756 -> 0.742 ms, FP32 0.694 ->
 *     0.671 ms; with the multi-pass rows first instead of the whole level by
 *     count: wide_4m's transpose, 2.4 % of whose rows take two passes, 0.928
 *     -> 0.890 ms, 1M rows with 2-10 dependencies 1.301 -> 1.279 ms, its
 *     transpose 1.352 -> 1.315 ms);
 *   - except in a level of CAPSP_WIDE_LEVEL rows or more that holds a
 *     multi-pass row, where all rows go by dependency count: there no warp
 *     waits on the chain, and rows of equal work finish a warp's passes
 *     together (the newest-dependency order for the single-pass rows cost the
 *     2,048 systems, 93k rows per level, 3 %).
 * level_start (n+2 ints, optional) receives the first position of every level.
 * Returns the number of levels, or -1 on allocation failure. */
int capsp_level_schedule(int n, const int *ptr, const int *idx, int upper, int *order, int *position,
                         int *level_start)
{
    int *lev = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int *cnt = (int *)calloc((size_t)n + 2, sizeof(int));
    if (!lev || !cnt) {
        free(lev);
        free(cnt);
        return -1;
    }
    int deepest = 0;
    for (int p = 0; p < n; ++p) {
        const int i = upper ? n - 1 - p : p;
        const int s = ptr[i] + (upper ? 1 : 0), e = ptr[i + 1] - (upper ? 0 : 1);
        int lv = 1;
        for (int j = s; j < e; ++j) {
            const int q = upper ? n - 1 - idx[j] : idx[j];
            if (lev[q] + 1 > lv)
                lv = lev[q] + 1;
        }
        lev[p] = lv;
        cnt[lv]++;
        if (lv > deepest)
            deepest = lv;
    }
    /* exclusive scan over levels 1..deepest: first position of each level */
    int run = 0, widest = 0;
    for (int l = 0; l <= deepest + 1; ++l) {
        int c = cnt[l];
        if (c > widest)
            widest = c;
        cnt[l] = run;
        run += c;
    }
    if (level_start)
        for (int l = 0; l <= deepest + 1; ++l)
            level_start[l] = cnt[l];
    for (int p = 0; p < n; ++p) {
        const int i = upper ? n - 1 - p : p;
        const int k = cnt[lev[p]]++;
        order[k] = i;
    }
    /* Stable counting sorts inside each level, levels in order (the positions
     * of every earlier level are final when a level's rows are keyed).  A
     * row's newest dependency always lies in the previous level (its deepest
     * dependency sets its level, and positions ascend with the level), so the
     * key of a single-pass level ranges over the previous level's positions. */
    int *tmp = lev; /* the row levels are no longer needed */
    int *hist = (int *)malloc(sizeof(int) * ((size_t)widest + 64 + 1));
    int *key = (int *)malloc(sizeof(int) * (size_t)(widest > 0 ? widest : 1));
    if (!hist || !key) {
        free(hist);
        free(key);
        free(lev);
        free(cnt);
        return -1;
    }
    for (int l = 1; l <= deepest; ++l) {
        /* cnt[l] now holds the end of level l, cnt[l - 1] its start */
        const int a = cnt[l - 1], b = cnt[l];
        if (b - a > 1) {
            /* the rows of a level are scattered over the matrix: a wide
             * level's passes over them run on all host threads */
            int most = 0;
#pragma omp parallel for schedule(static) reduction(max : most) if (b - a >= 2048)
            for (int k = a; k < b; ++k) {
                const int i = order[k];
                const int d = ptr[i + 1] - ptr[i] - 1;
                most = d > most ? d : most;
            }
            int range;
            /* a level of 32k rows or more keeps the GPU busy without waiting:
             * there rows of equal dependency count together finish a warp's
             * passes together */
            const int by_count = most > CAPSP_ROW_PASS && b - a >= CAPSP_WIDE_LEVEL;
            if (l > 1) {
                /* multi-pass rows first, by dependency count (bucket 0: 63+
                 * dependencies), then the single-pass rows by the position
                 * of their newest dependency (buckets 64 ...) */
                const int base = cnt[l - 2];
                range = by_count ? 64 : most > CAPSP_ROW_PASS ? 64 + (a - base) : a - base;
                const int off = most > CAPSP_ROW_PASS ? 64 : 0;
#pragma omp parallel for schedule(static) if (b - a >= 2048)
                for (int k = a; k < b; ++k) {
                    const int i = order[k];
                    const int d = ptr[i + 1] - ptr[i] - 1;
                    if (d > CAPSP_ROW_PASS || by_count) {
                        key[k - a] = 63 - (d < 63 ? d : 63);
                        continue;
                    }
                    const int s = ptr[i] + (upper ? 1 : 0), e = ptr[i + 1] - (upper ? 0 : 1);
                    int newest = base;
                    for (int j = s; j < e; ++j)
                        if (position[idx[j]] > newest)
                            newest = position[idx[j]];
                    key[k - a] = off + newest - base;
                }
            } else {
                range = 0; /* level 1: no dependencies, solve order */
            }
            if (range > 0) {
                memset(hist, 0, sizeof(int) * ((size_t)range + 1));
                for (int k = a; k < b; ++k)
                    hist[key[k - a] + 1]++;
                for (int t = 0; t < range; ++t)
                    hist[t + 1] += hist[t];
                for (int k = a; k < b; ++k)
                    tmp[a + hist[key[k - a]]++] = order[k];
                memcpy(order + a, tmp + a, sizeof(int) * (size_t)(b - a));
            }
        }
#pragma omp parallel for schedule(static) if (b - a >= 2048)
        for (int k = a; k < b; ++k)
            position[order[k]] = k;
    }
    free(hist);
    free(key);
    free(lev);
    free(cnt);
    return deepest;
}

static int cmp_u64(const void *x, const void *y)
{
    const unsigned long long a = *(const unsigned long long *)x, b = *(const unsigned long long *)y;
    return a < b ? -1 : a > b ? 1 : 0;
}

/* The transpose by a counting sort: a histogram of idx, its scan, a scatter
 * of (row, stored index) pairs into the new rows, then each new row sorted by
 * row.  The histogram and the scatter take atomic slots in parallel; the sort
 * restores the stored-row order (rows are distinct within a new row), so the
 * result is the serial stable one whatever the thread count. */
int capsp_transpose_structure(int n, int nnz, const int *ptr, const int *idx, int *tptr, int *tidx,
                              int *src)
{
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int k = 0; k < nnz; ++k)
        bad |= idx[k] < 0 || idx[k] >= n;
    if (bad)
        return -1;
    memset(tptr, 0, sizeof(int) * ((size_t)n + 1));
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nnz; ++k)
        __atomic_fetch_add(&tptr[idx[k] + 1], 1, __ATOMIC_RELAXED);
    for (int j = 0; j < n; ++j)
        tptr[j + 1] += tptr[j];
    int *fill = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!fill)
        return -1;
    memcpy(fill, tptr, sizeof(int) * (size_t)n);
#pragma omp parallel for schedule(static, 4096)
    for (int i = 0; i < n; ++i)
        for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
            const int p = __atomic_fetch_add(&fill[idx[k]], 1, __ATOMIC_RELAXED);
            tidx[p] = i;
            src[p] = k;
        }
    free(fill);
    int failed = 0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(| : failed)
    for (int j = 0; j < n; ++j) {
        const int a = tptr[j], e = tptr[j + 1];
        if (e - a <= 32) {
            for (int p = a + 1; p < e; ++p) { /* insertion sort by row */
                const int r = tidx[p], k = src[p];
                int q = p - 1;
                while (q >= a && tidx[q] > r) {
                    tidx[q + 1] = tidx[q];
                    src[q + 1] = src[q];
                    --q;
                }
                tidx[q + 1] = r;
                src[q + 1] = k;
            }
            continue;
        }
        /* a long new row (a heavily referenced index): (row, stored index)
         * packed into one key, sorted in O(m log m) */
        unsigned long long *key = (unsigned long long *)malloc(sizeof(unsigned long long) * (size_t)(e - a));
        if (!key) {
            failed = 1;
            continue;
        }
        for (int p = a; p < e; ++p)
            key[p - a] = ((unsigned long long)(unsigned)tidx[p] << 32) | (unsigned)src[p];
        qsort(key, (size_t)(e - a), sizeof(unsigned long long), cmp_u64);
        for (int p = a; p < e; ++p) {
            tidx[p] = (int)(key[p - a] >> 32);
            src[p] = (int)(key[p - a] & 0xffffffffull);
        }
        free(key);
    }
    return failed ? -1 : 0;
}

/* Dependency structure in schedule-position space: for position k (row
 * order[k]) its dependencies' positions, ascending, in dep_idx[dep_ptr[k] ..
 * dep_ptr[k+1]); dep_src gives the index of each dependency's value in the
 * original arrays and diag_src[k] that of the row's diagonal.  dep_ptr has
 * n+1 entries, dep_idx/dep_src nnz-n.  Returns 0 or -1 on a malformed row. */
int capsp_level_layout(int n, const int *ptr, const int *idx, int upper, const int *order,
                       const int *position, int *dep_ptr, int *dep_idx, int *dep_src, int *diag_src)
{
    dep_ptr[0] = 0;
    for (int k = 0; k < n; ++k) {
        const int i = order[k];
        dep_ptr[k + 1] = dep_ptr[k] + (ptr[i + 1] - ptr[i] - 1);
    }
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 4096)
    for (int k = 0; k < n; ++k) {
        const int i = order[k];
        const int s = ptr[i], e = ptr[i + 1];
        const int d = upper ? s : e - 1;
        if (idx[d] != i) {
            bad = 1;
            continue;
        }
        diag_src[k] = d;
        int w = dep_ptr[k];
        for (int j = s; j < e; ++j) {
            if (j == d)
                continue;
            /* insertion into the ascending run [dep_ptr[k], w) */
            const int q = position[idx[j]];
            int u = w - 1;
            while (u >= dep_ptr[k] && dep_idx[u] > q) {
                dep_idx[u + 1] = dep_idx[u];
                dep_src[u + 1] = dep_src[u];
                --u;
            }
            dep_idx[u + 1] = q;
            dep_src[u + 1] = j;
            ++w;
        }
    }
    return bad ? -1 : 0;
}

void capsp_indegree(int n, int nnz, const int *idx, int *indeg)
{
    memset(indeg, 0, sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int k = 0; k < nnz; ++k)
        indeg[idx[k]]++;
}

int capsp_validate(int n, int nnz, const int *ptr, const int *idx, int format, int uplo, char *msg,
                   int msg_len)
{
    char local[8];
    if (!msg || msg_len <= 0) {
        msg = local;
        msg_len = (int)sizeof(local);
    }
    msg[0] = 0;
    if (n < 1 || nnz < n) {
        snprintf(msg, (size_t)msg_len, "need n >= 1 and nnz >= n (got n=%d nnz=%d)", n, nnz);
        return -1;
    }
    if (ptr[0] != 0 || ptr[n] != nnz) {
        snprintf(msg, (size_t)msg_len, "ptr[0]=%d ptr[n]=%d, expected 0 and nnz=%d", ptr[0], ptr[n],
                 nnz);
        return -1;
    }
    const int diag_last = (format == CAPSP_FMT_CSR) == (uplo == CAPSP_LOWER);
    /* Rows are checked in parallel for the first bad one (each row checks its
     * own pointers before it reads idx), then that row again, serially, for
     * the message. */
    int first_bad = n;
#pragma omp parallel for schedule(static, 16384) reduction(min : first_bad)
    for (int i = 0; i < n; ++i) {
        const int s = ptr[i], e = ptr[i + 1];
        int bad = s < 0 || e <= s || e > nnz;
        if (!bad) {
            const int dpos = diag_last ? e - 1 : s;
            bad = idx[dpos] != i;
            for (int j = s; j < e && !bad; ++j) {
                const int c = idx[j];
                bad = j != dpos && !(diag_last ? (c >= 0 && c < i) : (c > i && c < n));
            }
        }
        if (bad && i < first_bad)
            first_bad = i;
    }
    for (int i = first_bad; i < n; ++i) {
        const int s = ptr[i], e = ptr[i + 1];
        if (s < 0 || e <= s || e > nnz) {
            snprintf(msg, (size_t)msg_len, "row/column %d is empty or its pointer is out of order", i);
            return -(i + 2);
        }
        const int dpos = diag_last ? e - 1 : s;
        if (idx[dpos] != i) {
            snprintf(msg, (size_t)msg_len, "row/column %d: diagonal missing from its %s position", i,
                     diag_last ? "last" : "first");
            return -(i + 2);
        }
        for (int j = s; j < e; ++j) {
            if (j == dpos)
                continue;
            const int c = idx[j];
            const int ok = diag_last ? (c >= 0 && c < i) : (c > i && c < n);
            if (!ok) {
                snprintf(msg, (size_t)msg_len,
                         "row/column %d: index %d is not on the triangular side of the diagonal", i, c);
                return -(i + 2);
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Matrix Market parsing (coordinate format)                           */
/* ------------------------------------------------------------------ */

typedef struct {
    int m, n, nnz;
    int field;     /* 0 real, 1 integer, 2 pattern */
    int symmetric; /* symmetric or hermitian: mirror off-diagonal entries */
} mm_header_t;

static void lower_str(char *s)
{
    for (; *s; ++s)
        *s = (char)tolower((unsigned char)*s);
}

static int mm_read_header(FILE *f, mm_header_t *hd)
{
    char line[1100], t0[64], t1[64], t2[64], t3[64], t4[64];
    if (!fgets(line, sizeof(line), f))
        return -2;
    if (sscanf(line, "%63s %63s %63s %63s %63s", t0, t1, t2, t3, t4) != 5)
        return -2;
    lower_str(t0);
    lower_str(t1);
    lower_str(t2);
    lower_str(t3);
    lower_str(t4);
    if (strcmp(t0, "%%matrixmarket") != 0 || strcmp(t1, "matrix") != 0)
        return -2;
    if (strcmp(t2, "coordinate") != 0)
        return -3;
    if (strcmp(t3, "complex") == 0)
        return -3;
    if (strcmp(t3, "real") == 0 || strcmp(t3, "double") == 0)
        hd->field = 0;
    else if (strcmp(t3, "integer") == 0)
        hd->field = 1;
    else if (strcmp(t3, "pattern") == 0)
        hd->field = 2;
    else
        return -3;
    hd->symmetric = (strcmp(t4, "symmetric") == 0 || strcmp(t4, "hermitian") == 0);
    do {
        if (!fgets(line, sizeof(line), f))
            return -4;
    } while (line[0] == '%' || line[0] == '\n' || line[0] == '\r');
    if (sscanf(line, "%d %d %d", &hd->m, &hd->n, &hd->nnz) != 3 || hd->m < 0 || hd->n < 0 ||
        hd->nnz < 0)
        return -4;
    return 0;
}

static int mm_read_entry(FILE *f, const mm_header_t *hd, int *a, int *b, double *v)
{
    if (hd->field == 2) {
        *v = 1.0;
        return fscanf(f, "%d %d", a, b) == 2 ? 0 : -1;
    }
    if (hd->field == 1) {
        long iv;
        if (fscanf(f, "%d %d %ld", a, b, &iv) != 3)
            return -1;
        *v = (double)iv;
        return 0;
    }
    return fscanf(f, "%d %d %lg", a, b, v) == 3 ? 0 : -1;
}

/* ------------------------------------------------------------------ */
/* value-type generic functions                                        */
/* ------------------------------------------------------------------ */

#define VT double
#define SFX(x) x##_f64
#include "preprocess_impl.h"
#undef VT
#undef SFX

#define VT float
#define SFX(x) x##_f32
#include "preprocess_impl.h"
#undef VT
#undef SFX
