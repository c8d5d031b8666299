/*
 * Seeded synthetic lower-triangular CSR generators.
 *
 * They stand in for the SuiteSparse matrices the reference benchmarks on
 * (matrix/matrix_name.txt), which are not available.  Every row draws from its
 * own splitmix64 stream keyed by (seed, stream, row); a first pass produces the
 * row pointer, a second pass regenerates each row's stream and writes columns
 * (ascending, diagonal last) and values.  The result does not depend on the
 * number of threads.
 *
 * Value rule (shared by all workloads): off-diagonals U[-1,1], diagonal
 * 1 + sum |off-diagonals|, which keeps L strictly diagonally dominant.
 */
#include "capsp.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define GEN_MAX_K 4096

static inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct { uint64_t s; } rng_t;

static inline uint64_t rng_next(rng_t *r)
{
    r->s += 0x9E3779B97F4A7C15ull;
    return mix64(r->s);
}

static inline rng_t rng_for(uint64_t seed, uint64_t stream, uint64_t row)
{
    rng_t r;
    r.s = mix64(mix64(seed + 0x632BE59BD9B4E019ull) ^ mix64(stream * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull)
                ^ (row * 0x9E3779B97F4A7C15ull));
    return r;
}

/* uniform integer in [0, m) (m >= 1), multiply-shift */
static inline uint64_t rng_below(rng_t *r, uint64_t m)
{
    return (uint64_t)(((unsigned __int128)rng_next(r) * (unsigned __int128)m) >> 64);
}

/* uniform double in [0, 1) */
static inline double rng_unit(rng_t *r)
{
    return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0);
}

typedef struct {
    double *cdf; /* cdf[k-1] = P(K <= k), k = 1..cap */
    int cap;
} zipf_t;

static int zipf_init(zipf_t *z, double s, int cap)
{
    z->cap = cap;
    z->cdf = (double *)malloc(sizeof(double) * (size_t)cap);
    if (!z->cdf)
        return -1;
    double tot = 0.0;
    for (int k = 1; k <= cap; ++k)
        tot += pow((double)k, -s);
    double acc = 0.0;
    for (int k = 1; k <= cap; ++k) {
        acc += pow((double)k, -s);
        z->cdf[k - 1] = acc / tot;
    }
    z->cdf[cap - 1] = 1.0;
    return 0;
}

static inline int zipf_draw(const zipf_t *z, rng_t *r)
{
    double u = rng_unit(r);
    int lo = 0, hi = z->cap - 1;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (z->cdf[mid] >= u)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo + 1;
}

/* Number of off-diagonals of row i (first draw(s) of the row stream). */
static inline int64_t row_k(const capsp_gen_params_t *p, const zipf_t *z, rng_t *r, int64_t i)
{
    int64_t k;
    if (p->kind == CAPSP_GEN_ZIPF_NEAR_FAR) {
        k = zipf_draw(z, r);
        if (k < p->kmin) /* optional floor on the drawn count */
            k = p->kmin;
        if (k > i)
            k = i;
    } else {
        k = p->kmin + (int64_t)rng_below(r, (uint64_t)(p->kmax - p->kmin + 1));
        int64_t lo = (p->band > 0 && i - p->band > 0) ? i - p->band : 0;
        if (k > i - lo)
            k = i - lo;
    }
    if (k < 0)
        k = 0;
    return k;
}

static int contains(const int *a, int cnt, int v)
{
    for (int t = 0; t < cnt; ++t)
        if (a[t] == v)
            return 1;
    return 0;
}

static int cmp_int(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

static void sort_small(int *a, int cnt)
{
    if (cnt > 32) {
        qsort(a, (size_t)cnt, sizeof(int), cmp_int);
        return;
    }
    for (int t = 1; t < cnt; ++t) {
        int v = a[t], u = t - 1;
        while (u >= 0 && a[u] > v) {
            a[u + 1] = a[u];
            --u;
        }
        a[u + 1] = v;
    }
}

/* distinct uniform draws from [lo, hi] (inclusive) appended to cols */
static void draw_distinct(rng_t *r, int *cols, int *cnt, int64_t want, int64_t lo, int64_t hi)
{
    uint64_t span = (uint64_t)(hi - lo + 1);
    int64_t got = 0;
    while (got < want) {
        int c = (int)(lo + (int64_t)rng_below(r, span));
        if (!contains(cols, *cnt, c)) {
            cols[(*cnt)++] = c;
            ++got;
        }
    }
}

static int check_params(const capsp_gen_params_t *p)
{
    if (!p || p->n < 1 || p->n > 0x7fffffffLL)
        return 0;
    if (p->kind == CAPSP_GEN_UNIFORM_BAND)
        return p->kmin >= 0 && p->kmax >= p->kmin && p->kmax < GEN_MAX_K;
    if (p->kind == CAPSP_GEN_ZIPF_NEAR_FAR)
        return p->zipf_cap >= 1 && p->zipf_cap < GEN_MAX_K && p->zipf_s > 0.0 && p->near_window >= 1 &&
               p->kmin >= 0 && p->kmin < GEN_MAX_K;
    return 0;
}

capsp_status_t capsp_gen_rowptr(const capsp_gen_params_t *p, int *rowptr)
{
    if (!check_params(p) || !rowptr)
        return CAPSP_ERR_INVALID;
    zipf_t z = {0, 0};
    if (p->kind == CAPSP_GEN_ZIPF_NEAR_FAR && zipf_init(&z, p->zipf_s, p->zipf_cap))
        return CAPSP_ERR_OOM;
    const int64_t n = p->n;
#pragma omp parallel for schedule(static, 8192)
    for (int64_t i = 0; i < n; ++i) {
        rng_t r = rng_for(p->seed, p->stream, (uint64_t)i);
        rowptr[i + 1] = (int)(row_k(p, &z, &r, i) + 1);
    }
    free(z.cdf);
    int64_t acc = 0;
    rowptr[0] = 0;
    for (int64_t i = 0; i < n; ++i) {
        acc += rowptr[i + 1];
        if (acc > 0x7fffffffLL)
            return CAPSP_ERR_INVALID;
        rowptr[i + 1] = (int)acc;
    }
    return CAPSP_OK;
}

capsp_status_t capsp_gen_fill_f64(const capsp_gen_params_t *p, const int *rowptr,
                                  int *colidx, double *val)
{
    if (!check_params(p) || !rowptr || !colidx || !val)
        return CAPSP_ERR_INVALID;
    zipf_t z = {0, 0};
    if (p->kind == CAPSP_GEN_ZIPF_NEAR_FAR && zipf_init(&z, p->zipf_s, p->zipf_cap))
        return CAPSP_ERR_OOM;
    const int64_t n = p->n;
    int bad = 0;
#pragma omp parallel
    {
        int cols[GEN_MAX_K];
#pragma omp for schedule(static, 8192)
        for (int64_t i = 0; i < n; ++i) {
            rng_t r = rng_for(p->seed, p->stream, (uint64_t)i);
            int64_t k = row_k(p, &z, &r, i);
            int cnt = 0;
            if (p->kind == CAPSP_GEN_ZIPF_NEAR_FAR) {
                int64_t knear = (k + 1) / 2;
                int64_t win = p->near_window < i ? p->near_window : i;
                if (knear > win)
                    knear = win;
                if (knear > 0)
                    draw_distinct(&r, cols, &cnt, knear, i - win, i - 1);
                if (k - knear > 0)
                    draw_distinct(&r, cols, &cnt, k - knear, 0, i - 1);
            } else if (k > 0) {
                int64_t lo = (p->band > 0 && i - p->band > 0) ? i - p->band : 0;
                draw_distinct(&r, cols, &cnt, k, lo, i - 1);
            }
            sort_small(cols, cnt);
            const int base = rowptr[i];
            if (rowptr[i + 1] - base != cnt + 1) {
                bad = 1;
                continue;
            }
            double sabs = 0.0;
            for (int t = 0; t < cnt; ++t) {
                double v = 2.0 * rng_unit(&r) - 1.0;
                colidx[base + t] = cols[t];
                val[base + t] = v;
                sabs += fabs(v);
            }
            colidx[base + cnt] = (int)i;
            val[base + cnt] = 1.0 + sabs;
        }
    }
    free(z.cdf);
    return bad ? CAPSP_ERR_INVALID : CAPSP_OK;
}

capsp_status_t capsp_gen_normal_f64(uint64_t seed, uint64_t stream, int64_t count, double *out)
{
    if (count < 0 || (count > 0 && !out))
        return CAPSP_ERR_INVALID;
    const int64_t pairs = (count + 1) / 2;
#pragma omp parallel for schedule(static, 16384)
    for (int64_t t = 0; t < pairs; ++t) {
        rng_t r = rng_for(seed, stream ^ 0xA5A5A5A5ull, (uint64_t)t);
        double u1 = rng_unit(&r), u2 = rng_unit(&r);
        if (u1 < 1e-300)
            u1 = 1e-300;
        double rad = sqrt(-2.0 * log(u1));
        double ang = 6.283185307179586476925286766559 * u2;
        out[2 * t] = rad * cos(ang);
        if (2 * t + 1 < count)
            out[2 * t + 1] = rad * sin(ang);
    }
    return CAPSP_OK;
}

capsp_status_t capsp_spmv_f64(int n, const int *rowptr, const int *colidx, const double *val,
                              int nrhs, const double *x, double *y)
{
    if (n < 0 || nrhs < 1 || !rowptr || !colidx || !val || !x || !y)
        return CAPSP_ERR_INVALID;
#pragma omp parallel for schedule(static, 4096)
    for (int i = 0; i < n; ++i) {
        for (int r = 0; r < nrhs; ++r) {
            double acc = 0.0;
            for (int j = rowptr[i]; j < rowptr[i + 1]; ++j)
                acc += val[j] * x[(int64_t)colidx[j] * nrhs + r];
            y[(int64_t)i * nrhs + r] = acc;
        }
    }
    return CAPSP_OK;
}

uint64_t capsp_digest(int n, int nnz, const int *rowptr, const int *colidx, const void *val,
                      int val_bytes)
{
    uint64_t h = 0xcbf29ce484222325ull;
#define FNV_BYTES(ptr, len)                                        \
    do {                                                           \
        const unsigned char *b_ = (const unsigned char *)(ptr);    \
        for (size_t t_ = 0; t_ < (size_t)(len); ++t_) {            \
            h ^= b_[t_];                                           \
            h *= 0x100000001b3ull;                                 \
        }                                                          \
    } while (0)
    FNV_BYTES(&n, sizeof(int));
    FNV_BYTES(&nnz, sizeof(int));
    if (rowptr)
        FNV_BYTES(rowptr, sizeof(int) * ((size_t)n + 1));
    if (colidx)
        FNV_BYTES(colidx, sizeof(int) * (size_t)nnz);
    if (val && val_bytes > 0)
        FNV_BYTES(val, (size_t)val_bytes * (size_t)nnz);
#undef FNV_BYTES
    return h;
}
