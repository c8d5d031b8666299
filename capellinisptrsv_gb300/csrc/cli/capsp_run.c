/*
 * capsp_run: the command-line driver of the reference's four CUDA variants
 * (CUDA/{ourWrtFst,our2Part,mix,SyncFree_csc}/main.cu), one program with the
 * variant picked at run time instead of one build per folder.
 *
 *   capsp_run [--alg wrtfst|twopart|mix|csc] [--f32] [--out result.csv] matrix.mtx
 *
 * Flow, as in the reference: read the Matrix Market file, square it to
 * min(m, n), extract the unit-valued lower triangle (change2tran), count its
 * levels (matrix_layer), run the variant's driver twice (the second run's
 * numbers are reported) and append the header line and one result row to the
 * CSV file in the reference's column order and number format
 * (README.md:56; mix/main.cu:104-106 adds warp_occupy and element_occupy).
 * Exit codes follow main.cu: 0 for m <= 1, -1 when the CSV cannot be opened,
 * -3 for an empty triangle; a failing read or driver returns 1.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "capsp.h"

enum { ALG_WRTFST, ALG_TWOPART, ALG_MIX, ALG_CSC };

typedef struct {
    int m, n, nnzL, layer;
    double parallelism, pre_time, solve_time, gflops, bandwidth, warp_occupy, element_occupy;
} Row;

/* One precision of the flow; VT is double or float, SFX _f64 or _f32. */
#define CAPSP_RUN_BODY(VT, SFX)                                                                   \
    static int run##SFX(const char *file, int alg, Row *r)                                         \
    {                                                                                               \
        int m = 0, n = 0, nnzA = 0, *rpA = NULL, *ciA = NULL, *rpL = NULL, *ciL = NULL;             \
        VT *vA = NULL, *vL = NULL;                                                                  \
        int rc = 1;                                                                                 \
        if (read_mtx##SFX(file, &m, &n, &nnzA, &rpA, &ciA, &vA) != 0) {                             \
            fprintf(stderr, "capsp_run: cannot read %s\n", file);                                   \
            return 1;                                                                               \
        }                                                                                           \
        if (m <= n)                                                                                 \
            n = m;                                                                                  \
        else                                                                                        \
            m = n;                                                                                  \
        r->m = m;                                                                                   \
        r->n = n;                                                                                   \
        if (m <= 1) {                                                                               \
            rc = 0;                                                                                 \
            r->m = -1;                                                                              \
            goto out;                                                                               \
        }                                                                                           \
        if (change2tran##SFX(m, nnzA, rpA, ciA, vA, &r->nnzL, &rpL, &ciL, &vL) != 0)                \
            goto out;                                                                               \
        if (r->nnzL == 0) {                                                                         \
            rc = -3;                                                                                \
            goto out;                                                                               \
        }                                                                                           \
        matrix_layer##SFX(m, n, r->nnzL, rpL, ciL, vL, &r->layer, &r->parallelism);                 \
        for (int rep = 0; rep < 2; ++rep) {                                                         \
            int st = 0;                                                                             \
            if (alg == ALG_WRTFST)                                                                  \
                st = spts_syncfree_cuda_csr_wrt##SFX(rpL, ciL, vL, m, n, r->nnzL, &r->solve_time,   \
                                                     &r->gflops, &r->bandwidth);                    \
            else if (alg == ALG_TWOPART)                                                            \
                st = spts_syncfree_cuda_csr##SFX(rpL, ciL, vL, m, n, r->nnzL, &r->solve_time,       \
                                                 &r->gflops, &r->bandwidth);                        \
            else if (alg == ALG_MIX)                                                                \
                st = spts_syncfree_cuda_csr_wrt_mix##SFX(rpL, ciL, vL, m, n, r->nnzL,               \
                                                         &r->solve_time, &r->gflops, &r->bandwidth, \
                                                         &r->pre_time, &r->warp_occupy,             \
                                                         &r->element_occupy);                       \
            else {                                                                                  \
                int *cp = (int *)malloc(sizeof(int) * ((size_t)n + 1));                             \
                int *ri = (int *)malloc(sizeof(int) * (size_t)r->nnzL);                             \
                VT *cv = (VT *)malloc(sizeof(VT) * (size_t)r->nnzL);                                \
                VT *xr = NULL, *b = NULL, *x = (VT *)malloc(sizeof(VT) * (size_t)n);                \
                if (!cp || !ri || !cv || !x) {                                                      \
                    st = -2;                                                                        \
                } else {                                                                            \
                    matrix_transposition##SFX(m, n, r->nnzL, rpL, ciL, vL, ri, cp, cv);             \
                    get_x_b##SFX(m, n, rpL, ciL, vL, &xr, &b);                                      \
                    st = sptrsv_syncfree_cuda##SFX(cp, ri, cv, m, n, r->nnzL, x, b, xr,             \
                                                   &r->pre_time, &r->solve_time, &r->gflops,        \
                                                   &r->bandwidth);                                  \
                }                                                                                   \
                free(cp);                                                                           \
                free(ri);                                                                           \
                free(cv);                                                                           \
                free(x);                                                                            \
                free(xr);                                                                           \
                free(b);                                                                            \
            }                                                                                       \
            if (st != 0) {                                                                          \
                fprintf(stderr, "capsp_run: driver returned %d (%s)\n", st, capsp_last_error());    \
                goto out;                                                                           \
            }                                                                                       \
        }                                                                                           \
        rc = 0;                                                                                     \
    out:                                                                                            \
        free(rpA);                                                                                  \
        free(ciA);                                                                                  \
        free(vA);                                                                                   \
        free(rpL);                                                                                  \
        free(ciL);                                                                                  \
        free(vL);                                                                                   \
        return rc;                                                                                  \
    }

CAPSP_RUN_BODY(double, _f64)
CAPSP_RUN_BODY(float, _f32)

static void usage(void)
{
    fprintf(stderr, "usage: capsp_run [--alg wrtfst|twopart|mix|csc] [--f32] [--out result.csv] matrix.mtx\n");
}

int main(int argc, char **argv)
{
    const char *file = NULL, *out = "result.csv";
    int alg = ALG_WRTFST, f32 = 0;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "--alg") && i + 1 < argc) {
            const char *a = argv[++i];
            if (!strcmp(a, "wrtfst"))
                alg = ALG_WRTFST;
            else if (!strcmp(a, "twopart"))
                alg = ALG_TWOPART;
            else if (!strcmp(a, "mix"))
                alg = ALG_MIX;
            else if (!strcmp(a, "csc"))
                alg = ALG_CSC;
            else {
                usage();
                return 2;
            }
        } else if (!strcmp(argv[i], "--f32")) {
            f32 = 1;
        } else if (!strcmp(argv[i], "--out") && i + 1 < argc) {
            out = argv[++i];
        } else if (argv[i][0] == '-') {
            usage();
            return 2;
        } else {
            file = argv[i];
        }
    }
    if (!file) {
        usage();
        return 2;
    }
    FILE *fp = fopen(out, "a");
    if (!fp)
        return -1;
    Row r;
    memset(&r, 0, sizeof(r));
    const int rc = f32 ? run_f32(file, alg, &r) : run_f64(file, alg, &r);
    if (rc != 0 || r.m < 0) {
        fclose(fp);
        return rc;
    }
    if (alg == ALG_MIX) {
        fprintf(fp, "filename,m,nnzL,nnzL/m,layer,parallelism,pre_time,solve_time,gflops,bandwith,"
                    "warp_occupy,element_occupy\n");
        fprintf(fp, "%s, %d, %d, %4.2f, %d, %4.2f, %4.2f, %4.2f, %4.2f, %4.2f, %4.2f, %4.2f\n", file, r.m,
                r.nnzL, (double)r.nnzL / r.m, r.layer, r.parallelism, r.pre_time, r.solve_time, r.gflops,
                r.bandwidth, r.warp_occupy, r.element_occupy);
    } else {
        fprintf(fp, "filename,m,nnzL,nnzL/m,layer,parallelism,pre_time,solve_time,gflops,bandwith\n");
        fprintf(fp, "%s, %d, %d, %4.2f, %d, %4.2f, %4.2f, %4.2f, %4.2f, %4.2f\n", file, r.m, r.nnzL,
                (double)r.nnzL / r.m, r.layer, r.parallelism, r.pre_time, r.solve_time, r.gflops,
                r.bandwidth);
    }
    fclose(fp);
    return 0;
}
