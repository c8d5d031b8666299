/*
 * ORACLE -- test infrastructure.  Value-type generic body of oracle.c
 * (included with OVT = double / float).
 */

/* sptrsv_syncfree_executor (openCL/SynFree_csc/sptrsv_syncfree_serialref.h:25-108):
 * columns in order (FORWARD) or reverse order (BACKWARD); x_i from b, the
 * accumulated left_sum and the diagonal; the column's other entries are then
 * scattered into left_sum row by row.  Multi-RHS storage is row-major
 * x[i*rhs + k]. */
int OSFX(oracle_executor)(const int *colptr, const int *rowidx, const OVT *val, const int *indeg, int m,
                          int n, int substitution, int rhs, const OVT *b, OVT *x)
{
    int *arrived = (int *)calloc((size_t)(m > 0 ? m : 1), sizeof(int));
    OVT *left = (OVT *)calloc((size_t)m * (size_t)rhs + 1, sizeof(OVT));
    if (!arrived || !left) {
        free(arrived);
        free(left);
        return -2;
    }
    int rc = 0;
    for (int step = 0; step < n && rc == 0; ++step) {
        const int i = substitution == ORACLE_FORWARD ? step : n - 1 - step;
        if (indeg[i] - 1 != arrived[i]) {
            rc = -1; /* the reference would wait here forever */
            break;
        }
        const int dpos = substitution == ORACLE_FORWARD ? colptr[i] : colptr[i + 1] - 1;
        for (int k = 0; k < rhs; ++k) {
            const size_t o = (size_t)i * rhs + k;
            OVT xi = (b[o] - left[o]) / val[dpos];
            x[o] = xi;
        }
        const int js = substitution == ORACLE_FORWARD ? colptr[i] + 1 : colptr[i];
        const int je = substitution == ORACLE_FORWARD ? colptr[i + 1] : colptr[i + 1] - 1;
        for (int j = js; j < je; ++j) {
            const int r = rowidx[j];
            for (int k = 0; k < rhs; ++k) {
                OVT prod = x[(size_t)i * rhs + k] * val[j];
                left[(size_t)r * rhs + k] = left[(size_t)r * rhs + k] + prod;
            }
            arrived[r] += 1;
        }
    }
    free(arrived);
    free(left);
    return rc;
}

/* matrix_transposition (CUDA/ourWrtFst/tranpose.h:36-75): counting sort by
 * column, rows ascending inside each column. */
void OSFX(oracle_transpose)(int m, int n, int nnz, const int *rowptr, const int *colidx, const OVT *val,
                            int *cscRowIdx, int *cscColPtr, OVT *cscVal)
{
    memset(cscColPtr, 0, sizeof(int) * ((size_t)n + 1));
    for (int k = 0; k < nnz; ++k)
        cscColPtr[colidx[k] + 1]++;
    for (int c = 0; c < n; ++c)
        cscColPtr[c + 1] += cscColPtr[c];
    int *fill = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    if (!fill)
        return;
    memcpy(fill, cscColPtr, sizeof(int) * ((size_t)n + 1));
    for (int row = 0; row < m; ++row)
        for (int j = rowptr[row]; j < rowptr[row + 1]; ++j) {
            const int d = fill[colidx[j]]++;
            cscRowIdx[d] = row;
            cscVal[d] = val[j];
        }
    free(fill);
}

/* Reference pipeline for a lower-triangular CSR matrix (SyncFree_csc/main.cu
 * path): transpose to CSC, in-degree analysis, FORWARD executor. */
int OSFX(oracle_solve_csr_lower)(int n, int nnz, const int *rowptr, const int *colidx, const OVT *val,
                                 int rhs, const OVT *b, OVT *x)
{
    int *cp = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    int *ri = (int *)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    OVT *cv = (OVT *)malloc(sizeof(OVT) * (size_t)(nnz > 0 ? nnz : 1));
    int *deg = (int *)malloc(sizeof(int) * (size_t)n);
    int rc = -2;
    if (cp && ri && cv && deg) {
        OSFX(oracle_transpose)(n, n, nnz, rowptr, colidx, val, ri, cp, cv);
        oracle_analyser(ri, n, nnz, deg);
        rc = OSFX(oracle_executor)(cp, ri, cv, deg, n, n, ORACLE_FORWARD, rhs, b, x);
    }
    free(cp);
    free(ri);
    free(cv);
    free(deg);
    return rc;
}

/* Serial adjoint y = L^{-T} g: the BACKWARD executor run directly on the CSR
 * arrays of L, which are the CSC arrays of L^T (serialref.h:73-102 with the
 * diagonal last in each column).  In-degree = histogram of the column indices. */
int OSFX(oracle_solve_csr_transpose)(int n, int nnz, const int *rowptr, const int *colidx, const OVT *val,
                                     int rhs, const OVT *g, OVT *y)
{
    int *deg = (int *)malloc(sizeof(int) * (size_t)n);
    if (!deg)
        return -2;
    oracle_analyser(colidx, n, nnz, deg);
    int rc = OSFX(oracle_executor)(rowptr, colidx, val, deg, n, n, ORACLE_BACKWARD, rhs, g, y);
    free(deg);
    return rc;
}

/* grad_val[k] = -sum_r y[row(k), r] * x[col(k), r]: derivative of a loss with
 * gradient g = dLoss/dx with respect to the stored values of L, given
 * y = L^{-T} g and x = L^{-1} b.  No reference counterpart (the reference has
 * no differentiation); sums over r in ascending order. */
void OSFX(oracle_grad_val)(int n, const int *rowptr, const int *colidx, int rhs, const OVT *y, const OVT *x,
                           OVT *grad)
{
    for (int i = 0; i < n; ++i)
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            OVT acc = (OVT)0;
            for (int r = 0; r < rhs; ++r) {
                OVT prod = y[(size_t)i * rhs + r] * x[(size_t)colidx[k] * rhs + r];
                acc = acc + prod;
            }
            grad[k] = -acc;
        }
}

/* b = A * ones over the stored entries of each row, accumulated in row order
 * in the value type: the known-answer right-hand side of get_x_b
 * (CUDA/ourWrtFst/read_mtx.h:260-278, whose x_ref is all ones, so each
 * product val * x_ref[col] is val itself). */
void OSFX(oracle_get_x_b)(int m, const int *rowptr, const OVT *val, OVT *b)
{
    for (int i = 0; i < m; ++i) {
        OVT acc = (OVT)0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; ++j) {
            OVT prod = val[j] * (OVT)1;
            acc = acc + prod;
        }
        b[i] = acc;
    }
}
