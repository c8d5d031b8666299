/*
 * Value-type generic part of the host preprocessing.  Included by
 * preprocess.c once with VT=double, SFX(x)=x##_f64 and once with VT=float,
 * SFX(x)=x##_f32, mirroring the reference's compile-time VALUE_TYPE
 * (CUDA/ourWrtFst/common.h:16-18).
 */

/* Lower-triangular extraction with the contract of change2tran
 * (CUDA/ourWrtFst/read_mtx.h:194-257): every row of A is sorted in place by
 * column, entries with col < row are kept with value 1, and a unit diagonal is
 * appended.  Unlike the reference, the output is sized by a counting pass, so
 * a matrix with fewer stored entries than rows cannot overrun it. */
int SFX(change2tran)(int m, int nnzA, int *csrRowPtrA, int *csrColIdxA, VT *csrValA,
                     int *nnzL_add, int **csrRowPtrL_tmp_add, int **csrColIdxL_tmp_add,
                     VT **csrValL_tmp_add)
{
    (void)nnzA;
    int *rowptr = (int *)malloc(sizeof(int) * ((size_t)m + 1));
    if (!rowptr)
        return -1;
    rowptr[0] = 0;
    long long total = 0;
    for (int i = 0; i < m; ++i) {
        const int s = csrRowPtrA[i], e = csrRowPtrA[i + 1];
        sort_row_pairs_generic(csrColIdxA + s, (unsigned char *)(csrValA + s), sizeof(VT), e - s);
        int keep = 0;
        for (int j = s; j < e && csrColIdxA[j] < i; ++j)
            ++keep;
        total += keep + 1;
        rowptr[i + 1] = (int)total;
    }
    const int nnzL = (int)total;
    int *colidx = (int *)malloc(sizeof(int) * (size_t)(nnzL > 0 ? nnzL : 1));
    VT *val = (VT *)malloc(sizeof(VT) * (size_t)(nnzL > 0 ? nnzL : 1));
    if (!colidx || !val) {
        free(rowptr);
        free(colidx);
        free(val);
        return -1;
    }
    for (int i = 0; i < m; ++i) {
        int w = rowptr[i];
        for (int j = csrRowPtrA[i]; j < csrRowPtrA[i + 1] && csrColIdxA[j] < i; ++j) {
            colidx[w] = csrColIdxA[j];
            val[w] = (VT)1;
            ++w;
        }
        colidx[w] = i;
        val[w] = (VT)1;
    }
    *nnzL_add = nnzL;
    *csrRowPtrL_tmp_add = rowptr;
    *csrColIdxL_tmp_add = colidx;
    *csrValL_tmp_add = val;
    return 0;
}

/* x_ref = ones and b = A * x_ref accumulated in VT, row by row in storage
 * order (CUDA/ourWrtFst/read_mtx.h:260-278). */
void SFX(get_x_b)(int m, int n, const int *csrRowPtrA, const int *csrColIdxA,
                  const VT *csrValA, VT **x_add, VT **b_add)
{
    VT *x_ref = (VT *)malloc(sizeof(VT) * (size_t)(n > 0 ? n : 1));
    VT *b = (VT *)malloc(sizeof(VT) * (size_t)(m > 0 ? m : 1));
    if (!x_ref || !b) {
        free(x_ref);
        free(b);
        *x_add = NULL;
        *b_add = NULL;
        return;
    }
    for (int i = 0; i < n; ++i)
        x_ref[i] = (VT)1;
    for (int i = 0; i < m; ++i) {
        VT acc = (VT)0;
        for (int j = csrRowPtrA[i]; j < csrRowPtrA[i + 1]; ++j) {
            VT prod = csrValA[j] * x_ref[csrColIdxA[j]];
            acc = acc + prod;
        }
        b[i] = acc;
    }
    *x_add = x_ref;
    *b_add = b;
}

/* Level recurrence of matrix_layer (CUDA/ourWrtFst/tranpose.h:78-142). */
int SFX(matrix_layer)(const int m, const int n, const int nnz, const int *csrRowPtr,
                      const int *csrColIdx, const VT *csrVal, int *layer_add,
                      double *parallelism_add)
{
    (void)n;
    (void)nnz;
    (void)csrVal;
    int *level = (int *)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    if (!level) {
        *layer_add = 0;
        *parallelism_add = 0.0;
        return 0;
    }
    int levels = capsp_row_levels(m, csrRowPtr, csrColIdx, level, NULL);
    free(level);
    *layer_add = levels;
    *parallelism_add = levels > 0 ? (double)m / levels : 0.0;
    return levels;
}

/* Counting-sort transposition (CUDA/ourWrtFst/tranpose.h:36-75). */
void SFX(matrix_transposition)(const int m, const int n, const int nnz, const int *csrRowPtr,
                               const int *csrColIdx, const VT *csrVal, int *cscRowIdx,
                               int *cscColPtr, VT *cscVal)
{
    memset(cscColPtr, 0, sizeof(int) * ((size_t)n + 1));
    for (int k = 0; k < nnz; ++k)
        cscColPtr[csrColIdx[k]]++;
    capsp_exclusive_scan(cscColPtr, n + 1);
    int *fill = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    if (!fill)
        return;
    memcpy(fill, cscColPtr, sizeof(int) * ((size_t)n + 1));
    for (int row = 0; row < m; ++row) {
        for (int j = csrRowPtr[row]; j < csrRowPtr[row + 1]; ++j) {
            const int col = csrColIdx[j];
            const int dst = fill[col]++;
            cscRowIdx[dst] = row;
            cscVal[dst] = csrVal[j];
        }
    }
    free(fill);
}

/* Mix selector (CUDA/mix/tranpose.h:1423-1483) over 32-row groups. */
void SFX(matrix_warp4)(const int m, const int n, const int nnz, const int *csrRowPtr,
                       const int *csrColIdx, const VT *csrVal, const int border,
                       int *Len_add, int *warp_num, double *warp_occupy_add,
                       double *element_occupy_add)
{
    (void)n;
    (void)csrColIdx;
    (void)csrVal;
    double wo = 0.0, eo = 0.0;
    int len = mix_table_impl(m, csrRowPtr, 0, 32, border, nnz, warp_num, &wo, &eo);
    *Len_add = len;
    *warp_occupy_add = wo;
    *element_occupy_add = eo;
}

/* Matrix Market reader with the contract of read_mtx
 * (CUDA/ourWrtFst/read_mtx.h:6-191): real, integer or pattern data, general or
 * symmetric (mirrored off-diagonal entries), 1-based coordinates, entries
 * placed row by row in file order. */
int SFX(read_mtx)(const char *filename, int *m_add, int *n_add, int *nnzA_add,
                  int **csrRowPtrA_add, int **csrColIdxA_add, VT **csrValA_add)
{
    mm_header_t hd;
    FILE *f = fopen(filename, "r");
    if (!f)
        return -1;
    int rc = mm_read_header(f, &hd);
    if (rc != 0) {
        fclose(f);
        return rc;
    }
    const int m = hd.m, n = hd.n, nrep = hd.nnz;
    int *cnt = (int *)calloc((size_t)m + 1, sizeof(int));
    int *ri = (int *)malloc(sizeof(int) * (size_t)(nrep > 0 ? nrep : 1));
    int *ci = (int *)malloc(sizeof(int) * (size_t)(nrep > 0 ? nrep : 1));
    double *vv = (double *)malloc(sizeof(double) * (size_t)(nrep > 0 ? nrep : 1));
    if (!cnt || !ri || !ci || !vv) {
        fclose(f);
        free(cnt);
        free(ri);
        free(ci);
        free(vv);
        return -2;
    }
    for (int t = 0; t < nrep; ++t) {
        int a, b;
        double v = 1.0;
        if (mm_read_entry(f, &hd, &a, &b, &v) != 0 || a < 1 || b < 1 || a > m || b > n) {
            fclose(f);
            free(cnt);
            free(ri);
            free(ci);
            free(vv);
            return -5;
        }
        ri[t] = a - 1;
        ci[t] = b - 1;
        vv[t] = v;
        cnt[ri[t]]++;
        if (hd.symmetric && ri[t] != ci[t])
            cnt[ci[t]]++;
    }
    fclose(f);
    capsp_exclusive_scan(cnt, m + 1);
    const int nnz = cnt[m];
    int *rowptr = (int *)malloc(sizeof(int) * ((size_t)m + 1));
    int *colidx = (int *)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    VT *val = (VT *)malloc(sizeof(VT) * (size_t)(nnz > 0 ? nnz : 1));
    if (!rowptr || !colidx || !val) {
        free(cnt);
        free(ri);
        free(ci);
        free(vv);
        free(rowptr);
        free(colidx);
        free(val);
        return -2;
    }
    memcpy(rowptr, cnt, sizeof(int) * ((size_t)m + 1));
    for (int t = 0; t < nrep; ++t) {
        int dst = cnt[ri[t]]++;
        colidx[dst] = ci[t];
        val[dst] = (VT)vv[t];
        if (hd.symmetric && ri[t] != ci[t]) {
            dst = cnt[ci[t]]++;
            colidx[dst] = ri[t];
            val[dst] = (VT)vv[t];
        }
    }
    free(cnt);
    free(ri);
    free(ci);
    free(vv);
    *m_add = m;
    *n_add = n;
    *nnzA_add = nnz;
    *csrRowPtrA_add = rowptr;
    *csrColIdxA_add = colidx;
    *csrValA_add = val;
    return 0;
}
