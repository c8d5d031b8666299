/*
 * ORACLE -- test infrastructure, not product code.  CPU restatement of the
 * reference's serial sync-free solve; see oracle.c.
 */
#ifndef CAPSP_ORACLE_H
#define CAPSP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_FORWARD 0  /* SUBSTITUTION_FORWARD, openCL/SynFree_csc/common.h:27 */
#define ORACLE_BACKWARD 1 /* SUBSTITUTION_BACKWARD, openCL/SynFree_csc/common.h:28 */

void oracle_analyser(const int *idx, int m, int nnz, int *histo);

int oracle_executor_f64(const int *colptr, const int *rowidx, const double *val, const int *indeg, int m,
                        int n, int substitution, int rhs, const double *b, double *x);
int oracle_executor_f32(const int *colptr, const int *rowidx, const float *val, const int *indeg, int m,
                        int n, int substitution, int rhs, const float *b, float *x);
void oracle_transpose_f64(int m, int n, int nnz, const int *rowptr, const int *colidx, const double *val,
                          int *cscRowIdx, int *cscColPtr, double *cscVal);
void oracle_transpose_f32(int m, int n, int nnz, const int *rowptr, const int *colidx, const float *val,
                          int *cscRowIdx, int *cscColPtr, float *cscVal);
int oracle_solve_csr_lower_f64(int n, int nnz, const int *rowptr, const int *colidx, const double *val,
                               int rhs, const double *b, double *x);
int oracle_solve_csr_lower_f32(int n, int nnz, const int *rowptr, const int *colidx, const float *val,
                               int rhs, const float *b, float *x);
int oracle_solve_csr_transpose_f64(int n, int nnz, const int *rowptr, const int *colidx,
                                   const double *val, int rhs, const double *g, double *y);
int oracle_solve_csr_transpose_f32(int n, int nnz, const int *rowptr, const int *colidx, const float *val,
                                   int rhs, const float *g, float *y);
void oracle_grad_val_f64(int n, const int *rowptr, const int *colidx, int rhs, const double *y,
                         const double *x, double *grad);
void oracle_grad_val_f32(int n, const int *rowptr, const int *colidx, int rhs, const float *y,
                         const float *x, float *grad);

void oracle_get_x_b_f64(int m, const int *rowptr, const double *val, double *b);
void oracle_get_x_b_f32(int m, const int *rowptr, const float *val, float *b);

#ifdef __cplusplus
}
#endif

#endif
