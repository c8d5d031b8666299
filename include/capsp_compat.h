/*
 * capsp_compat.h -- drop-in names for code written against CapelliniSpTRSV.
 *
 * The reference compiles every driver for one VALUE_TYPE chosen in common.h
 * (CUDA/ourWrtFst/common.h:16-18).  libcapsp exports each driver twice
 * (_f64 / _f32); this header restores the reference's unsuffixed names and
 * picks the variant from the type of the value-array argument:
 *   - C++: inline overloads on const double* / const float*;
 *   - C11: _Generic macros.
 *
 * Solve drivers are always mapped.  The reference's mix driver shares its name
 * with the ourWrtFst driver (both are spts_syncfree_cuda_csr_wrt, told apart
 * by three extra out-parameters); in C++ both overloads are provided, in C
 * define CAPSP_COMPAT_MIX to map the name to the mix driver.
 * Host preprocessing (change2tran, get_x_b, matrix_layer,
 * matrix_transposition, matrix_warp4, read_mtx) is mapped only when
 * CAPSP_COMPAT_HOST is defined, so the header can coexist with the
 * reference's own read_mtx.h / tranpose.h in one translation unit.
 */
#ifndef CAPSP_COMPAT_H
#define CAPSP_COMPAT_H

#include "capsp.h"

#ifdef __cplusplus

/* CUDA/ourWrtFst/spts_syncfree_cuda_csr_wrt.h:66-75 */
inline int spts_syncfree_cuda_csr_wrt(const int *r, const int *c, const double *v, const int m,
                                      const int n, const int nnz, double *t, double *g, double *bw)
{ return spts_syncfree_cuda_csr_wrt_f64(r, c, v, m, n, nnz, t, g, bw); }
inline int spts_syncfree_cuda_csr_wrt(const int *r, const int *c, const float *v, const int m,
                                      const int n, const int nnz, double *t, double *g, double *bw)
{ return spts_syncfree_cuda_csr_wrt_f32(r, c, v, m, n, nnz, t, g, bw); }

/* CUDA/mix/spts_syncfree_cuda_csr_wrt.h:146-158 */
inline int spts_syncfree_cuda_csr_wrt(const int *r, const int *c, const double *v, const int m,
                                      const int n, const int nnz, double *t, double *g, double *bw,
                                      double *pre, double *wo, double *eo)
{ return spts_syncfree_cuda_csr_wrt_mix_f64(r, c, v, m, n, nnz, t, g, bw, pre, wo, eo); }
inline int spts_syncfree_cuda_csr_wrt(const int *r, const int *c, const float *v, const int m,
                                      const int n, const int nnz, double *t, double *g, double *bw,
                                      double *pre, double *wo, double *eo)
{ return spts_syncfree_cuda_csr_wrt_mix_f32(r, c, v, m, n, nnz, t, g, bw, pre, wo, eo); }

/* CUDA/our2Part/spts_syncfree_cuda_csr.h:133-142 */
inline int spts_syncfree_cuda_csr(const int *r, const int *c, const double *v, const int m,
                                  const int n, const int nnz, double *t, double *g, double *bw)
{ return spts_syncfree_cuda_csr_f64(r, c, v, m, n, nnz, t, g, bw); }
inline int spts_syncfree_cuda_csr(const int *r, const int *c, const float *v, const int m,
                                  const int n, const int nnz, double *t, double *g, double *bw)
{ return spts_syncfree_cuda_csr_f32(r, c, v, m, n, nnz, t, g, bw); }

/* CUDA/SyncFree_csc/spts_syncfree_cuda2.h:89-102 */
inline int sptrsv_syncfree_cuda(const int *cp, const int *ri, const double *cv, const int m,
                                const int n, const int nnz, double *x, const double *b,
                                const double *xr, double *pre, double *t, double *g, double *bw)
{ return sptrsv_syncfree_cuda_f64(cp, ri, cv, m, n, nnz, x, b, xr, pre, t, g, bw); }
inline int sptrsv_syncfree_cuda(const int *cp, const int *ri, const float *cv, const int m,
                                const int n, const int nnz, float *x, const float *b,
                                const float *xr, double *pre, double *t, double *g, double *bw)
{ return sptrsv_syncfree_cuda_f32(cp, ri, cv, m, n, nnz, x, b, xr, pre, t, g, bw); }

#ifdef CAPSP_COMPAT_HOST
inline void change2tran(int m, int nnzA, int *rp, int *ci, double *v, int *nnzL, int **lrp,
                        int **lci, double **lv)
{ change2tran_f64(m, nnzA, rp, ci, v, nnzL, lrp, lci, lv); }
inline void change2tran(int m, int nnzA, int *rp, int *ci, float *v, int *nnzL, int **lrp,
                        int **lci, float **lv)
{ change2tran_f32(m, nnzA, rp, ci, v, nnzL, lrp, lci, lv); }
inline void get_x_b(int m, int n, const int *rp, const int *ci, const double *v, double **x, double **b)
{ get_x_b_f64(m, n, rp, ci, v, x, b); }
inline void get_x_b(int m, int n, const int *rp, const int *ci, const float *v, float **x, float **b)
{ get_x_b_f32(m, n, rp, ci, v, x, b); }
inline int matrix_layer(const int m, const int n, const int nnz, const int *rp, const int *ci,
                        const double *v, int *layer, double *par)
{ return matrix_layer_f64(m, n, nnz, rp, ci, v, layer, par); }
inline int matrix_layer(const int m, const int n, const int nnz, const int *rp, const int *ci,
                        const float *v, int *layer, double *par)
{ return matrix_layer_f32(m, n, nnz, rp, ci, v, layer, par); }
inline void matrix_transposition(const int m, const int n, const int nnz, const int *rp, const int *ci,
                                 const double *v, int *ri, int *cp, double *cv)
{ matrix_transposition_f64(m, n, nnz, rp, ci, v, ri, cp, cv); }
inline void matrix_transposition(const int m, const int n, const int nnz, const int *rp, const int *ci,
                                 const float *v, int *ri, int *cp, float *cv)
{ matrix_transposition_f32(m, n, nnz, rp, ci, v, ri, cp, cv); }
inline void matrix_warp4(const int m, const int n, const int nnz, const int *rp, const int *ci,
                         const double *v, const int border, int *len, int *wn, double *wo, double *eo)
{ matrix_warp4_f64(m, n, nnz, rp, ci, v, border, len, wn, wo, eo); }
inline void matrix_warp4(const int m, const int n, const int nnz, const int *rp, const int *ci,
                         const float *v, const int border, int *len, int *wn, double *wo, double *eo)
{ matrix_warp4_f32(m, n, nnz, rp, ci, v, border, len, wn, wo, eo); }
inline void exclusive_scan(int *input, int length) { capsp_exclusive_scan(input, length); }
#endif /* CAPSP_COMPAT_HOST */

#else /* C11 */

#ifdef CAPSP_COMPAT_MIX
#define spts_syncfree_cuda_csr_wrt(r, c, v, ...)                                                  \
    _Generic((v), const float *: spts_syncfree_cuda_csr_wrt_mix_f32,                              \
             float *: spts_syncfree_cuda_csr_wrt_mix_f32,                                         \
             default: spts_syncfree_cuda_csr_wrt_mix_f64)(r, c, v, __VA_ARGS__)
#else
#define spts_syncfree_cuda_csr_wrt(r, c, v, ...)                                                  \
    _Generic((v), const float *: spts_syncfree_cuda_csr_wrt_f32,                                  \
             float *: spts_syncfree_cuda_csr_wrt_f32,                                             \
             default: spts_syncfree_cuda_csr_wrt_f64)(r, c, v, __VA_ARGS__)
#endif
#define spts_syncfree_cuda_csr(r, c, v, ...)                                                      \
    _Generic((v), const float *: spts_syncfree_cuda_csr_f32, float *: spts_syncfree_cuda_csr_f32, \
             default: spts_syncfree_cuda_csr_f64)(r, c, v, __VA_ARGS__)
#define sptrsv_syncfree_cuda(cp, ri, cv, ...)                                                     \
    _Generic((cv), const float *: sptrsv_syncfree_cuda_f32, float *: sptrsv_syncfree_cuda_f32,    \
             default: sptrsv_syncfree_cuda_f64)(cp, ri, cv, __VA_ARGS__)

#ifdef CAPSP_COMPAT_HOST
#define change2tran(m, nnzA, rp, ci, v, ...)                                                      \
    _Generic((v), float *: change2tran_f32, default: change2tran_f64)(m, nnzA, rp, ci, v, __VA_ARGS__)
#define get_x_b(m, n, rp, ci, v, ...)                                                             \
    _Generic((v), const float *: get_x_b_f32, float *: get_x_b_f32,                               \
             default: get_x_b_f64)(m, n, rp, ci, v, __VA_ARGS__)
#define matrix_layer(m, n, nnz, rp, ci, v, ...)                                                   \
    _Generic((v), const float *: matrix_layer_f32, float *: matrix_layer_f32,                     \
             default: matrix_layer_f64)(m, n, nnz, rp, ci, v, __VA_ARGS__)
#define matrix_transposition(m, n, nnz, rp, ci, v, ...)                                           \
    _Generic((v), const float *: matrix_transposition_f32, float *: matrix_transposition_f32,     \
             default: matrix_transposition_f64)(m, n, nnz, rp, ci, v, __VA_ARGS__)
#define matrix_warp4(m, n, nnz, rp, ci, v, ...)                                                   \
    _Generic((v), const float *: matrix_warp4_f32, float *: matrix_warp4_f32,                     \
             default: matrix_warp4_f64)(m, n, nnz, rp, ci, v, __VA_ARGS__)
#define exclusive_scan(input, length) capsp_exclusive_scan(input, length)
#endif /* CAPSP_COMPAT_HOST */

#endif /* __cplusplus */

#endif /* CAPSP_COMPAT_H */
