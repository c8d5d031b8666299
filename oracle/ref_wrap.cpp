// ORACLE -- test infrastructure.  Wrapper translation unit compiled directly
// against the reference's own headers where they lie (the recipe in
// oracle/Makefile passes -I to the reference directory); no reference source
// is copied into this repository.  It exports the reference's serial solve
// and host preprocessing under C names so tests can compare the oracle
// restatement and the product's host code against the reference itself.
//
//   REF_SERIAL: openCL/SynFree_csc/{common.h, tranpose.h, sptrsv_syncfree_serialref.h}
//   REF_PRE:    CUDA/mix/{common.h, mmio.h, read_mtx.h, tranpose.h}
//               (byte-identical to the CUDA/ourWrtFst copies of those helpers)
//
// Built twice per group, with -DVALUE_TYPE=double -DREF_SFX=_f64 and with
// -DVALUE_TYPE=float -DREF_SFX=_f32.
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <time.h>

#include <iostream>

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define REFN(name) CAT(ref_##name, REF_SFX)

#if defined(REF_SERIAL)
#include "common.h"
#include "tranpose.h"
#include "sptrsv_syncfree_serialref.h"

extern "C" int REFN(executor)(const int *colptr, const int *rowidx, const VALUE_TYPE *val,
                              const int *indeg, int m, int n, int substitution, int rhs,
                              const VALUE_TYPE *b, VALUE_TYPE *x)
{
    return sptrsv_syncfree_executor(colptr, rowidx, val, indeg, m, n, substitution, rhs, b, x);
}

extern "C" int REFN(analyser)(const int *rowidx, int m, int n, int nnz, int *histo)
{
    return sptrsv_syncfree_analyser(rowidx, m, n, nnz, histo);
}

extern "C" void REFN(transposition)(int m, int n, int nnz, const int *rowptr, const int *colidx,
                                    const VALUE_TYPE *val, int *cscRowIdx, int *cscColPtr,
                                    VALUE_TYPE *cscVal)
{
    matrix_transposition(m, n, nnz, rowptr, colidx, val, cscRowIdx, cscColPtr, cscVal);
}

#elif defined(REF_PRE)
#include "common.h"
#include "mmio.h"
#include "read_mtx.h"
#include "tranpose.h"

extern "C" void REFN(change2tran)(int m, int nnzA, int *rowptrA, int *colidxA, VALUE_TYPE *valA,
                                  int *nnzL, int **rowptrL, int **colidxL, VALUE_TYPE **valL)
{
    change2tran(m, nnzA, rowptrA, colidxA, valA, nnzL, rowptrL, colidxL, valL);
}

extern "C" void REFN(get_x_b)(int m, int n, const int *rowptr, const int *colidx,
                              const VALUE_TYPE *val, VALUE_TYPE **x, VALUE_TYPE **b)
{
    get_x_b(m, n, rowptr, colidx, val, x, b);
}

extern "C" int REFN(matrix_layer)(int m, int n, int nnz, const int *rowptr, const int *colidx,
                                  const VALUE_TYPE *val, int *layer, double *parallelism)
{
    return matrix_layer(m, n, nnz, rowptr, colidx, val, layer, parallelism);
}

extern "C" void REFN(matrix_transposition)(int m, int n, int nnz, const int *rowptr,
                                           const int *colidx, const VALUE_TYPE *val,
                                           int *cscRowIdx, int *cscColPtr, VALUE_TYPE *cscVal)
{
    matrix_transposition(m, n, nnz, rowptr, colidx, val, cscRowIdx, cscColPtr, cscVal);
}

extern "C" void REFN(matrix_warp4)(int m, int n, int nnz, const int *rowptr, const int *colidx,
                                   const VALUE_TYPE *val, int border, int *len, int *warp_num,
                                   double *warp_occupy, double *element_occupy)
{
    matrix_warp4(m, n, nnz, rowptr, colidx, val, border, len, warp_num, warp_occupy,
                 element_occupy);
}

extern "C" int REFN(read_mtx)(char *filename, int *m, int *n, int *nnz, int **rowptr, int **colidx,
                              VALUE_TYPE **val)
{
    return read_mtx(filename, m, n, nnz, rowptr, colidx, val);
}

extern "C" void REFN(free)(void *p) { free(p); }

#else
#error "define REF_SERIAL or REF_PRE"
#endif
