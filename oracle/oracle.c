/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A CPU restatement of the reference's serial sync-free triangular solve,
 * used only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline to
 * check the CUDA path.  It follows, operation for operation and in the same
 * order, the serial executor of CapelliniSpTRSV:
 *
 *   sptrsv_syncfree_analyser   openCL/SynFree_csc/sptrsv_syncfree_serialref.h:6-23
 *   sptrsv_syncfree_executor   openCL/SynFree_csc/sptrsv_syncfree_serialref.h:25-108
 *     FORWARD  :44-72   (diagonal first in each CSC column)
 *     BACKWARD :73-102  (diagonal last in each column)
 *   matrix_transposition       CUDA/ourWrtFst/tranpose.h:36-75
 *
 * Compiled with -ffp-contract=off so that left_sum += x*v is a rounded product
 * followed by a rounded sum on every host (x86-64 and aarch64 alike), which
 * makes its results bit-identical to the reference executor compiled the same
 * way (checked by tests/test_oracle.py against oracle/_ref and the committed
 * golden vectors).
 *
 * Differences from the reference, none of which changes a result:
 *   - the executor's busy-wait on the simulated in-degree counter
 *     (serialref.h:51-56, :80-85) can only fail for a malformed matrix, where
 *     the reference spins forever; here it returns -1 instead;
 *   - buffers are caller-allocated.
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>

void oracle_analyser(const int *idx, int m, int nnz, int *histo)
{
    memset(histo, 0, sizeof(int) * (size_t)(m > 0 ? m : 1));
    for (int k = 0; k < nnz; ++k)
        histo[idx[k]]++;
}

#define OVT double
#define OSFX(x) x##_f64
#include "oracle_impl.h"
#undef OVT
#undef OSFX

#define OVT float
#define OSFX(x) x##_f32
#include "oracle_impl.h"
#undef OVT
#undef OSFX
