// Structure checks and the in-degree histogram (type independent).
#include "capsp_internal.h"

namespace capsp {

// One thread per row/column: pointer order, diagonal position and the side of
// the diagonal every other index lies on.  Records the first bad row in *bad.
__global__ void validate_kernel(const int *__restrict__ ptr, const int *__restrict__ idx, int n,
                                int nnz, int diag_last, int *bad)
{
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long ii = tid; ii < n; ii += stride) {
        const int i = (int)ii;
        const int s = ptr[i], e = ptr[i + 1];
        bool ok = s >= 0 && e > s && e <= nnz;
        if (i == 0 && s != 0)
            ok = false;
        if (i == n - 1 && e != nnz)
            ok = false;
        if (ok) {
            const int dpos = diag_last ? e - 1 : s;
            ok = idx[dpos] == i;
            for (int j = s; ok && j < e; ++j) {
                if (j == dpos)
                    continue;
                const int c = idx[j];
                ok = diag_last ? (c >= 0 && c < i) : (c > i && c < n);
            }
        }
        if (!ok)
            atomicMin(bad, i);
    }
}

cudaError_t launch_validate(const int *ptr, const int *idx, int n, int nnz, int diag_last, int *bad,
                            cudaStream_t st)
{
    long long blocks = ((long long)n + 255) / 256;
    if (blocks > 8192)
        blocks = 8192;
    validate_kernel<<<(unsigned)blocks, 256, 0, st>>>(ptr, idx, n, nnz, diag_last, bad);
    return cudaGetLastError();
}

// In-degree analyser (CUDA/SyncFree_csc/spts_syncfree_cuda2.h:10-21).
__global__ void histogram_kernel(const int *__restrict__ idx, int nnz, int *out)
{
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = tid; k < nnz; k += stride)
        atomicAdd(out + idx[k], 1);
}

cudaError_t launch_histogram(const int *idx, int nnz, int *out, cudaStream_t st)
{
    long long blocks = ((long long)nnz + 255) / 256;
    if (blocks > 8192)
        blocks = 8192;
    if (blocks < 1)
        blocks = 1;
    histogram_kernel<<<(unsigned)blocks, 256, 0, st>>>(idx, nnz, out);
    return cudaGetLastError();
}

}  // namespace capsp
