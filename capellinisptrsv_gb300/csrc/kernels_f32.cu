// Explicit instantiation of the solve kernels for VALUE_TYPE float.  One
// translation unit per value type so the two compile in parallel.
#include "kernels_col.cuh"
#include "kernels_row.cuh"

namespace capsp {

template cudaError_t launch_row_solve<float>(const RowArgs<float> &, int, int, int, int, int, bool, bool,
                                                cudaStream_t);
template cudaError_t launch_col_solve<float>(const ColArgs<float> &, int, int, int, cudaStream_t);
template cudaError_t launch_fill_pending<float>(float *, int, int, long long, unsigned *, int, int *,
                                              cudaStream_t);
template cudaError_t launch_inv_diag<float>(const int *, const float *, float *, int, int, int *, cudaStream_t);
template cudaError_t launch_level_values<float>(const int *, const int *, const int *, int, const float *, float *, float *, int *, cudaStream_t);
template cudaError_t launch_grad_val<float>(const int *, const int *, const float *, const float *, float *, int,
                                          int, long long, int, cudaStream_t);

}  // namespace capsp
