// Explicit instantiation of the solve kernels for VALUE_TYPE double.  One
// translation unit per value type so the two compile in parallel.
#include "kernels_col.cuh"
#include "kernels_row.cuh"

namespace capsp {

template cudaError_t launch_row_solve<double>(const RowArgs<double> &, int, int, int, int, int, bool, bool,
                                                cudaStream_t);
template cudaError_t launch_col_solve<double>(const ColArgs<double> &, int, int, int, cudaStream_t);
template cudaError_t launch_fill_pending<double>(double *, int, int, long long, unsigned *, int, int *,
                                              cudaStream_t);
template cudaError_t launch_inv_diag<double>(const int *, const double *, double *, int, int, int *, cudaStream_t);
template cudaError_t launch_level_values<double>(const int *, const int *, const int *, int, const double *, double *, double *, int *, cudaStream_t);
template cudaError_t launch_grad_val<double>(const int *, const int *, const double *, const double *, double *, int,
                                          int, long long, int, cudaStream_t);

}  // namespace capsp
