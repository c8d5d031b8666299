// Reference-compatible benchmark drivers.  Each keeps the argument list,
// ownership and reporting contract of a CapelliniSpTRSV driver:
//   * host arrays in (read only); device memory allocated, used and freed here;
//   * the CSR drivers build x_ref = ones and b = L*x_ref themselves (get_x_b);
//   * capsp_compat_repeat() timed solves, averaged into *solve_time (ms);
//   * gflops = 2*nnz / (1e6*ms) and bandwidth = dataSize / (1e6*ms) with the
//     reference's byte formula;
//   * validation failure prints a message and reports solve_time = -1 and
//     zero throughput; a non-square matrix returns -1.
// Underneath they run the native analyse/solve path with the matching
// algorithm.  Timing uses CUDA events around each solve (fill + kernel).
#include "capsp.h"
#include "capsp_internal.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

static int g_repeat = 100;  // BENCH_REPEAT (CUDA/ourWrtFst/common.h:20-22)

extern "C" int capsp_compat_set_repeat(int repeat)
{
    const int prev = g_repeat;
    if (repeat >= 1)
        g_repeat = repeat;
    return prev;
}

extern "C" int capsp_compat_repeat(void) { return g_repeat; }

namespace {

template <typename T>
struct HostVec {
    T *p = nullptr;
    ~HostVec() { free(p); }
};

template <typename T>
void get_x_b_t(int m, int n, const int *rp, const int *ci, const T *v, T **x, T **b);
template <>
void get_x_b_t<double>(int m, int n, const int *rp, const int *ci, const double *v, double **x, double **b)
{
    get_x_b_f64(m, n, rp, ci, v, x, b);
}
template <>
void get_x_b_t<float>(int m, int n, const int *rp, const int *ci, const float *v, float **x, float **b)
{
    get_x_b_f32(m, n, rp, ci, v, x, b);
}

template <typename T>
constexpr int dtype_of();
template <>
constexpr int dtype_of<double>() { return CAPSP_R_64F; }
template <>
constexpr int dtype_of<float>() { return CAPSP_R_32F; }

// Shared body of the three CSR drivers.  pre_ms receives the host selector time
// (mix only).
template <typename T>
int csr_driver(const int *rowptr, const int *colidx, const T *val, int m, int n, int nnzL, int algorithm,
               double *solve_time, double *gflops, double *bandwidth, double *pre_ms,
               double *warp_occupy, double *element_occupy)
{
    if (m != n) {
        printf("This is not a square matrix, return.\n");
        return -1;
    }
    HostVec<T> x_ref, b;
    get_x_b_t<T>(m, n, rowptr, colidx, val, &x_ref.p, &b.p);
    if (!x_ref.p || !b.p) {
        printf("capsp: host allocation failed\n");
        return -2;
    }
    const int repeat = g_repeat;
    int len = 0;
    if (algorithm == CAPSP_ALG_MIX) {
        // the reference times its host selector BENCH_REPEAT times (mix/...:185-193)
        std::vector<int> table((size_t)m + 1);
        double wo = 0.0, eo = 0.0, tot = 0.0;
        for (int r = 0; r < repeat; ++r) {
            const auto t0 = std::chrono::steady_clock::now();
            len = capsp_mix_table(m, rowptr, 0, 32, 10, table.data(), &wo, &eo);
            tot += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        }
        if (pre_ms)
            *pre_ms = tot / repeat;
        if (warp_occupy)
            *warp_occupy = wo;
        if (element_occupy)
            *element_occupy = eo;
    }
    capsp_handle_t h = nullptr;
    if (capsp_analyse(n, nnzL, rowptr, colidx, val, dtype_of<T>(), CAPSP_FMT_CSR, CAPSP_LOWER, 0, &h) !=
        CAPSP_OK) {
        printf("capsp: %s\n", capsp_last_error());
        *solve_time = -1;
        *gflops = 0;
        *bandwidth = 0;
        return -3;
    }
    capsp_set_algorithm(h, algorithm);
    if (algorithm == CAPSP_ALG_MIX)
        capsp_set_mix_border(h, 10);
    T *d_b = nullptr, *d_x = nullptr;
    std::vector<T> x((size_t)n);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool ok = cudaMalloc(&d_b, sizeof(T) * (size_t)n) == cudaSuccess &&
              cudaMalloc(&d_x, sizeof(T) * (size_t)n) == cudaSuccess &&
              cudaMemcpy(d_b, b.p, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
    double total_ms = 0.0;
    int passed = 0;
    for (int r = 0; ok && r < repeat; ++r) {
        cudaEventRecord(e0, 0);
        ok = capsp_solve(h, d_b, d_x, 1, 1, 0) == CAPSP_OK;
        cudaEventRecord(e1, 0);
        ok = ok && cudaEventSynchronize(e1) == cudaSuccess;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        total_ms += ms;
        ok = ok && capsp_status_sync(h, 0) == CAPSP_OK;
        ok = ok && cudaMemcpy(x.data(), d_x, sizeof(T) * (size_t)n, cudaMemcpyDeviceToHost) == cudaSuccess;
        int errs = 0;
        for (int i = 0; ok && i < n; ++i)
            if (std::fabs((double)x_ref.p[i] - (double)x[i]) > 0.01 * std::fabs((double)x_ref.p[i]))
                ++errs;
        if (ok && !errs)
            ++passed;
    }
    if (!ok)
        printf("capsp: %s\n", capsp_last_error());
    const double ms = total_ms / repeat;
    double data = (double)(n + 1) * sizeof(int) + (double)(nnzL + m) * sizeof(int) + (double)nnzL * sizeof(T) +
                  2.0 * n * sizeof(T);
    if (algorithm == CAPSP_ALG_MIX)
        data += (double)len * sizeof(int);  // mix/spts_syncfree_cuda_csr_wrt.h:305
    *solve_time = ms;
    *gflops = 2.0 * nnzL / (1e6 * ms);
    *bandwidth = data / (1e6 * ms);
    if (passed != repeat) {
        printf("cuda syncfree SpTS on L failed!\n");
        *solve_time = -1;
        *gflops = 0;
        *bandwidth = 0;
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    cudaFree(d_b);
    cudaFree(d_x);
    capsp_destroy(h);
    return 0;
}

template <typename T>
int csc_driver(const int *colptr, const int *rowidx, const T *val, int m, int n, int nnz, T *x, const T *b,
               const T *x_ref, double *pre_time, double *solve_time, double *gflops, double *bandwidth)
{
    if (m != n) {
        printf("This is not a square matrix, return.\n");
        return -1;
    }
    const int repeat = g_repeat;
    capsp_handle_t h = nullptr;
    if (capsp_analyse(n, nnz, colptr, rowidx, val, dtype_of<T>(), CAPSP_FMT_CSC, CAPSP_LOWER, 0, &h) !=
        CAPSP_OK) {
        printf("capsp: %s\n", capsp_last_error());
        *solve_time = -1;
        return -3;
    }
    T *d_b = nullptr, *d_x = nullptr;
    int *d_deg = nullptr, *d_idx = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool ok = cudaMalloc(&d_b, sizeof(T) * (size_t)n) == cudaSuccess &&
              cudaMalloc(&d_x, sizeof(T) * (size_t)n) == cudaSuccess &&
              cudaMalloc(&d_deg, sizeof(int) * (size_t)n) == cudaSuccess &&
              cudaMalloc(&d_idx, sizeof(int) * (size_t)nnz) == cudaSuccess &&
              cudaMemcpy(d_b, b, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(d_idx, rowidx, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
    // analysis time: the in-degree histogram, averaged like the reference (:151-166)
    double pre = 0.0;
    for (int r = 0; ok && r < repeat; ++r) {
        cudaEventRecord(e0, 0);
        ok = cudaMemsetAsync(d_deg, 0, sizeof(int) * (size_t)n, 0) == cudaSuccess &&
             capsp::launch_histogram(d_idx, nnz, d_deg, 0) == cudaSuccess;
        cudaEventRecord(e1, 0);
        ok = ok && cudaEventSynchronize(e1) == cudaSuccess;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        pre += ms;
    }
    *pre_time = pre / repeat;
    double total_ms = 0.0;
    for (int r = 0; ok && r < repeat; ++r) {
        cudaEventRecord(e0, 0);
        ok = capsp_solve(h, d_b, d_x, 1, 1, 0) == CAPSP_OK;
        cudaEventRecord(e1, 0);
        ok = ok && cudaEventSynchronize(e1) == cudaSuccess;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        total_ms += ms;
    }
    ok = ok && capsp_status_sync(h, 0) == CAPSP_OK;
    ok = ok && cudaMemcpy(x, d_x, sizeof(T) * (size_t)n, cudaMemcpyDeviceToHost) == cudaSuccess;
    if (!ok)
        printf("capsp: %s\n", capsp_last_error());
    const double ms = total_ms / repeat;
    const double data = (double)(n + 1) * sizeof(int) + (double)(nnz + n) * sizeof(int) +
                        (double)nnz * sizeof(T) + 2.0 * n * sizeof(T);
    *solve_time = ms;
    *gflops = 2.0 * nnz / (1e6 * ms);
    *bandwidth = data / (1e6 * ms);
    // L1 relative error check, spts_syncfree_cuda2.h:245-264
    double ref = 0.0, res = 0.0;
    for (int i = 0; ok && i < n; ++i) {
        ref += std::fabs((double)x_ref[i]);
        res += std::fabs((double)x[i] - (double)x_ref[i]);
    }
    res = ref == 0.0 ? res : res / ref;
    if (!ok || !(res < 1e-4)) {
        printf("cuda syncfree SpTRSV executor _NOT_ passed! |x-xref|/|xref| = %8.2e\n", res);
        *solve_time = -1;
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    cudaFree(d_b);
    cudaFree(d_x);
    cudaFree(d_deg);
    cudaFree(d_idx);
    capsp_destroy(h);
    return 0;
}

}  // namespace

#define CSR_DRIVER(NAME, T, ALG)                                                                         \
    extern "C" int NAME(const int *csrRowPtrL_tmp, const int *csrColIdxL_tmp, const T *csrValL_tmp,      \
                        const int m, const int n, const int nnzL, double *solve_time_add,                \
                        double *gflops_add, double *bandwith_add)                                        \
    {                                                                                                    \
        return csr_driver<T>(csrRowPtrL_tmp, csrColIdxL_tmp, csrValL_tmp, m, n, nnzL, ALG,               \
                             solve_time_add, gflops_add, bandwith_add, nullptr, nullptr, nullptr);       \
    }

CSR_DRIVER(spts_syncfree_cuda_csr_wrt_f64, double, CAPSP_ALG_WRTFST)
CSR_DRIVER(spts_syncfree_cuda_csr_wrt_f32, float, CAPSP_ALG_WRTFST)
CSR_DRIVER(spts_syncfree_cuda_csr_f64, double, CAPSP_ALG_TWOPART)
CSR_DRIVER(spts_syncfree_cuda_csr_f32, float, CAPSP_ALG_TWOPART)

#define MIX_DRIVER(NAME, T)                                                                              \
    extern "C" int NAME(const int *csrRowPtrL_tmp, const int *csrColIdxL_tmp, const T *csrValL_tmp,      \
                        const int m, const int n, const int nnzL, double *solve_time_add,                \
                        double *gflops_add, double *bandwith_add, double *pre_time_add,                  \
                        double *warp_occupy_add, double *element_occupy_add)                             \
    {                                                                                                    \
        return csr_driver<T>(csrRowPtrL_tmp, csrColIdxL_tmp, csrValL_tmp, m, n, nnzL, CAPSP_ALG_MIX,     \
                             solve_time_add, gflops_add, bandwith_add, pre_time_add, warp_occupy_add,    \
                             element_occupy_add);                                                        \
    }

MIX_DRIVER(spts_syncfree_cuda_csr_wrt_mix_f64, double)
MIX_DRIVER(spts_syncfree_cuda_csr_wrt_mix_f32, float)

#define CSC_DRIVER(NAME, T)                                                                              \
    extern "C" int NAME(const int *cscColPtrTR, const int *cscRowIdxTR, const T *cscValTR, const int m,  \
                        const int n, const int nnzTR, T *x, const T *b, const T *x_ref,                  \
                        double *pre_time_add, double *solve_time_add, double *gflops_add,                \
                        double *bandwidth_add)                                                           \
    {                                                                                                    \
        return csc_driver<T>(cscColPtrTR, cscRowIdxTR, cscValTR, m, n, nnzTR, x, b, x_ref, pre_time_add, \
                             solve_time_add, gflops_add, bandwidth_add);                                 \
    }

CSC_DRIVER(sptrsv_syncfree_cuda_f64, double)
CSC_DRIVER(sptrsv_syncfree_cuda_f32, float)
