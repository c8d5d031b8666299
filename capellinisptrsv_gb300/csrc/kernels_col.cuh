// Column-driven sync-free triangular solve for sm_103a: one warp per column,
// the SyncFree design of sptrsv_syncfree_cuda_executor_update
// (CUDA/SyncFree_csc/spts_syncfree_cuda2.h:24-86) and of the serial executor
// (openCL/SynFree_csc/sptrsv_syncfree_serialref.h:25-108).
//
// A column j waits until every other entry of its row has been scattered
// (arrived[j] == indeg[j] - 1), computes x_j = (b_j - left_sum_j) * (1/diag),
// then scatters x_j * L_rj into left_sum[r] for the column's off-diagonal
// rows and counts them in arrived[r].  FORWARD visits columns 0..n-1 with the
// diagonal first in each column; BACKWARD visits n-1..0 with the diagonal
// last.  BACKWARD on the CSR arrays of a lower-triangular L is the transpose
// solve L^T y = g without building L^T: row i of L is column i of L^T.
//
// Differences from the reference kernel:
//   * counters count up from zero (no in-degree restore copy per solve);
//   * every waiting lane performs its own acquire load, then reads left_sum
//     through L2; producers issue all their fp64 reductions, one fence, a
//     warp barrier, then the counter increments;
//   * multi-RHS: G = next_pow2(nrhs) lanes per entry, one right-hand side
//     each; 32/G entries per warp pass;
//   * optional fused gradient: while column j's values y_j are in registers
//     the warp also writes grad_val[k] = -sum_r y[j,r] * xf[idx[k], r] for
//     every stored entry k of the column (diagonal included);
//   * bounded waits with the same Spin budget as the row kernels.
#pragma once

#include "capsp_internal.h"

namespace capsp {

// A target's partial sum and arrival count for one right-hand side, kept in one
// atomic word: FP64 {sum bits, count} in 16 bytes, FP32 {count << 32 | sum
// bits} in 8.  A producer's contribution is one compare-and-swap (sum + c,
// count + 1), so the consumer that sees the full count holds the final sum in
// the same read: no left_sum read after the wait and no fence between the
// producer's sum and its count.
template <typename T>
struct SumCount;

template <>
struct SumCount<double> {
    typedef ulonglong2 W;
    // atomic read: a compare that never matches (no count is all ones)
    static __device__ __forceinline__ W read(W *p)
    {
        return cas128(p, make_ulonglong2(0ull, ~0ull), make_ulonglong2(0ull, ~0ull));
    }
    // the producer's first guess of the current value (a torn read only costs a retry)
    static __device__ __forceinline__ W guess(const W *p)
    {
        W r;
        asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(r.x), "=l"(r.y) : "l"(p));
        return r;
    }
    static __device__ __forceinline__ double sum(W w) { return __longlong_as_double((long long)w.x); }
    static __device__ __forceinline__ unsigned long long count(W w) { return w.y; }
    static __device__ __forceinline__ W add(W w, double c)
    {
        return make_ulonglong2((unsigned long long)__double_as_longlong(sum(w) + c), w.y + 1ull);
    }
    static __device__ __forceinline__ bool same(W a, W b) { return a.x == b.x && a.y == b.y; }
    static __device__ __forceinline__ W cas(W *p, W cmp, W val) { return cas128(p, cmp, val); }
};

template <>
struct SumCount<float> {
    typedef unsigned long long W;
    static __device__ __forceinline__ W read(W *p) { return ld_relaxed(p); }  // 8-byte single-copy atomic
    static __device__ __forceinline__ W guess(const W *p) { return ld_relaxed(p); }
    static __device__ __forceinline__ float sum(W w) { return __uint_as_float((unsigned)(w & 0xffffffffull)); }
    static __device__ __forceinline__ unsigned long long count(W w) { return w >> 32; }
    static __device__ __forceinline__ W add(W w, float c)
    {
        return ((count(w) + 1ull) << 32) | (unsigned long long)__float_as_uint(sum(w) + c);
    }
    static __device__ __forceinline__ bool same(W a, W b) { return a == b; }
    static __device__ __forceinline__ W cas(W *p, W cmp, W val) { return atomicCAS(p, cmp, val); }
};

// Column-driven solve on sum-and-count words (a.slots, zeroed before the
// launch, word (i, r) at i*lsld + r): the same schedule, waits and fused
// gradient as col_solve_kernel below.  A failed compare-and-swap means another
// producer of the same target succeeded, so a producer retries at most as
// often as the target has producers; kCasRetries only backstops that bound.
// entry passes whose guesses are fetched before the wait: enough for columns of
// 8 entries or more at every width (one pass covers 32/G entries), no more, so
// the narrow builds keep their registers (1 RHS: 1.54 -> 1.48 ms on grad_1m)
constexpr int kCasPassesMax = 4;
constexpr int kCasRetries = 1 << 20;

template <typename T, int G>
__global__ void __launch_bounds__(512) col_solve_packed_kernel(const ColArgs<T> a)
{
    typedef VBits<T> VB;
    typedef SumCount<T> SC;
    typedef typename SC::W W;
    constexpr int EPW = 32 / G;
    constexpr int kCasPasses = G >= 8 ? kCasPassesMax : (G >= 2 ? 2 : 1);
    const int lane = threadIdx.x & 31;
    const int es = lane / G, g = lane % G;
    const bool active = g < a.nrhs;
    W *slots = reinterpret_cast<W *>(a.slots);
    for (;;) {
        unsigned tk = 0, stop = 0;
        if (lane == 0) {
            tk = atomicAdd(a.ticket, 1u);
            stop = ld_relaxed(reinterpret_cast<const unsigned *>(a.err));
        }
        tk = __shfl_sync(kFullMask, tk, 0);
        stop = __shfl_sync(kFullMask, stop, 0);
        if (stop || tk >= (unsigned)a.n)
            break;
        const int j = a.order != nullptr ? __ldg(a.order + tk) : (a.backward ? a.n - 1 - (int)tk : (int)tk);
        const int s0 = __ldg(a.ptr + j), e0 = __ldg(a.ptr + j + 1);
        const int s = a.backward ? s0 : s0 + 1;
        const int e = a.backward ? e0 - 1 : e0;
        const int need = __ldg(a.indeg + j) - 1;
        const T dinv = __ldg(a.inv_diag + j);
        // before the wait: the first passes of entries, each target word's
        // current value as the compare-and-swap guess, and the fused gradient's
        // first x value
        int rr[kCasPasses];
        T vv[kCasPasses];
        W gw[kCasPasses];
#pragma unroll
        for (int q = 0; q < kCasPasses; ++q) {
            const int k = s + es + q * EPW;
            rr[q] = 0;
            vv[q] = T(0);
            gw[q] = W();
            if (k < e) {
                rr[q] = __ldg(a.idx + k);
                vv[q] = __ldg(a.val + k);
                if (active)
                    gw[q] = SC::guess(slots + (size_t)rr[q] * (size_t)a.lsld + g);
            }
        }
        const int kg1 = s0 + es;
        T xg1 = T(0);
        if (a.grad_val != nullptr && kg1 < e0 && active)
            xg1 = __ldg(a.xf + (size_t)__ldg(a.idx + kg1) * (size_t)a.ld + g);
        bool aborted = false;
        T xj = T(0);
        if (es == 0 && active) {
            const size_t xo = (size_t)j * (size_t)a.ld + g;
            const T bj = __ldg(a.b + xo);
            T ls = T(0);
            if (need > 0) {
                W *mine = slots + (size_t)j * (size_t)a.lsld + g;
                Spin sp;
                W w = SC::read(mine);
                while (SC::count(w) != (unsigned long long)need) {
                    if (sp.next(a.err, a.wait, j, j)) {
                        aborted = true;
                        break;
                    }
                    w = SC::read(mine);
                }
                ls = SC::sum(w);
            }
            xj = aborted ? VB::from(VB::kQNaN) : (bj - ls) * dinv;
            a.x[xo] = xj;
        }
        xj = __shfl_sync(kFullMask, xj, g);
        if (j != a.stuck_row && active) {
            // all prefetched passes' compare-and-swaps in flight together,
            // then the (rare) retries
            W got[kCasPasses];
#pragma unroll
            for (int q = 0; q < kCasPasses; ++q) {
                got[q] = W();
                if (s + es + q * EPW < e)
                    got[q] = SC::cas(slots + (size_t)rr[q] * (size_t)a.lsld + g, gw[q], SC::add(gw[q], xj * vv[q]));
            }
#pragma unroll
            for (int q = 0; q < kCasPasses; ++q) {
                if (s + es + q * EPW < e && !SC::same(got[q], gw[q])) {
                    W *p = slots + (size_t)rr[q] * (size_t)a.lsld + g;
                    W old = got[q];
                    for (int it = 0;; ++it) {
                        const W now = SC::cas(p, old, SC::add(old, xj * vv[q]));
                        if (SC::same(now, old))
                            break;
                        old = now;
                        if (it > kCasRetries) {
                            if (atomicCAS(a.err + kErrStatus, 0, kStatusTimeout) == 0) {
                                a.err[kErrRow] = rr[q];
                                a.err[kErrWaitedOn] = j;
                            }
                            break;
                        }
                    }
                }
            }
            // passes beyond the prefetched ones: guess, then compare-and-swap
            for (int k = s + es + kCasPasses * EPW; k < e; k += EPW) {
                W *p = slots + (size_t)__ldg(a.idx + k) * (size_t)a.lsld + g;
                const T c = xj * __ldg(a.val + k);
                W old = SC::guess(p);
                for (int it = 0;; ++it) {
                    const W now = SC::cas(p, old, SC::add(old, c));
                    if (SC::same(now, old))
                        break;
                    old = now;
                    if (it > kCasRetries) {
                        if (atomicCAS(a.err + kErrStatus, 0, kStatusTimeout) == 0) {
                            a.err[kErrRow] = (int)(p - slots) / (int)a.lsld;
                            a.err[kErrWaitedOn] = j;
                        }
                        break;
                    }
                }
            }
        }
        __syncwarp();
        if (a.grad_val != nullptr) {
            for (int kb = s0; kb < e0; kb += EPW) {
                const int k = kb + es;
                T prod = T(0);
                if (k < e0 && active)
                    prod = xj * (k == kg1 ? xg1 : __ldg(a.xf + (size_t)__ldg(a.idx + k) * (size_t)a.ld + g));
#pragma unroll
                for (int off = G / 2; off >= 1; off >>= 1)
                    prod += __shfl_xor_sync(kFullMask, prod, off);
                if (k < e0 && g == 0)
                    a.grad_val[k] = a.grad_accumulate ? a.grad_val[k] - prod : -prod;
            }
        }
    }
}

template <typename T, int G>
__global__ void __launch_bounds__(512) col_solve_kernel(const ColArgs<T> a)
{
    typedef VBits<T> VB;
    typedef typename VB::U U;
    constexpr int EPW = 32 / G;
    const int lane = threadIdx.x & 31;
    const int es = lane / G, g = lane % G;
    const bool active = g < a.nrhs;
    for (;;) {
        unsigned tk = 0, stop = 0;
        if (lane == 0) {
            tk = atomicAdd(a.ticket, 1u);
            stop = ld_relaxed(reinterpret_cast<const unsigned *>(a.err));
        }
        tk = __shfl_sync(kFullMask, tk, 0);
        stop = __shfl_sync(kFullMask, stop, 0);
        if (stop || tk >= (unsigned)a.n)
            break;
        const int j = a.order != nullptr ? __ldg(a.order + tk) : (a.backward ? a.n - 1 - (int)tk : (int)tk);
        const int s0 = __ldg(a.ptr + j), e0 = __ldg(a.ptr + j + 1);
        const int s = a.backward ? s0 : s0 + 1;
        const int e = a.backward ? e0 - 1 : e0;
        const int need = __ldg(a.indeg + j) - 1;
        const T dinv = __ldg(a.inv_diag + j);
        // the column's first pass of entries (and, for the fused gradient, the
        // x values they pair with) do not depend on readiness: fetch them
        // before the wait so the work after the last arrival hits registers
        const int k1 = s + es;
        int r1 = 0;
        T v1 = T(0);
        if (k1 < e) {
            r1 = __ldg(a.idx + k1);
            v1 = __ldg(a.val + k1);
        }
        const int kg1 = s0 + es;
        T xg1 = T(0);
        if (a.grad_val != nullptr && kg1 < e0 && active)
            xg1 = __ldg(a.xf + (size_t)__ldg(a.idx + kg1) * (size_t)a.ld + g);
        bool aborted = false;
        T xj = T(0);
        if (es == 0 && active) {
            const size_t xo = (size_t)j * (size_t)a.ld + g;
            const T bj = __ldg(a.b + xo);
            Spin sp;
            while (ld_acquire(a.arrived + j) != need) {
                if (sp.next(a.err, a.wait, j, j)) {
                    aborted = true;
                    break;
                }
            }
            const T ls = VB::from(ld_relaxed(reinterpret_cast<const U *>(a.left_sum) +
                                             (size_t)j * (size_t)a.lsld + g));
            xj = aborted ? VB::from(VB::kQNaN) : (bj - ls) * dinv;
            a.x[xo] = xj;
        }
        xj = __shfl_sync(kFullMask, xj, g);
        if (j != a.stuck_row) {
            for (int k = k1; k < e; k += EPW) {
                const int r = k == k1 ? r1 : __ldg(a.idx + k);
                const T v = k == k1 ? v1 : __ldg(a.val + k);
                if (active)
                    atomicAdd(a.left_sum + (size_t)r * (size_t)a.lsld + g, xj * v);
            }
            __threadfence();
            __syncwarp();
            if (g == 0) {
                for (int k = k1; k < e; k += EPW)
                    atomicAdd(a.arrived + (k == k1 ? r1 : __ldg(a.idx + k)), 1);
            }
        }
        if (a.grad_val != nullptr) {
            for (int kb = s0; kb < e0; kb += EPW) {
                const int k = kb + es;
                T prod = T(0);
                if (k < e0 && active)
                    prod = xj * (k == kg1 ? xg1 : __ldg(a.xf + (size_t)__ldg(a.idx + k) * (size_t)a.ld + g));
#pragma unroll
                for (int off = G / 2; off >= 1; off >>= 1)
                    prod += __shfl_xor_sync(kFullMask, prod, off);
                if (k < e0 && g == 0)
                    a.grad_val[k] = a.grad_accumulate ? a.grad_val[k] - prod : -prod;
            }
        }
    }
}

template <typename T, int G>
static cudaError_t launch_col_impl(const ColArgs<T> &a, int block, int bps, int num_sms,
                                   cudaStream_t st)
{
    auto kern = a.slots != nullptr ? col_solve_packed_kernel<T, G> : col_solve_kernel<T, G>;
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, block, 0);
    if (e != cudaSuccess)
        return e;
    if (occ < 1)
        occ = 1;
    const int per_sm = (bps > 0 && bps < occ) ? bps : occ;
    long long grid = (long long)per_sm * num_sms;
    const long long need = ((long long)a.n + block / 32 - 1) / (block / 32);
    if (grid > need)
        grid = need;
    if (grid < 1)
        grid = 1;
    kern<<<(unsigned)grid, block, 0, st>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_col_solve(const ColArgs<T> &a, int block, int blocks_per_sm, int num_sms,
                             cudaStream_t st)
{
    switch (lanes_for_rhs(a.nrhs)) {
    case 1: return launch_col_impl<T, 1>(a, block, blocks_per_sm, num_sms, st);
    case 2: return launch_col_impl<T, 2>(a, block, blocks_per_sm, num_sms, st);
    case 4: return launch_col_impl<T, 4>(a, block, blocks_per_sm, num_sms, st);
    case 8: return launch_col_impl<T, 8>(a, block, blocks_per_sm, num_sms, st);
    case 16: return launch_col_impl<T, 16>(a, block, blocks_per_sm, num_sms, st);
    default: return launch_col_impl<T, 32>(a, block, blocks_per_sm, num_sms, st);
    }
}

// ---------------------------------------------------------------------------
// analysis helpers and the standalone gradient
// ---------------------------------------------------------------------------

template <typename T>
__global__ void inv_diag_kernel(const int *__restrict__ ptr, const T *__restrict__ val,
                                T *__restrict__ inv, int n, int diag_last, int *bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int pos = diag_last ? ptr[i + 1] - 1 : ptr[i];
    const T d = val[pos];
    if (!(d != T(0)) || !isfinite(d))
        atomicMin(bad, i);
    inv[i] = T(1) / d;
}

template <typename T>
cudaError_t launch_inv_diag(const int *ptr, const T *val, T *inv, int n, int diag_last, int *bad,
                            cudaStream_t st)
{
    inv_diag_kernel<T><<<(n + 255) / 256, 256, 0, st>>>(ptr, val, inv, n, diag_last, bad);
    return cudaGetLastError();
}

// 16-byte vector of T (the rows of own/other are read in these when every
// row starts on a 16-byte boundary)
template <typename T>
struct Vec16;
template <>
struct Vec16<double> {
    typedef double2 V;
    static constexpr int W = 2;
    static __device__ __forceinline__ void put(V v, double *r)
    {
        r[0] = v.x;
        r[1] = v.y;
    }
};
template <>
struct Vec16<float> {
    typedef float4 V;
    static constexpr int W = 4;
    static __device__ __forceinline__ void put(V v, float *r)
    {
        r[0] = v.x;
        r[1] = v.y;
        r[2] = v.z;
        r[3] = v.w;
    }
};

// r[0..NR) = p[0..nrhs), zero beyond nrhs; VEC: nrhs == NR, 16-byte aligned
template <typename T, int NR, bool VEC>
__device__ __forceinline__ void load_rhs(const T *__restrict__ p, int nrhs, T (&r)[NR])
{
    if (VEC) {
        typedef Vec16<T> VT;
#pragma unroll
        for (int v = 0; v < NR / VT::W; ++v)
            VT::put(__ldg(reinterpret_cast<const typename VT::V *>(p) + v), r + v * VT::W);
    } else {
#pragma unroll
        for (int q = 0; q < NR; ++q)
            r[q] = q < nrhs ? __ldg(p + q) : T(0);
    }
}

// grad[k] = -sum_r own[i, r] * other[idx[k], r] for every stored entry k of
// row i.  A warp takes 32 consecutive rows and walks their entries one per
// lane (each lane finds its entry's row among the group's row starts), so
// every lane does the same work: each entry's sum over the right-hand sides
// is one FMA chain in its lane, and the FP64 pipe -- the bound on GB300 --
// issues no instruction for idle lanes.  (One thread per row idles the lanes
// of short rows while the warp's longest row finishes: grad_1m with 16 RHS
// 0.357 -> 0.268 ms, wide_4m 1.37 -> 0.743 ms; lanes split by right-hand
// side add a shuffle reduction per entry: 0.58 ms.)
template <typename T, int NR, bool VEC>
__global__ void __launch_bounds__(256) grad_val_kernel(const int *__restrict__ rowptr,
                                                       const int *__restrict__ colidx,
                                                       const T *__restrict__ own, const T *__restrict__ other,
                                                       T *__restrict__ grad, int n, int nrhs, long long ld,
                                                       int accumulate)
{
    const int lane = threadIdx.x & 31;
    const long long r0 = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
    if (r0 >= n)
        return;
    const int nr = (int)min(32LL, (long long)n - r0);
    const int start = lane < nr ? __ldg(rowptr + r0 + lane) : INT_MAX;
    const int eb = __shfl_sync(kFullMask, start, 0);
    const int ee = __ldg(rowptr + r0 + nr);
    for (int kb = eb; kb < ee; kb += 32) {
        const int k = kb + lane;
        const int l = group_row_of(start, k, nr);
        if (k < ee) {
            T yi[NR], xr[NR];
            load_rhs<T, NR, VEC>(own + (size_t)(r0 + l) * ld, nrhs, yi);
            load_rhs<T, NR, VEC>(other + (size_t)__ldg(colidx + k) * ld, nrhs, xr);
            T acc = T(0);
#pragma unroll
            for (int q = 0; q < NR; ++q)
                acc = fma(yi[q], xr[q], acc);
            grad[k] = accumulate ? grad[k] - acc : -acc;
        }
    }
}

template <typename T, int NR>
static cudaError_t launch_grad_nr(const int *rowptr, const int *colidx, const T *own, const T *other, T *grad,
                                  int n, int nrhs, long long ld, int accumulate, cudaStream_t st)
{
    const unsigned blocks = (unsigned)(((long long)n + 255) / 256);  // a warp per 32 rows
    const int w = Vec16<T>::W;
    const bool vec = NR % w == 0 && nrhs == NR && ld % w == 0 && ((uintptr_t)own & 15) == 0 &&
                     ((uintptr_t)other & 15) == 0;
    if (vec)
        grad_val_kernel<T, NR, (NR % Vec16<T>::W == 0)>
            <<<blocks, 256, 0, st>>>(rowptr, colidx, own, other, grad, n, nrhs, ld, accumulate);
    else
        grad_val_kernel<T, NR, false><<<blocks, 256, 0, st>>>(rowptr, colidx, own, other, grad, n, nrhs, ld,
                                                              accumulate);
    return cudaGetLastError();
}

// nrhs <= 32 right-hand sides, rows at stride ld
template <typename T>
cudaError_t launch_grad_val(const int *rowptr, const int *colidx, const T *own, const T *other,
                            T *grad_val, int n, int nrhs, long long ld, int accumulate,
                            cudaStream_t st)
{
    switch (lanes_for_rhs(nrhs)) {
    case 1: return launch_grad_nr<T, 1>(rowptr, colidx, own, other, grad_val, n, nrhs, ld, accumulate, st);
    case 2: return launch_grad_nr<T, 2>(rowptr, colidx, own, other, grad_val, n, nrhs, ld, accumulate, st);
    case 4: return launch_grad_nr<T, 4>(rowptr, colidx, own, other, grad_val, n, nrhs, ld, accumulate, st);
    case 8: return launch_grad_nr<T, 8>(rowptr, colidx, own, other, grad_val, n, nrhs, ld, accumulate, st);
    case 16: return launch_grad_nr<T, 16>(rowptr, colidx, own, other, grad_val, n, nrhs, ld, accumulate, st);
    default: return launch_grad_nr<T, 32>(rowptr, colidx, own, other, grad_val, n, nrhs, ld, accumulate, st);
    }
}

}  // namespace capsp
