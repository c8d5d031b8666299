// Row-driven sync-free triangular solve kernels for sm_103a.
//
// One family covers the reference's three CSR executors:
//   * WRTFST  - thread per row, write-first: every lane polls all of its
//               row's dependencies and consumes whichever are ready
//               (CUDA/ourWrtFst/spts_syncfree_cuda_csr_wrt.h:10-57);
//   * TWOPART - thread per row, dependencies outside the warp's row chunk
//               awaited one by one in storage order, then the in-chunk ones
//               write-first (CUDA/our2Part/spts_syncfree_cuda_csr.h:10-124);
//   * MIX     - virtual warps from the selector table: a light group of rows
//               runs thread-per-row, a heavy row gets a whole warp with a
//               shuffle reduction (CUDA/mix/spts_syncfree_cuda_csr_wrt.h:15-137).
//
// GB300 design (what differs from the reference):
//   * Persistent grid sized from the SM count and occupancy; a warp takes
//     its next chunk of consecutive rows from one atomic ticket.  Rows are
//     therefore started in solve order by warps that are already running, so
//     the lowest unfinished row always has a running owner whose
//     dependencies are finished: forward progress needs no assumption about
//     block scheduling.  (The reference takes one ticket per thread and maps
//     lanes from threadIdx, mix/...:32-45.)
//   * Value-as-flag readiness (capsp_device.cuh): no flag array, no fence.
//   * Dependencies inside the warp's own chunk are read from a per-warp
//     shared-memory mirror of the chunk's x values instead of from L2.
//   * Each lane fetches up to kBatch column indices and values of its row
//     at once and keeps all of their polls in flight together.
//   * Partial sums are accumulated in storage (column) order whatever the
//     arrival order, so WRTFST and TWOPART produce bit-identical results.
//   * 1/diag is precomputed at analysis; x = (b - sum) * (1/diag).
//   * Multi-RHS: G = next_pow2(nrhs) lanes share a row, one right-hand side
//     each; every (row, rhs) element is published and polled independently.
//   * Every wait is bounded (Spin); a lane that gives up publishes a quiet
//     NaN so its dependants finish, and the error word records TIMEOUT.
#pragma once

#include "capsp_internal.h"

namespace capsp {

constexpr int kBatch = 8;  // dependencies one lane keeps in flight

template <typename T, int G, bool TWO>
__device__ __forceinline__ void thread_row(const RowArgs<T> &a, const int p, const int g,
                                           const int lo, volatile typename VBits<T>::U *cache)
{
    typedef VBits<T> VB;
    typedef typename VB::U U;
    const int i = a.upper ? a.n - 1 - p : p;
    int s = __ldg(a.ptr + i), e = __ldg(a.ptr + i + 1);
    if (a.upper)
        ++s;
    else
        --e;
    const size_t xo = (size_t)i * (size_t)a.ld + (size_t)g;
    const T bi = __ldg(a.b + xo);
    const T dinv = __ldg(a.inv_diag + i);
    const U *xb = reinterpret_cast<const U *>(a.x);
    T acc = T(0);
    bool aborted = false;
    for (int j0 = s; j0 < e && !aborted; j0 += kBatch) {
        const int cnt = min(kBatch, e - j0);
        int c[kBatch];
        T v[kBatch];
        U w[kBatch];
#pragma unroll
        for (int t = 0; t < kBatch; ++t) {
            c[t] = 0;
            v[t] = T(0);
            w[t] = 0;
            if (t < cnt) {
                c[t] = __ldg(a.idx + j0 + t);
                v[t] = __ldg(a.val + j0 + t);
            }
        }
        unsigned pend = (1u << cnt) - 1u;
        if (TWO) {
            // phase 1: dependencies outside this warp's chunk, one at a time
#pragma unroll
            for (int t = 0; t < kBatch; ++t) {
                if (!aborted && ((pend >> t) & 1u)) {
                    const int q = a.upper ? a.n - 1 - c[t] : c[t];
                    if (q < lo) {
                        const U *src = xb + (size_t)c[t] * (size_t)a.ld + g;
                        U u = ld_relaxed(src);
                        Spin sp;
                        while (u == VB::kPending) {
                            if (sp.next(a.err, a.wait, i, c[t])) {
                                aborted = true;
                                break;
                            }
                            u = ld_relaxed(src);
                        }
                        w[t] = u;
                        pend &= ~(1u << t);
                    }
                }
            }
        }
        // write-first: consume whichever dependencies are ready, re-poll the rest
        Spin sp;
        int waited = 0;
        while (pend && !aborted) {
#pragma unroll
            for (int t = 0; t < kBatch; ++t) {
                if ((pend >> t) & 1u) {
                    const int q = a.upper ? a.n - 1 - c[t] : c[t];
                    const U u = (q >= lo) ? cache[(q - lo) * G + g]
                                          : ld_relaxed(xb + (size_t)c[t] * (size_t)a.ld + g);
                    if (u != VB::kPending) {
                        w[t] = u;
                        pend &= ~(1u << t);
                    } else {
                        waited = c[t];
                    }
                }
            }
            if (pend && sp.next(a.err, a.wait, i, waited))
                aborted = true;
        }
#pragma unroll
        for (int t = 0; t < kBatch; ++t)
            if (t < cnt)
                acc = fma(v[t], VB::from(w[t]), acc);
    }
    U ub = aborted ? VB::kQNaN : VB::to((bi - acc) * dinv);
    if (ub == VB::kPending)
        ub = VB::kQNaN;
    if (i != a.stuck_row) {
        cache[(p - lo) * G + g] = ub;
        st_relaxed(reinterpret_cast<U *>(a.x) + xo, ub);
    }
}

// One heavy row per warp: 32/G slices of the row's entries x G right-hand
// sides; slices are reduced with butterfly shuffles.
template <typename T, int G>
__device__ __forceinline__ void warp_row(const RowArgs<T> &a, const int p, const int sl,
                                         const int g)
{
    constexpr int NS = 32 / G;
    typedef VBits<T> VB;
    typedef typename VB::U U;
    const int i = a.upper ? a.n - 1 - p : p;
    int s = __ldg(a.ptr + i), e = __ldg(a.ptr + i + 1);
    if (a.upper)
        ++s;
    else
        --e;
    const bool active = g < a.nrhs;
    const size_t xo = (size_t)i * (size_t)a.ld + (size_t)g;
    T bi = T(0), dinv = T(0);
    if (active && sl == 0) {
        bi = __ldg(a.b + xo);
        dinv = __ldg(a.inv_diag + i);
    }
    const U *xb = reinterpret_cast<const U *>(a.x);
    T acc = T(0);
    bool aborted = false;
    if (active) {
        for (int j0 = s + sl; j0 < e && !aborted; j0 += NS * kBatch) {
            int c[kBatch];
            T v[kBatch];
            U w[kBatch];
            unsigned pend = 0;
#pragma unroll
            for (int t = 0; t < kBatch; ++t) {
                const int j = j0 + t * NS;
                c[t] = 0;
                v[t] = T(0);
                w[t] = 0;
                if (j < e) {
                    c[t] = __ldg(a.idx + j);
                    v[t] = __ldg(a.val + j);
                    pend |= 1u << t;
                }
            }
            const unsigned have = pend;
            Spin sp;
            int waited = 0;
            while (pend && !aborted) {
#pragma unroll
                for (int t = 0; t < kBatch; ++t) {
                    if ((pend >> t) & 1u) {
                        const U u = ld_relaxed(xb + (size_t)c[t] * (size_t)a.ld + g);
                        if (u != VB::kPending) {
                            w[t] = u;
                            pend &= ~(1u << t);
                        } else {
                            waited = c[t];
                        }
                    }
                }
                if (pend && sp.next(a.err, a.wait, i, waited))
                    aborted = true;
            }
#pragma unroll
            for (int t = 0; t < kBatch; ++t)
                if ((have >> t) & 1u)
                    acc = fma(v[t], VB::from(w[t]), acc);
        }
    }
#pragma unroll
    for (int off = 16; off >= G; off >>= 1)
        acc += __shfl_xor_sync(kFullMask, acc, off);
    aborted = __any_sync(kFullMask, aborted);
    if (sl == 0 && active && i != a.stuck_row) {
        U ub = aborted ? VB::kQNaN : VB::to((bi - acc) * dinv);
        if (ub == VB::kPending)
            ub = VB::kQNaN;
        st_relaxed(reinterpret_cast<U *>(a.x) + xo, ub);
    }
}

template <typename T, int G, int R, int KIND>
__global__ void __launch_bounds__(512) row_solve_kernel(const RowArgs<T> a)
{
    typedef typename VBits<T>::U U;
    constexpr int RPW = 32 / G;
    constexpr int CH = RPW * R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    volatile U *cache = reinterpret_cast<volatile U *>(smem_raw) + (size_t)(threadIdx.x >> 5) * (32 * R);
    const int rl = lane / G, g = lane % G;
    for (;;) {
        unsigned tk = 0, stop = 0;
        if (lane == 0) {
            tk = atomicAdd(a.ticket, KIND == kRowMix ? 1u : (unsigned)CH);
            stop = ld_relaxed(reinterpret_cast<const unsigned *>(a.err));
        }
        tk = __shfl_sync(kFullMask, tk, 0);
        stop = __shfl_sync(kFullMask, stop, 0);
        if (stop)
            break;
        if (KIND != kRowMix) {
            if (tk >= (unsigned)a.n)
                break;
            const int lo = (int)tk;
#pragma unroll
            for (int r = 0; r < R; ++r)
                cache[r * 32 + lane] = VBits<T>::kPending;
            __syncwarp();
#pragma unroll 1
            for (int r = 0; r < R; ++r) {
                const int p = lo + r * RPW + rl;
                if (p < a.n && g < a.nrhs)
                    thread_row<T, G, KIND == kRowTwoPart>(a, p, g, lo, cache);
            }
            __syncwarp();
        } else {
            if (tk + 1u >= (unsigned)a.table_len)
                break;
            const int lo = __ldg(a.table + tk), hi = __ldg(a.table + tk + 1);
            if (hi - lo > 1) {
                cache[lane] = VBits<T>::kPending;
                __syncwarp();
                const int p = lo + rl;
                if (p < hi && g < a.nrhs)
                    thread_row<T, G, false>(a, p, g, lo, cache);
                __syncwarp();
            } else {
                warp_row<T, G>(a, lo, rl, g);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------

template <typename T, int G, int R, int KIND>
static cudaError_t launch_row_impl(const RowArgs<T> &a, int block, int bps, int num_sms,
                                   cudaStream_t st)
{
    constexpr int RPW = 32 / G;
    auto kern = row_solve_kernel<T, G, R, KIND>;
    const size_t smem = (size_t)(block / 32) * 32 * R * sizeof(typename VBits<T>::U);
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, block, smem);
    if (e != cudaSuccess)
        return e;
    if (occ < 1)
        occ = 1;
    const int per_sm = (bps > 0 && bps < occ) ? bps : occ;
    long long grid = (long long)per_sm * num_sms;
    const long long chunks =
        KIND == kRowMix ? (long long)a.table_len - 1 : ((long long)a.n + RPW * R - 1) / (RPW * R);
    const long long need = (chunks + block / 32 - 1) / (block / 32);
    if (grid > need)
        grid = need;
    if (grid < 1)
        grid = 1;
    kern<<<(unsigned)grid, block, smem, st>>>(a);
    return cudaGetLastError();
}

template <typename T, int G>
static cudaError_t launch_row_g(const RowArgs<T> &a, int kind, int R, int block, int bps,
                                int num_sms, cudaStream_t st)
{
    if (kind == kRowMix)
        return launch_row_impl<T, G, 1, kRowMix>(a, block, bps, num_sms, st);
    // the two-phase schedule is the reference's single-RHS design; multi-RHS
    // launches use the write-first schedule
    if constexpr (G == 1) {
        if (kind == kRowTwoPart) {
            switch (R) {
            case 4: return launch_row_impl<T, G, 4, kRowTwoPart>(a, block, bps, num_sms, st);
            case 2: return launch_row_impl<T, G, 2, kRowTwoPart>(a, block, bps, num_sms, st);
            default: return launch_row_impl<T, G, 1, kRowTwoPart>(a, block, bps, num_sms, st);
            }
        }
    }
    switch (R) {
    case 4: return launch_row_impl<T, G, 4, kRowWrtFst>(a, block, bps, num_sms, st);
    case 2: return launch_row_impl<T, G, 2, kRowWrtFst>(a, block, bps, num_sms, st);
    default: return launch_row_impl<T, G, 1, kRowWrtFst>(a, block, bps, num_sms, st);
    }
}

template <typename T>
cudaError_t launch_row_solve(const RowArgs<T> &a, int kind, int rows_per_thread, int block,
                             int blocks_per_sm, int num_sms, cudaStream_t st)
{
    switch (lanes_for_rhs(a.nrhs)) {
    case 1: return launch_row_g<T, 1>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, st);
    case 2: return launch_row_g<T, 2>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, st);
    case 4: return launch_row_g<T, 4>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, st);
    case 8: return launch_row_g<T, 8>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, st);
    case 16: return launch_row_g<T, 16>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, st);
    default: return launch_row_g<T, 32>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, st);
    }
}

// ---------------------------------------------------------------------------
// fill x with the pending pattern, reset ticket counters and the error word
// ---------------------------------------------------------------------------

template <typename U>
__global__ void fill_pending_kernel(U *__restrict__ x, int n, int nrhs, long long ld, U pattern,
                                    uint4 pattern16, unsigned *ticket, int nticket, int *err)
{
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    if (tid < nticket)
        ticket[tid] = 0u;
    if (err != nullptr && tid < 4)
        err[tid] = 0;
    const long long total = (long long)n * nrhs;
    if (ld == nrhs) {
        constexpr int PER = 16 / sizeof(U);
        const uintptr_t addr = reinterpret_cast<uintptr_t>(x);
        long long head = (addr & 15) ? (long long)((16 - (addr & 15)) / sizeof(U)) : 0;
        if (head > total)
            head = total;
        for (long long k = tid; k < head; k += stride)
            x[k] = pattern;
        uint4 *body = reinterpret_cast<uint4 *>(x + head);
        const long long nb = (total - head) / PER;
        for (long long k = tid; k < nb; k += stride)
            body[k] = pattern16;
        for (long long k = head + nb * PER + tid; k < total; k += stride)
            x[k] = pattern;
    } else {
        for (long long k = tid; k < total; k += stride) {
            const long long i = k / nrhs, r = k - i * nrhs;
            x[i * ld + r] = pattern;
        }
    }
}

template <typename T>
cudaError_t launch_fill_pending(T *x, int n, int nrhs, long long ld, unsigned *ticket, int nticket,
                                int *err, cudaStream_t st)
{
    typedef typename VBits<T>::U U;
    const U pat = VBits<T>::kPending;
    uint4 p16;
    if (sizeof(U) == 8) {
        const unsigned long long w = (unsigned long long)pat;
        p16.x = (unsigned)(w & 0xffffffffull);
        p16.y = (unsigned)(w >> 32);
        p16.z = p16.x;
        p16.w = p16.y;
    } else {
        p16.x = p16.y = p16.z = p16.w = (unsigned)pat;
    }
    const long long total = (long long)n * nrhs;
    long long blocks = (total / (16 / (long long)sizeof(U)) + 255) / 256;
    if (blocks > 4096)
        blocks = 4096;
    if (blocks < 1)
        blocks = 1;
    fill_pending_kernel<U><<<(unsigned)blocks, 256, 0, st>>>(reinterpret_cast<U *>(x), n, nrhs, ld,
                                                            pat, p16, ticket, nticket, err);
    return cudaGetLastError();
}

}  // namespace capsp
