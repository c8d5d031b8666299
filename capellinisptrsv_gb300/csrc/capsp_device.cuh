// Device-side building blocks shared by the sync-free solve kernels (sm_103a).
//
// Readiness protocol ("value as flag").  The reference keeps a separate
// int flag per row and publishes x[i] with  x store -> __threadfence() ->
// flag store  (CUDA/ourWrtFst/spts_syncfree_cuda_csr_wrt.h:49-52); a consumer
// needs one L2 round trip for the flag and another for x.  Here every x
// element is first filled with a signalling-NaN bit pattern (kPending) that
// no floating-point operation can produce (IEEE arithmetic quietens NaNs), and
// the producer publishes the value itself with one relaxed gpu-scope store.
// A consumer polls the x element with relaxed gpu-scope loads (served by L2,
// never by a stale L1 line) until it differs from kPending; the value it reads
// is the dependency.  Aligned 32/64-bit accesses are single-copy atomic, so a
// reader sees either kPending or the complete value.  One store, no fence,
// one round trip per hop.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace capsp {

constexpr unsigned kFullMask = 0xffffffffu;

// device error word layout (int[4]): status, row that gave up, index it waited on
enum { kErrStatus = 0, kErrRow = 1, kErrWaitedOn = 2 };
constexpr int kStatusTimeout = 2;  // == CAPSP_ERR_TIMEOUT

template <typename T>
struct VBits;

template <>
struct VBits<double> {
    typedef unsigned long long U;
    static constexpr U kPending = 0x7FF4000000000BADull;  // signalling NaN (quiet bit clear)
    static constexpr U kQNaN = 0x7FF8000000000000ull;
    __device__ __forceinline__ static U to(double v) { return (U)__double_as_longlong(v); }
    __device__ __forceinline__ static double from(U u) { return __longlong_as_double((long long)u); }
};

template <>
struct VBits<float> {
    typedef unsigned int U;
    static constexpr U kPending = 0x7FA00BADu;  // signalling NaN (quiet bit clear)
    static constexpr U kQNaN = 0x7FC00000u;
    __device__ __forceinline__ static U to(float v) { return __float_as_uint(v); }
    __device__ __forceinline__ static float from(U u) { return __uint_as_float(u); }
};

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// bring a global line into L2 (no register result, no ordering)
__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned int ld_relaxed(const unsigned int *p)
{
    unsigned int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ void st_relaxed(unsigned int *p, unsigned int v)
{
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// L2 eviction policies.  The matrix arrays are streamed once per solve and
// marked evict_first; the publication vector (a few tens of MB that every
// dependency poll and every publication touches) is marked evict_last, so the
// streamed data does not push it out of the 129 MB L2 and a poll or a
// publication never pays a DRAM round trip.
__device__ __forceinline__ unsigned long long l2_policy_evict_first()
{
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ unsigned long long l2_policy_evict_last()
{
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ unsigned long long l2_policy_evict_normal()
{
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// read-only streamed loads with an L2 policy
__device__ __forceinline__ int ld_stream(const int *p, unsigned long long pol)
{
    int v;
    asm("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ double ld_stream(const double *p, unsigned long long pol)
{
    double v;
    asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ float ld_stream(const float *p, unsigned long long pol)
{
    float v;
    asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
    return v;
}

// relaxed gpu-scope poll / publication with an L2 policy
// Polls carry no "memory" clobber: they must be re-issued every round
// (volatile) but need not be ordered against the warp's shared-memory
// traffic, and without the clobber consecutive polls go out back to back.
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p, unsigned long long pol)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.L2::cache_hint.b64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ unsigned int ld_relaxed(const unsigned int *p, unsigned long long pol)
{
    unsigned int v;
    asm volatile("ld.relaxed.gpu.global.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ void st_relaxed(unsigned long long *p, unsigned long long v, unsigned long long pol)
{
    asm volatile("st.relaxed.gpu.global.L2::cache_hint.b64 [%0], %1, %2;" ::"l"(p), "l"(v), "l"(pol) : "memory");
}

__device__ __forceinline__ void st_relaxed(unsigned int *p, unsigned int v, unsigned long long pol)
{
    asm volatile("st.relaxed.gpu.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}

__device__ __forceinline__ void st_stream(unsigned long long *p, unsigned long long v, unsigned long long pol)
{
    asm volatile("st.global.L2::cache_hint.b64 [%0], %1, %2;" ::"l"(p), "l"(v), "l"(pol) : "memory");
}

__device__ __forceinline__ void st_stream(unsigned int *p, unsigned int v, unsigned long long pol)
{
    asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}

__device__ __forceinline__ unsigned long long global_timer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// 16-byte asynchronous global -> shared copy (both addresses 16-byte aligned),
// L2 policy as for the streamed loads.  Completion: cp_async_wait_all().
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, unsigned long long pol)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(s), "l"(gmem), "l"(pol)
                 : "memory");
}

// commit this thread's outstanding cp.async copies and wait for all of them
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// 16-byte compare-and-swap (gpu scope, relaxed); returns the previous value
__device__ __forceinline__ ulonglong2 cas128(ulonglong2 *p, ulonglong2 cmp, ulonglong2 val)
{
    ulonglong2 r;
    asm volatile("{\n\t.reg .b128 c, v, o;\n\t"
                 "mov.b128 c, {%2, %3};\n\t"
                 "mov.b128 v, {%4, %5};\n\t"
                 "atom.relaxed.gpu.global.cas.b128 o, [%6], c, v;\n\t"
                 "mov.b128 {%0, %1}, o;\n\t}"
                 : "=l"(r.x), "=l"(r.y)
                 : "l"(cmp.x), "l"(cmp.y), "l"(val.x), "l"(val.y), "l"(p)
                 : "memory");
    return r;
}

// Budget of one dependency wait.
struct WaitCfg {
    unsigned long long timeout_ns;  // wall-clock budget of a single wait
    unsigned max_iters;             // iteration cap (backstop for the timer)
    unsigned sleep_max_ns;          // ceiling of the exponential __nanosleep backoff
};

// Bounded spin with exponential backoff.  next() returns true when the wait
// must be abandoned: the budget ran out (this thread records TIMEOUT in the
// error word) or another thread already recorded an error.
struct Spin {
    unsigned it;
    unsigned long long t0;
    __device__ __forceinline__ Spin() : it(0), t0(0) {}
    __device__ __forceinline__ bool next(int *err, const WaitCfg &w, int row, int waited_on)
    {
        ++it;
        if (it > 4u && w.sleep_max_ns) {
            unsigned s = 32u << (it - 5u < 6u ? it - 5u : 6u);
            __nanosleep(s < w.sleep_max_ns ? s : w.sleep_max_ns);
        }
        if ((it & 15u) == 0u) {
            if (ld_relaxed(reinterpret_cast<const unsigned *>(err)) != 0u)
                return true;
            const unsigned long long now = global_timer_ns();
            if (t0 == 0ull) {
                t0 = now;
            } else if (now - t0 > w.timeout_ns || it > w.max_iters) {
                if (atomicCAS(err + kErrStatus, 0, kStatusTimeout) == 0) {
                    err[kErrRow] = row;
                    err[kErrWaitedOn] = waited_on;
                }
                return true;
            }
        }
        return false;
    }
};

// Owner, among a warp's 32-row group, of entry k: the largest lane l < nr whose
// row start (held in `start` by lane l) is <= k; rows without entries share
// their successor's start and never own one.  Every lane must call it.
__device__ __forceinline__ int group_row_of(int start, int k, int nr)
{
    int lo = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
        const int cand = lo + step;
        const int sv = __shfl_sync(kFullMask, start, cand & 31);
        if (cand < nr && sv <= k)
            lo = cand;
    }
    return lo;
}

}  // namespace capsp
