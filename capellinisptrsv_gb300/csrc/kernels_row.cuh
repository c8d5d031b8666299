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
//     its next chunk of consecutive schedule positions from one atomic
//     ticket.  Positions are therefore started in schedule order by warps
//     that are already running, so the lowest unfinished position always has
//     a running owner whose dependencies are finished: forward progress needs
//     no assumption about block scheduling.  (The reference takes one ticket
//     per thread and maps lanes from threadIdx, mix/...:32-45.)
//   * Two schedules.  NATURAL visits rows in index order (no preprocessing,
//     like the reference).  LEVEL visits rows sorted by dependency level
//     (built at analysis): a warp's chunk then holds rows that become ready
//     together, so no lane idles behind a row several levels deeper, far
//     fewer rows need to be in flight, and chains through consecutive levels
//     stay inside one warp.  LEVEL works in schedule-position space:
//     dependencies are stored as positions and values are published into a
//     position-ordered scratch vector (plus the caller's x).
//   * Value-as-flag readiness (capsp_device.cuh): no flag array, no fence.
//   * Dependencies inside the warp's own chunk are read from a per-warp
//     shared-memory mirror of the chunk's values instead of from L2.
//   * Polling: a fresh batch of dependencies is swept once; afterwards each
//     lane probes only the dependency that blocks its in-order fold, and the
//     next round's probe is issued before the current round folds and
//     publishes, so the poll's round trip overlaps that work.  A row whose
//     last dependency lands in a probe, with everything before it folded,
//     takes its one FMA and publishes right there, without waiting for the
//     warp's fold/publish pass.
//   * Partial sums are accumulated in storage order whatever the arrival
//     order, so repeated solves and the WRTFST / TWOPART schedules are
//     bit-identical.
//   * 1/diag is precomputed at analysis; x = (b - sum) * (1/diag).  The
//     level schedule pre-scales the values instead (x = b/d + sum (-v/d) x_j),
//     so a single FMA follows the last dependency.
//   * Multi-RHS: G = next_pow2(nrhs) lanes share a row, one right-hand side
//     each (more than 16: 8 lanes with RPL = 4 right-hand sides each); every
//     (row, rhs) element is published and polled independently.
//   * Every wait is bounded (Spin); a lane that gives up publishes a quiet
//     NaN so its dependants finish, and the error word records TIMEOUT.
#pragma once

#include "capsp_internal.h"

namespace capsp {

// dependencies one lane keeps in flight (the level schedule in
// host/preprocess.c sorts rows by this pass size: CAPSP_ROW_PASS)
constexpr int kBatch = 8;

// Where a row's data lives, for the natural and the level schedule.
template <typename T, bool LEVEL>
struct RowView {
    int i;         // row index (output / b / trace)
    int s, e;      // dependency range in idx/val
    const int *idx;
    const T *val;
    T dinv;
    typename VBits<T>::U *pub;  // publication vector (x or xp)
    long long pld;              // its row stride
    long long pslot;            // this row's slot in pub (row i or position p)

    __device__ __forceinline__ RowView(const RowArgs<T> &a, int p, unsigned long long pol)
    {
        typedef typename VBits<T>::U U;
        if (LEVEL) {
            i = ld_stream(a.perm + p, pol);
            s = ld_stream(a.lptr + p, pol);
            e = ld_stream(a.lptr + p + 1, pol);
            idx = a.lidx;
            val = a.lval;
            dinv = ld_stream(a.linv + p, pol);
            pub = reinterpret_cast<U *>(a.xp);
            pld = a.ldp;
            pslot = p;
        } else {
            i = a.upper ? a.n - 1 - p : p;
            s = ld_stream(a.ptr + i, pol);
            e = ld_stream(a.ptr + i + 1, pol);
            if (a.upper)
                ++s;
            else
                --e;
            idx = a.idx;
            val = a.val;
            dinv = ld_stream(a.inv_diag + i, pol);
            pub = reinterpret_cast<U *>(a.x);
            pld = a.ld;
            pslot = i;
        }
    }
    // schedule position of the dependency stored as c
    __device__ __forceinline__ int pos_of(const RowArgs<T> &a, int c) const
    {
        return LEVEL ? c : (a.upper ? a.n - 1 - c : c);
    }
    // newest pending dependency: highest position (storage order ascends in
    // position except for the natural upper view, where it descends)
    __device__ __forceinline__ unsigned newest(const RowArgs<T> &a, unsigned pend) const
    {
        return (!LEVEL && a.upper) ? (pend & (0u - pend)) : (1u << (31 - __clz(pend)));
    }
};

// L2 policies of one kernel launch (see capsp_device.cuh)
struct L2Pol {
    unsigned long long stream;  // evict_first: matrix arrays, b, the output x of the level schedule
    unsigned long long keep;    // evict_last: the publication vector
};

template <typename T, bool LEVEL>
__device__ __forceinline__ void publish(const RowArgs<T> &a, const RowView<T, LEVEL> &rv, int g,
                                        typename VBits<T>::U ub, const L2Pol &pol)
{
    typedef typename VBits<T>::U U;
    st_relaxed(rv.pub + (size_t)rv.pslot * (size_t)rv.pld + g, ub, pol.keep);
    if (LEVEL)
        st_stream(reinterpret_cast<U *>(a.x) + (size_t)rv.i * (size_t)a.ld + g, ub, pol.stream);
}

// Per-warp shared-memory slot storage: for each lane, the values and the
// received dependency values of its current batch, so that the in-order fold
// can run a data-dependent loop (a fully unrolled, predicated FMA chain would
// wait ~64 cycles per slot on this GPU's FP64 pipe even when predicated off).
template <typename T>
struct Slots {
    T *v;                          // dependency values, [t * 32 + lane]
    typename VBits<T>::U *w;       // received x values
    int *q;                        // dependency positions
    int *si;                       // staged entries of the sub-chunk: positions ...
    T *sv;                         // ... and values (staged launches only)
};

// Entries of a 32-row sub-chunk staged in shared memory (STAGE launches: one
// lane per row, level schedule): up to kStage of them, from a 16-byte boundary.
constexpr int kStage = 384;

// bytes of dynamic shared memory per warp: chunk mirror (32R elements of RPL
// right-hand sides) + slot storage (kBatch / RPL dependencies of RPL values)
// + the staging buffers.  Every part is a multiple of 16 bytes.
template <typename T>
__host__ __device__ constexpr size_t warp_smem_bytes(int R, int RPL = 1, bool stage = false)
{
    return (size_t)32 * R * RPL * sizeof(typename VBits<T>::U) +
           (size_t)(kBatch / RPL) * 32 * (sizeof(T) + sizeof(int)) +
           (size_t)kBatch * 32 * sizeof(typename VBits<T>::U) +
           (stage ? (size_t)kStage * (sizeof(int) + sizeof(T)) : 0);
}

// The 16-byte staging copies need every warp's block, and the staging buffers
// inside it (after the mirror and slot parts; positions, then kStage values
// later), to start on a 16-byte boundary.
template <typename T>
__host__ __device__ constexpr bool staging_aligned()
{
    return warp_smem_bytes<T>(1, 1, true) % 16 == 0 && warp_smem_bytes<T>(2, 1, true) % 16 == 0 &&
           warp_smem_bytes<T>(4, 1, true) % 16 == 0 && warp_smem_bytes<T>(1, 1, false) % 16 == 0 &&
           warp_smem_bytes<T>(2, 1, false) % 16 == 0 && warp_smem_bytes<T>(4, 1, false) % 16 == 0 &&
           warp_smem_bytes<T>(1, 4, false) % 16 == 0 && (kStage * sizeof(int)) % 16 == 0;
}
static_assert(staging_aligned<double>() && staging_aligned<float>(), "shared-memory parts must be 16-byte multiples");

// Convergent chunk solve.  The warp's chunk holds schedule positions
// [lo, lo + CH); in each pass over a sub-chunk of 32/G positions starting at
// `sub`, lane (rl, g) owns the element (position p = sub + rl, rhs g).  All
// lanes advance together in rounds, so a warp never splits into long-lived
// divergent paths (which the hardware runs one at a time):
//   A. every lane issues the polls it selected for dependencies before the
//      chunk (relaxed gpu-scope loads), all in flight together;
//   B. runs only when something changed: a ballot of the lanes that have
//      published tells every lane whether a producer of one of its
//      dependencies inside the sub-chunk has published; those values come
//      from the shared-memory mirror; contributions are folded in storage
//      order as soon as the ready prefix grows, so when the last dependency
//      lands a single FMA remains; complete rows publish, and B repeats while
//      lanes publish, so a chain through the sub-chunk resolves in one round;
//   C. a round in which nothing moved backs off and checks the wait budget.
// Level schedule: values are pre-scaled at analysis, x = b/d + sum (-v/d) x_j,
// so no FP64 work is left after the last dependency but that FMA (one
// warp-wide DFMA occupies an SM sub-partition's FP64 pipe for ~64 cycles).
// TWO (the two-phase schedule of the reference's our2Part) polls the outside
// dependencies one at a time in storage order.
// b's element (i, r).  HOSTIO launches (capsp_solve_host) may run while a
// copy stream is still uploading b: there b is read at gpu scope (the warp
// has waited for the row's segment), past the non-coherent path.
template <typename T, bool HOSTIO>
__device__ __forceinline__ T load_b(const RowArgs<T> &a, int i, int r, unsigned long long pol)
{
    typedef typename VBits<T>::U U;
    const T *p = a.b + (size_t)i * (size_t)a.ld + r;
    if (HOSTIO && a.b_ready != nullptr)
        return VBits<T>::from(ld_relaxed(reinterpret_cast<const U *>(p), pol));
    return ld_stream(p, pol);
}

// While a copy stream is uploading b: wait (bounded) until every row of the
// positions [lo, hi) has its b in place.  One flag per chunk, polled by lane 0.
template <typename T>
__device__ __forceinline__ void wait_b_chunk(const RowArgs<T> &a, int lo, int hi)
{
    const int lane = threadIdx.x & 31;
    const int q0 = lo >> 5, q1 = (hi - 1) >> 5;
    const int seg = __reduce_max_sync(kFullMask, q0 + lane <= q1 ? (int)a.b_group_seg[q0 + lane] : 0);
    if (lane == 0) {
        const unsigned *f = reinterpret_cast<const unsigned *>(a.b_ready + seg);
        Spin sp;
        while (ld_acquire(f) == 0u)
            if (sp.next(a.err, a.wait, lo, -1))
                break;
    }
    __syncwarp();
}

template <typename T, int G, bool TWO, bool LEVEL, int RPL, bool STAGE, bool HOSTIO>
__device__ __forceinline__ void chunk_rows(const RowArgs<T> &a, const int lo, const int sub, const int p,
                                           const bool mine, const int g,
                                           volatile typename VBits<T>::U *cache, const Slots<T> &sl,
                                           const unsigned long long t_pick, const L2Pol &pol)
{
    typedef VBits<T> VB;
    typedef typename VB::U U;
    const int lane = threadIdx.x & 31;
    constexpr int KB = kBatch / RPL;       // dependencies in flight per lane (RPL values each)
    const int r0 = g * RPL;                // this lane's first right-hand side
    const int nq = mine ? min(RPL, a.nrhs - r0) : 0;
    // right-hand side r of this lane exists; with one per lane that is implied
    // wherever it is asked (only lanes that own a row load, store or poll), and
    // the test compiles away (keeping it cost the single-RHS solve 2-5 %)
    const auto has_rhs = [nq](int r) { return RPL == 1 || r < nq; };
    int i = 0, j0 = 0, e = 0;
    const int *idxp = nullptr;
    const T *valp = nullptr;
    T dinv = T(0), bi[RPL], acc[RPL];
#pragma unroll
    for (int r = 0; r < RPL; ++r)
        bi[r] = acc[r] = T(0);
    U *pub = nullptr;
    long long pld = 0, pslot = 0;
    if (mine) {
        const RowView<T, LEVEL> rv(a, p, pol.stream);
        i = rv.i;
        j0 = rv.s;
        e = rv.e;
        idxp = rv.idx;
        valp = rv.val;
        dinv = rv.dinv;
        pub = rv.pub;
        pld = rv.pld;
        pslot = rv.pslot;
#pragma unroll
        for (int r = 0; r < RPL; ++r) {
            if (has_rhs(r))
                bi[r] = load_b<T, HOSTIO>(a, i, r0 + r, pol.stream);
            if (LEVEL)
                acc[r] = bi[r] * dinv;  // x = b/d + sum (-v/d) x_j
        }
    }
    // Stage the sub-chunk's entries.  Its rows' entries are consecutive in the
    // level layout, so 16-byte copies by all lanes read them with full sectors;
    // a lane walking its own row touches a different line with every load.
    int sbase = 0;
    bool staged = false;
    static_assert(!STAGE || (LEVEL && G == 1 && RPL == 1), "staging: one lane per row, level schedule");
    if constexpr (STAGE) {
        const int lo_e = __reduce_min_sync(kFullMask, mine ? j0 : INT_MAX);
        const int hi_e = __reduce_max_sync(kFullMask, mine ? e : INT_MIN);
        const int s4 = lo_e & ~3, e4 = (hi_e + 3) & ~3;  // 16-byte boundaries of the positions
        if (hi_e > lo_e && e4 - s4 <= kStage) {
            staged = true;
            sbase = s4;
            const int nidx = (e4 - s4) / 4;
            const int nval = (e4 - s4) * (int)sizeof(T) / 16;
            for (int k = lane; k < nidx; k += 32)
                cp_async16(sl.si + 4 * k, a.lidx + s4 + 4 * k, pol.stream);
            for (int k = lane; k < nval; k += 32)
                cp_async16(reinterpret_cast<char *>(sl.sv) + 16 * k,
                           reinterpret_cast<const char *>(a.lval + s4) + 16 * k, pol.stream);
            cp_async_wait_all();
        }
        __syncwarp();
    }
    int c[KB];                    // dependency index (position, or row in natural order)
    unsigned pend = 0, ext = 0, need = 0;
    int nacc = 0, cnt = 0;
    bool sweep_next = false;          // a fresh batch is swept once, then probed
    auto load_batch = [&]() {
        sweep_next = true;
        cnt = min(KB, e - j0);
        pend = ext = need = 0;
        nacc = 0;
#pragma unroll
        for (int t = 0; t < KB; ++t) {
            c[t] = 0;
            if (t < cnt) {
                const int cc = staged ? sl.si[j0 + t - sbase] : ld_stream(idxp + j0 + t, pol.stream);
                const int q = LEVEL ? cc : (a.upper ? a.n - 1 - cc : cc);
                c[t] = cc;
                sl.v[t * 32 + lane] = staged ? sl.sv[j0 + t - sbase] : ld_stream(valp + j0 + t, pol.stream);
                sl.q[t * 32 + lane] = q;
                if (q < lo) {
                    ext |= 1u << t;
                    pend |= 1u << t;
                } else if (q < sub) {  // earlier sub-chunk of this chunk: already in the mirror
#pragma unroll
                    for (int r = 0; r < RPL; ++r)
                        sl.w[(t * RPL + r) * 32 + lane] = cache[((q - lo) * G + g) * RPL + r];
                } else {
                    pend |= 1u << t;
                    need |= 1u << ((q - sub) * G + g);
                }
            }
        }
    };
    // fold the contributions of the ready prefix [nacc, first pending).  Not
    // unrolled: an unrolled copy issues predicated-off FMAs, and every warp
    // FP64 instruction holds the sub-partition's FP64 pipe for ~64 cycles.
    auto fold = [&]() {
        const int lim = pend ? __ffs(pend) - 1 : cnt;
#pragma unroll 1
        for (int t = nacc; t < lim; ++t) {
            const T v = sl.v[t * 32 + lane];
#pragma unroll
            for (int r = 0; r < RPL; ++r)
                acc[r] = fma(v, VB::from(sl.w[(t * RPL + r) * 32 + lane]), acc[r]);
        }
        nacc = lim;
    };
    bool done = !mine, published = !mine;
    if (mine && j0 < e)
        load_batch();
    bool aborted = false;
    U u_next[RPL];                    // probe issued at the end of the previous round
#pragma unroll
    for (int r = 0; r < RPL; ++r)
        u_next[r] = VB::kPending;
    unsigned top_next = 0u;           // ... and the slot it polls
    unsigned long long t_ready = 0;
    Spin sp;
    int waited = 0;
    bool first = true;
    unsigned long long t_first = 0;
    if (a.trace != nullptr)
        t_first = global_timer_ns();
    // the row is complete: publish into the mirror, the publication vector
    // and (level schedule) the caller's x
    auto finish = [&]() {
        if (a.trace != nullptr && t_ready == 0)
            t_ready = global_timer_ns();
        if (i != a.stuck_row) {
#pragma unroll
            for (int r = 0; r < RPL; ++r) {
                if (has_rhs(r)) {
                    U ub = VB::to(LEVEL ? acc[r] : (bi[r] - acc[r]) * dinv);
                    if (ub == VB::kPending)
                        ub = VB::kQNaN;
                    cache[((p - lo) * G + g) * RPL + r] = ub;
                    st_relaxed(pub + (size_t)pslot * (size_t)pld + r0 + r, ub, pol.keep);
                    if (LEVEL)
                        st_stream(reinterpret_cast<U *>(a.x) + (size_t)i * (size_t)a.ld + r0 + r, ub, pol.stream);
                }
            }
            published = true;
        }
        if (a.trace != nullptr && g == 0) {
            a.trace[4 * (size_t)i] = t_pick;
            a.trace[4 * (size_t)i + 1] = t_first;
            a.trace[4 * (size_t)i + 2] = t_ready;
            a.trace[4 * (size_t)i + 3] = global_timer_ns();
        }
        done = true;
    };
    for (;;) {
        // ---- A: polls of dependencies before the chunk ---------------------
        // A fresh batch is swept once: every outstanding dependency polled,
        // all loads in flight together.  After that each lane probes one
        // dependency per round, its first pending one in storage order (the
        // one that blocks the in-order fold), so by the time the last one
        // lands everything before it has been folded.  The two-phase
        // schedule never sweeps.  Each round issues the next round's probe
        // at its end, so the poll travels while this round folds, publishes
        // and backs off.
        bool changed = first;
        first = false;
        const unsigned ext_pend = done ? 0u : (pend & ext);
        const unsigned top = ext_pend & (0u - ext_pend);
        const bool sweep = !TWO && ext_pend != 0u && sweep_next;
        sweep_next = false;
        if (!__any_sync(kFullMask, sweep)) {
            // probe round (warp-uniform): the value polled at the end of the
            // previous round when it was for this slot, else a fresh load
            U u0[RPL];
#pragma unroll
            for (int r = 0; r < RPL; ++r)
                u0[r] = u_next[r];
            if (top != 0u && top != top_next) {
                const U *addr = pub;
#pragma unroll
                for (int t = 0; t < KB; ++t)
                    if ((top >> t) & 1u)
                        addr = pub + (size_t)c[t] * (size_t)pld + r0;
#pragma unroll
                for (int r = 0; r < RPL; ++r)
                    u0[r] = has_rhs(r) ? ld_relaxed(addr + r, pol.keep) : (U)0;
            }
            bool landed = true;
#pragma unroll
            for (int r = 0; r < RPL; ++r)
                landed = landed && (!has_rhs(r) || u0[r] != VB::kPending);
            if (top) {
                if (landed) {
#pragma unroll
                    for (int t = 0; t < KB; ++t)
                        if ((top >> t) & 1u) {
#pragma unroll
                            for (int r = 0; r < RPL; ++r)
                                sl.w[(t * RPL + r) * 32 + lane] = u0[r];
                        }
                    pend &= ~top;
                    changed = true;
                    if (a.trace != nullptr && pend == 0 && j0 + KB >= e)
                        t_ready = global_timer_ns();  // last dependency value received
                    if (pend == 0 && nacc == cnt - 1 && top == (1u << (cnt - 1)) && j0 + KB >= e) {
                        // the row's last dependency, everything before it
                        // folded: one FMA per right-hand side (same order as
                        // the fold) and the row publishes now instead of after
                        // the warp's B pass
                        const T v = sl.v[(cnt - 1) * 32 + lane];
#pragma unroll
                        for (int r = 0; r < RPL; ++r)
                            acc[r] = fma(v, VB::from(u0[r]), acc[r]);
                        nacc = cnt;
                        finish();
                    }
                } else {
                    int w = 0;
#pragma unroll
                    for (int t = 0; t < KB; ++t)
                        if ((top >> t) & 1u)
                            w = c[t];
                    waited = w;
                }
            }
        } else if (ext_pend) {
            // sweep round: every outstanding outside dependency, all loads in
            // flight together before any result is consumed (in-order issue
            // would otherwise stall on the first result)
            U u[KB][RPL];
#pragma unroll
            for (int t = 0; t < KB; ++t)
#pragma unroll
                for (int r = 0; r < RPL; ++r)
                    u[t][r] = ((ext_pend >> t) & 1u) && has_rhs(r)
                                  ? ld_relaxed(pub + (size_t)c[t] * (size_t)pld + r0 + r, pol.keep)
                                  : (U)0;
            unsigned got = 0;
#pragma unroll
            for (int t = 0; t < KB; ++t) {
                if ((ext_pend >> t) & 1u) {
                    bool ok = true;
#pragma unroll
                    for (int r = 0; r < RPL; ++r)
                        ok = ok && u[t][r] != VB::kPending;
                    if (ok) {
#pragma unroll
                        for (int r = 0; r < RPL; ++r)
                            sl.w[(t * RPL + r) * 32 + lane] = u[t][r];
                        got |= 1u << t;
                    } else {
                        waited = c[t];
                    }
                }
            }
            pend &= ~got;
            changed = changed || got != 0;
            if (a.trace != nullptr && got != 0 && pend == 0 && j0 + KB >= e)
                t_ready = global_timer_ns();  // last dependency value received
        }
        {
            // next round's probe (B and C leave the outside part of pend alone;
            // a batch loaded in B is swept instead)
            const unsigned np = done ? 0u : (pend & ext);
            top_next = np & (0u - np);
#pragma unroll
            for (int r = 0; r < RPL; ++r)
                u_next[r] = VB::kPending;
            if (top_next != 0u) {
                const U *addr = pub;
#pragma unroll
                for (int t = 0; t < KB; ++t)
                    if ((top_next >> t) & 1u)
                        addr = pub + (size_t)c[t] * (size_t)pld + r0;
#pragma unroll
                for (int r = 0; r < RPL; ++r)
                    u_next[r] = has_rhs(r) ? ld_relaxed(addr + r, pol.keep) : (U)0;
            }
        }
        // a lane whose current batch is complete but not yet folded also needs B
        const bool progress = __any_sync(kFullMask, changed || (!done && pend == 0u));
        // ---- B: in-sub-chunk pickup, fold, publish ------------------------
        if (progress) {
            __syncwarp();  // mirror stores of rows finished in A visible to the pickups
            for (;;) {
                const unsigned pubmask = __ballot_sync(kFullMask, published);
                bool moved = false;
                if (!done) {
                    if (need & pubmask) {
                        unsigned m = pend & ~ext;
                        while (m) {
                            const int t = __ffs(m) - 1;
                            m &= m - 1;
                            const int q = sl.q[t * 32 + lane];
                            if ((pubmask >> ((q - sub) * G + g)) & 1u) {
#pragma unroll
                                for (int r = 0; r < RPL; ++r)
                                    sl.w[(t * RPL + r) * 32 + lane] = cache[((q - lo) * G + g) * RPL + r];
                                pend &= ~(1u << t);
                            }
                        }
                        need &= ~pubmask;
                    }
                    if (nacc < cnt)
                        fold();
                    if (pend == 0 && nacc >= cnt) {
                        j0 += KB;
                        if (j0 < e) {
                            load_batch();  // a row with more than KB dependencies
                            moved = true;
                        } else {
                            finish();
                            moved = true;
                        }
                    }
                }
                __syncwarp();  // mirror stores visible to the next pickup
                // another pass can only help a lane that still waits on a
                // dependency inside the sub-chunk
                if (!__any_sync(kFullMask, moved) ||
                    !__any_sync(kFullMask, !done && (pend == 0u || (pend & ~ext) != 0u)))
                    break;
            }
        }
        if (__all_sync(kFullMask, done))
            break;
        // ---- C: back off when nothing moved; bounded wait -----------------
        if (!progress) {
            if (sp.next(a.err, a.wait, i, waited))
                aborted = true;
        } else {
            sp.it = 0;
        }
        if (__any_sync(kFullMask, aborted)) {
            // give up: unfinished rows publish a quiet NaN so their dependants end
            if (!done && i != a.stuck_row) {
#pragma unroll
                for (int r = 0; r < RPL; ++r) {
                    if (has_rhs(r)) {
                        cache[((p - lo) * G + g) * RPL + r] = VB::kQNaN;
                        st_relaxed(pub + (size_t)pslot * (size_t)pld + r0 + r, VB::kQNaN, pol.keep);
                        if (LEVEL)
                            st_stream(reinterpret_cast<U *>(a.x) + (size_t)i * (size_t)a.ld + r0 + r, VB::kQNaN,
                                      pol.stream);
                    }
                }
            }
            __syncwarp();
            break;
        }
    }
}

// One heavy row per warp: 32/G slices of the row's entries x G right-hand
// sides, advanced in convergent rounds; slices are reduced with butterfly
// shuffles once every lane has consumed its entries.
template <typename T, int G, bool LEVEL, bool HOSTIO>
__device__ __forceinline__ void warp_row(const RowArgs<T> &a, const int p, const int sl_idx, const int g,
                                         const Slots<T> &sl, const L2Pol &pol)
{
    constexpr int NS = 32 / G;
    typedef VBits<T> VB;
    typedef typename VB::U U;
    const int lane = threadIdx.x & 31;
    const RowView<T, LEVEL> rv(a, p, pol.stream);
    const int i = rv.i;
    const bool active = g < a.nrhs;
    // The row's newest dependency (last in position order; first in storage
    // order for the natural upper view) is kept out of the slices: the warp
    // folds and reduces everything else while it waits, and the lanes of
    // slice 0 add its term with one FMA when it lands, so a chain through
    // heavy rows pays one hop per row, not a hop plus a full reduction.
    const bool upper_nat = !LEVEL && a.upper;
    const bool has_last = rv.e > rv.s;
    const int j_last = upper_nat ? rv.s : rv.e - 1;
    const int rs = (upper_nat && has_last) ? rv.s + 1 : rv.s;
    const int re = (!upper_nat && has_last) ? rv.e - 1 : rv.e;
    const bool owner = active && sl_idx == 0;  // lanes that finish the row
    T bi = T(0), v_last = T(0);
    int c_last = 0;
    if (owner) {
        bi = load_b<T, HOSTIO>(a, i, g, pol.stream);
        if (has_last) {
            c_last = ld_stream(rv.idx + j_last, pol.stream);
            v_last = ld_stream(rv.val + j_last, pol.stream);
        }
    }
    const U *pb = rv.pub;
    T acc = T(0);
    int c[kBatch];
    unsigned pend = 0;
    int cnt = 0;
    int j0 = rs + sl_idx;
    auto load_batch = [&]() {
        pend = 0;
        cnt = 0;
#pragma unroll
        for (int t = 0; t < kBatch; ++t) {
            const int j = j0 + t * NS;
            c[t] = 0;
            if (j < re) {
                c[t] = ld_stream(rv.idx + j, pol.stream);
                sl.v[t * 32 + lane] = ld_stream(rv.val + j, pol.stream);
                pend |= 1u << t;
                ++cnt;
            }
        }
    };
    bool done = !active || j0 >= re;
    if (!done)
        load_batch();
    bool probe_only = false, aborted = false;
    Spin sp;
    int waited = 0;
    for (;;) {
        bool progress = false;
        if (!done) {
            const unsigned top = rv.newest(a, pend);
            const unsigned sel = probe_only ? top : pend;
            U u[kBatch];
#pragma unroll
            for (int t = 0; t < kBatch; ++t)
                u[t] = ((sel >> t) & 1u) ? ld_relaxed(pb + (size_t)c[t] * (size_t)rv.pld + g, pol.keep)
                                         : VB::kPending;
            unsigned got = 0;
#pragma unroll
            for (int t = 0; t < kBatch; ++t) {
                if ((sel >> t) & 1u) {
                    if (u[t] != VB::kPending) {
                        sl.w[t * 32 + lane] = u[t];
                        got |= 1u << t;
                    } else {
                        waited = c[t];
                    }
                }
            }
            pend &= ~got;
            probe_only = pend != 0 && !(got & top);
            progress = got != 0;
            if (pend == 0) {
#pragma unroll 1
                for (int t = 0; t < cnt; ++t)
                    acc = fma(sl.v[t * 32 + lane], VB::from(sl.w[t * 32 + lane]), acc);
                j0 += NS * kBatch;
                if (j0 < re) {
                    load_batch();
                    probe_only = false;
                } else {
                    done = true;
                }
            }
        }
        if (__all_sync(kFullMask, done))
            break;
        if (!__any_sync(kFullMask, progress)) {
            if (sp.next(a.err, a.wait, i, waited))
                aborted = true;
        } else {
            sp.it = 0;
        }
        if (__any_sync(kFullMask, aborted))
            break;
    }
    aborted = __any_sync(kFullMask, aborted);
#pragma unroll
    for (int off = 16; off >= G; off >>= 1)
        acc += __shfl_xor_sync(kFullMask, acc, off);
    // the newest dependency: the slice-0 lanes wait for it and finish the row
    if (owner && has_last && !aborted) {
        const U *addr = pb + (size_t)c_last * (size_t)rv.pld + g;
        Spin wait_last;
        for (;;) {
            const U u_last = ld_relaxed(addr, pol.keep);
            if (u_last != VB::kPending) {
                acc = fma(v_last, VB::from(u_last), acc);
                break;
            }
            if (wait_last.next(a.err, a.wait, i, c_last)) {
                aborted = true;
                break;
            }
        }
    }
    unsigned long long t_ready = 0;
    if (a.trace != nullptr)
        t_ready = global_timer_ns();
    if (owner && i != a.stuck_row) {
        // level schedule: values are pre-scaled (x = b/d + sum), else x = (b - sum)/d
        U ub = aborted ? VB::kQNaN : VB::to(LEVEL ? fma(bi, rv.dinv, acc) : (bi - acc) * rv.dinv);
        if (ub == VB::kPending)
            ub = VB::kQNaN;
        publish<T, LEVEL>(a, rv, g, ub, pol);
    }
    if (a.trace != nullptr && sl_idx == 0 && g == 0) {
        a.trace[4 * (size_t)i] = t_ready;
        a.trace[4 * (size_t)i + 1] = t_ready;
        a.trace[4 * (size_t)i + 2] = t_ready;
        a.trace[4 * (size_t)i + 3] = global_timer_ns();
    }
}

// After the positions [lo, hi) of a warp's chunk have finished, count their
// rows into the completion counters of their row segments: one atomic per
// segment present in the chunk, after a fence that makes the chunk's stores
// of x visible device-wide, so a copy that waits for a segment's full count
// reads finished rows only.
template <typename T>
__device__ __forceinline__ void count_finished_rows(const RowArgs<T> &a, int lo, int hi)
{
    const int lane = threadIdx.x & 31;
    __threadfence();
    __syncwarp();
    for (int base = lo; base < hi; base += 32) {
        const int p = base + lane;
        const int seg = p < hi ? __ldg(a.perm + p) / a.seg_rows : -1;
        const unsigned grp = __match_any_sync(kFullMask, seg);
        if (seg >= 0 && lane == __ffs(grp) - 1)
            atomicAdd(a.seg_count + seg, __popc(grp));
    }
}

// CAP limits registers to 64 so that every warp an SM can hold fits: with G >= 4
// lanes per row on wide levels a warp holds few rows and residency decides
// (measured on GB300: 16 RHS on wide_4m 2.55 -> 1.84 ms).  Narrow levels and
// one or two lanes per row run faster with the full register budget.
// RPL: right-hand sides per lane (G lanes per row cover G * RPL of them), so a
// warp holds 32 / G rows however many right-hand sides there are.
// HOSTIO: a capsp_solve_host launch (one lane per row, level schedule): it
// waits for b's segments while a copy stream uploads them and counts finished
// rows per segment of x for the copy stream that takes them back.  A separate
// build, so that the other launches keep their registers.
template <typename T, int G, int R, int KIND, bool LEVEL, bool CAP = false, int RPL = 1, bool STAGE = false,
          bool HOSTIO = false>
__global__ void __launch_bounds__(512, (CAP ? 2 : 1)) row_solve_kernel(const RowArgs<T> a)
{
    typedef typename VBits<T>::U U;
    static_assert(RPL == 1 || KIND == kRowWrtFst, "several right-hand sides per lane: write-first only");
    constexpr int RPW = 32 / G;
    constexpr int CH = RPW * R;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    unsigned char *wbase = smem_raw + (size_t)wib * warp_smem_bytes<T>(R, RPL, STAGE);
    volatile U *cache = reinterpret_cast<volatile U *>(wbase);
    Slots<T> sl;
    sl.v = reinterpret_cast<T *>(wbase + (size_t)32 * R * RPL * sizeof(U));
    sl.w = reinterpret_cast<U *>(sl.v + (kBatch / RPL) * 32);
    sl.q = reinterpret_cast<int *>(sl.w + kBatch * 32);
    sl.si = sl.q + (kBatch / RPL) * 32;
    sl.sv = reinterpret_cast<T *>(sl.si + kStage);
    const int rl = lane / G, g = lane % G;
    L2Pol pol;
    pol.stream = l2_policy_evict_first();
    pol.keep = a.keep_hint ? l2_policy_evict_last() : l2_policy_evict_normal();
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
        const unsigned long long t_pick = a.trace != nullptr ? global_timer_ns() : 0ull;
        if (KIND != kRowMix) {
            if (tk >= (unsigned)a.n)
                break;
            const int lo = (int)tk;
            // One lane per row: prefetch into L2 the position metadata of the
            // chunk that the warps will take one round from now, so its
            // set-up starts from L2 instead of DRAM (measured on GB300:
            // wide_4m 0.738 -> 0.724 ms, 2,048 systems 1.661 -> 1.653 ms,
            // grad_1m 1.279 -> 1.268 ms; half a round or two rounds ahead gave
            // the same to 0.3 %; with 16 lanes per row it cost grad_1m 7 %, so
            // multi-RHS launches do without).
            if (LEVEL && G == 1) {
                const long long ahead = (long long)lo + (long long)gridDim.x * (blockDim.x >> 5) * CH + lane;
                if (ahead < a.n) {
                    prefetch_l2(a.perm + ahead);
                    prefetch_l2(a.lptr + ahead);
                    prefetch_l2(a.linv + ahead);
                }
            }
            if (HOSTIO && a.b_ready != nullptr)
                wait_b_chunk(a, lo, min(lo + CH, a.n));
#pragma unroll
            for (int r = 0; r < R * RPL; ++r)
                cache[r * 32 + lane] = VBits<T>::kPending;
            __syncwarp();
#pragma unroll 1
            for (int r = 0; r < R; ++r) {
                const int sub = lo + r * RPW;
                const int p = sub + rl;
                chunk_rows<T, G, KIND == kRowTwoPart, LEVEL, RPL, STAGE, HOSTIO>(
                    a, lo, sub, p, p < a.n && g * RPL < a.nrhs, g, cache, sl, t_pick, pol);
            }
            __syncwarp();
            if (HOSTIO && a.seg_count != nullptr)
                count_finished_rows(a, lo, min(lo + CH, a.n));
        } else {
            if (tk + 1u >= (unsigned)a.table_len)
                break;
            const int lo = ld_stream(a.table + tk, pol.stream), hi = ld_stream(a.table + tk + 1, pol.stream);
            if (HOSTIO && a.b_ready != nullptr)
                wait_b_chunk(a, lo, hi);
            if (hi - lo > 1) {
                cache[lane] = VBits<T>::kPending;
                __syncwarp();
                const int p = lo + rl;
                chunk_rows<T, G, false, LEVEL, 1, STAGE, HOSTIO>(a, lo, lo, p, p < hi && g < a.nrhs, g, cache, sl,
                                                                t_pick, pol);
                __syncwarp();
            } else {
                warp_row<T, G, LEVEL, HOSTIO>(a, lo, rl, g, sl, pol);
            }
            __syncwarp();
            if (HOSTIO && a.seg_count != nullptr)
                count_finished_rows(a, lo, hi);
        }
    }
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------

template <typename T, int G, int R, int KIND, bool LEVEL, bool CAP = false, int RPL = 1, bool STAGE = false,
          bool HOSTIO = false>
static cudaError_t launch_row_impl(const RowArgs<T> &a, int block, int bps, int num_sms,
                                   cudaStream_t st)
{
    constexpr int RPW = 32 / G;
    auto kern = row_solve_kernel<T, G, R, KIND, LEVEL, CAP, RPL, STAGE, HOSTIO>;
    const size_t smem = (size_t)(block / 32) * warp_smem_bytes<T>(R, RPL, STAGE);
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, block, smem);
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
    if (a.win_bytes == 0) {
        kern<<<(unsigned)grid, block, smem, st>>>(a);
        return cudaGetLastError();
    }
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[0].val.accessPolicyWindow.base_ptr = a.win_base;
    attr[0].val.accessPolicyWindow.num_bytes = a.win_bytes;
    attr[0].val.accessPolicyWindow.hitRatio = a.win_hit;
    attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a);
}

// one lane per row on the level schedule, entries staged in shared memory
template <typename T>
static cudaError_t launch_row_staged(const RowArgs<T> &a, int kind, int R, int block, int bps, int num_sms,
                                     cudaStream_t st)
{
    if (kind == kRowMix)
        return launch_row_impl<T, 1, 1, kRowMix, true, false, 1, true>(a, block, bps, num_sms, st);
    if (kind == kRowTwoPart) {
        switch (R) {
        case 4: return launch_row_impl<T, 1, 4, kRowTwoPart, true, false, 1, true>(a, block, bps, num_sms, st);
        case 2: return launch_row_impl<T, 1, 2, kRowTwoPart, true, false, 1, true>(a, block, bps, num_sms, st);
        default: return launch_row_impl<T, 1, 1, kRowTwoPart, true, false, 1, true>(a, block, bps, num_sms, st);
        }
    }
    switch (R) {
    case 4: return launch_row_impl<T, 1, 4, kRowWrtFst, true, false, 1, true>(a, block, bps, num_sms, st);
    case 2: return launch_row_impl<T, 1, 2, kRowWrtFst, true, false, 1, true>(a, block, bps, num_sms, st);
    default: return launch_row_impl<T, 1, 1, kRowWrtFst, true, false, 1, true>(a, block, bps, num_sms, st);
    }
}

template <typename T, int G, bool LEVEL>
static cudaError_t launch_row_g(const RowArgs<T> &a, int kind, int R, int block, int bps,
                                int num_sms, bool cap, bool stage, cudaStream_t st)
{
    if constexpr (G == 1 && LEVEL && sizeof(T) == 8) {
        if (stage)
            return launch_row_staged<T>(a, kind, R, block, bps, num_sms, st);
    }
    if constexpr (G >= 4 && LEVEL) {
        if (cap && kind == kRowWrtFst && R == 1)
            return launch_row_impl<T, G, 1, kRowWrtFst, LEVEL, true>(a, block, bps, num_sms, st);
    }
    if (kind == kRowMix)
        return launch_row_impl<T, G, 1, kRowMix, LEVEL>(a, block, bps, num_sms, st);
    // the two-phase schedule is the reference's single-RHS design; multi-RHS
    // launches use the write-first schedule
    if constexpr (G == 1) {
        if (kind == kRowTwoPart) {
            switch (R) {
            case 4: return launch_row_impl<T, G, 4, kRowTwoPart, LEVEL>(a, block, bps, num_sms, st);
            case 2: return launch_row_impl<T, G, 2, kRowTwoPart, LEVEL>(a, block, bps, num_sms, st);
            default: return launch_row_impl<T, G, 1, kRowTwoPart, LEVEL>(a, block, bps, num_sms, st);
            }
        }
    }
    switch (R) {
    case 4: return launch_row_impl<T, G, 4, kRowWrtFst, LEVEL>(a, block, bps, num_sms, st);
    case 2: return launch_row_impl<T, G, 2, kRowWrtFst, LEVEL>(a, block, bps, num_sms, st);
    default: return launch_row_impl<T, G, 1, kRowWrtFst, LEVEL>(a, block, bps, num_sms, st);
    }
}

// Write-first launches with more than 16 right-hand sides pack four of them
// per lane: 8 lanes per row instead of 32, so a warp keeps 4 rows in flight
// instead of 1 (measured on GB300: wide_4m with 32 RHS 3.34 -> 2.75 ms).  With
// fewer right-hand sides a lane per right-hand side is faster: the packed
// lane's serial loads, stores and FMAs lengthen every round (4 RHS: 1.02 ms
// unpacked, 1.92 ms packed).
template <typename T, bool LEVEL>
static cudaError_t launch_row_packed(const RowArgs<T> &a, int block, int bps, int num_sms, bool cap,
                                     cudaStream_t st)
{
    if (cap)
        return launch_row_impl<T, 8, 1, kRowWrtFst, LEVEL, true, 4>(a, block, bps, num_sms, st);
    return launch_row_impl<T, 8, 1, kRowWrtFst, LEVEL, false, 4>(a, block, bps, num_sms, st);
}

template <typename T, bool LEVEL>
static cudaError_t launch_row_sched(const RowArgs<T> &a, int kind, int rows_per_thread, int block,
                                    int blocks_per_sm, int num_sms, bool cap, bool stage, cudaStream_t st)
{
    if (kind == kRowWrtFst && rows_per_thread == 1 && a.nrhs > 16)
        return launch_row_packed<T, LEVEL>(a, block, blocks_per_sm, num_sms, cap, st);
    switch (lanes_for_rhs(a.nrhs)) {
    case 1: return launch_row_g<T, 1, LEVEL>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, cap, stage, st);
    case 2: return launch_row_g<T, 2, LEVEL>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, cap, stage, st);
    case 4: return launch_row_g<T, 4, LEVEL>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, cap, stage, st);
    case 8: return launch_row_g<T, 8, LEVEL>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, cap, stage, st);
    case 16: return launch_row_g<T, 16, LEVEL>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, cap, stage, st);
    default: return launch_row_g<T, 32, LEVEL>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, cap, stage, st);
    }
}

template <typename T>
cudaError_t launch_row_solve(const RowArgs<T> &a, int kind, int rows_per_thread, int block,
                             int blocks_per_sm, int num_sms, bool regcap, bool stage, cudaStream_t st)
{
    if (a.b_ready != nullptr || a.seg_count != nullptr) {
        if (a.perm == nullptr || regcap || !row_hostio_supported(kind, rows_per_thread, a.nrhs))
            return cudaErrorNotSupported;
        if constexpr (sizeof(T) == 8) {
            if (stage)
                return kind == kRowMix
                           ? launch_row_impl<T, 1, 1, kRowMix, true, false, 1, true, true>(a, block, blocks_per_sm,
                                                                                          num_sms, st)
                           : launch_row_impl<T, 1, 1, kRowWrtFst, true, false, 1, true, true>(a, block, blocks_per_sm,
                                                                                             num_sms, st);
        }
        return kind == kRowMix
                   ? launch_row_impl<T, 1, 1, kRowMix, true, false, 1, false, true>(a, block, blocks_per_sm, num_sms, st)
                   : launch_row_impl<T, 1, 1, kRowWrtFst, true, false, 1, false, true>(a, block, blocks_per_sm, num_sms,
                                                                                      st);
    }
    if (a.perm != nullptr)
        return launch_row_sched<T, true>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, regcap, stage,
                                         st);
    return launch_row_sched<T, false>(a, kind, rows_per_thread, block, blocks_per_sm, num_sms, regcap, false, st);
}

// ---------------------------------------------------------------------------
// fill the publication vector with the pending pattern, reset ticket
// counters and the error word
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

// ---------------------------------------------------------------------------
// level-schedule values
// ---------------------------------------------------------------------------

// Level-schedule values: linv[p] = 1/d_p and, for every dependency k of
// position p, lval[k] = -val[dep_src[k]] / d_p.  A warp takes 32 consecutive
// positions (lane l computes position l's 1/d) and walks their dependencies
// one per lane, each taking its position's 1/d from the owning lane, so the
// reads of dep_src and the writes of lval are coalesced.
template <typename T>
__global__ void __launch_bounds__(256) level_values_kernel(const int *__restrict__ lptr,
                                                           const int *__restrict__ dep_src,
                                                           const int *__restrict__ diag_src, int n,
                                                           const T *__restrict__ val, T *__restrict__ lval,
                                                           T *__restrict__ linv, int *bad)
{
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long p0 = warp * 32; p0 < n; p0 += nwarps * 32) {
        const int nr = (int)min(32LL, (long long)n - p0);
        T d = T(0);
        int start = INT_MAX;
        if (lane < nr) {
            const T dg = val[diag_src[p0 + lane]];
            if (!(dg != T(0)) || !isfinite(dg))
                atomicMin(bad, (int)(p0 + lane));
            d = T(1) / dg;
            linv[p0 + lane] = d;
            start = lptr[p0 + lane];
        }
        const int eb = __shfl_sync(kFullMask, start, 0);
        const int ee = lptr[p0 + nr];
        for (int kb = eb; kb < ee; kb += 32) {
            const int k = kb + lane;
            const int l = group_row_of(start, k, nr);
            const T dl = __shfl_sync(kFullMask, d, l);
            // pre-scaled dependencies: x_p = b/d_p + sum (-v/d_p) x_q
            if (k < ee)
                lval[k] = -val[dep_src[k]] * dl;
        }
    }
}

template <typename T>
cudaError_t launch_level_values(const int *lptr, const int *dep_src, const int *diag_src, int n,
                                const T *val, T *lval, T *linv, int *bad, cudaStream_t st)
{
    long long blocks = ((long long)n + 255) / 256;  // a warp per 32 positions
    if (blocks > 16384)
        blocks = 16384;
    if (blocks < 1)
        blocks = 1;
    level_values_kernel<T><<<(unsigned)blocks, 256, 0, st>>>(lptr, dep_src, diag_src, n, val, lval, linv, bad);
    return cudaGetLastError();
}

}  // namespace capsp
