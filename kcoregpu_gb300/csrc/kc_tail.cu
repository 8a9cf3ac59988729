// Tail of the single-graph peel for sm_103a: one CTA finishes the
// level-synchronous peel (src/ours.cc:117-160) on the induced subgraph of the
// survivors that the persistent kernel built when it stopped (local ids,
// kc_peel_impl.cuh tail_handoff).  The states live in shared memory, so a
// decrement is a shared-memory atomic and a level costs CTA barriers instead
// of the grid-wide arrival protocol.  The walk follows the reference rule:
// a neighbour whose degree is above the level is decremented, the decrement
// that takes it to the level adds it to this level's queue, and a decrement
// that raced below the level is undone (ours.cc:91-106).  Launched after the
// persistent kernel on the same stream; it returns at once when no hand-off
// happened.
//
// The induced CSR pads every adjacency to a multiple of 4 entries (pad =
// 0xFFFFFFFF), so the walk reads 16-byte quads that never straddle two
// vertices: each thread keeps kTailQuads quads (16 arcs) in flight.
#include "kc_device.cuh"
#include "kc_peel.cuh"

namespace kc {
namespace {

constexpr int kTailQuads = 4;   // 16-byte quads per thread per walk step

struct TailSmem {
    uint32_t st[kTailV];              // remaining degree; the core number once peeled
    uint32_t off[kTailV + 4];         // induced CSR offsets (multiples of 4); the bulk copy's round-up
    uint32_t q[kTailV];               // local ids in peel order
    uint32_t pref[kTailItems + 1];    // quad prefix of the items of one walk round
    uint32_t start[kTailItems];       // first quad of each item
    uint32_t warp_tot[kTailWarps];
    uint32_t wmin[2][kTailWarps];     // each warp's smallest survivor state, by level parity
    uint32_t qtail;
    uint32_t total;
    unsigned long long bar;           // mbarrier of the bulk copies that stage the offsets and cursors
};
static_assert(offsetof(TailSmem, off) % 16 == 0 && offsetof(TailSmem, st) % 16 == 0 &&
              offsetof(TailSmem, bar) % 8 == 0, "bulk-copy destinations and the mbarrier are aligned");

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Stages `bytes` (a multiple of 16) from global `src` into shared `dst` with
// one bulk copy (the TMA engine) that completes on mbarrier `bar`.
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Block-wide exclusive prefix sum of one value per thread.
__device__ __forceinline__ uint32_t tail_scan(uint32_t x, TailSmem& s, uint32_t* total) {
    const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t wt;
    const uint32_t ex = warp_excl_scan(x, &wt);
    if (lane == 0) s.warp_tot[wid] = wt;
    __syncthreads();
    if (wid == 0) {
        uint32_t all;
        const uint32_t te = warp_excl_scan(lane < kTailWarps ? s.warp_tot[lane] : 0u, &all);
        if (lane < kTailWarps) s.warp_tot[lane] = te;
        if (lane == 0) s.total = all;
    }
    __syncthreads();
    *total = s.total;
    return s.warp_tot[wid] + ex;
}

__global__ void __launch_bounds__(kTailThreads, 1) peel_tail_kernel(const __grid_constant__ PeelArgs a) {
    extern __shared__ __align__(16) unsigned char tail_smem[];
    TailSmem& s = *reinterpret_cast<TailSmem*>(tail_smem);
    PeelCtl* ctl = a.ctl;
    const unsigned tid = threadIdx.x, lane = tid & 31;
    const uint32_t n = ctl->tail_n;
    if (n == 0 || ctl->err != 0 || ctl->hx.tail_solved) return;   // (the cluster h-index tail finished it)
    if (n > kTailV || n > a.tail_cap_v) {
        if (tid == 0) record_error(ctl, kErrOverflow, ctl->tail_level);
        return;
    }
    const uint32_t max_level = a.max_level == kFull ? ctl->maxdeg : a.max_level;
    const uint32_t peeled0 = ctl->tail_peeled;
    const uint32_t nquads = ctl->tail_arcs / 4;
    const uint4* nbr4 = reinterpret_cast<const uint4*>(a.tail_nbr);
    uint32_t level = ctl->tail_level;
    uint32_t it = ctl->tail_iter;
    const uint32_t it0 = it;
    const unsigned long long t_entry = now_ns();
    {   // Offsets, and degrees from the fill cursors (they stopped at offset +
        // degree): two bulk copies stage both arrays in shared memory, the
        // cursors into the state array, which then becomes cursor - offset.
        const uint32_t off_bytes = ((n + 1) * 4u + 15u) & ~15u;   // <= (kTailV + 4) * 4
        const uint32_t cur_bytes = (n * 4u + 15u) & ~15u;         // <= kTailV * 4
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s.bar)) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&s.bar)),
                         "r"(off_bytes + cur_bytes)
                         : "memory");
            bulk_to_smem(s.off, a.tail_off, off_bytes, &s.bar);
            bulk_to_smem(s.st, a.tail_cur, cur_bytes, &s.bar);
        }
        __syncthreads();   // the barrier is initialised before anyone polls it
        // every thread waits for phase 0, bounded in time (the copies are
        // 128 KB at most: a stuck wait means a broken device)
        bool arrived = false;
        const unsigned long long t0 = now_ns();
        const unsigned long long limit = (unsigned long long)a.wait_us * 1000ull;
        while (!(arrived = mbar_try_wait(&s.bar, 0)) && now_ns() - t0 < limit) {}
        if (!__syncthreads_and(arrived)) {
            if (tid == 0) record_error(ctl, kErrTimeout, ctl->tail_level);
            // the copies may still land: wait for them once more before leaving,
            // bounded by at least 2 s whatever the wait limit (a shortened
            // limit must not let the CTA exit with its copies in flight)
            const unsigned long long t1 = now_ns();
            const unsigned long long drain = limit > 2000000000ull ? limit : 2000000000ull;
            while (!mbar_try_wait(&s.bar, 0) && now_ns() - t1 < drain) {}
            return;
        }
        for (uint32_t i = tid; i < n; i += kTailThreads) s.st[i] -= s.off[i];
        if (tid == 0) s.qtail = 0;
        __syncthreads();   // states and the queue end are set before the first scan
    }

    bool failed = false;
    // The queue end at the start of the level; every thread holds the same
    // value (read before the barrier that closed the previous level).
    uint32_t lvl_start = 0;
    for (;;) {
        const unsigned long long t_start = (a.trace && tid == 0) ? now_ns() : 0ull;
        const uint32_t par = it & 1u;
        // scan: every vertex whose degree equals the level (ours.cc:15-25);
        // peeled vertices keep the level they were peeled at, below this one.
        // 16-byte reads of 4 states, up to 4 groups per lane with their loads
        // in flight together, and one warp-aggregated append for all of them
        // (a shared-memory atomic on one word costs ~30 cycles per warp, in
        // series).  The smallest survivor state is kept per warp, with no
        // atomic: only a level that peels nothing needs it.
        uint32_t mymin = kFull, hit = 0;
        {
            const uint32_t wb = (tid >> 5) * 128 + 4 * lane;
            uint4 x[kTailV / (4 * kTailThreads)];
#pragma unroll
            for (uint32_t r = 0; r < kTailV / (4 * kTailThreads); ++r) {
                const uint32_t b = wb + r * 4 * kTailThreads;
                x[r] = b < n ? *reinterpret_cast<const uint4*>(s.st + b) : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (uint32_t r = 0; r < kTailV / (4 * kTailThreads); ++r) {
                const uint32_t b = wb + r * 4 * kTailThreads;
                const uint32_t d[4] = {x[r].x, x[r].y, x[r].z, x[r].w};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (b + k < n && d[k] > level) mymin = min(mymin, d[k]);
                    if (b + k < n && d[k] == level) hit |= 1u << (4 * r + k);
                }
            }
            if (__any_sync(kFull, hit != 0)) {
                uint32_t htot;
                const uint32_t hex = warp_excl_scan(__popc(hit), &htot);
                uint32_t pos = 0;
                if (lane == 0) pos = atomicAdd(&s.qtail, htot);
                pos = __shfl_sync(kFull, pos, 0) + hex;
                for (uint32_t m = hit; m; m &= m - 1u) {
                    const uint32_t bit = __ffs(m) - 1;
                    if (pos < kTailV) s.q[pos] = wb + (bit >> 2) * 4 * kTailThreads + (bit & 3u);
                    ++pos;
                }
            }
        }
        mymin = __reduce_min_sync(kFull, mymin);
        if (lane == 0) s.wmin[par][tid >> 5] = mymin;
        __syncthreads();

        // walk rounds over the queue, including the vertices the walk itself
        // appends (same level)
        uint32_t head = lvl_start, tail = min(s.qtail, n);   // each vertex is queued once
        uint32_t rounds = 0, quads = 0;
        // Once every vertex is claimed (queued), the walks still queued can
        // only decrement peeled vertices, whose state (their core number) is
        // at or below the level: the reference rule skips those (ours.cc:94),
        // so they change nothing and are not run.  The final collapse of a
        // dense core is where this pays.
        while (head < tail && tail < n) {
            ++rounds;
            const uint32_t m = min(tail - head, kTailItems);
            const uint32_t i0 = 2 * tid, i1 = 2 * tid + 1;
            uint32_t total;
            if (m <= 64) {   // one warp holds every item: a warp scan and one barrier
                if (tid < 32) {
                    uint32_t s0 = 0, s1 = 0, l0 = 0, l1 = 0;
                    if (i0 < m) { const uint32_t v = s.q[head + i0]; s0 = s.off[v] >> 2; l0 = (s.off[v + 1] >> 2) - s0; }
                    if (i1 < m) { const uint32_t v = s.q[head + i1]; s1 = s.off[v] >> 2; l1 = (s.off[v + 1] >> 2) - s1; }
                    uint32_t wt;
                    const uint32_t ex = warp_excl_scan(l0 + l1, &wt);
                    if (i0 < m) { s.pref[i0] = ex; s.start[i0] = s0; }
                    if (i1 < m) { s.pref[i1] = ex + l0; s.start[i1] = s1; }
                    if (tid == 0) { s.pref[m] = wt; s.total = wt; }
                }
                __syncthreads();
                total = s.total;
            } else {
                uint32_t s0 = 0, s1 = 0, l0 = 0, l1 = 0;
                if (i0 < m) { const uint32_t v = s.q[head + i0]; s0 = s.off[v] >> 2; l0 = (s.off[v + 1] >> 2) - s0; }
                if (i1 < m) { const uint32_t v = s.q[head + i1]; s1 = s.off[v] >> 2; l1 = (s.off[v + 1] >> 2) - s1; }
                const uint32_t ex = tail_scan(l0 + l1, s, &total);
                if (i0 < m) { s.pref[i0] = ex; s.start[i0] = s0; }
                if (i1 < m) { s.pref[i1] = ex + l0; s.start[i1] = s1; }
                if (tid == 0) s.pref[m] = total;
                __syncthreads();
            }
            // Quads are spread over all threads (thread t takes quads b + j *
            // kTailThreads + t) so that a small round costs one quad per
            // thread; warps past the round's end skip with a uniform branch.
            const uint32_t wq = (tid & ~31u);   // this warp's first quad offset
            uint32_t lo = 0;
            for (uint32_t b = 0; b < total; b += kTailQuads * kTailThreads) {
                if (b + wq >= total) break;   // warp-uniform
                if (*(volatile uint32_t*)&s.qtail >= n) break;   // all claimed (see above); one load, warp-uniform
                uint4 x[kTailQuads];
#pragma unroll
                for (int j = 0; j < kTailQuads; ++j) {
                    const uint32_t qi = b + j * kTailThreads + tid;
                    x[j] = make_uint4(kFull, kFull, kFull, kFull);
                    if (qi < total) {
                        uint32_t hi = m;
                        while (hi - lo > 1) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (s.pref[mid] <= qi) lo = mid; else hi = mid;
                        }
                        const uint32_t p = s.start[lo] + (qi - s.pref[lo]);
                        if (p < nquads) x[j] = __ldcg(nbr4 + p);
                    }
                }
                // decrements (ours.cc:91-106); pads and out-of-range ids are
                // skipped.  The degree pre-checks are read first: they only
                // filter, the atomic's result decides.
                uint32_t hit = 0;
#pragma unroll
                for (int j = 0; j < kTailQuads; ++j) {
                    if (b + j * kTailThreads + wq >= total) break;   // warp-uniform
                    const uint32_t u[4] = {x[j].x, x[j].y, x[j].z, x[j].w};
                    uint32_t d[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) d[k] = u[k] < n ? s.st[u[k]] : 0u;
                    uint32_t old[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) old[k] = d[k] > level ? atomicSub(&s.st[u[k]], 1u) : 0u;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if (d[k] <= level) continue;
                        if (old[k] == level + 1) hit |= 1u << (4 * j + k);
                        else if (old[k] <= level) atomicAdd(&s.st[u[k]], 1u);   // undo (ours.cc:102-105)
                    }
                }
                // the decrements that took a vertex to the level queue it
                if (__any_sync(kFull, hit != 0)) {
                    uint32_t htot;
                    const uint32_t hex = warp_excl_scan(__popc(hit), &htot);
                    uint32_t pos = 0;
                    if (lane == 0) pos = atomicAdd(&s.qtail, htot);
                    pos = __shfl_sync(kFull, pos, 0) + hex;
#pragma unroll
                    for (int j = 0; j < kTailQuads; ++j) {
                        const uint32_t u[4] = {x[j].x, x[j].y, x[j].z, x[j].w};
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            if ((hit >> (4 * j + k)) & 1u) { if (pos < kTailV) s.q[pos] = u[k]; ++pos; }
                    }
                }
            }
            quads += total;
            __syncthreads();
            head += m;
            tail = min(s.qtail, n);
        }
        ++it;
        const uint32_t peeled = peeled0 + tail;
        if (tid == 0) {
            if (a.trace && it - 1 < a.trace_cap) {
                // Tail rows: 0 level start (the first: this kernel's entry),
                // 3 level end, 4 vertices peeled so far, 6 walk rounds, 7
                // quads walked; 1, 2 and 5 = level end, except in the first
                // row, which keeps the hand-off's times there (both barriers
                // passed, CTA 0's fill done).
                unsigned long long* row = a.trace + (size_t)(it - 1) * kTraceFields;
                const unsigned long long t_end = now_ns();
                row[0] = it - 1 == it0 ? t_entry : t_start;
                row[3] = t_end;
                row[4] = peeled;
                row[6] = rounds;
                row[7] = quads;
                if (it - 1 != it0) { row[1] = t_end; row[2] = t_end; row[5] = t_end; }
            }
            if (a.shells && level + 1 < a.shell_cap) a.shells[level + 1] = peeled;
        }
        if (tail >= n) break;
        // A level that peeled nothing changed no degree: jump to the smallest
        // survivor degree (every level in between is empty).
        uint32_t next = level + 1;
        if (tail == lvl_start) {
            uint32_t mn = kFull;
            for (uint32_t w = 0; w < kTailWarps; ++w) mn = min(mn, s.wmin[par][w]);
            if (mn != kFull && mn > next) next = mn;
        }
        if (next > max_level) {   // cannot happen for a valid CSR: every vertex is peeled by its degree
            if (tid == 0) record_error(ctl, kErrOverflow, level);
            failed = true;
            break;
        }
        if (tid == 0 && a.shells)
            for (uint32_t l = level + 2; l <= next && l < a.shell_cap; ++l) a.shells[l] = peeled;
        level = next;
        lvl_start = tail;
        __syncthreads();   // every thread has read the queue end and the minima
    }
    if (failed) return;
    // Outputs: the state of a peeled vertex is its core number; the queue is
    // the peel order of the tail.
    for (uint32_t i = tid; i < n; i += kTailThreads) {
        const uint32_t v = __ldcg(a.tail_ids + i);
        if (v < a.V) a.core[v] = s.st[i];
    }
    if (a.order) {
        for (uint32_t p = tid; p < n; p += kTailThreads) {
            const uint32_t lid = s.q[p];
            if (lid < n && peeled0 + p < a.V) a.order[peeled0 + p] = __ldcg(a.tail_ids + lid);
        }
    }
    if (tid == 0) {
        ctl->kmax = level;
        ctl->levels = level + 1;
        ctl->iterations = it;
    }
}

}  // namespace

const void* peel_tail_fn() { return reinterpret_cast<const void*>(&peel_tail_kernel); }
size_t peel_tail_smem() { return sizeof(TailSmem); }

}  // namespace kc
