// Batched peel for sm_103a: thousands of independent graphs in one persistent
// launch.  Each CTA takes the next graph from a device work counter (graphs
// ordered largest first by the host autotuner) and peels it alone with the
// reference's level-synchronous method (src/ours.cc:117-160), synchronising
// its levels and walk rounds with CTA barriers only.  A CTA owns its graph, so
// the state array is the graph's slice of the output: when the graph is done
// it holds the core numbers, exactly like the reference's degree array.
#pragma once
#include "kc_batch.cuh"
#include "kc_device.cuh"

namespace kc {
namespace {

struct BatchShared {
    uint32_t pref[kBatchChunk + 1];  // arc prefix of the items of one walk round
    uint32_t start[kBatchChunk];     // first arc of each item
    uint32_t warp_tot[kBatchWarps];
    uint32_t qtail;                  // vertices peeled so far in this graph
    uint32_t level_start;            // qtail when the level began (set before the level's barrier)
    uint32_t alen;                   // survivors appended to the next alive list
    uint32_t minv;                   // smallest survivor degree seen by a level's scan
    uint32_t g;                      // schedule index of the current graph
};

// Block-wide exclusive prefix sum of one value per thread.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x, BatchShared& sh, uint32_t* total) {
    const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t wt;
    const uint32_t ex = warp_excl_scan(x, &wt);
    if (lane == 0) sh.warp_tot[wid] = wt;
    __syncthreads();
    if (wid == 0) {
        const uint32_t t = lane < kBatchWarps ? sh.warp_tot[lane] : 0u;
        uint32_t tt;
        const uint32_t te = warp_excl_scan(t, &tt);
        if (lane < kBatchWarps) sh.warp_tot[lane] = te;
        if (lane == 0) sh.pref[kBatchChunk] = tt;   // stash the total
    }
    __syncthreads();
    *total = sh.pref[kBatchChunk];
    return sh.warp_tot[wid] + ex;
}

// Appends the vertices v of the lanes with `pred` at the position counter
// *tail of buffer q (the CTA's queue, or an alive list).
__device__ __forceinline__ void append_at(uint32_t* tail, uint32_t* q, bool pred, uint32_t v) {
    const unsigned m = __ballot_sync(kFull, pred);
    if (!m) return;
    const unsigned lane = threadIdx.x & 31;
    uint32_t pos = 0;
    if (lane == 0) pos = atomicAdd(tail, (unsigned)__popc(m));
    pos = __shfl_sync(kFull, pos, 0);
    if (pred) q[pos + __popc(m & lanemask_lt())] = v;
}

// Appends the vertices v of the lanes with `pred` to the CTA's queue.
__device__ __forceinline__ void enqueue(BatchShared& sh, uint32_t* q, bool pred, uint32_t v) {
    append_at(&sh.qtail, q, pred, v);
}

// Sets bit v of the shared-memory bitmap for the lanes with `pred`.
__device__ __forceinline__ void mark_peeled(uint32_t* bits, bool pred, uint32_t v) {
    if (pred) atomicOr(bits + (v >> 5), 1u << (v & 31u));
}

// Peels one graph (V vertices, graph-local CSR off/nb) with this CTA alone.
// w (V entries) receives the core numbers, q (>= V entries) is the CTA's
// queue / peel order, lists (2*qcap entries) holds two alive lists: once at
// most half the scanned vertices survive, a level's scan appends its
// survivors to a list and the next level scans that list instead of every
// vertex.  Thread 0 writes kmax and the level iterations run.
//
// bits (shared memory, bits_cap vertices, or null): a bitmap of the vertices
// queued so far.  With it the walk tests a neighbour's bit instead of reading
// its state from L2 first: an arc to a peeled vertex costs no L2 request, an
// arc to a live one costs one atomicSub, whose result decides as the
// reference's rule does (ours.cc:91-106; a neighbour queued by another thread
// of the same round whose bit was not yet visible is decremented and undone).
__device__ void peel_graph_cta(const uint32_t* off, const uint32_t* nb, uint32_t* w, uint32_t V, uint32_t* q,
                               uint32_t* lists, uint32_t qcap, int* err, uint32_t* kmax_out, uint32_t* iters_out,
                               BatchShared& sh, uint32_t* bits = nullptr, uint32_t bits_cap = 0) {
    const unsigned tid = threadIdx.x;
    if (V == 0) {   // the reference loop never runs: kmax = level-1 = 0xFFFFFFFF
        if (tid == 0) { *kmax_out = 0xFFFFFFFFu; *iters_out = 0; }
        return;
    }
    if (V > qcap) {
        if (tid == 0) atomicCAS(err, 0, kErrOverflow);
        return;
    }
    for (uint32_t b = 0; b < V; b += 4 * kBatchThreads) {
        uint32_t o[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t v = b + k * kBatchThreads + tid;
            o[k] = v < V ? KC_LDG(off + v + 1) - KC_LDG(off + v) : 0u;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t v = b + k * kBatchThreads + tid;
            if (v < V) w[v] = o[k];
        }
    }
    const bool use_bits = bits != nullptr && V <= bits_cap;
    if (use_bits)
        for (uint32_t i = tid; i < (V + 31) / 32; i += kBatchThreads) bits[i] = 0u;
    if (tid == 0) sh.qtail = 0;
    __syncthreads();

    uint32_t level = 0, iters = 0;
    // scan source: every vertex (src == nullptr) or the alive list src[0, nscan)
    const uint32_t* src = nullptr;
    uint32_t nscan = V, cur = 0;
    bool compact = false;   // this level's scan writes the next alive list
    for (;;) {
        if (tid == 0) { sh.minv = kFull; sh.level_start = sh.qtail; sh.alen = 0; }
        __syncthreads();
        // a snapshot taken before the barrier: the scan below appends at once
        const uint32_t lvl_start = sh.level_start;
        uint32_t* dst = lists + (size_t)(cur ^ 1u) * qcap;
        // scan: every vertex whose degree equals the level (ours.cc:15-25),
        // kScanLoads independent loads in flight per thread; survivors go to
        // the next alive list when compacting
        constexpr uint32_t kScanLoads = 8;
        uint32_t mymin = kFull;
        for (uint32_t base = 0; base < nscan; base += kBatchThreads * kScanLoads) {
            uint32_t vv[kScanLoads], d[kScanLoads];
#pragma unroll
            for (uint32_t k = 0; k < kScanLoads; ++k) {
                const uint32_t i = base + k * kBatchThreads + tid;
                vv[k] = i < nscan ? (src ? __ldcg(src + i) : i) : kFull;
            }
#pragma unroll
            for (uint32_t k = 0; k < kScanLoads; ++k) d[k] = vv[k] < V ? __ldcg(w + vv[k]) : kFull;
#pragma unroll
            for (uint32_t k = 0; k < kScanLoads; ++k) {
                const bool surv = d[k] != kFull && d[k] > level;
                if (surv) mymin = min(mymin, d[k]);
                enqueue(sh, q, d[k] == level, vv[k]);
                if (use_bits) mark_peeled(bits, d[k] == level, vv[k]);
                if (compact) append_at(&sh.alen, dst, surv, vv[k]);
            }
        }
        mymin = __reduce_min_sync(kFull, mymin);
        if ((tid & 31) == 0 && mymin != kFull) atomicMin(&sh.minv, mymin);
        __syncthreads();

        // walk rounds over the queue, including vertices appended by the walk
        // itself (same level, ours.cc:60-107)
        // Once every vertex is queued (claimed), the walks still queued can
        // only reach peeled vertices, which are never live (ours.cc:94): they
        // change nothing and are not run.
        uint32_t head = lvl_start;
        uint32_t tail = sh.qtail;
        while (head < tail && tail < V) {
            const uint32_t n = min(tail - head, kBatchChunk);
            uint32_t l0 = 0, l1 = 0, s0 = 0, s1 = 0;
            const uint32_t i0 = 2 * tid, i1 = 2 * tid + 1;
            if (i0 < n) { const uint32_t v = q[head + i0]; s0 = KC_LDG(off + v); l0 = KC_LDG(off + v + 1) - s0; }
            if (i1 < n) { const uint32_t v = q[head + i1]; s1 = KC_LDG(off + v); l1 = KC_LDG(off + v + 1) - s1; }
            uint32_t total;
            const uint32_t ex = block_excl_scan(l0 + l1, sh, &total);
            if (i0 < n) { sh.pref[i0] = ex; sh.start[i0] = s0; }
            if (i1 < n) { sh.pref[i1] = ex + l0; sh.start[i1] = s1; }
            __syncthreads();
            if (tid == 0) sh.pref[n] = total;
            __syncthreads();
            // kWalkArcs arcs per thread: neighbour ids, then degree pre-checks,
            // then the atomics, each group in flight together
            constexpr int kWalkArcs = 4;
            uint32_t lo = 0;
            for (uint32_t b = 0; b < total; b += kWalkArcs * kBatchThreads) {
                if (*(volatile uint32_t*)&sh.qtail >= V) break;   // all claimed (see above)
                uint32_t u[kWalkArcs];
#pragma unroll
                for (int j = 0; j < kWalkArcs; ++j) {
                    const uint32_t arc = b + j * kBatchThreads + tid;
                    u[j] = kFull;
                    if (arc < total) {
                        uint32_t hi = n;
                        while (hi - lo > 1) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (sh.pref[mid] <= arc) lo = mid; else hi = mid;
                        }
                        u[j] = KC_LDG(nb + sh.start[lo] + (arc - sh.pref[lo]));
                    }
                }
                // live: the reference's deg[u] > level test, from the bitmap or
                // from a read of the state
                bool live[kWalkArcs];
                if (use_bits) {
#pragma unroll
                    for (int j = 0; j < kWalkArcs; ++j)
                        live[j] = u[j] < V && !((bits[u[j] >> 5] >> (u[j] & 31u)) & 1u);
                } else {
                    uint32_t d[kWalkArcs];
#pragma unroll
                    for (int j = 0; j < kWalkArcs; ++j) d[j] = u[j] < V ? __ldcg(w + u[j]) : 0u;
#pragma unroll
                    for (int j = 0; j < kWalkArcs; ++j) live[j] = u[j] < V && d[j] > level;
                }
                uint32_t old[kWalkArcs];
#pragma unroll
                for (int j = 0; j < kWalkArcs; ++j) old[j] = live[j] ? atomicSub(w + u[j], 1u) : 0u;
#pragma unroll
                for (int j = 0; j < kWalkArcs; ++j) {
                    // (ours.cc:91-106): the decrement that took u to the level
                    // queues it; one that raced below the level is undone
                    if (live[j] && old[j] <= level) atomicAdd(w + u[j], 1u);
                    const bool hit = live[j] && old[j] == level + 1;
                    if (use_bits) mark_peeled(bits, hit, u[j]);
                    enqueue(sh, q, hit, u[j]);
                }
            }
            __syncthreads();
            head += n;
            tail = sh.qtail;
            __syncthreads();
        }
        ++iters;
        if (tail >= V) {
            if (tid == 0) { *kmax_out = level; *iters_out = iters; }
            return;
        }
        // The next level scans the list this level wrote; it writes a new one
        // once at most half of what it scans can survive.
        if (compact) {
            src = dst;
            nscan = min(sh.alen, qcap);
            cur ^= 1u;
        }
        compact = V - tail <= nscan / 2;
        // A level that peeled nothing changed no degree: jump to the smallest
        // survivor degree (every level in between is empty).
        uint32_t next = level + 1;
        const uint32_t mn = sh.minv;
        if (tail == lvl_start && mn != kFull && mn > next) next = mn;
        if (next > V) {   // cannot happen for a valid CSR: every vertex is peeled by its degree
            if (tid == 0) atomicCAS(err, 0, kErrOverflow);
            return;
        }
        level = next;
        __syncthreads();
    }
}

}  // namespace
}  // namespace kc
