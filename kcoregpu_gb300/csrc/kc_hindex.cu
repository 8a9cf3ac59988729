// h-index peel of one graph for sm_103a: the same core numbers as the level
// peel (src/ours.cc:117-160), found as the fixed point of the h-index operator
// instead of level by level.
//
// Start from est[v] = deg(v) and replace est[v] by min(est[v], h) where h is
// the h-index of the neighbours' estimates (the largest h such that at least h
// neighbours have an estimate >= h).  Every estimate stays an upper bound of
// the core number whatever values the update reads, as long as each value read
// is itself such an upper bound, and once est[v] <= h holds for every v the
// estimates are the core numbers: for each k the vertices with estimate >= k
// then have at least k neighbours among themselves, so they lie in the k-core,
// while the core numbers are themselves a fixed point reached from above
// (Lu, Zhou, Zhang and Stanley, "The H-index of a network node and its
// relation to degree and coreness", Nature Communications 7, 2016;
// Montresor, De Pellegrini and Miorandi, "Distributed k-core decomposition",
// IEEE TPDS 24, 2013).  The benchmark graphs converge in 35 to 61
// iterations, where the level peel needs 175 to 253 levels, 85 of them
// grid-wide, plus hundreds of dependent rounds in its one-CTA tail.
//
// Work is kept to the vertices whose estimate can change.  cnt[v] counts the
// neighbours whose estimate was >= est[v] in the reads that found est[v], so
// cnt[v] >= est[v].  A neighbour whose estimate later drops from `old` to
// `new` with new < est[v] <= old takes one off cnt[v], and the decrement that
// takes cnt[v] below est[v] (exactly one per drop below) queues v.  cnt[v]
// never exceeds the true count: a neighbour read before its drop is taken off
// again by that drop, one read after it may be taken off twice, which only
// queues v once more.  One iteration is
//   phase A: each queued vertex recomputes min(est, h) and the count at the
//            new value, both from one read of its neighbours' estimates (reads
//            of estimates that other vertices change in the same pass are
//            older or newer upper bounds); a drop records the old value and
//            queues update tasks;
//   phase B: each vertex that dropped scans its neighbours and decrements the
//            counts its drop crossed (no estimate changes in phase B).
// The estimates are final when phase B queues nothing.
//
// Kernel shape: one cooperative launch of one 512-thread CTA per SM.  Phases
// and the window passes below are separated by a time-bounded grid barrier.
//   * Iteration 1 reads every vertex: a lane computes the h-index of a vertex
//     with at most kHxLaneArcs arcs from values in registers; larger vertices
//     are queued.
//   * A vertex of at most kHxWarpArcs arcs is one warp: 8 values a lane in
//     registers, binary search on h with warp reductions.
//   * A larger vertex gets a window slot and is split into chunk tasks of
//     kHxChunk arcs spread over the grid.  Each chunk bins its neighbours'
//     estimates into 32 bins of a window [lo, hi] (plus one bin above hi) in
//     global counters; the warp that finishes the last chunk of the pass reads
//     the bins, and either finds h (bins one wide) or narrows the window to
//     the bin holding h (or the range below it) for another pass.  Every pass
//     counts afresh, so the final h and its count come from one pass's reads.
// Once the frontier is small, the last iterations go to a 16-CTA cluster
// kernel (kc_hxtail.cu): the set of vertices at or above a floor T, handed
// over only when every member has at least T neighbours in it (try_handoff
// below), so that the vertices outside it are already final.
// A graph that needs more than max_iters iterations (long paths converge one
// hop per iteration) is left to the level peel: the kernel returns without
// setting HxCtl::solved and the persistent and tail kernels run as usual.
#include "kc_device.cuh"
#include "kc_peel.cuh"

namespace kc {
namespace {

constexpr uint32_t kWarps = kPeelThreads / 32;
constexpr uint32_t kNoBin = 0xFFu;
constexpr uint32_t kBatchVals = 512;   // neighbour estimates a warp gathers into shared memory at once
// CTA entries per CTA in one pass before they go to window searches instead
// (2 and 4 measured: 4 took 3.5% off the Chung-Lu 2.4M peel, the R-MAT
// graphs within 0.5%)
constexpr uint32_t kCtaEntries = 4;
constexpr uint32_t kListTask = 0x80000000u;   // update task flag: scan the active list, not the adjacency
constexpr uint32_t kListMargin = 64;   // a rebuilt list also keeps neighbours this far below the window
constexpr uint32_t kListGuard = 4;     // an estimate this close to its list's floor rebuilds the list first
constexpr uint32_t kListFlag = 0x80000000u;   // warp-frontier entry flag: a large vertex read from its active list

struct HxShared {
    unsigned long long bt_stage[kWarps][32];   // per-warp staging of update tasks
    uint32_t rm_stage[kWarps][32];             // per-warp staging of frontier entries
    uint32_t wbin[kWarps][33];                 // per-warp bin counts of one chunk; phase B: task prefix
    uint32_t tstart[kWarps][32];               // phase B: first arc, old and new estimate of 32 tasks
    uint32_t told[kWarps][32];
    uint32_t tnew[kWarps][32];
    uint32_t vals[kWarps][kBatchVals];         // phase A: gathered neighbour estimates of a batch
    int bar_ok;
    unsigned bar_k;   // grid barriers passed (thread 0)
    uint32_t red[kWarps];   // CTA reductions
    uint32_t cpos;          // CTA path: active-list append cursor
};
static_assert(sizeof(uint32_t) * kWarps * kBatchVals == sizeof(uint32_t) * kHxCtaVals, "the CTA path uses every warp's values");

// Grid barrier of the cooperative launch, bounded in time; false when the wait
// ran out or an error was recorded (every CTA then returns).  Arrivals only
// add to one counter (barrier k is complete at k * grid arrivals), so the
// last arrival needs no reset and the waiters one load: a fence, an add and
// the poll are the whole cost.
__device__ bool hx_barrier(const HxArgs& a, HxShared& sh) {
    __syncthreads();
    if (threadIdx.x == 0) {
        PeelCtl* ctl = a.ctl;
        int ok = 1;
        const unsigned target = ++sh.bar_k * gridDim.x;
        __threadfence();
        asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" ::"l"(&ctl->hx.bar) : "memory");
        const unsigned long long t0 = now_ns(), lim = (unsigned long long)a.wait_us * 1000ull;
        uint32_t polls = 0;
        while (ld_acquire(&ctl->hx.bar) < target) {
            if ((++polls & 31u) == 0) {
                if (ld_err(&ctl->err)) { ok = 0; break; }
                if (now_ns() - t0 > lim) { record_error(ctl, kErrTimeout, ctl->hx.iters); ok = 0; break; }
            }
        }
        if (ld_err(&ctl->err)) ok = 0;
        sh.bar_ok = ok;
    }
    __syncthreads();
    return sh.bar_ok != 0;
}

// Per-warp staging of list appends: entries collect in shared memory and go
// to the global list 32 at a time, one atomic per flush.
struct Stager {
    uint32_t n_bt = 0, n_rm = 0;
};

__device__ __forceinline__ void flush_bt(const HxArgs& a, HxShared& sh, Stager& s, uint32_t p) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    if (s.n_bt == 0) return;
    __syncwarp();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&a.ctl->hx.bt_n[p], s.n_bt);
    base = __shfl_sync(kFull, base, 0);
    if (lane < s.n_bt) {
        if (base + lane < a.cap_bt) a.bt[p][base + lane] = sh.bt_stage[wid][lane];
        else record_error(a.ctl, kErrOverflow, 0);
    }
    s.n_bt = 0;
    __syncwarp();
}

// Lanes in `mask` append one update task each.
__device__ __forceinline__ void stage_bt(const HxArgs& a, HxShared& sh, Stager& s, uint32_t p, unsigned mask,
                                         unsigned long long task) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    const uint32_t k = __popc(mask);
    if (k == 0) return;
    if (s.n_bt + k > 32) flush_bt(a, sh, s, p);
    if (mask & (1u << lane)) sh.bt_stage[wid][s.n_bt + __popc(mask & lanemask_lt())] = task;
    s.n_bt += k;
    __syncwarp();
    if (s.n_bt == 32) flush_bt(a, sh, s, p);
}

__device__ __forceinline__ void flush_rm(const HxArgs& a, HxShared& sh, Stager& s, uint32_t q) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    if (s.n_rm == 0) return;
    __syncwarp();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&a.ctl->hx.rm_n[q], s.n_rm);
    base = __shfl_sync(kFull, base, 0);
    if (lane < s.n_rm) {
        if (base + lane < a.V) a.rm[q][base + lane] = sh.rm_stage[wid][lane];
        else record_error(a.ctl, kErrOverflow, 0);
    }
    s.n_rm = 0;
    __syncwarp();
}

__device__ __forceinline__ void stage_rm(const HxArgs& a, HxShared& sh, Stager& s, uint32_t q, unsigned mask,
                                         uint32_t v) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    const uint32_t k = __popc(mask);
    if (k == 0) return;
    if (s.n_rm + k > 32) flush_rm(a, sh, s, q);
    if (mask & (1u << lane)) sh.rm_stage[wid][s.n_rm + __popc(mask & lanemask_lt())] = v;
    s.n_rm += k;
    __syncwarp();
    if (s.n_rm == 32) flush_rm(a, sh, s, q);
}

__device__ __forceinline__ uint32_t bin_shift(uint32_t lo, uint32_t hi) {
    uint32_t sh = 0;
    while (((hi - lo) >> sh) >= 32u) ++sh;   // (hi - lo + 1) <= 32 << sh
    return sh;
}

// Queues the chunk tasks of slot s (pass over `len` entries) for sub-phase r+1.
__device__ __forceinline__ void queue_chunks(const HxArgs& a, uint32_t r, uint32_t s, uint32_t nch, unsigned lane,
                                             unsigned step) {
    HxCtl* hx = &a.ctl->hx;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&hx->cl_n[(r + 1) % 3], nch);
    if (step == 32) base = __shfl_sync(kFull, base, 0);
    if (base + nch > a.cap_cl) {
        if (lane == 0) record_error(a.ctl, kErrOverflow, 0);
        return;
    }
    for (uint32_t c = lane; c < nch; c += step) a.cl[(r + 1) % 3][base + c] = ((unsigned long long)s << 32) | c;
}

// One lane opens a window slot for large vertex v (d arcs, estimate e) in the
// frontier of parity q, searching [lo, hi] in the active list (mode 1, len
// entries) or the adjacency (mode 0, which rebuilds the list), and queues its
// chunk tasks for sub-phase r+1.
__device__ void open_window(const HxArgs& a, uint32_t q, uint32_t r, uint32_t v, uint32_t e, uint32_t lo, uint32_t hi,
                            uint32_t mode, uint32_t len) {
    HxCtl* hx = &a.ctl->hx;
    const uint32_t s = atomicAdd(&hx->rl_n[q], 1u);
    if (s >= a.cap_l) { record_error(a.ctl, kErrOverflow, 0); return; }
    HxSlot sl;
    sl.v = v;
    sl.e = e;
    sl.lo = lo;
    sl.hi = hi;
    sl.mode = mode;
    sl.len = len;
    if (mode == 0) a.alen[v] = lo > kListMargin ? 0u : kFull;   // the pass rebuilds the list (none from floor 0)
    sl.sh = bin_shift(lo, hi);
    sl.done = 0;
    sl.nch = (len + kHxChunk - 1) / kHxChunk;
    sl.pad[0] = sl.pad[1] = sl.pad[2] = 0;
    const uint32_t nch = sl.nch;
    a.slots[q][s] = sl;
    uint4* b = reinterpret_cast<uint4*>(a.bins[q] + (size_t)s * kHxBinWords);
#pragma unroll
    for (int i = 0; i < (int)(kHxBinWords / 4); ++i) b[i] = make_uint4(0, 0, 0, 0);
    queue_chunks(a, r, s, nch, 0, 1);
}

// One lane queues large vertex v (entry flag kListFlag: read its active list)
// for the CTA path of sub-phase r+1.
__device__ __forceinline__ void push_cta(const HxArgs& a, uint32_t r, uint32_t ent) {
    const uint32_t i = atomicAdd(&a.ctl->hx.rc_n[(r + 1) % 3], 1u);
    if (i < a.cap_l) a.rc[(r + 1) % 3][i] = ent;
    else record_error(a.ctl, kErrOverflow, 0);
}

// The window of a large vertex queued for recomputation: its active list from
// the top 32 values down (when it has one), else the adjacency, from [0, e]
// when coarse (iterations 1 and 2, where estimates fall far) or the top 32
// values.
__device__ void open_slot(const HxArgs& a, uint32_t q, uint32_t r, uint32_t v, uint32_t e, uint32_t d, bool coarse) {
    const uint32_t al = coarse ? kFull : __ldcg(a.alen + v);
    const uint32_t l0 = coarse ? 0u : __ldcg(a.alo + v);
    const uint32_t top = e >= 31u ? e - 31u : 0u;
    if (al != kFull && al != 0 && l0 <= e) open_window(a, q, r, v, e, max(l0, top), e, 1, al);
    else open_window(a, q, r, v, e, coarse ? 0u : top, e, 0, d);
}

// Largest h in [fl, e] with ge(h) >= h, where ge(h) counts values >= h (non-
// increasing in h); kFull when ge(fl) < fl.  Probes e, e-1, e-3, e-7, ...
// (late drops are small), then bisects the last step.
template <class Ge>
__device__ __forceinline__ uint32_t gallop_hindex(Ge ge, uint32_t fl, uint32_t e) {
    uint32_t bad = e + 1, t = 1, lo;
    for (;;) {
        const uint32_t cand = e - fl >= t - 1 ? e - (t - 1) : fl;
        if (ge(cand) >= cand) { lo = cand; break; }
        bad = cand;
        if (cand == fl) return kFull;
        t <<= 1;
    }
    uint32_t hi = bad - 1;   // ge(bad) < bad
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (ge(mid) >= mid) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Largest h in [fl, e] with ge(h) >= h by bisection; kFull when ge(fl) < fl.
// For iterations 1 and 2, where estimates fall far: about log2(e - fl) probes
// against galloping's two per halving of the drop (1-2% off the benchmark
// peels).
template <class Ge>
__device__ __forceinline__ uint32_t bisect_hindex(Ge ge, uint32_t fl, uint32_t e) {
    if (ge(fl) < fl) return kFull;
    uint32_t lo = fl, hi = e;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (ge(mid) >= mid) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Largest h in [fl, e] with at least h of the d values xs[0..d) >= h (d <=
// kBatchVals, in shared memory), and the count at that h; kFull when fewer
// than fl values are >= fl (the h-index lies below the floor).  One warp.
__device__ __forceinline__ uint32_t warp_hindex(const uint32_t* xs, uint32_t d, uint32_t fl, uint32_t e,
                                                uint32_t* count, bool far) {
    const unsigned lane = lane_id();
    constexpr int kPer = kBatchVals / 32;
    uint32_t x[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
        const uint32_t idx = lane + 32u * j;
        x[j] = idx < d ? xs[idx] : 0u;
    }
    auto ge = [&](uint32_t h) {
        uint32_t c = 0;
#pragma unroll
        for (int j = 0; j < kPer; ++j) c += (lane + 32u * j < d && x[j] >= h) ? 1u : 0u;
        return __reduce_add_sync(kFull, c);
    };
    const uint32_t h = far ? bisect_hindex(ge, fl, e) : gallop_hindex(ge, fl, e);   // warp-uniform
    if (h != kFull) *count = ge(h);
    return h;
}

// Phase A for the warp frontier, up to 8 list entries per warp step: vertices of
// at most kHxWarpArcs arcs (their adjacency) and large vertices whose active
// list holds at most kBatchVals entries (entry flag kListFlag; the search
// starts at the list's floor).  The neighbours' estimates of as many whole
// entries as fit kBatchVals values are gathered into shared memory with all
// loads in flight (the dependent load chain is paid once per batch, not once
// per vertex); then a lane (all degrees <= 32) or the warp finds each
// h-index from shared memory.  An h-index below a list's floor sends the
// vertex to a window search over its adjacency in the next pass.
__device__ void warp_batch(const HxArgs& a, HxShared& sh, Stager& st, uint32_t p, uint32_t r, const uint32_t* list,
                           uint32_t n, uint32_t wr, uint32_t nw, bool far) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    uint32_t* vals = sh.vals[wid];
    uint32_t* pref = sh.wbin[wid];   // 33 words: exclusive prefix of the degrees + total
    uint32_t* ss = sh.tnew[wid];
    // entries per warp step: enough for every warp to get a share, at most 8
    // (a long list is dealt out in small blocks, so that no warp draws a run
    // of the largest entries; 32 measured 1.4-2.5% slower on the benchmark
    // graphs)
    const uint32_t B = min(8u, max(1u, (n + nw - 1) / nw));
    for (uint32_t i0 = wr * B; i0 < n; i0 += nw * B) {
        const uint32_t i = i0 + lane;
        uint32_t v = kFull, s0 = 0, d = 0, e = 0, fl = 0, dfull = 0;
        bool listed = false, below = false;
        if (lane < B && i < n) {
            const uint32_t ent = __ldcg(list + i);
            v = ent & ~kListFlag;
            listed = (ent & kListFlag) != 0;
            if (v < a.V) {
                s0 = KC_LDG(a.off + v);
                dfull = KC_LDG(a.off + v + 1) - s0;
                e = __ldcg(a.est + v);
                if (listed) {
                    const uint32_t al = __ldcg(a.alen + v);
                    fl = __ldcg(a.alo + v);
                    if (al == kFull || al > kBatchVals || al > dfull || fl > e) below = true;   // (cannot happen)
                    else d = al;
                } else {
                    d = min(dfull, kHxWarpArcs);
                }
            } else {
                v = kFull;
            }
        }
        const unsigned listm = __ballot_sync(kFull, listed);
        uint32_t total;
        const uint32_t ex = warp_excl_scan(d, &total);
        __syncwarp();
        ss[lane] = s0;
        pref[lane] = ex;
        if (lane == 0) pref[32] = total;
        __syncwarp();
        uint32_t k0 = 0;
        while (k0 < 32) {   // warp-uniform
            // the batch: entries k0..k1-1, the most whose values fit kBatchVals
            // (at least one: an entry holds at most kBatchVals)
            const uint32_t base = pref[k0];
            const unsigned fit = __ballot_sync(kFull, lane >= k0 && pref[lane + 1] - base <= kBatchVals);
            const uint32_t k1 = k0 + max(1u, (uint32_t)__popc(fit));
            const uint32_t nv = pref[k1] - base;
            uint32_t lo = k0;
            for (uint32_t q0 = 0; q0 < nv; q0 += 128) {
                uint32_t u[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t qi = q0 + 32u * j + lane;
                    u[j] = kFull;
                    if (qi < nv) {
                        const uint32_t qa = qi + base;
                        uint32_t hi = k1;
                        while (hi - lo > 1) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (pref[mid] <= qa) lo = mid; else hi = mid;
                        }
                        const uint32_t at = ss[lo] + (qa - pref[lo]);
                        u[j] = (listm >> lo) & 1u ? __ldcg(a.act + at) : KC_LDG(a.nbr + at);
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t qi = q0 + 32u * j + lane;
                    if (qi < nv) vals[qi] = u[j] < a.V ? __ldcg(a.est + u[j]) : 0u;
                }
            }
            __syncwarp();
            const bool mine = lane >= k0 && lane < k1 && v != kFull;
            uint32_t h = kFull, c = 0;
            // entries of at most 32 values: a lane each, from shared memory
            if (mine && !below && d <= 32) {
                const uint32_t* xs = vals + (ex - base);
                auto ge = [&](uint32_t t) {
                    uint32_t k = 0;
                    for (uint32_t i2 = 0; i2 < d; ++i2) k += xs[i2] >= t ? 1u : 0u;
                    return k;
                };
                h = far ? bisect_hindex(ge, fl, e) : gallop_hindex(ge, fl, e);
                if (h != kFull) c = ge(h);
            }
            // larger entries: the warp, one after another
            unsigned big = __ballot_sync(kFull, mine && !below && d > 32);
            while (big) {
                const uint32_t k = __ffs(big) - 1;
                big &= big - 1;
                const uint32_t dk = pref[k + 1] - pref[k];
                const uint32_t ek = __shfl_sync(kFull, e, k), fk = __shfl_sync(kFull, fl, k);
                uint32_t ck = 0;
                const uint32_t hk = warp_hindex(vals + (pref[k] - base), dk, fk, ek, &ck, far);
                if (lane == k) { h = hk; c = ck; }
            }
            // results: the lane of each entry writes it
            bool drop = false, two = false;
            if (mine) {
                if (below || h == kFull) {
                    // h-index below the list's floor: search the adjacency, the
                    // 32 values under the floor first
                    if (dfull <= kHxCtaVals) {
                        push_cta(a, r, v);   // the adjacency, read whole by a CTA next pass
                    } else {
                        const uint32_t hi = below ? e : fl - 1;
                        open_window(a, p, r, v, e, hi >= 31u ? hi - 31u : 0u, hi, 0, dfull);
                    }
                } else {
                    a.cnt[v] = c;
                    if (h < e) {
                        a.old[v] = e;
                        a.est[v] = h;
                        drop = true;
                        two = listed && d > kHxChunk;
                    }
                }
            }
            const unsigned long long t0 = ((unsigned long long)v << 32) | (listed ? kListTask : 0u);
            stage_bt(a, sh, st, p, __ballot_sync(kFull, drop), t0);
            stage_bt(a, sh, st, p, __ballot_sync(kFull, two), t0 | 1u);
            __syncwarp();
            k0 = k1;
        }
    }
}

// CTA-wide sum of one value per thread (every thread gets it).
__device__ __forceinline__ uint32_t cta_sum(uint32_t x, HxShared& sh) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    x = __reduce_add_sync(kFull, x);
    __syncthreads();   // earlier readers of red[] are done
    if (lane == 0) sh.red[wid] = x;
    __syncthreads();
    return __reduce_add_sync(kFull, lane < kWarps ? sh.red[lane] : 0u);
}

// Phase A for a large vertex read whole by one CTA (at most kHxCtaVals
// entries): its active list (from the list's floor) or its adjacency (from 0,
// rebuilding the list), gathered into shared memory; the h-index is exact in
// one pass, with CTA reductions.  An h-index below the list's floor sends the
// CTA on to the adjacency, or, above kHxCtaVals arcs, to a window search in
// the next pass.
__device__ void cta_entry(const HxArgs& a, HxShared& sh, uint32_t p, uint32_t r, uint32_t ent, bool far) {
    const unsigned tid = threadIdx.x, lane = lane_id();
    const uint32_t v = ent & ~kListFlag;
    if (v >= a.V) return;
    const uint32_t s0 = KC_LDG(a.off + v);
    const uint32_t d = KC_LDG(a.off + v + 1) - s0;
    const uint32_t e = __ldcg(a.est + v);
    const uint32_t al = __ldcg(a.alen + v), fl0 = __ldcg(a.alo + v);
    bool list = (ent & kListFlag) != 0 && al != kFull && al != 0 && al <= kHxCtaVals && al <= d && fl0 <= e;
    uint32_t* vals = &sh.vals[0][0];
    constexpr int kPer = kHxCtaVals / kPeelThreads;
    for (int round = 0; round < 2; ++round) {   // the list, then (below its floor) the adjacency
        const uint32_t len = list ? al : d;
        const uint32_t fl = list ? fl0 : 0u;
        if (len > kHxCtaVals) {   // (adjacency only) a window search in the next pass
            if (tid == 0) {
                const uint32_t hi = round == 0 ? e : fl0 - 1;
                open_window(a, p, r, v, e, hi >= 31u ? hi - 31u : 0u, hi, 0, d);
            }
            break;
        }
        for (uint32_t i = tid; i < len; i += kPeelThreads) {
            const uint32_t u = list ? __ldcg(a.act + s0 + i) : KC_LDG(a.nbr + s0 + i);
            vals[i] = u < a.V ? __ldcg(a.est + u) : 0u;
        }
        __syncthreads();
        uint32_t x[kPer];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t idx = tid + kPeelThreads * j;
            x[j] = idx < len ? vals[idx] : 0u;
        }
        auto ge = [&](uint32_t h) {
            uint32_t c = 0;
#pragma unroll
            for (int j = 0; j < kPer; ++j) c += (tid + kPeelThreads * j < len && x[j] >= h) ? 1u : 0u;
            return cta_sum(c, sh);
        };
        const uint32_t h = far ? bisect_hindex(ge, fl, e) : gallop_hindex(ge, fl, e);   // CTA-uniform
        if (h == kFull) {   // below the list's floor
            list = false;
            __syncthreads();
            continue;
        }
        const uint32_t c = ge(h);
        uint32_t L = al;
        if (!list) {
            // rebuild the active list: the neighbours at or above h - kListMargin
            const uint32_t nf = h > kListMargin ? h - kListMargin : 0u;
            if (tid == 0) sh.cpos = 0;
            __syncthreads();
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const uint32_t idx = tid + kPeelThreads * j;
                const bool keep = idx < len && x[j] >= nf;
                const unsigned m = __ballot_sync(kFull, keep);
                if (!m) continue;
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(&sh.cpos, (uint32_t)__popc(m));
                base = __shfl_sync(kFull, base, 0);
                if (keep) a.act[s0 + base + __popc(m & lanemask_lt())] = KC_LDG(a.nbr + s0 + idx);
            }
            __syncthreads();
            L = sh.cpos;
            if (tid == 0) {
                a.alen[v] = L;
                a.alo[v] = nf;
            }
        }
        if (tid == 0) {
            a.cnt[v] = c;
            if (h < e) {
                a.old[v] = e;
                a.est[v] = h;
            }
        }
        if (h < e && tid < 32) {   // update tasks over the active list
            const uint32_t n = (L + kHxChunk - 1) / kHxChunk;
            uint32_t base = 0;
            if (lane == 0 && n) base = atomicAdd(&a.ctl->hx.bt_n[p], n);
            base = __shfl_sync(kFull, base, 0);
            for (uint32_t cc = lane; cc < n; cc += 32) {
                if (base + cc < a.cap_bt) a.bt[p][base + cc] = ((unsigned long long)v << 32) | kListTask | cc;
                else record_error(a.ctl, kErrOverflow, 0);
            }
        }
        break;
    }
    __syncthreads();   // shared values reused by the next entry
}

// The warp that finished the last chunk of slot `s` reads the pass's bins.
// Found (bins one wide): the h-index and its count; a drop queues update tasks
// over the active list.  Otherwise the next pass narrows the window to the bin
// that holds h, or, when h lies below the window, reads the range below it
// (the whole adjacency once h is below the active list's floor).
__device__ void resolve_slot(const HxArgs& a, HxShared& sh, Stager& st, uint32_t p, uint32_t r, uint32_t s) {
    const unsigned lane = lane_id();
    HxSlot* sl = a.slots[p] + s;
    uint32_t* bins = a.bins[p] + (size_t)s * kHxBinWords;
    const uint32_t v = __ldcg(&sl->v), e = __ldcg(&sl->e), lo = __ldcg(&sl->lo), hi = __ldcg(&sl->hi);
    const uint32_t shft = __ldcg(&sl->sh), mode = __ldcg(&sl->mode);
    const uint32_t nb = ((hi - lo) >> shft) + 1;
    __threadfence();
    const uint32_t cb = lane < nb ? __ldcg(bins + lane) : 0u;
    const uint32_t above = __ldcg(bins + 32);
    // clear for the next pass (or the next vertex of this slot)
    bins[lane] = 0;
    if (lane == 0) bins[32] = 0;
    // S(b) = count of estimates >= lo + b << shft
    uint32_t suf = cb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_down_sync(kFull, suf, o);
        if (lane + o < 32) suf += y;
    }
    const uint32_t S = suf + above;
    const uint32_t start = lo + (lane << shft);
    const unsigned ok = __ballot_sync(kFull, lane < nb && S >= start);
    uint32_t nlo, nhi, nmode = mode;
    if (ok) {
        const uint32_t bs = 31 - __clz(ok);
        const uint32_t Sb = __shfl_sync(kFull, S, bs);
        const uint32_t sb = lo + (bs << shft);
        if (shft == 0) {   // found: h = sb, counted Sb
            // a pass over the adjacency leaves the list of neighbours >= lo -
            // kListMargin (none from a window at or below kListMargin: the
            // update then reads the adjacency)
            const bool listed = mode == 1 || lo > kListMargin;
            const uint32_t L = mode == 1 ? __ldcg(&sl->len)
                                         : (listed ? __ldcg(a.alen + v) : KC_LDG(a.off + v + 1) - KC_LDG(a.off + v));
            if (lane == 0) {
                if (mode == 0 && listed) a.alo[v] = lo - kListMargin;
                a.cnt[v] = Sb;
                if (sb < e) {
                    a.old[v] = e;
                    a.est[v] = sb;
                }
            }
            if (sb < e) {
                // update tasks over the active list: a neighbour whose count
                // this drop crosses has an estimate above sb >= alo[v]
                const uint32_t n = (L + kHxChunk - 1) / kHxChunk;
                HxCtl* hx = &a.ctl->hx;
                uint32_t base = 0;
                if (lane == 0 && n) base = atomicAdd(&hx->bt_n[p], n);
                base = __shfl_sync(kFull, base, 0);
                for (uint32_t c = lane; c < n; c += 32) {
                    if (base + c < a.cap_bt) a.bt[p][base + c] = ((unsigned long long)v << 32) | (listed ? kListTask : 0u) | c;
                    else record_error(a.ctl, kErrOverflow, 0);
                }
            }
            return;
        }
        nlo = sb;
        nhi = min(sb + (1u << shft) - 1u, hi);
        // this pass over the adjacency rebuilt the list of the neighbours at or
        // above lo - kListMargin: it holds every neighbour that can still reach
        // the narrower window, so the next pass reads it when it is at most
        // half the adjacency
        if (mode == 0 && lo > kListMargin && 2u * __ldcg(a.alen + v) <= KC_LDG(a.off + v + 1) - KC_LDG(a.off + v))
            nmode = 1;
    } else {   // h < lo (lo > 0 here: at lo = 0 bin 0 always qualifies)
        // the list still holds every neighbour down to its floor; below that
        // the adjacency is read
        const uint32_t fl = mode == 1 ? __ldcg(a.alo + v) : 0u;
        nhi = lo - 1;
        if (mode == 1 && fl < lo) {
            nlo = fl;
        } else {
            // the adjacency: once the 32 values under a top window or under
            // the list's floor, then everything below
            nlo = ((mode == 1 || hi == e) && nhi >= 31u) ? nhi - 31u : 0u;
            nmode = 0;
        }
    }
    uint32_t len = __ldcg(&sl->len);
    if (nmode == 0 && mode == 1) len = KC_LDG(a.off + v + 1) - KC_LDG(a.off + v);
    if (nmode == 1 && mode == 0) len = __ldcg(a.alen + v);
    const uint32_t nch = (len + kHxChunk - 1) / kHxChunk;
    if (lane == 0) {
        sl->lo = nlo;
        sl->hi = nhi;
        sl->sh = bin_shift(nlo, nhi);
        sl->mode = nmode;
        sl->len = len;
        sl->nch = nch;
        sl->done = 0;
        if (nmode == 0) a.alen[v] = nlo > kListMargin ? 0u : kFull;   // the next pass rebuilds the list
        if (nmode == 1 && mode == 0) a.alo[v] = lo > kListMargin ? lo - kListMargin : 0u;
        atomicAdd(&a.ctl->hx.passes, 1u);
    }
    queue_chunks(a, r, s, nch, lane, 32);
}

// Phase A for one chunk task of a large vertex: bin its neighbours' estimates
// (of the adjacency or of the active list).  A pass over the adjacency also
// appends every neighbour at or above the window's floor to the active list.
__device__ void chunk_task(const HxArgs& a, HxShared& sh, Stager& st, uint32_t p, uint32_t r,
                           unsigned long long task, bool degrees) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    const uint32_t s = (uint32_t)(task >> 32), c = (uint32_t)task;
    if (s >= a.cap_l) return;
    HxSlot* sl = a.slots[p] + s;
    const uint32_t v = __ldcg(&sl->v), lo = __ldcg(&sl->lo), hi = __ldcg(&sl->hi), shft = __ldcg(&sl->sh);
    const uint32_t nch = __ldcg(&sl->nch), mode = __ldcg(&sl->mode), total = __ldcg(&sl->len);
    if (v >= a.V) return;
    const uint32_t s0 = KC_LDG(a.off + v);
    const uint32_t d = KC_LDG(a.off + v + 1) - s0;
    const uint32_t b0 = c * kHxChunk;
    const uint32_t len = (b0 < total && total <= d) ? min(kHxChunk, total - b0) : 0u;
    uint32_t bin[8], uu[8], xv[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t i = lane + 32u * k;
        uu[k] = kFull;
        if (i < len) uu[k] = mode ? __ldcg(a.act + s0 + b0 + i) : KC_LDG(a.nbr + s0 + b0 + i);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        bin[k] = kNoBin;
        xv[k] = 0;
        if (uu[k] < a.V) {
            const uint32_t u = uu[k];
            uint32_t x;
            if (!degrees) {
                x = __ldcg(a.est + u);
            } else if (a.after_peel) {   // iteration 1 after a level peel: remaining degree or core number
                const uint32_t wu = __ldcg(a.w + u);
                x = (wu & kClaim) ? __ldcg(a.est + u) : wu - kBias;
            } else {
                x = KC_LDG(a.off + u + 1) - KC_LDG(a.off + u);
            }
            xv[k] = x;
            bin[k] = x > hi ? 32u : (x >= lo ? (x - lo) >> shft : kNoBin);
        }
    }
    if (mode == 0 && lo > kListMargin) {   // rebuild the active list: the neighbours at or above lo - kListMargin
        // (a window from at most kListMargin keeps no list: it would hold every neighbour)
        const uint32_t lfl = lo - kListMargin;
        unsigned keep[8];
        uint32_t nk = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            keep[k] = __ballot_sync(kFull, uu[k] < a.V && xv[k] >= lfl);
            nk += __popc(keep[k]);
        }
        if (nk) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(a.alen + v, nk);
            base = __shfl_sync(kFull, base, 0);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if (keep[k] & (1u << lane)) {
                    const uint32_t pos = base + __popc(keep[k] & lanemask_lt());
                    if (pos < d) a.act[s0 + pos] = uu[k];
                    else record_error(a.ctl, kErrOverflow, 0);
                }
                base += __popc(keep[k]);
            }
        }
    }
    uint32_t* wb = sh.wbin[wid];
    wb[lane] = 0;
    if (lane == 0) wb[32] = 0;
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (!__any_sync(kFull, bin[k] != kNoBin)) continue;
        const unsigned m = __match_any_sync(kFull, bin[k]);
        if (bin[k] != kNoBin && lane == (unsigned)(__ffs(m) - 1)) wb[bin[k]] += __popc(m);
        __syncwarp();
    }
    uint32_t* gb = a.bins[p] + (size_t)s * kHxBinWords;
    const uint32_t mine = wb[lane];
    if (mine) atomicAdd(gb + lane, mine);
    if (lane == 0 && wb[32]) atomicAdd(gb + 32, wb[32]);
    __threadfence();
    __syncwarp();
    uint32_t prev = 0;
    if (lane == 0) prev = atomicAdd(&sl->done, 1u);
    prev = __shfl_sync(kFull, prev, 0);
    if (prev + 1 == nch) resolve_slot(a, sh, st, p, r, s);
}

// Phase B: the flattened arcs of 32 update tasks per warp step.  A neighbour w
// whose estimate x satisfies new < x <= old loses one count; the decrement
// that takes its count below x queues it.
__device__ void update_tasks(const HxArgs& a, HxShared& sh, Stager& st, uint32_t p, uint32_t r, uint32_t nbt,
                             uint32_t wr, uint32_t nw, bool coarse) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    const uint32_t q = p ^ 1u;
    // per-warp task table in the (free) bin area: prefix, first arc, old, new
    uint32_t* pref = sh.wbin[wid];   // 33 words: exclusive prefix of 32 tasks + total
    uint32_t* tstart = sh.tstart[wid];
    uint32_t* told = sh.told[wid];
    uint32_t* tnew = sh.tnew[wid];
    // Warp wr takes tasks wr, wr + nw, wr + 2nw, ..., T per step (T: enough
    // for every warp to get a share, at most 32): a vertex's chunk tasks sit
    // side by side in the list, and this spreads them over the warps.
    const uint32_t T = min(32u, max(1u, (nbt + nw - 1) / nw));
    for (uint64_t m0 = 0; m0 * nw + wr < nbt; m0 += T) {
        const uint64_t i64 = (m0 + lane) * nw + wr;
        const uint32_t i = (uint32_t)i64;
        uint32_t len = 0, s1 = 0, ol = 0, nw_ = 0;
        bool listed = false;
        if (lane < T && i64 < nbt) {
            const unsigned long long tk = __ldcg(a.bt[p] + i);
            const uint32_t u = (uint32_t)(tk >> 32), c = (uint32_t)tk & ~kListTask;
            listed = ((uint32_t)tk & kListTask) != 0;
            if (u < a.V) {
                const uint32_t s0 = KC_LDG(a.off + u);
                const uint32_t d = KC_LDG(a.off + u + 1) - s0;
                const uint32_t n = listed ? min(__ldcg(a.alen + u), d) : d;
                const uint32_t b0 = c * kHxChunk;
                len = b0 < n ? min(kHxChunk, n - b0) : 0u;
                s1 = s0 + b0;
                ol = __ldcg(a.old + u);
                nw_ = __ldcg(a.est + u);
            }
        }
        const unsigned listm = __ballot_sync(kFull, listed);   // tasks that read an active list
        uint32_t total;
        const uint32_t ex = warp_excl_scan(len, &total);
        pref[lane] = ex;
        if (lane == 0) pref[32] = total;
        tstart[lane] = s1;
        told[lane] = ol;
        tnew[lane] = nw_;
        __syncwarp();
        uint32_t lo = 0;
        for (uint32_t q0 = 0; q0 < total; q0 += 256) {
            // neighbour ids, then their estimates, then the decrements: each
            // step's loads are all in flight before the next step uses them
            uint32_t wv[8], kk[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const uint32_t qi = q0 + 32u * j + lane;
                wv[j] = kFull;
                kk[j] = 0;
                if (qi < total) {
                    uint32_t hi = 32;
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (pref[mid] <= qi) lo = mid; else hi = mid;
                    }
                    kk[j] = lo;
                    const uint32_t at = tstart[lo] + (qi - pref[lo]);
                    wv[j] = (listm >> lo) & 1u ? __ldcg(a.act + at) : KC_LDG(a.nbr + at);
                }
            }
            uint32_t xv[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) xv[j] = wv[j] < a.V ? __ldcg(a.est + wv[j]) : 0u;
            uint32_t y[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                y[j] = kFull;
                if (wv[j] < a.V && tnew[kk[j]] < xv[j] && xv[j] <= told[kk[j]]) y[j] = atomicSub(a.cnt + wv[j], 1u);
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                bool queue = y[j] != kFull && y[j] == xv[j];
                // queue: small and mid-size vertices to the warp list, large ones to a slot
                uint32_t ent = wv[j];
                if (queue) {
                    const uint32_t dq = KC_LDG(a.off + wv[j] + 1) - KC_LDG(a.off + wv[j]);
                    if (dq > kHxWarpArcs) {
                        // a short active list: the warp path; up to kHxCtaVals entries
                        // (list or adjacency): the CTA path; else a window slot
                        // (a list whose floor is within kListGuard of the estimate is
                        // rebuilt now, before the h-index can fall below it)
                        const uint32_t al = __ldcg(a.alen + wv[j]);
                        const bool usable = al != kFull && al != 0 && __ldcg(a.alo + wv[j]) + kListGuard <= xv[j];
                        if (usable && al <= kBatchVals) {
                            ent |= kListFlag;
                        } else {
                            if (usable && al <= kHxCtaVals) push_cta(a, r, wv[j] | kListFlag);
                            else if (!usable && dq <= kHxCtaVals) push_cta(a, r, wv[j]);
                            else open_slot(a, q, r, wv[j], xv[j], dq, coarse);
                            queue = false;
                        }
                    }
                }
                stage_rm(a, sh, st, q, __ballot_sync(kFull, queue), ent);
            }
        }
        __syncwarp();
    }
    flush_rm(a, sh, st, q);
}

// The CTAs of an iteration.  cta/ncta: this CTA's rank and the CTAs taking
// part; gw: warp rank for linear sweeps; wr/nw: warp rank for work lists
// (consecutive ranks on different SMs) and the warps taking part.
struct Exec {
    uint32_t cta, ncta, gw, wr, nw;
    bool lead;
};

// One iteration (phase A passes, then phase B) from sub-phase r; t and r
// advance.  Returns 0: another iteration has work, 1: converged, 2: the
// iteration budget is spent, -1: a barrier failed (error recorded).
__device__ int hx_iteration(const HxArgs& a, HxShared& sh, Stager& st, uint32_t& t, uint32_t& r, const Exec& ex) {
    HxCtl* hx = &a.ctl->hx;
    const unsigned lane = lane_id();
    const uint32_t p = t & 1u;
    // ---- phase A: window passes; the first also takes the warp frontier.
    // Every pass narrows each open window or ends it, so the passes are few;
    // the cap only turns a broken invariant into an error instead of a loop.
    bool first = true;
    for (uint32_t npass = 0;; ++npass) {
        if (npass > 4096) {   // (every CTA counts the same passes)
            if (ex.lead) record_error(a.ctl, kErrOverflow, t);
            return -1;
        }
        const uint32_t ncl = min(ld_relaxed(&hx->cl_n[r % 3]), a.cap_cl);
        const uint32_t nrc = min(ld_relaxed(&hx->rc_n[r % 3]), a.cap_l);
        const uint32_t nrm = first ? min(ld_relaxed(&hx->rm_n[p]), a.V) : 0u;
        if (ncl == 0 && nrm == 0 && nrc == 0) break;   // every thread reads the same counts
        if (ex.lead) {
            hx->cl_n[(r + 2) % 3] = 0;
            hx->rc_n[(r + 2) % 3] = 0;
        }
        if (nrc <= kCtaEntries * ex.ncta) {   // a CTA each, one after another
            for (uint32_t i = ex.cta; i < nrc; i += ex.ncta) cta_entry(a, sh, p, r, __ldcg(a.rc[r % 3] + i), t <= 2);
        } else {
            // too many for the CTAs: window searches spread over every warp,
            // from the next pass
            for (uint32_t i = ex.gw * 32 + lane; i < nrc; i += ex.nw * 32) {
                const uint32_t ent = __ldcg(a.rc[r % 3] + i), v = ent & ~kListFlag;
                if (v < a.V) {
                    const uint32_t d = KC_LDG(a.off + v + 1) - KC_LDG(a.off + v);
                    open_slot(a, p, r, v, __ldcg(a.est + v), d, t == 2);
                }
            }
        }
        if (nrm) warp_batch(a, sh, st, p, r, a.rm[p], nrm, ex.wr, ex.nw, t <= 2);
        for (uint32_t i = ex.wr; i < ncl; i += ex.nw) chunk_task(a, sh, st, p, r, __ldcg(a.cl[r % 3] + i), t == 1);
        flush_bt(a, sh, st, p);
        if (!hx_barrier(a, sh)) return -1;
        ++r;
        first = false;
    }
    // ---- phase B (sub-phase r)
    if (ex.lead) {
        hx->cl_n[(r + 2) % 3] = 0;
        hx->rc_n[(r + 2) % 3] = 0;
        hx->bt_n[p ^ 1u] = 0;
        hx->rm_n[p] = 0;
        hx->rl_n[p] = 0;
    }
    const uint32_t nbt = min(ld_relaxed(&hx->bt_n[p]), a.cap_bt);
    // (the large vertices queued for iteration 2 fall far again: their windows
    // start over the whole range, as in iteration 1)
    update_tasks(a, sh, st, p, r, nbt, ex.wr, ex.nw, t == 1);
    if (!hx_barrier(a, sh)) return -1;
    ++r;
    const uint32_t nm = ld_relaxed(&hx->rm_n[p ^ 1u]), nl = ld_relaxed(&hx->rl_n[p ^ 1u]);
    const uint32_t nc = ld_relaxed(&hx->rc_n[r % 3]);
    if (nm == 0 && nl == 0 && nc == 0) return 1;
    ++t;
    if (t > a.max_iters) {   // the level peel takes over
        if (ex.lead) hx->iters = t;
        return 2;
    }
    return 0;
}

// ------------------------------------------------------------ cluster hand-off
// Late iterations touch few vertices but each still costs two or three grid
// barriers and their chains of L2 round trips; a 16-CTA cluster runs them
// about twice as fast (kc_hxtail.cu).  The set handed over is S = {v : est[v]
// >= T} with T at most the smallest estimate in the next frontier, so that
// every queued vertex is in S.  The hand-off is made only when every vertex
// of S has at least T neighbours in S: S then lies in the T-core, so every
// core number in S is at least T and no estimate in S falls below T; the
// vertices outside S, none of them queued and none of them ever crossed by a
// drop in S (their estimates are below T), are final.  Inside S the counts
// stay valid (every neighbour they count has an estimate >= est >= T).  The
// cluster continues the same iteration on the induced CSR of S from these
// estimates and counts.  T is the smallest of T0/2, 5T0/8, ... T0 (T0 the
// frontier's smallest estimate) that leaves at most kHoV vertices in S.

constexpr uint32_t kHoMark = 0xFFFFFFFEu;   // lmap: a queued vertex (before the local ids are given)
constexpr uint32_t kHoTask = 256;           // entries per chunk task of the hand-off
constexpr int kHoCand = 5;                  // candidate floors

__device__ __forceinline__ uint32_t cand_floor(uint32_t T0, int k) {
    return max(1u, (uint32_t)(((unsigned long long)T0 * (4u + k)) / 8u));
}

// Visits the next frontier (iteration t, sub-phase r): f(v) per queued vertex.
template <class F>
__device__ __forceinline__ void for_frontier(const HxArgs& a, uint32_t t, uint32_t r, uint32_t gw, uint32_t nw, F f) {
    HxCtl* hx = &a.ctl->hx;
    const unsigned lane = lane_id();
    const uint32_t q = t & 1u;
    const uint32_t nm = min(ld_relaxed(&hx->rm_n[q]), a.V), nl = min(ld_relaxed(&hx->rl_n[q]), a.cap_l);
    const uint32_t nc = min(ld_relaxed(&hx->rc_n[r % 3]), a.cap_l);
    for (uint32_t base = gw * 32; base < nm + nl + nc; base += nw * 32) {   // warp-uniform
        const uint32_t i = base + lane;
        uint32_t v = kFull;
        if (i < nm) v = __ldcg(a.rm[q] + i) & ~kListFlag;
        else if (i < nm + nl) v = __ldcg(&a.slots[q][i - nm].v);
        else if (i < nm + nl + nc) v = __ldcg(a.rc[r % 3] + (i - nm - nl)) & ~kListFlag;
        f(v < a.V ? v : kFull);
    }
}

// A chunk task of the hand-off: the low word is the position of its first
// entry in the member's source (the adjacency, or its active list when that
// is complete for the floor: the vertex is not queued, so no window pass is
// rebuilding it, and its list floor is at or below T); the high word holds
// the member's local id (bits 0-14), the source (bit 15: the list) and the
// entry count - 1 (bits 16-23).
constexpr uint32_t kHoListed = 1u << 15;

// A task's entries, 8 a lane, all loads in flight; u = 0xFFFFFFFF past the end.
__device__ __forceinline__ void ho_load(const HxArgs& a, unsigned long long tk, uint32_t& lid,
                                        uint32_t (&u)[kHoTask / 32]) {
    const unsigned lane = lane_id();
    const uint32_t hi = (uint32_t)(tk >> 32), pos = (uint32_t)tk;
    lid = hi & 0x7FFFu;
    const bool listed = (hi & kHoListed) != 0;
    const uint32_t m = ((hi >> 16) & 0xFFu) + 1u;
#pragma unroll
    for (uint32_t j = 0; j < kHoTask / 32; ++j) {
        const uint32_t x = 32u * j + lane;
        u[j] = x < m ? (listed ? __ldcg(a.act + pos + x) : KC_LDG(a.nbr + pos + x)) : kFull;
    }
}

// Builds the induced CSR of S (local ids; each adjacency in a span as long as
// its source, padded to quads) in the tail buffers and checks that every
// member has at least T neighbours in S.  Returns 1 when S is handed over, 0
// when no floor leaves S small enough, 2 when S failed the certificate (or
// did not fit), -1 on a failed barrier; the grid goes on after 0 and 2.
// Every CTA calls it with the same attempt number k.
__device__ int try_handoff(const HxArgs& a, HxShared& sh, uint32_t t, uint32_t r, uint32_t k, const Exec& ex) {
    HxCtl* hx = &a.ctl->hx;
    const unsigned lane = lane_id();
    const uint32_t P = k & 1u;
    unsigned long long* tasks = a.bt[t & 1u];   // both update-task lists are free between iterations
    constexpr uint32_t kU = kHoTask / 32;
    // 0: the frontier's smallest estimate; queued vertices marked in lmap
    {
        uint32_t mn = kFull;
        for_frontier(a, t, r, ex.gw, ex.nw, [&](uint32_t v) {
            if (v != kFull) {
                mn = min(mn, __ldcg(a.est + v));
                a.lmap[v] = kHoMark;
            }
        });
        mn = __reduce_min_sync(kFull, mn);
        if (lane == 0 && mn != kFull) atomicMin(&hx->ho_min[P], mn);
    }
    if (!hx_barrier(a, sh)) return -1;
    if (ex.lead) {   // the next attempt's counters (no CTA touches them until then)
        hx->ho_min[P ^ 1u] = kFull;
        for (int c = 0; c < kHoCand; ++c) hx->ho_cnt[P ^ 1u][c] = 0;
        hx->ho_m[P ^ 1u] = 0;
        hx->ho_fail[P ^ 1u] = 0;
        hx->ho_tasks[P ^ 1u] = 0;
        hx->ho_arcs[P ^ 1u] = 0;
    }
    const uint32_t T0 = ld_relaxed(&hx->ho_min[P]);
    if (T0 == kFull || T0 < 2) return 0;
    // 1: |S| for each candidate floor
    {
        uint32_t c[kHoCand] = {};
        uint32_t fl[kHoCand];
#pragma unroll
        for (int j = 0; j < kHoCand; ++j) fl[j] = cand_floor(T0, j);
        for (uint32_t base = ex.gw * 32 * kU; base < a.V; base += ex.nw * 32 * kU) {
            uint32_t e[kU];
#pragma unroll
            for (uint32_t u = 0; u < kU; ++u) {
                const uint32_t v = base + 32u * u + lane;
                e[u] = v < a.V ? __ldcg(a.est + v) : 0u;
            }
#pragma unroll
            for (uint32_t u = 0; u < kU; ++u)
#pragma unroll
                for (int j = 0; j < kHoCand; ++j) c[j] += e[u] >= fl[j] ? 1u : 0u;
        }
#pragma unroll
        for (int j = 0; j < kHoCand; ++j) {
            const uint32_t x = __reduce_add_sync(kFull, c[j]);
            if (lane == 0 && x) atomicAdd(&hx->ho_cnt[P][j], x);
        }
    }
    if (!hx_barrier(a, sh)) return -1;
    int pick = -1;
    const uint32_t nmax = min(a.ho_max, kHoV);
    for (int j = 0; j < kHoCand && pick < 0; ++j) {
        const uint32_t x = ld_relaxed(&hx->ho_cnt[P][j]);
        if (x > 0 && x <= nmax) pick = j;
    }
    if (pick < 0) return 0;
    const uint32_t T = cand_floor(T0, pick), n = ld_relaxed(&hx->ho_cnt[P][pick]);
    // 2: members: local ids, estimates, counts (a queued vertex's as zero: it
    // may have been taken below zero by decrements of neighbours it had not
    // counted, and zero queues it in the cluster too), spans, chunk tasks
    for (uint32_t base = ex.gw * 32 * kU; base < a.V; base += ex.nw * 32 * kU) {   // warp-uniform
        uint32_t e[kU];
#pragma unroll
        for (uint32_t u = 0; u < kU; ++u) {
            const uint32_t v = base + 32u * u + lane;
            e[u] = v < a.V ? __ldcg(a.est + v) : 0u;
        }
#pragma unroll
        for (uint32_t u = 0; u < kU; ++u) {
            const uint32_t v = base + 32u * u + lane;
            const bool in = v < a.V && e[u] >= T;
            const unsigned m = __ballot_sync(kFull, in);
            if (!m) continue;
            uint32_t s0 = 0, len = 0, tag = 0;
            bool queued = false;
            if (in) {
                queued = __ldcg(a.lmap + v) == kHoMark;
                s0 = KC_LDG(a.off + v);
                const uint32_t d = KC_LDG(a.off + v + 1) - s0;
                len = d;
                if (!queued) {
                    const uint32_t al = __ldcg(a.alen + v);
                    if (al != kFull && __ldcg(a.alo + v) <= T) {
                        len = min(al, d);
                        tag = kHoListed;
                    }
                }
            }
            // (a span longer than the whole buffer fails below anyway; the clamp
            // keeps a warp's sum of spans within 32 bits)
            const uint32_t nch = (len + kHoTask - 1) / kHoTask;
            const uint32_t span = min((len + 3u) & ~3u, a.tail_cap_arcs + 4u);
            uint32_t ntot, stot;
            const uint32_t cex = warp_excl_scan(nch, &ntot);
            const uint32_t sex = warp_excl_scan(span, &stot);
            uint32_t b = 0, tb = 0;
            unsigned long long ab64 = 0;
            if (lane == 0) {
                b = atomicAdd(&hx->ho_m[P], (uint32_t)__popc(m));
                if (ntot) tb = atomicAdd(&hx->ho_tasks[P], ntot);
                if (stot) ab64 = atomicAdd(&hx->ho_arcs[P], (unsigned long long)stot);
            }
            b = __shfl_sync(kFull, b, 0);
            tb = __shfl_sync(kFull, tb, 0) + cex;
            ab64 = __shfl_sync(kFull, ab64, 0) + sex;
            if (in) {
                const uint32_t lid = b + __popc(m & lanemask_lt());
                if (lid < n && ab64 + span <= a.tail_cap_arcs && tb + nch <= a.cap_bt) {
                    const uint32_t ab = (uint32_t)ab64;
                    a.lmap[v] = lid;
                    a.tail_ids[lid] = v;
                    a.tail_est[lid] = e[u];
                    a.tail_cnt[lid] = queued ? 0u : __ldcg(a.cnt + v);
                    a.tail_off[lid] = ab;
                    a.tail_cur[lid] = ab;
                    for (uint32_t c = 0; c < nch; ++c) {
                        const uint32_t cnt = min(kHoTask, len - c * kHoTask);
                        tasks[tb + c] = ((unsigned long long)(lid | tag | ((cnt - 1u) << 16)) << 32) |
                                        (s0 + c * kHoTask);
                    }
                } else {
                    atomicOr(&hx->ho_fail[P], 1u);
                }
            }
        }
    }
    if (!hx_barrier(a, sh)) return -1;
    if (ld_relaxed(&hx->ho_fail[P])) return 2;
    const uint32_t ntask = min(ld_relaxed(&hx->ho_tasks[P]), a.cap_bt);
    // 3: each member's neighbours in S as local ids, appended to its span
    for (uint32_t i = ex.wr; i < ntask; i += ex.nw) {
        uint32_t lid, u[kU];
        ho_load(a, __ldcg(tasks + i), lid, u);
        uint32_t x[kU];
#pragma unroll
        for (uint32_t j = 0; j < kU; ++j) x[j] = u[j] < a.V ? __ldcg(a.est + u[j]) : 0u;
#pragma unroll
        for (uint32_t j = 0; j < kU; ++j) x[j] = (u[j] < a.V && x[j] >= T) ? __ldcg(a.lmap + u[j]) : kFull;
        uint32_t c = 0;
#pragma unroll
        for (uint32_t j = 0; j < kU; ++j) c += x[j] < n ? 1u : 0u;
        uint32_t tot;
        const uint32_t cx = warp_excl_scan(c, &tot);
        if (tot == 0 || lid >= n) continue;
        uint32_t pb = 0;
        if (lane == 0) pb = atomicAdd(a.tail_cur + lid, tot);
        uint32_t at = __shfl_sync(kFull, pb, 0) + cx;
#pragma unroll
        for (uint32_t j = 0; j < kU; ++j) {
            if (x[j] < n) {
                if (at < a.tail_cap_arcs) a.tail_nbr[at] = x[j];
                else atomicOr(&hx->ho_fail[P], 1u);
                ++at;
            }
        }
    }
    if (!hx_barrier(a, sh)) return -1;
    // 4: the certificate; the pads after each adjacency
    for (uint32_t i = ex.gw * 32 + lane; i < n; i += ex.nw * 32) {
        const uint32_t o = __ldcg(a.tail_off + i), end = __ldcg(a.tail_cur + i);
        if (end - o < T) atomicOr(&hx->ho_fail[P], 1u);
        for (uint32_t q = end; q < ((end + 3u) & ~3u) && q < a.tail_cap_arcs; ++q) a.tail_nbr[q] = kFull;
    }
    if (ex.lead) a.ctl->tail_arcs = (uint32_t)min(__ldcg(&hx->ho_arcs[P]), (unsigned long long)a.tail_cap_arcs);
    if (!hx_barrier(a, sh)) return -1;
    if (ld_relaxed(&hx->ho_fail[P])) return 2;
    if (ex.lead) {
        hx->ho_floor = T;
        hx->ho_n = n;
        hx->iters = t - 1;
        hx->handoff = 1;
    }
    return 1;
}

__global__ void __launch_bounds__(kPeelThreads, 1) peel_hindex_kernel(const __grid_constant__ HxArgs a) {
    __shared__ HxShared sh;
    PeelCtl* ctl = a.ctl;
    HxCtl* hx = &ctl->hx;
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    const uint32_t gw = blockIdx.x * kWarps + wid, nw = gridDim.x * kWarps;
    // rank for work lists: consecutive ranks sit on different SMs, so a short
    // list is spread over the whole GPU instead of the first CTAs
    const uint32_t wr = wid * gridDim.x + blockIdx.x;
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    if (a.max_level == kFull && ld_err(&ctl->err)) return;   // the device validation refused the CSR
    // after a level peel: nothing to do when it finished, or failed
    if (a.after_peel && (ld_relaxed(&ctl->hx.peel_done) || !ld_relaxed(&ctl->hx.stopped) || ld_err(&ctl->err)))
        return;
    if (threadIdx.x == 0) sh.bar_k = 0;
    if (lead) {   // the first hand-off attempt's counters (seen by every CTA after the first barrier)
        hx->ho_min[0] = kFull;
        for (int c = 0; c < kHoCand; ++c) hx->ho_cnt[0][c] = 0;
        hx->ho_m[0] = 0;
        hx->ho_fail[0] = 0;
        hx->ho_tasks[0] = 0;
        hx->ho_arcs[0] = 0;
    }
    Stager st;

    // Sub-phase 0: est = degree (after a level peel: a survivor's remaining
    // degree; a peeled vertex keeps its core number, below every survivor's),
    // no active lists.
    for (uint32_t v = gw * 32 + lane; v < a.V; v += nw * 32) {
        if (a.after_peel) {
            const uint32_t x = __ldcg(a.w + v);
            if (!(x & kClaim)) a.est[v] = x - kBias;
        } else {
            a.est[v] = KC_LDG(a.off + v + 1) - KC_LDG(a.off + v);
        }
        a.alen[v] = kFull;
    }
    if (!hx_barrier(a, sh)) return;

    // Iteration 1, first sweep (sub-phase 1): a lane per vertex of at most
    // kHxLaneArcs arcs, two such vertices in flight per lane (blocks of 64
    // consecutive vertices per warp); larger vertices are queued for phase A
    // (parity 1).
    uint32_t r = 1;
    {
        for (uint32_t base = gw * 64; base < a.V; base += nw * 64) {
            uint32_t vv[2], s0[2], d[2], e0[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                vv[h] = base + 32u * h + lane;
                s0[h] = 0;
                d[h] = 0;
                e0[h] = 0;
                if (vv[h] < a.V) {
                    s0[h] = KC_LDG(a.off + vv[h]);
                    d[h] = KC_LDG(a.off + vv[h] + 1) - s0[h];
                    e0[h] = d[h];
                    if (a.after_peel) {   // a peeled vertex takes no part; a survivor starts at its remaining degree
                        const uint32_t x = __ldcg(a.w + vv[h]);
                        if (x & kClaim) vv[h] = kFull;
                        else e0[h] = x - kBias;
                    }
                }
            }
            uint32_t x[2][kHxLaneArcs];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t dl = (vv[h] < a.V && d[h] <= kHxLaneArcs) ? d[h] : 0u;
#pragma unroll
                for (uint32_t i = 0; i < kHxLaneArcs; ++i) x[h][i] = i < dl ? KC_LDG(a.nbr + s0[h] + i) : kFull;
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
#pragma unroll
                for (uint32_t i = 0; i < kHxLaneArcs; ++i) x[h][i] = x[h][i] < a.V ? __ldcg(a.est + x[h][i]) : 0u;
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t v = vv[h], dv = d[h], ev = e0[h];
                const bool small = v < a.V && dv <= kHxLaneArcs;
                bool drop = false;
                if (small) {
                    uint32_t lo = 0, hi = ev;
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi + 1) >> 1;
                        uint32_t c = 0;
#pragma unroll
                        for (uint32_t i = 0; i < kHxLaneArcs; ++i) c += (i < dv && x[h][i] >= mid) ? 1u : 0u;
                        if (c >= mid) lo = mid; else hi = mid - 1;
                    }
                    uint32_t c = 0;
#pragma unroll
                    for (uint32_t i = 0; i < kHxLaneArcs; ++i) c += (i < dv && x[h][i] >= lo) ? 1u : 0u;
                    a.cnt[v] = c;
                    if (lo < ev) {
                        a.old[v] = ev;
                        a.est[v] = lo;
                        drop = true;
                    }
                }
                stage_bt(a, sh, st, 1, __ballot_sync(kFull, drop), (unsigned long long)v << 32);
                const bool mid = v < a.V && dv > kHxLaneArcs && dv <= kHxWarpArcs;
                stage_rm(a, sh, st, 1, __ballot_sync(kFull, mid), v);
                if (v < a.V && dv > kHxWarpArcs) open_slot(a, 1, 0, v, ev, dv, true);
            }
        }
        flush_bt(a, sh, st, 1);
        flush_rm(a, sh, st, 1);
    }
    if (!hx_barrier(a, sh)) return;
    // (the first sweep queued chunk tasks into list (0 + 1) % 3 = 1, consumed at r = 1)

    uint32_t t = 1;
    const Exec grid{blockIdx.x, gridDim.x, gw, wr, nw, lead};
    // hand-off attempts: every other iteration while no floor leaves S small
    // enough; after a failed certificate, twice as long a wait each time
    uint32_t last_try = 0, attempts = 0, gap = 2;
    for (;;) {
        const int state = hx_iteration(a, sh, st, t, r, grid);
        if (state == 0 && a.handoff && t >= 3 && t >= last_try + gap) {
            // (every CTA reads the same counts after the iteration's last barrier)
            const uint32_t nf = min(ld_relaxed(&hx->rm_n[t & 1u]), a.V) + min(ld_relaxed(&hx->rl_n[t & 1u]), a.cap_l) +
                                min(ld_relaxed(&hx->rc_n[r % 3]), a.cap_l);
            if (nf <= a.ho_front) {
                last_try = t;
                const int ho = try_handoff(a, sh, t, r, attempts++, grid);
                if (ho == 1 || ho < 0) return;   // handed over, or an error
                if (ho == 2) gap *= 2;
            }
        }
        if (state == 1) break;
        if (state != 0) {   // an error, or the budget: the level peel takes over
            if (state == 2 && lead && a.after_peel) {
                // it starts over: the level counters the stopped level peel
                // left behind go back to their initial values
                for (int i = 0; i < 4; ++i) {
                    LevelSlot* sl = &ctl->slot[i];
                    sl->units_tail = 0; sl->head = 0; sl->peeled = 0; sl->arrived = 0;
                    sl->alive_next = 0; sl->min_next = kFull; sl->arcs_next = 0;
                }
                ctl->iters_done = 0;
                __threadfence();
            }
            return;
        }
    }

    // Converged: est holds the core numbers.
    uint32_t mx = 0;
    for (uint32_t v = gw * 32 + lane; v < a.V; v += nw * 32) mx = max(mx, __ldcg(a.est + v));
    mx = __reduce_max_sync(kFull, mx);
    if (lane == 0 && mx) atomicMax(&ctl->kmax, mx);
    if (lead) {
        hx->iters = t;
        ctl->iterations = (a.after_peel ? ctl->iterations : 0u) + t;
        hx->solved = 1;
    }
}

}  // namespace

const void* peel_hindex_fn() { return reinterpret_cast<const void*>(&peel_hindex_kernel); }

}  // namespace kc
