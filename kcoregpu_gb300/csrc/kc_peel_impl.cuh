// Device code of the persistent single-graph peel for sm_103a: every level of
// the level-synchronous peel (src/ours.cc:117-160) in one cooperative launch,
// with no host round trip and no grid barrier inside a level.  See
// kc_device.cuh for the claim protocol.  Included by kc_peel.cu (the normal and
// the bounds-checked kernel) and by kc_serve.cu (gangs of the serve kernel,
// with KC_PEEL_NO_KERNEL and its own KC_VNS).
#pragma once
#include "kc_device.cuh"
#include "kc_peel.cuh"

#ifndef KC_VNS
#ifdef KC_CHECKED
#define KC_VNS checked_variant
#else
#define KC_VNS fast_variant
#endif
#endif

namespace kc {
namespace KC_VNS {   // the normal and the bounds-checked build link into one library

// Bounds check at an access site of warp `w` (no-op unless built with KC_CHECKED).
#define IN(idx, size, site) KC_IN(w.a.ctl, (idx), (size), (site), w.level)

struct WarpBatch {
    uint32_t start[kItemCap];     // first arc of each item
    uint32_t pref[kItemCap + 1];  // lengths, then exclusive prefix
    uint32_t nstart[kItemCap];    // cascade list (next batch)
    uint32_t nlen[kItemCap];
};

struct CtaShared {
    WarpBatch wb[kPeelWarps];
    unsigned int arrive[4];
    unsigned int peeled[4];
    unsigned int minv[4];
    unsigned long long arcs[4];
    unsigned int poll_lock;
    int bar_ok;
    unsigned int hint_level;
    unsigned int hint_avail;
    unsigned int hint_done;
    int hint_err;
};

// Scan modes of a level.  Once few vertices remain, the scan reads a list of
// the still-alive vertices instead of the whole state array; the list is
// rebuilt (compacted) whenever it is more than half dead.
enum ScanMode : uint32_t { kDense = 0, kDenseCompact = 1, kList = 2, kListCompact = 3 };

struct Warp {
    const PeelArgs& a;
    WarpBatch& b;
    CtaShared& sh;
    LevelSlot* slot;
    unsigned long long task_base;
    uint32_t level;
    uint32_t kk;       // level + kBias
    uint32_t nitems;   // items staged in b.start / b.pref (lengths)
    uint32_t nnext;    // cascade entries in b.nstart / b.nlen
    uint32_t peeled;   // claims not yet published
    uint32_t nwt;      // warps of all participants
    uint32_t nparts;   // participating CTAs (the whole grid, or a gang of the serve kernel)
    uint32_t mode;     // ScanMode of this level
    uint32_t list_len; // entries in the current alive list
    uint32_t list_cur; // which alive buffer is current
    uint32_t it;       // level iteration (levels may be skipped, iterations are consecutive)
    uint32_t minv;     // smallest survivor state this lane's scan saw
    uint32_t arcs;     // sum of the survivor degrees this lane's scan saw (tail hand-off only)
    uint32_t narcs;    // arcs of the entries in the cascade list
};

// Optional per-level trace (kc_graph_trace): kTraceFields words per level.
__device__ __forceinline__ void trace(const PeelArgs& a, uint32_t level, int field, unsigned long long v) {
    if (a.trace && level < a.trace_cap) a.trace[(size_t)level * kTraceFields + field] = v;
}

// Pushes the arc range [start, start+len) of every lane with `pred` to the
// level's task queue, split into chunks of a.chunk_arcs arcs.
__device__ __noinline__ void push_tasks(Warp& w, bool pred, uint32_t start, uint32_t len) {
    const unsigned lane = lane_id();
    const uint32_t ch = w.a.chunk_arcs;
    uint32_t nch = pred ? (len + ch - 1) / ch : 0;
    uint32_t tot;
    uint32_t ex = warp_excl_scan(nch, &tot);
    if (tot == 0) return;
    uint32_t base = 0;
    if (lane == 0) base = (uint32_t)atomicAdd(&w.slot->units_tail, (unsigned long long)tot);
    base = __shfl_sync(kFull, base, 0);
    const unsigned long long first = w.task_base + base;
    if (first + tot > w.a.task_cap) {
        if (lane == 0) record_error(w.a.ctl, kErrOverflow, w.level);
        return;
    }
    unsigned m = __ballot_sync(kFull, nch != 0);
    while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const uint32_t s0 = __shfl_sync(kFull, start, src);
        const uint32_t l0 = __shfl_sync(kFull, len, src);
        const uint32_t e0 = __shfl_sync(kFull, ex, src);
        const uint32_t c0 = (l0 + ch - 1) / ch;
        for (uint32_t c = lane; c < c0; c += 32) {
            const uint32_t cs = s0 + c * ch;
            const uint32_t cl = min(ch, l0 - c * ch);
            if (IN(first + e0 + c, w.a.task_cap, 1))
                st_relaxed64(&w.a.tasks[first + e0 + c], make_task(cs, cl, w.level, w.a.epoch));
        }
    }
}

// Handles the vertices claimed by this warp in one walk step (their arc
// range [start, start+len) was loaded with the claiming atomic): records the
// core number (and peel order), then queues their adjacency on the cascade
// list or, for hubs and list overflow, on the global task queue.
__device__ __forceinline__ void on_claimed(Warp& w, bool found, uint32_t u, uint32_t start, uint32_t len) {
    const unsigned m = __ballot_sync(kFull, found);
    if (!m) return;
    const unsigned lane = lane_id();
    const uint32_t cnt = __popc(m);
    w.peeled += cnt;
    if (!(found && IN(u, w.a.V, 2))) { start = 0; len = 0; }
    else w.a.core[u] = w.level;
    if (w.a.order) {
        uint32_t pos = 0;
        if (lane == 0) pos = atomicAdd(&w.a.ctl->order_tail, cnt);
        pos = __shfl_sync(kFull, pos, 0);
        const uint32_t op = pos + __popc(m & lanemask_lt());
        if (found && IN(op, w.a.V, 4)) w.a.order[op] = u;
    }
    // The cascade list keeps at most local_budget arcs: the rest of a wide
    // cascade goes to the level's task queue, where idle warps take it,
    // instead of being walked by this warp alone, 128 arcs a step.
    bool local = found && len <= w.a.hub_arcs;
    uint32_t lsum;
    const uint32_t lex = warp_excl_scan(local ? len : 0u, &lsum);
    if (local && w.narcs + lex + len > w.a.local_budget) local = false;
    unsigned lm = __ballot_sync(kFull, local);
    if (w.nnext + __popc(lm) > kItemCap) { local = false; lm = 0; }
    if (local) {
        const uint32_t idx = w.nnext + __popc(lm & lanemask_lt());
        if (!IN(idx, kItemCap, 24)) return;
        w.b.nstart[idx] = start;
        w.b.nlen[idx] = len;
    }
    w.nnext += __popc(lm);
    w.narcs += __reduce_add_sync(kFull, local ? len : 0u);
    const bool glob = found && !local;
    if (__ballot_sync(kFull, glob)) push_tasks(w, glob, start, len);
}

// Starts moving the first adjacency line(s) of a vertex just claimed, arcs
// [start, start+len), into L1: the walk step that reads them comes one claim
// later, and the adjacency is read-only while the peel runs.  Hubs go to the
// task queue, where another SM reads them, and get none.
__device__ __forceinline__ void prefetch_adjacency(const PeelArgs& a, uint32_t start, uint32_t len) {
    if (len == 0 || len > a.hub_arcs) return;
    asm volatile("prefetch.global.L1 [%0];" ::"l"(a.nbr + start));
    if ((start & 31u) + len > 32u) asm volatile("prefetch.global.L1 [%0];" ::"l"(a.nbr + ((start | 31u) + 1u)));
}

// The neighbours u[j] of vertices peeled at this level (ours.cc:91-106), d[j]
// their states as read before: f[j] is set when this thread's decrement took
// u[j] to the level and claimed it, with u[j]'s arc range in start[j] / len[j].
// When d says the decrement will take u to the level, one atomicCAS
// decrements and claims at once, and u's offsets are loaded while it is in
// flight; otherwise one atomicSub.  All four atomics are issued before any
// result is examined, so they are in flight together.  A CAS that lost a
// race falls back to the reference's rule with the value it saw; a
// decrement that took u to the level claims it with atomicOr; one that found
// u at or below the level is undone (ours.cc:102-105).
__device__ __forceinline__ void decrement4(const PeelArgs& a, const uint32_t (&u)[4], const uint32_t (&d)[4],
                                           uint32_t kk, bool (&f)[4], uint32_t (&start)[4], uint32_t (&len)[4]) {
    uint32_t old[4], s0[4], s1[4];
    unsigned cas = 0, sub = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        f[j] = false; start[j] = 0; len[j] = 0; old[j] = 0; s0[j] = 0; s1[j] = 0;
        if (u[j] == kFull) continue;
        if (d[j] == kk + 1) {
            s0[j] = KC_LDG(a.off + u[j]);
            s1[j] = KC_LDG(a.off + u[j] + 1);
            old[j] = atomicCAS(a.w + u[j], kk + 1, kClaim | kk);
            cas |= 1u << j;
        } else if (d[j] > kk && d[j] < kClaim) {
            old[j] = atomicSub(a.w + u[j], 1u);
            sub |= 1u << j;
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (cas & (1u << j)) {
            if (old[j] == kk + 1) {
                f[j] = true; start[j] = s0[j]; len[j] = s1[j] - s0[j];
                prefetch_adjacency(a, start[j], len[j]);
                continue;
            }
            if (!(old[j] > kk && old[j] < kClaim)) continue;
            old[j] = atomicSub(a.w + u[j], 1u);   // lost race: the plain rule with the value seen
        } else if (!(sub & (1u << j))) {
            continue;
        }
        if (old[j] == kk + 1) {
            const uint32_t t0 = KC_LDG(a.off + u[j]), t1 = KC_LDG(a.off + u[j] + 1);
            if (atomicOr(a.w + u[j], kClaim) & kClaim) continue;
            f[j] = true; start[j] = t0; len[j] = t1 - t0;
            prefetch_adjacency(a, start[j], len[j]);
        } else if (old[j] <= kk || old[j] >= kClaim) {
            atomicAdd(a.w + u[j], 1u);   // undo
        }
    }
}

// Plain decrements issued by a walk step whose results have not been
// examined yet (u = kFull: none).
struct PendingDec {
    uint32_t u[4];
    uint32_t old[4];
};

// Examines the deferred decrements (ours.cc:96-105): one that took u to the
// level claims it with atomicOr and walks it in this level; one that found u
// at or below the level is undone.
__device__ __forceinline__ void resolve_pending(Warp& w, PendingDec& pd) {
    const uint32_t kk = w.kk;
    unsigned race = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (pd.u[j] == kFull) continue;
        const uint32_t o = pd.old[j];
        if (o == kk + 1) race |= 1u << j;
        else if (o <= kk || o >= kClaim) atomicAdd(w.a.w + pd.u[j], 1u);   // undo
    }
    if (__ballot_sync(kFull, race != 0)) {
        uint32_t t0[4], t1[4], r[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            t0[j] = 0; t1[j] = 0; r[j] = kClaim;
            if (race & (1u << j)) {
                t0[j] = KC_LDG(w.a.off + pd.u[j]);
                t1[j] = KC_LDG(w.a.off + pd.u[j] + 1);
                r[j] = atomicOr(w.a.w + pd.u[j], kClaim);
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const bool f = !(r[j] & kClaim);
            on_claimed(w, f, pd.u[j], t0[j], t1[j] - t0[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) pd.u[j] = kFull;
}

// Decrements the neighbours u[j] of vertices peeled at this level
// (ours.cc:91-106).  A level's progress is a chain of dependent hops
// (decrement -> claim -> walk of the claimed vertex), so a hop waits for one
// atomic: without reading the state first, one atomicCAS(level+1 -> level |
// claim) per neighbour decrements and claims at once, with the neighbour's
// offsets loaded while it is in flight.  A CAS that failed returned the
// state: a neighbour above level+1 gets a plain atomicSub whose result is
// examined by the next step (or by the flush at the end of the walk), off
// the hop's path; claimed neighbours and those at or below the level get
// nothing (the reference's deg[u] > level test).  The previous step's
// deferred decrements are resolved while these CASes are in flight.  f[j] is
// set for the neighbours this thread claimed, with their arc ranges.
__device__ __forceinline__ void claim_or_defer(Warp& w, const uint32_t (&u)[4], PendingDec& pd, bool (&f)[4],
                                               uint32_t (&start)[4], uint32_t (&len)[4]) {
    const PeelArgs& a = w.a;
    const uint32_t kk = w.kk;
    uint32_t old[4], s0[4], s1[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        old[j] = kClaim; s0[j] = 0; s1[j] = 0;
        if (u[j] == kFull) continue;
        s0[j] = KC_LDG(a.off + u[j]);
        s1[j] = KC_LDG(a.off + u[j] + 1);
        old[j] = atomicCAS(a.w + u[j], kk + 1, kClaim | kk);
    }
    resolve_pending(w, pd);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        f[j] = false; start[j] = 0; len[j] = 0;
        if (u[j] == kFull) continue;
        if (old[j] == kk + 1) {
            f[j] = true; start[j] = s0[j]; len[j] = s1[j] - s0[j];
            prefetch_adjacency(a, start[j], len[j]);
        } else if (old[j] > kk + 1 && old[j] < kClaim) {
            pd.u[j] = u[j];
            pd.old[j] = atomicSub(a.w + u[j], 1u);
        }
    }
}

// Walks every arc of the staged items (b.start / b.pref hold first arc and
// length), lanes striding over the concatenated arcs (ours.cc:82-107); each
// lane keeps four arcs in flight.  With claim_cas, decrements whose results
// are not examined yet carry over in pd to the next step; without, each
// step reads the neighbours' states first and settles its decrements.
__device__ __forceinline__ void walk_items(Warp& w, PendingDec& pd) {
    const unsigned lane = lane_id();
    const uint32_t n = w.nitems;
    w.nitems = 0;
    if (n == 0) return;
    // lengths -> exclusive prefix, 4 items per lane
    uint32_t l[4], s4 = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t i = lane * 4 + j;
        l[j] = i < n ? w.b.pref[i] : 0;
        s4 += l[j];
    }
    uint32_t total;
    uint32_t ex = warp_excl_scan(s4, &total);
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t i = lane * 4 + j;
        if (i < n) w.b.pref[i] = ex;
        ex += l[j];
    }
    if (lane == 0) w.b.pref[n] = total;
    __syncwarp();
    // Neighbour ids of arcs [base, base+128), 4 per lane.  (Issuing the next
    // step's loads before this step's atomics measured 1-5% slower: it made
    // the kernel spill registers.)
    uint32_t lo = 0;
    auto load_step = [&](uint32_t base, uint32_t (&u)[4]) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t a = base + 32 * j + lane;
            u[j] = 0xFFFFFFFFu;
            if (a < total) {
                uint32_t hi = n;
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (w.b.pref[mid] <= a) lo = mid; else hi = mid;
                }
                const uint32_t arc = w.b.start[lo] + (a - w.b.pref[lo]);
                if (IN(lo, kItemCap, 22) && IN(arc, w.a.E, 5)) {
                    u[j] = KC_LDG(w.a.nbr + arc);
                    if (!IN(u[j], w.a.V, 6)) u[j] = 0xFFFFFFFFu;
                }
            }
        }
    };
    for (uint32_t base = 0; base < total; base += 128) {
        uint32_t u[4];
        load_step(base, u);
        bool f[4];
        uint32_t cs[4], cl[4];
        if (w.a.claim_cas) {
            claim_or_defer(w, u, pd, f, cs, cl);
        } else {
            uint32_t d[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) d[j] = (u[j] != kFull) ? __ldcg(w.a.w + u[j]) : 0u;
            decrement4(w.a, u, d, w.kk, f, cs, cl);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) on_claimed(w, f[j], u[j], cs[j], cl[j]);
    }
    __syncwarp();
}

// Walks the staged items and then, while the cascade list is non-empty, the
// vertices it discovered in the same level.
__device__ void walk_with_cascades(Warp& w) {
    PendingDec pd;
#pragma unroll
    for (int j = 0; j < 4; ++j) { pd.u[j] = kFull; pd.old[j] = 0; }
    walk_items(w, pd);
    const unsigned lane = lane_id();
    for (;;) {
        while (w.nnext) {
            const uint32_t n = w.nnext;
            for (uint32_t i = lane; i < n; i += 32) {
                w.b.start[i] = w.b.nstart[i];
                w.b.pref[i] = w.b.nlen[i];
            }
            __syncwarp();
            w.nnext = 0;
            w.narcs = 0;
            w.nitems = n;
            walk_items(w, pd);
        }
        // the deferred decrements of the last steps; a raced claim among
        // them starts another cascade
        bool any = false;
#pragma unroll
        for (int j = 0; j < 4; ++j) any |= pd.u[j] != kFull;
        if (!__any_sync(kFull, any)) break;
        resolve_pending(w, pd);
    }
}

// Stages the claimed vertices v[j] (mask bits, up to 4 per lane; arcs
// [s0[j], s1[j])) as walk items; hubs go to the task queue.  Flushes the
// batch first when it could overflow.
__device__ __forceinline__ void stage_claims(Warp& w, const uint32_t (&v)[4], unsigned mine, const uint32_t (&s0)[4],
                                             const uint32_t (&s1)[4]) {
    uint32_t st[4], ln[4];
    unsigned localm = 0, hubm = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        st[j] = 0; ln[j] = 0;
        if (mine & (1u << j)) {
            if (!IN(v[j], w.a.V, 8)) continue;
            st[j] = s0[j];
            ln[j] = s1[j] - s0[j];
            if (ln[j] == 0) continue;
            if (ln[j] <= w.a.hub_arcs) localm |= 1u << j; else hubm |= 1u << j;
        }
    }
    const uint32_t cnt = __popc(localm);
    uint32_t tot;
    const uint32_t ex = warp_excl_scan(cnt, &tot);
    if (tot && w.nitems + tot > kItemCap) walk_with_cascades(w);
    uint32_t pos = w.nitems + ex;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if ((localm & (1u << j)) && IN(pos, kItemCap, 23)) { w.b.start[pos] = st[j]; w.b.pref[pos] = ln[j]; ++pos; }
    w.nitems += tot;
    __syncwarp();
    if (__ballot_sync(kFull, hubm != 0)) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const bool h = (hubm >> j) & 1u;
            if (__ballot_sync(kFull, h)) push_tasks(w, h, st[j], ln[j]);
        }
    }
}

// Appends this lane's survivors (mask bits of v[]) to the next alive list.
__device__ __forceinline__ void append_survivors(Warp& w, const uint32_t (&v)[4], unsigned surv) {
    const unsigned lane = lane_id();
    uint32_t tot;
    const uint32_t ex = warp_excl_scan(__popc(surv), &tot);
    if (tot == 0) return;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&w.slot->alive_next, tot);
    base = __shfl_sync(kFull, base, 0);
    if (base + tot > w.a.V) {   // cannot happen: each vertex is appended once per level
        if (lane == 0) record_error(w.a.ctl, kErrOverflow, w.level);
        return;
    }
    base += ex;
    uint32_t* out = w.a.alive[w.list_cur ^ 1u];
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if ((surv & (1u << j)) && IN(base, w.a.V, 9)) out[base++] = v[j];
}

// Claims (atomicOr) the hit vertices v[j], their offsets s0/s1 loaded while
// the atomics are in flight; returns the mask of those this lane claimed,
// recording their core number.
__device__ __forceinline__ unsigned claim_hits(Warp& w, const uint32_t (&v)[4], unsigned hit, uint32_t (&s0)[4],
                                               uint32_t (&s1)[4]) {
    unsigned o[4] = {kClaim, kClaim, kClaim, kClaim};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        s0[j] = 0; s1[j] = 0;
        if ((hit & (1u << j)) && IN(v[j], w.a.V, 10)) {
            s0[j] = KC_LDG(w.a.off + v[j]);
            s1[j] = KC_LDG(w.a.off + v[j] + 1);
            o[j] = atomicOr(w.a.w + v[j], kClaim);
        }
    }
    unsigned mine = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (!(o[j] & kClaim)) {
            mine |= 1u << j;
            w.a.core[v[j]] = w.level;
            if (w.level > 0) prefetch_adjacency(w.a, s0[j], s1[j] - s0[j]);
        }
    return mine;
}

// Common tail of one scan step: publishes claims (peel order, count) and
// stages their walk.
__device__ __forceinline__ void after_claims(Warp& w, const uint32_t (&v)[4], unsigned mine, const uint32_t (&s0)[4],
                                             const uint32_t (&s1)[4]) {
    const unsigned lane = lane_id();
    uint32_t tot;
    const uint32_t ex = warp_excl_scan(__popc(mine), &tot);
    if (tot == 0) return;
    w.peeled += tot;
    if (w.a.order) {
        uint32_t pos = 0;
        if (lane == 0) pos = atomicAdd(&w.a.ctl->order_tail, tot);
        pos = __shfl_sync(kFull, pos, 0) + ex;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if ((mine & (1u << j)) && IN(pos, w.a.V, 12)) w.a.order[pos++] = v[j];
    }
    if (w.level > 0) stage_claims(w, v, mine, s0, s1);
}

// Scan of this warp's share of the vertices for level w.level (ours.cc:15-25):
// either 128-vertex groups of the state array (uint4 loads) or 32-entry
// groups of the alive list; every claimed vertex is walked inline.
__device__ void scan_level(Warp& w, uint32_t gw) {
    const unsigned lane = lane_id();
    const PeelArgs& a = w.a;
    const uint32_t kk = w.kk;
    const bool compact = (w.mode == kDenseCompact || w.mode == kListCompact);
    if (w.it == 0 && a.zero_tasks) {
        // Level 0 pushes no task (its vertices have no arcs) and the next level
        // starts only after every participant has arrived, so the queue can be
        // cleared here instead of by a separate memset.
        for (unsigned long long i = (unsigned long long)gw * 32 + lane; i < a.task_cap; i += (unsigned long long)w.nwt * 32)
            a.tasks[i] = 0ull;
    }
    if (w.mode == kList || w.mode == kListCompact) {
        const uint32_t* list = a.alive[w.list_cur];
        const uint32_t n = w.list_len;
        // When every warp has several steps of the list (a small gang), a step
        // takes 128 entries, 4 per lane with their loads in flight together;
        // otherwise 32, one per lane, so that a short list still spreads over
        // all warps.
        const uint32_t nj = (n >= w.nwt * 128u * 2u) ? 4u : 1u;
        for (uint32_t i0 = gw * 32 * nj; i0 < n; i0 += w.nwt * 32 * nj) {
            uint32_t v[4];
#pragma unroll
            for (uint32_t j = 0; j < 4; ++j) {
                const uint32_t i = i0 + j * 32 + lane;
                v[j] = (j < nj && i < n && IN(i, a.V, 13)) ? __ldcg(list + i) : kFull;
            }
            uint32_t d[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                d[j] = kClaim;
                if (v[j] < a.V) d[j] = __ldcg(a.w + v[j]);
                else if (v[j] != kFull) record_error(a.ctl, kErrOverflow, w.level);   // defensive: never index past V
            }
            unsigned hit = 0, surv = 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (d[j] == kk) hit |= 1u << j;
                if (d[j] > kk && d[j] < kClaim) { surv |= 1u << j; w.minv = min(w.minv, d[j]); w.arcs += d[j] - kBias; }
            }
            if (compact) append_survivors(w, v, surv);
            if (!__ballot_sync(kFull, hit != 0)) continue;
            uint32_t s0[4], s1[4];
            const unsigned mine = claim_hits(w, v, hit, s0, s1);
            after_claims(w, v, mine, s0, s1);
        }
    } else {
        const uint32_t ngroups = (a.V + 127) / 128;
        uint4* w4 = reinterpret_cast<uint4*>(a.w);
        // When every warp has several groups (a small gang), a step takes two
        // 128-vertex groups with both loads in flight together.
        const uint4 kNone = make_uint4(kClaim, kClaim, kClaim, kClaim);
        const uint32_t ng = (ngroups >= 4 * w.nwt) ? 2u : 1u;
        for (uint32_t g0 = gw; w.level != 0 && g0 < ngroups; g0 += ng * w.nwt) {
            const uint32_t g1 = g0 + w.nwt;
            uint4 xg[2];
            xg[0] = IN(g0 * 32 + lane, (a.V + 127) / 128 * 32, 18) ? __ldcg(w4 + g0 * 32 + lane) : kNone;
            xg[1] = (ng == 2 && g1 < ngroups && IN(g1 * 32 + lane, (a.V + 127) / 128 * 32, 18)) ? __ldcg(w4 + g1 * 32 + lane)
                                                                                                : kNone;
#pragma unroll
            for (uint32_t r = 0; r < 2; ++r) {
                if (r >= ng) break;
                const uint32_t vb = (r ? g1 : g0) * 128 + lane * 4;
                const uint32_t v[4] = {vb, vb + 1, vb + 2, vb + 3};
                const uint32_t xs[4] = {xg[r].x, xg[r].y, xg[r].z, xg[r].w};
                unsigned hit = 0, surv = 0;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (xs[j] == kk) hit |= 1u << j;
                    if (xs[j] > kk && xs[j] < kClaim) { surv |= 1u << j; w.minv = min(w.minv, xs[j]); w.arcs += xs[j] - kBias; }
                }
                if (compact) append_survivors(w, v, surv);
                if (__ballot_sync(kFull, hit != 0)) {
                    uint32_t s0[4], s1[4];
                    const unsigned mine = claim_hits(w, v, hit, s0, s1);
                    after_claims(w, v, mine, s0, s1);
                }
            }
        }
        for (uint32_t g = gw; w.level == 0 && g < ngroups; g += w.nwt) {
            const uint32_t vb = g * 128 + lane * 4;
            const uint32_t v[4] = {vb, vb + 1, vb + 2, vb + 3};
            {
                // Level 0 also initialises the state from the offsets: isolated
                // vertices are peeled here and have nothing to walk.
                uint32_t st[4];
                unsigned mine = 0;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (v[j] < a.V) {
                        const uint32_t dg = KC_LDG(a.off + v[j] + 1) - KC_LDG(a.off + v[j]);
                        if (dg == 0) { st[j] = kClaim | kBias; mine |= 1u << j; a.core[v[j]] = 0; }
                        else st[j] = dg + kBias;
                    } else {
                        st[j] = kClaim | kBias;   // padding never matches
                    }
                }
                if (IN(g * 32 + lane, (a.V + 127) / 128 * 32, 17))
                    __stcg(w4 + g * 32 + lane, make_uint4(st[0], st[1], st[2], st[3]));
                unsigned surv = 0;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (!(st[j] & kClaim)) { surv |= 1u << j; w.minv = min(w.minv, st[j]); w.arcs += st[j] - kBias; }
                if (compact) append_survivors(w, v, surv);
                const uint32_t none[4] = {0u, 0u, 0u, 0u};   // level 0 stages no walk
                after_claims(w, v, mine, none, none);
            }
        }
    }
    walk_with_cascades(w);
}

// CTA-wide view of the level state: one warp at a time reads the global
// counters (level completion, queue depth, error word) with independent
// relaxed loads and leaves a hint in shared memory for the others, so idle
// warps do not hammer one L2 line.  Returns 1 when the level is complete, -1
// on a recorded error, else 0.
__device__ __forceinline__ int level_state(Warp& w, uint32_t* avail) {
    CtaShared& sh = w.sh;
    const unsigned lane = lane_id();
    unsigned done_v = 0, lvl = 0, av = 0;
    int err = 0;
    if (lane == 0) {
        if (atomicCAS(&sh.poll_lock, 0u, 1u) == 0u) {
            const unsigned long long ut = ld_relaxed64(&w.slot->units_tail);
            const unsigned h = ld_relaxed(&w.slot->head);
            const int e = ld_err(&w.a.ctl->err);
            const unsigned t = (unsigned)ut;
            // hint_done only grows: a warp of the CTA may already poll the
            // next iteration while another still polls this one
            if ((unsigned)(ut >> 32) == w.nparts + t && *(volatile unsigned*)&sh.hint_done < w.it + 1)
                *(volatile unsigned*)&sh.hint_done = w.it + 1;
            *(volatile unsigned*)&sh.hint_avail = t > h ? t - h : 0u;
            *(volatile unsigned*)&sh.hint_level = w.it;
            *(volatile int*)&sh.hint_err = e;
            __threadfence_block();
            atomicExch(&sh.poll_lock, 0u);
        }
        done_v = *(volatile unsigned*)&sh.hint_done;
        lvl = *(volatile unsigned*)&sh.hint_level;
        av = *(volatile unsigned*)&sh.hint_avail;
        err = *(volatile int*)&sh.hint_err;
    }
    done_v = __shfl_sync(kFull, done_v, 0);
    lvl = __shfl_sync(kFull, lvl, 0);
    av = __shfl_sync(kFull, av, 0);
    err = __shfl_sync(kFull, err, 0);
    *avail = (lvl == w.it) ? av : 0u;
    if (done_v > w.it) return 1;
    return err ? -1 : 0;
}

// Finishes `n` work units of the level (a participant's scan, or tasks).
// The caller has fenced its writes.  Only a traced run waits for the add's
// result, to time-stamp the event that completed the level.
__device__ __forceinline__ void finish_units(Warp& w, uint32_t n) {
    const unsigned long long add = (unsigned long long)n << 32;
    const unsigned long long ut = atomicAdd(&w.slot->units_tail, add) + add;
    if (w.a.trace && (unsigned)(ut >> 32) == w.nparts + (unsigned)ut) trace(w.a, w.it, 2, now_ns());
}

// Publishes `ndone` finished tasks and the vertices this warp claimed in them.
__device__ __forceinline__ void finish_tasks(Warp& w, uint32_t ndone) {
    if (lane_id() == 0) {
        if (w.peeled) atomicAdd(&w.slot->peeled, w.peeled);
        fence_acq_rel();   // pushes, claims and the count before the completion
        finish_units(w, ndone);
    }
    w.peeled = 0;
}

// Claims and walks queued tasks until the level is complete.  Returns false
// on error.
__device__ bool drain_level(Warp& w) {
    const unsigned lane = lane_id();
    const PeelArgs& a = w.a;
    unsigned pend = 0;
    uint32_t cbase = 0;
    unsigned long long waited_since = now_ns();
    const unsigned long long limit_ns = (unsigned long long)a.wait_us * 1000ull;
    uint32_t sleep_ns = 32;
    for (;;) {
        if (pend == 0) {
            uint32_t avail;
            const int ls = level_state(w, &avail);
            if (ls > 0) return true;
            if (ls < 0) return false;
            if (avail) {
                const uint32_t share = avail / max(1u, w.nwt / 2u);
                const uint32_t B = min(32u, max(1u, share));
                uint32_t c = 0;
                if (lane == 0) c = atomicAdd(&w.slot->head, B);
                cbase = __shfl_sync(kFull, c, 0);
                pend = (B == 32) ? kFull : ((1u << B) - 1u);
                waited_since = now_ns();
                sleep_ns = 32;
            } else {
                if (now_ns() - waited_since > limit_ns) { if (lane == 0) record_error(a.ctl, kErrTimeout, w.level); return false; }
                __nanosleep(sleep_ns);
                sleep_ns = min(sleep_ns * 2, 128u);
                continue;
            }
        }
        bool ready = false;
        unsigned long long e = 0;
        if (pend & (1u << lane)) {
            const unsigned long long pos = w.task_base + cbase + lane;
            if (pos < a.task_cap) {
                e = ld_relaxed64(&a.tasks[pos]);
                ready = task_ready(e, w.level, a.epoch);
            }
        }
        const unsigned rm = __ballot_sync(kFull, ready);
        if (rm) {
            if (ready) {
                const uint32_t idx = __popc(rm & lanemask_lt());
                w.b.start[idx] = (uint32_t)(e >> 32);
                w.b.pref[idx] = (uint32_t)((e >> 24) & 0xFF) + 1u;
            }
            __syncwarp();
            w.nitems = __popc(rm);
            walk_with_cascades(w);
            pend &= ~rm;
            finish_tasks(w, __popc(rm));
            waited_since = now_ns();
            sleep_ns = 32;
            continue;
        }
        uint32_t avail;
        const int ls = level_state(w, &avail);
        if (ls > 0) return true;   // claimed slots beyond the final tail
        if (ls < 0) return false;
        if (now_ns() - waited_since > limit_ns) { if (lane == 0) record_error(a.ctl, kErrTimeout, w.level); return false; }
        __nanosleep(sleep_ns);
        sleep_ns = min(sleep_ns * 2, 128u);
    }
}

// ------------------------------------------------------------ tail hand-off
// Once few vertices remain, every later level touches a small induced
// subgraph whose vertices still carry their full adjacency, and each level
// costs the grid-wide arrival protocol.  The participants then build the
// induced CSR of the survivors with local ids (their remaining degree is
// their state, so the offsets need no count pass) and stop; peel_tail_kernel
// finishes the peel in one CTA with the states in shared memory.

// Barrier of the `nparts` co-resident participants, bounded in time.  Every
// thread of the CTA calls it; false when the wait ran out or a participant
// recorded an error.
__device__ bool part_barrier(const PeelArgs& a, CtaShared& sh, uint32_t nparts, uint32_t level) {
    __syncthreads();
    if (threadIdx.x == 0) {
        PeelCtl* ctl = a.ctl;
        int ok = 1;
        const unsigned gen = ld_acquire(&ctl->bar_gen);
        __threadfence();
        if (atomicAdd(&ctl->bar_count, 1u) == nparts - 1) {
            atomicExch(&ctl->bar_count, 0u);
            __threadfence();
            atomicAdd(&ctl->bar_gen, 1u);
        } else {
            const unsigned long long t0 = now_ns(), lim = (unsigned long long)a.wait_us * 1000ull;
            while (ld_acquire(&ctl->bar_gen) == gen) {
                if (ld_err(&ctl->err)) { ok = 0; break; }
                if (now_ns() - t0 > lim) { record_error(ctl, kErrTimeout, level); ok = 0; break; }
                __nanosleep(64);
            }
        }
        if (ld_err(&ctl->err)) ok = 0;
        sh.bar_ok = ok;
    }
    __syncthreads();
    return sh.bar_ok != 0;
}

// Pass 1: every survivor (claim bit clear) gets a local id, its remaining
// degree as the length of its induced adjacency, and fill work items of at
// most kFillChunk raw arcs (first arc << 32 | local id << 9 | length-1).  The
// candidates are the current alive list when the scans keep one (a superset
// of the survivors), else every vertex.
__device__ void tail_collect(Warp& w, uint32_t gw, const uint32_t* list, uint32_t count) {
    const PeelArgs& a = w.a;
    const unsigned lane = lane_id();
    const bool dense = list == nullptr;
    const uint32_t nsteps = dense ? (a.V + 127) / 128 : (count + 127) / 128;
    for (uint32_t g = gw; g < nsteps; g += w.nwt) {
        uint32_t v[4], xs[4];
        if (dense) {
            const uint4 x = __ldcg(reinterpret_cast<const uint4*>(a.w) + g * 32 + lane);
            xs[0] = x.x; xs[1] = x.y; xs[2] = x.z; xs[3] = x.w;
#pragma unroll
            for (int j = 0; j < 4; ++j) v[j] = g * 128 + lane * 4 + j;
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t i = g * 128 + j * 32 + lane;
                v[j] = i < count ? __ldcg(list + i) : kFull;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) xs[j] = v[j] < a.V ? __ldcg(a.w + v[j]) : kClaim;
        }
        uint32_t st[4], rd[4], nit[4], cnt = 0, items = 0;
        unsigned alive = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            st[j] = 0; rd[j] = 0; nit[j] = 0;
            if (!(xs[j] & kClaim) && v[j] < a.V) {
                alive |= 1u << j;
                st[j] = KC_LDG(a.off + v[j]);
                rd[j] = KC_LDG(a.off + v[j] + 1) - st[j];
                nit[j] = (rd[j] + kFillChunk - 1) / kFillChunk;
                ++cnt;
                items += nit[j];
            }
        }
        if (!__ballot_sync(kFull, alive != 0)) continue;
        uint32_t ctot, itot;
        const uint32_t cex = warp_excl_scan(cnt, &ctot);
        const uint32_t iex = warp_excl_scan(items, &itot);
        uint32_t cb = 0, ib = 0;
        if (lane == 0) {
            cb = atomicAdd(&a.ctl->tail_n, ctot);
            ib = atomicAdd(&a.ctl->tail_items, itot);
        }
        cb = __shfl_sync(kFull, cb, 0) + cex;
        ib = __shfl_sync(kFull, ib, 0) + iex;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (!(alive & (1u << j))) continue;
            if (cb < a.tail_cap_v && ib + nit[j] <= a.tail_items_cap) {
                a.tail_ids[cb] = v[j];
                a.tail_off[cb + 1] = xs[j] - kBias;
                for (uint32_t c = 0; c < nit[j]; ++c) {
                    const uint32_t len = min(kFillChunk, rd[j] - c * kFillChunk);
                    a.tail_items[ib + c] = ((unsigned long long)(st[j] + c * kFillChunk) << 32) |
                                           ((unsigned long long)cb << 9) | (len - 1);
                }
            } else {
                record_error(a.ctl, kErrOverflow, w.level);
            }
            ++cb;
            ib += nit[j];
        }
    }
}

// Pass 2: the state word of each survivor becomes its local id (claim bit
// clear, so the fill pass tells survivors from peeled vertices by the same
// bit), the induced CSR is preset to the pad value 0xFFFFFFFF up to its bound
// (arcs_bound entries), and CTA 0 turns the degrees into offsets and fill
// cursors.  Each adjacency is padded to a multiple of 4 entries so that the
// tail walk can read 16-byte quads; a cursor ends at offset + degree.
__device__ void tail_offsets(Warp& w, CtaShared& sh, uint32_t gw, uint32_t part, unsigned long long arcs_bound) {
    const PeelArgs& a = w.a;
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    const uint32_t n = min(ld_relaxed(&a.ctl->tail_n), a.tail_cap_v);
    for (uint32_t i = gw * 32 + lane; i < n; i += w.nwt * 32) {
        const uint32_t v = __ldcg(a.tail_ids + i);
        if (v < a.V) a.w[v] = i;
    }
    const uint32_t nq = (uint32_t)(min(arcs_bound, (unsigned long long)a.tail_cap_arcs) / 4);
    uint4* nbr4 = reinterpret_cast<uint4*>(a.tail_nbr);
    for (uint32_t i = gw * 32 + lane; i < nq; i += w.nwt * 32) __stcg(nbr4 + i, make_uint4(kFull, kFull, kFull, kFull));
    if (part != 0) return;
    // Block-wide scan in tiles of kTile degrees staged in shared memory (the
    // walk batches are free here): coalesced loads and stores, each thread
    // scanning kTile/kPeelThreads consecutive entries of a tile.
    constexpr uint32_t kTile = 4096;
    constexpr uint32_t kPer = kTile / kPeelThreads;
    static_assert(sizeof(sh.wb) >= sizeof(uint32_t) * (kTile + kPeelWarps + 1), "scan scratch");
    uint32_t* buf = reinterpret_cast<uint32_t*>(&sh.wb[0]);
    uint32_t* tot = buf + kTile;
    uint32_t carry = 0;
    for (uint32_t t0 = 0; t0 < n; t0 += kTile) {
        const uint32_t m = min(kTile, n - t0);
        uint32_t d[kPer];
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) {
            const uint32_t i = threadIdx.x + k * kPeelThreads;
            d[k] = i < m ? (__ldcg(a.tail_off + t0 + i + 1) + 3u) & ~3u : 0u;
        }
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) buf[threadIdx.x + k * kPeelThreads] = d[k];
        __syncthreads();
        uint32_t loc[kPer], sum = 0;
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) { loc[k] = buf[threadIdx.x * kPer + k]; sum += loc[k]; }
        uint32_t wt;
        const uint32_t ex = warp_excl_scan(sum, &wt);
        if (lane == 0) tot[wid] = wt;
        __syncthreads();
        if (wid == 0) {
            const uint32_t t = lane < kPeelWarps ? tot[lane] : 0u;
            uint32_t all;
            const uint32_t te = warp_excl_scan(t, &all);
            if (lane < kPeelWarps) tot[lane] = te;
            if (lane == 0) tot[kPeelWarps] = all;
        }
        __syncthreads();
        uint32_t run = carry + tot[wid] + ex;
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) { run += loc[k]; buf[threadIdx.x * kPer + k] = run; }   // inclusive
        __syncthreads();
#pragma unroll
        for (uint32_t k = 0; k < kPer; ++k) {
            const uint32_t i = threadIdx.x + k * kPeelThreads;
            if (i < m) {
                const uint32_t incl = buf[i];
                a.tail_off[t0 + i + 1] = incl;
                a.tail_cur[t0 + i] = incl - d[k];
            }
        }
        carry += tot[kPeelWarps];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.tail_off[0] = 0;
        a.ctl->tail_arcs = carry;
        if (carry > nq * 4u) record_error(a.ctl, kErrOverflow, w.level);   // beyond the preset bound
    }
}

// Pass 3: fill items, kFillBatch per warp step; the survivors among an item's
// neighbours are appended, as local ids, at the vertex's fill cursor.  The
// order of a vertex's induced neighbours is immaterial.
__device__ void tail_fill(Warp& w, uint32_t gw) {
    const PeelArgs& a = w.a;
    const unsigned lane = lane_id();
    const uint32_t n = min(ld_relaxed(&a.ctl->tail_n), a.tail_cap_v);
    const uint32_t ni = min(ld_relaxed(&a.ctl->tail_items), a.tail_items_cap);
    constexpr int kPer = kFillChunk / 32;
    constexpr int kFillBatch = 4;
    for (uint32_t i0 = gw; i0 < ni; i0 += kFillBatch * w.nwt) {
        uint32_t lid[kFillBatch], u[kFillBatch][kPer];
#pragma unroll
        for (int r = 0; r < kFillBatch; ++r) {
            const uint32_t i = i0 + r * w.nwt;
            const unsigned long long item = i < ni ? __ldcg(a.tail_items + i) : 0ull;
            const uint32_t s0 = (uint32_t)(item >> 32);
            const uint32_t len = i < ni ? ((uint32_t)item & 0x1FFu) + 1u : 0u;
            lid[r] = i < ni ? ((uint32_t)item >> 9) : kFull;
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const uint32_t k = j * 32 + lane;
                u[r][j] = (k < len && s0 + k < a.E) ? KC_LDG(a.nbr + s0 + k) : kFull;
            }
        }
        unsigned keep[kFillBatch] = {};
#pragma unroll
        for (int r = 0; r < kFillBatch; ++r) {
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                if (u[r][j] < a.V) {
                    const uint32_t x = __ldcg(a.w + u[r][j]);
                    if (!(x & kClaim)) { keep[r] |= 1u << j; u[r][j] = x; }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < kFillBatch; ++r) {
            uint32_t tot;
            const uint32_t ex = warp_excl_scan(__popc(keep[r]), &tot);
            if (tot == 0) continue;
            if (lid[r] >= n) { if (lane == 0) record_error(a.ctl, kErrOverflow, w.level); continue; }
            uint32_t base = 0, end = 0;
            if (lane == 0) {
                base = atomicAdd(a.tail_cur + lid[r], tot);
                end = __ldcg(a.tail_off + lid[r] + 1);
            }
            base = __shfl_sync(kFull, base, 0);
            end = __shfl_sync(kFull, end, 0);
            if (base + tot > end || end > a.tail_cap_arcs) {   // a state disagrees with the adjacency
                if (lane == 0) record_error(a.ctl, kErrOverflow, w.level);
                continue;
            }
            uint32_t pos = base + ex;
#pragma unroll
            for (int j = 0; j < kPer; ++j)
                if (keep[r] & (1u << j)) a.tail_nbr[pos++] = u[r][j];
        }
    }
}

// Builds the induced CSR of the survivors for the tail peel, which starts at
// level `next` with `peeled_total` vertices peeled in `iters` iterations.
__device__ void tail_handoff(Warp& w, CtaShared& sh, uint32_t gw, uint32_t part, uint32_t nparts, uint32_t next,
                             uint32_t peeled_total, uint32_t iters, const uint32_t* list, uint32_t count,
                             unsigned long long arcs_bound) {
    const PeelArgs& a = w.a;
    if (part == 0 && threadIdx.x == 0) {
        a.ctl->tail_level = next;
        a.ctl->tail_peeled = peeled_total;
        a.ctl->tail_iter = iters;
    }
    // trace of the hand-off in the first tail row: fields 1, 2 and 5 = the
    // two barriers passed and CTA 0's fill done
    const bool lead = part == 0 && threadIdx.x == 0;
    tail_collect(w, gw, list, count);
    if (!part_barrier(a, sh, nparts, w.level)) return;
    if (lead) trace(a, iters, 1, now_ns());
    tail_offsets(w, sh, gw, part, arcs_bound);
    if (!part_barrier(a, sh, nparts, w.level)) return;
    if (lead) trace(a, iters, 2, now_ns());
    tail_fill(w, gw);
    __syncthreads();
    if (lead) trace(a, iters, 5, now_ns());
}

// The whole peel of one graph by `nparts` co-resident CTAs; this CTA is
// participant `part`.  Every thread of the CTA calls it.  The persistent
// kernel runs it with the whole grid; the serve kernel with a gang of CTAs.
__device__ void peel_body(const PeelArgs& a, CtaShared& sh, uint32_t part, uint32_t nparts) {
    const unsigned lane = lane_id();
    const unsigned wid = threadIdx.x >> 5;
    __syncthreads();
    if (threadIdx.x < 4) {
        sh.arrive[threadIdx.x] = 0; sh.peeled[threadIdx.x] = 0; sh.minv[threadIdx.x] = kFull; sh.arcs[threadIdx.x] = 0;
    }
    if (threadIdx.x == 0) { sh.poll_lock = 0; sh.hint_level = 0xFFFFFFFFu; sh.hint_avail = 0; sh.hint_done = 0; sh.hint_err = 0; }
    __syncthreads();

    Warp w{a, sh.wb[wid], sh, nullptr, 0ull, 0u, kBias, 0u, 0u, 0u, nparts * kPeelWarps, nparts, kDense, 0u, 0u,
           0u, kFull, 0u, 0u};
    const uint32_t gw = part * kPeelWarps + wid;
    PeelCtl* ctl = a.ctl;
    const bool lists = a.alive[0] != nullptr && a.alive[1] != nullptr;
    const bool lead = part == 0 && threadIdx.x == 0;
    if (lead && a.shells && a.shell_cap) a.shells[0] = 0;
    uint32_t peeled_total = 0;
    // max_level from the device-side validation that ran before this launch;
    // nothing is peeled when it found the CSR invalid
    uint32_t max_level = a.max_level;
    if (max_level == kFull) {
        if (ld_err(&ctl->err)) return;
        max_level = ld_relaxed(&ctl->maxdeg);
    }

    for (uint32_t level = 0, it = 0;; ++it) {
        w.level = level;
        w.it = it;
        w.kk = level + kBias;
        w.slot = &ctl->slot[it & 3];
        w.minv = kFull;
        w.arcs = 0;
        if (lead) {
            trace(a, it, 0, now_ns());
            LevelSlot* r = &ctl->slot[(it + 2) & 3];
            r->units_tail = 0; r->head = 0; r->peeled = 0; r->arrived = 0;
            r->alive_next = 0; r->min_next = kFull; r->arcs_next = 0;
            __threadfence();
        }
        scan_level(w, gw);

        // CTA arrival.  Each warp releases its writes at CTA scope and counts
        // itself in shared memory; the last warp of the CTA publishes the
        // CTA's claims and smallest survivor with one GPU-scope fence and one
        // 64-bit atomic, and the arrival that completes the level announces it.
        const uint32_t wmin = __reduce_min_sync(kFull, w.minv);
        const uint32_t warcs = __reduce_add_sync(kFull, w.arcs);
        if (lane == 0) {
            const unsigned r = it & 3;
            if (w.peeled) atomicAdd(&sh.peeled[r], w.peeled);
            if (wmin != kFull) atomicMin(&sh.minv[r], wmin);
            if (warcs) atomicAdd(&sh.arcs[r], (unsigned long long)warcs);
            __threadfence_block();
            const unsigned x = atomicAdd(&sh.arrive[r], 1u);
            if (x == kPeelWarps - 1) {
                __threadfence_block();
                const unsigned p = atomicExch(&sh.peeled[r], 0u);
                const unsigned m = atomicExch(&sh.minv[r], kFull);
                const unsigned long long ca = atomicExch(&sh.arcs[r], 0ull);
                atomicExch(&sh.arrive[r], 0u);
                if (m != kFull) atomicMin(&w.slot->min_next, m);
                if (ca) atomicAdd(&w.slot->arcs_next, ca);
                if (p) atomicAdd(&w.slot->peeled, p);
                __threadfence();
                if (part == 0) trace(a, it, 1, now_ns());
                finish_units(w, 1);
                if (a.trace && atomicAdd(&w.slot->arrived, 1u) + 1u == nparts) trace(a, it, 5, now_ns());
            }
        }
        w.peeled = 0;
        __syncwarp();

        if (!drain_level(w)) return;
        fence_acq_rel();

        unsigned t = 0, an = 0, mn = 0, pi = 0;
        unsigned long long ae = 0;
        if (lane == 0) {
            t = (unsigned)ld_relaxed64(&w.slot->units_tail);
            an = ld_relaxed(&w.slot->alive_next);
            mn = ld_relaxed(&w.slot->min_next);
            pi = ld_relaxed(&w.slot->peeled);
            ae = ld_relaxed64(&w.slot->arcs_next);
        }
        t = __shfl_sync(kFull, t, 0);
        an = __shfl_sync(kFull, an, 0);
        mn = __shfl_sync(kFull, mn, 0);
        pi = __shfl_sync(kFull, pi, 0);
        ae = __shfl_sync(kFull, ae, 0);
        w.task_base += t;
        peeled_total += pi;
        if (lead) {
            ctl->iters_done = it + 1;
            ctl->tasks += t;
            trace(a, it, 3, now_ns());
            trace(a, it, 4, peeled_total);
            if (a.shells && level + 1 < a.shell_cap) a.shells[level + 1] = peeled_total;
        }
        if (peeled_total >= a.V) {
            if (lead) {
                ctl->kmax = level;
                ctl->levels = level + 1;
                ctl->iterations = it + 1;
                ctl->hx.peel_done = 1;
            }
            return;
        }
        if (level >= max_level) {
            if (lane == 0) record_error(ctl, kErrOverflow, level);
            return;
        }
        // Next level.  A level that peeled nothing changed no degree, so every
        // level below the smallest survivor state its scan saw is empty too and
        // is skipped (its k-shell offset repeats).
        uint32_t next = level + 1;
        if (pi == 0 && mn != kFull && mn - kBias > next) next = mn - kBias;
        if (lead && a.shells)
            for (uint32_t l = level + 2; l <= next && l < a.shell_cap; ++l) a.shells[l] = peeled_total;
        // Stop for the h-index peel once few vertices survive: every survivor
        // has more than `level` surviving neighbours, so its core number is at
        // least `next`, and its remaining degree is an upper bound of it.
        if (a.stop_alive && a.V - peeled_total <= a.stop_alive) {
            if (lead) {
                ctl->hx.stopped = 1;
                ctl->iterations = it + 1;
            }
            return;
        }
        // Hand the rest to the tail peel once it fits: few survivors, and the
        // survivor degrees seen by this level's scans (an upper bound of the
        // induced arcs) plus padding within the tail's CSR capacity.
        if (a.tail_cap_v && a.V - peeled_total <= a.tail_cap_v &&
            ae + 3ull * (a.V - peeled_total) <= a.tail_cap_arcs) {
            // candidates: the list this level's scans appended to, or read
            const bool appended = w.mode == kDenseCompact || w.mode == kListCompact;
            const uint32_t* list = appended ? a.alive[w.list_cur ^ 1u] : (w.mode == kList ? a.alive[w.list_cur] : nullptr);
            const uint32_t count = appended ? min(an, a.V) : w.list_len;
            tail_handoff(w, sh, gw, part, nparts, next, peeled_total, it + 1, lists ? list : nullptr, count,
                         (ae + 3ull * (a.V - peeled_total) + 3ull) & ~3ull);
            return;
        }
        level = next;
        // Scan mode of the next level (identical in every warp: it depends only
        // on the peeled count and the list length, both final here).
        if (w.mode == kDenseCompact || w.mode == kListCompact) {
            w.list_cur ^= 1u;
            w.list_len = min(an, a.V);
        }
        const uint32_t alive = a.V - peeled_total;
        if (!lists) {
            w.mode = kDense;
        } else if (w.mode == kDense) {
            w.mode = (alive <= a.V / 4) ? kDenseCompact : kDense;
        } else {
            w.mode = (alive <= w.list_len / 2) ? kListCompact : kList;
        }
    }
}


#ifndef KC_PEEL_NO_KERNEL
#ifdef KC_CHECKED
#define KC_PEEL_KERNEL peel_persistent_kernel_checked
#define KC_PEEL_FN peel_persistent_fn_checked
#else
#define KC_PEEL_KERNEL peel_persistent_kernel
#define KC_PEEL_FN peel_persistent_fn
#endif

__global__ void __launch_bounds__(kPeelThreads, 1) KC_PEEL_KERNEL(const __grid_constant__ PeelArgs a) {
    __shared__ CtaShared sh;
    // the h-index peel launched before this kernel found every core number, or
    // a level peel launched before it finished
    if (ld_relaxed(&a.ctl->hx.solved) || ld_relaxed(&a.ctl->hx.peel_done)) return;
    peel_body(a, sh, blockIdx.x, gridDim.x);
}
#endif

}  // namespace KC_VNS

#ifndef KC_PEEL_NO_KERNEL
const void* KC_PEEL_FN() { return reinterpret_cast<const void*>(&KC_VNS::KC_PEEL_KERNEL); }
#endif

}  // namespace kc
