// Persistent single-graph peel for sm_103a: every level of the level-
// synchronous peel (src/ours.cc:117-160) in one cooperative launch, with no
// host round trip and no grid barrier inside a level.  See kc_device.cuh for
// the claim protocol.
#include "kc_device.cuh"
#include "kc_peel.cuh"

namespace kc {

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
    unsigned int poll_lock;
    unsigned int hint_level;
    unsigned int hint_avail;
    unsigned int hint_done;
};

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
    uint32_t nwt;      // warps in the grid
};

// Pushes the arc range [start, start+len) of every lane with `pred` to the
// level's task queue, split into chunks of kChunk arcs.
__device__ __noinline__ void push_tasks(Warp& w, bool pred, uint32_t start, uint32_t len) {
    const unsigned lane = lane_id();
    uint32_t nch = pred ? (len + kChunk - 1) / kChunk : 0;
    uint32_t tot;
    uint32_t ex = warp_excl_scan(nch, &tot);
    if (tot == 0) return;
    uint32_t base = 0;
    if (lane == 0) {
        base = atomicAdd(&w.slot->tail, tot);
        atomicAdd(&w.a.ctl->tasks, (unsigned long long)tot);
    }
    base = __shfl_sync(kFull, base, 0);
    const unsigned long long first = w.task_base + base;
    const bool fits = first + tot <= w.a.task_cap;
    if (!fits) {
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
        const uint32_t c0 = (l0 + kChunk - 1) / kChunk;
        for (uint32_t c = lane; c < c0; c += 32) {
            const uint32_t cs = s0 + c * kChunk;
            const uint32_t cl = min(kChunk, l0 - c * kChunk);
            st_relaxed64(&w.a.tasks[first + e0 + c], make_task(cs, cl, w.level, w.a.epoch));
        }
    }
}

// Handles the vertices claimed by this warp in one walk step: records the
// core number (and peel order), then queues their adjacency on the cascade
// list or, for hubs and list overflow, on the global task queue.
__device__ __forceinline__ void on_claimed(Warp& w, bool found, uint32_t u) {
    const unsigned m = __ballot_sync(kFull, found);
    if (!m) return;
    const unsigned lane = lane_id();
    const uint32_t cnt = __popc(m);
    w.peeled += cnt;
    uint32_t start = 0, len = 0;
    if (found) {
        w.a.core[u] = w.level;
        start = __ldg(w.a.off + u);
        len = __ldg(w.a.off + u + 1) - start;
    }
    if (w.a.order) {
        uint32_t pos = 0;
        if (lane == 0) pos = atomicAdd(&w.a.ctl->order_tail, cnt);
        pos = __shfl_sync(kFull, pos, 0);
        if (found) w.a.order[pos + __popc(m & lanemask_lt())] = u;
    }
    bool local = found && len <= kLocalArcs;
    unsigned lm = __ballot_sync(kFull, local);
    if (w.nnext + __popc(lm) > kItemCap) { local = false; lm = 0; }
    if (local) {
        const uint32_t idx = w.nnext + __popc(lm & lanemask_lt());
        w.b.nstart[idx] = start;
        w.b.nlen[idx] = len;
    }
    w.nnext += __popc(lm);
    const bool glob = found && !local;
    if (__ballot_sync(kFull, glob)) push_tasks(w, glob, start, len);
}

// Walks every arc of the staged items (b.start / b.pref hold first arc and
// length), lanes striding over the concatenated arcs (ours.cc:82-107).
__device__ void walk_items(Warp& w) {
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
    const uint32_t kk = w.kk;
    uint32_t lo = 0;
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t a = base + lane;
        bool found = false;
        uint32_t u = 0;
        if (a < total) {
            uint32_t hi = n;
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (w.b.pref[mid] <= a) lo = mid; else hi = mid;
            }
            const uint32_t arc = w.b.start[lo] + (a - w.b.pref[lo]);
            u = __ldg(w.a.nbr + arc);
            const uint32_t d = __ldcg(w.a.w + u);
            if (d > kk && d < kClaim) {
                const uint32_t old = atomicSub(w.a.w + u, 1u);
                if (old == kk + 1) {
                    const uint32_t o2 = atomicOr(w.a.w + u, kClaim);
                    found = !(o2 & kClaim);
                } else if (old <= kk || old >= kClaim) {
                    atomicAdd(w.a.w + u, 1u);   // undo (ours.cc:102-105)
                }
            }
        }
        on_claimed(w, found, u);
    }
    __syncwarp();
}

// Walks the staged items and then, while the cascade list is non-empty, the
// vertices it discovered in the same level.
__device__ void walk_with_cascades(Warp& w) {
    walk_items(w);
    const unsigned lane = lane_id();
    while (w.nnext) {
        const uint32_t n = w.nnext;
        for (uint32_t i = lane; i < n; i += 32) {
            w.b.start[i] = w.b.nstart[i];
            w.b.pref[i] = w.b.nlen[i];
        }
        __syncwarp();
        w.nnext = 0;
        w.nitems = n;
        walk_items(w);
    }
}

// Stages up to 4 claimed vertices per lane (mask bits) as walk items; hubs go
// to the task queue.  Flushes the batch first when it could overflow.
__device__ __forceinline__ void stage_claims(Warp& w, uint32_t vbase, unsigned mine) {
    const unsigned lane = lane_id();
    uint32_t st[4], ln[4];
    unsigned localm = 0, hubm = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        st[j] = 0; ln[j] = 0;
        if (mine & (1u << j)) {
            const uint32_t v = vbase + j;
            st[j] = __ldg(w.a.off + v);
            ln[j] = __ldg(w.a.off + v + 1) - st[j];
            if (ln[j] == 0) continue;
            if (ln[j] <= kLocalArcs) localm |= 1u << j; else hubm |= 1u << j;
        }
    }
    const uint32_t cnt = __popc(localm);
    uint32_t tot;
    const uint32_t ex = warp_excl_scan(cnt, &tot);
    if (tot && w.nitems + tot > kItemCap) walk_with_cascades(w);
    uint32_t pos = w.nitems + ex;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (localm & (1u << j)) { w.b.start[pos] = st[j]; w.b.pref[pos] = ln[j]; ++pos; }
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

// Scan of this warp's vertex groups for level w.level (ours.cc:15-25), with
// the walk of every vertex it claims done inline.
__device__ void scan_level(Warp& w, uint32_t gw) {
    const unsigned lane = lane_id();
    const PeelArgs& a = w.a;
    const uint32_t ngroups = (a.V + 127) / 128;
    uint4* w4 = reinterpret_cast<uint4*>(a.w);
    for (uint32_t g = gw; g < ngroups; g += w.nwt) {
        const uint32_t vbase = g * 128 + lane * 4;
        unsigned mine = 0;
        if (w.level == 0) {
            // Level 0 also initialises the state from the offsets: isolated
            // vertices are peeled here and have nothing to walk.
            uint32_t st[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t v = vbase + j;
                if (v < a.V) {
                    const uint32_t d = __ldg(a.off + v + 1) - __ldg(a.off + v);
                    if (d == 0) { st[j] = kClaim | kBias; mine |= 1u << j; a.core[v] = 0; }
                    else st[j] = d + kBias;
                } else {
                    st[j] = kClaim | kBias;   // padding never matches
                }
            }
            __stcg(w4 + g * 32 + lane, make_uint4(st[0], st[1], st[2], st[3]));
        } else {
            const uint4 x = __ldcg(w4 + g * 32 + lane);
            const uint32_t kk = w.kk;
            unsigned hit = (x.x == kk ? 1u : 0u) | (x.y == kk ? 2u : 0u) | (x.z == kk ? 4u : 0u) |
                           (x.w == kk ? 8u : 0u);
            if (!__ballot_sync(kFull, hit != 0)) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (hit & (1u << j)) {
                    const uint32_t v = vbase + j;
                    const uint32_t o = atomicOr(a.w + v, kClaim);
                    if (!(o & kClaim)) { mine |= 1u << j; a.core[v] = w.level; }
                }
        }
        const uint32_t cnt = __popc(mine);
        uint32_t tot;
        const uint32_t ex = warp_excl_scan(cnt, &tot);
        if (tot == 0) continue;
        w.peeled += tot;
        if (a.order) {
            uint32_t pos = 0;
            if (lane == 0) pos = atomicAdd(&a.ctl->order_tail, tot);
            pos = __shfl_sync(kFull, pos, 0) + ex;
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (mine & (1u << j)) a.order[pos++] = vbase + j;
        }
        if (w.level > 0) stage_claims(w, vbase, mine);
    }
    walk_with_cascades(w);
}

// CTA-wide view of the level state: one warp at a time reads the global
// counters and leaves a hint in shared memory for the others.
__device__ __forceinline__ bool level_over(Warp& w, uint32_t* avail) {
    CtaShared& sh = w.sh;
    const unsigned lane = lane_id();
    unsigned done_v = 0, lvl = 0, av = 0;
    if (lane == 0) {
        if (atomicCAS(&sh.poll_lock, 0u, 1u) == 0u) {
            const unsigned ld = ld_acquire(&w.a.ctl->levels_done);
            const unsigned t = ld_relaxed(&w.slot->tail);
            const unsigned h = ld_relaxed(&w.slot->head);
            *(volatile unsigned*)&sh.hint_done = ld;
            *(volatile unsigned*)&sh.hint_avail = t > h ? t - h : 0u;
            *(volatile unsigned*)&sh.hint_level = w.level;
            __threadfence_block();
            atomicExch(&sh.poll_lock, 0u);
        }
        done_v = *(volatile unsigned*)&sh.hint_done;
        lvl = *(volatile unsigned*)&sh.hint_level;
        av = *(volatile unsigned*)&sh.hint_avail;
    }
    done_v = __shfl_sync(kFull, done_v, 0);
    lvl = __shfl_sync(kFull, lvl, 0);
    av = __shfl_sync(kFull, av, 0);
    *avail = (lvl == w.level) ? av : 0u;
    return done_v > w.level;
}

// Publishes `ndone` finished tasks; the event that completes the level
// announces it.
__device__ __forceinline__ void finish_tasks(Warp& w, uint32_t ndone) {
    if (lane_id() == 0) {
        if (w.peeled) atomicAdd(&w.a.ctl->peeled, w.peeled);
        __threadfence();
        const unsigned nd = atomicAdd(&w.slot->done, ndone) + ndone;
        __threadfence();
        const unsigned ar = ld_acquire(&w.slot->arrivals);
        const unsigned t = ld_acquire(&w.slot->tail);
        if (ar == gridDim.x && t == nd) atomicMax(&w.a.ctl->levels_done, w.level + 1);
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
    uint32_t spins = 0;
    uint32_t sleep_ns = 32;
    for (;;) {
        if (pend == 0) {
            uint32_t avail;
            if (level_over(w, &avail)) return true;
            if (avail) {
                const uint32_t share = avail / max(1u, w.nwt / 2u);
                const uint32_t B = min(32u, max(1u, share));
                uint32_t c = 0;
                if (lane == 0) c = atomicAdd(&w.slot->head, B);
                cbase = __shfl_sync(kFull, c, 0);
                pend = (B == 32) ? kFull : ((1u << B) - 1u);
                spins = 0;
                sleep_ns = 32;
            } else {
                if (ld_err(&a.ctl->err)) return false;
                if (++spins > a.spin_limit) { if (lane == 0) record_error(a.ctl, kErrTimeout, w.level); return false; }
                __nanosleep(sleep_ns);
                sleep_ns = min(sleep_ns * 2, 256u);
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
            spins = 0;
            sleep_ns = 32;
            continue;
        }
        uint32_t avail;
        if (level_over(w, &avail)) return true;   // claimed slots beyond the final tail
        if (ld_err(&a.ctl->err)) return false;
        if (++spins > a.spin_limit) { if (lane == 0) record_error(a.ctl, kErrTimeout, w.level); return false; }
        __nanosleep(sleep_ns);
        sleep_ns = min(sleep_ns * 2, 256u);
    }
}

__global__ void __launch_bounds__(kPeelThreads, 2) peel_persistent_kernel(const __grid_constant__ PeelArgs a) {
    __shared__ CtaShared sh;
    const unsigned lane = lane_id();
    const unsigned wid = threadIdx.x >> 5;
    if (threadIdx.x < 4) { sh.arrive[threadIdx.x] = 0; sh.peeled[threadIdx.x] = 0; }
    if (threadIdx.x == 0) { sh.poll_lock = 0; sh.hint_level = 0xFFFFFFFFu; sh.hint_avail = 0; sh.hint_done = 0; }
    __syncthreads();

    Warp w{a, sh.wb[wid], sh, nullptr, 0ull, 0u, kBias, 0u, 0u, 0u, gridDim.x * kPeelWarps};
    const uint32_t gw = blockIdx.x * kPeelWarps + wid;
    PeelCtl* ctl = a.ctl;
    if (blockIdx.x == 0 && threadIdx.x == 0 && a.shells && a.shell_cap) a.shells[0] = 0;

    for (uint32_t level = 0;; ++level) {
        w.level = level;
        w.kk = level + kBias;
        w.slot = &ctl->slot[level & 3];
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            LevelSlot* r = &ctl->slot[(level + 2) & 3];
            r->tail = 0; r->head = 0; r->done = 0; r->arrivals = 0;
            __threadfence();
        }
        scan_level(w, gw);

        // CTA arrival: the last warp of the CTA publishes its claims and
        // arrives; the arrival that completes the level announces it.
        if (lane == 0) {
            atomicAdd(&sh.peeled[level & 3], w.peeled);
            __threadfence();
            const unsigned x = atomicAdd(&sh.arrive[level & 3], 1u);
            if (x == kPeelWarps - 1) {
                __threadfence();
                const unsigned p = atomicExch(&sh.peeled[level & 3], 0u);
                atomicExch(&sh.arrive[level & 3], 0u);
                if (p) atomicAdd(&ctl->peeled, p);
                __threadfence();
                const unsigned ar = atomicAdd(&w.slot->arrivals, 1u) + 1u;
                if (ar == gridDim.x) {
                    __threadfence();
                    const unsigned d = ld_acquire(&w.slot->done);
                    const unsigned t = ld_acquire(&w.slot->tail);
                    if (d == t) atomicMax(&ctl->levels_done, level + 1);
                }
            }
        }
        w.peeled = 0;
        __syncwarp();

        if (!drain_level(w)) return;

        unsigned t = 0, p = 0;
        if (lane == 0) {
            t = ld_acquire(&w.slot->tail);
            p = ld_acquire(&ctl->peeled);
        }
        t = __shfl_sync(kFull, t, 0);
        p = __shfl_sync(kFull, p, 0);
        w.task_base += t;
        if (blockIdx.x == 0 && threadIdx.x == 0 && a.shells && level + 1 < a.shell_cap) a.shells[level + 1] = p;
        if (p >= a.V) {
            if (blockIdx.x == 0 && threadIdx.x == 0) { ctl->kmax = level; ctl->levels = level + 1; }
            return;
        }
        if (level >= a.max_level) {
            if (lane == 0) record_error(ctl, kErrOverflow, level);
            return;
        }
    }
}

const void* peel_persistent_fn() { return reinterpret_cast<const void*>(&peel_persistent_kernel); }

}  // namespace kc
