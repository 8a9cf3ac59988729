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

struct HxShared {
    unsigned long long bt_stage[kWarps][32];   // per-warp staging of update tasks
    uint32_t rm_stage[kWarps][32];             // per-warp staging of frontier entries
    uint32_t wbin[kWarps][33];                 // per-warp bin counts of one chunk; phase B: task prefix
    uint32_t tstart[kWarps][32];               // phase B: first arc, old and new estimate of 32 tasks
    uint32_t told[kWarps][32];
    uint32_t tnew[kWarps][32];
    uint32_t vals[kWarps][kBatchVals];         // phase A: gathered neighbour estimates of a batch
    int bar_ok;
};

// Grid barrier of the cooperative launch, bounded in time; false when the wait
// ran out or an error was recorded (every CTA then returns).
__device__ bool hx_barrier(const HxArgs& a, HxShared& sh) {
    __syncthreads();
    if (threadIdx.x == 0) {
        PeelCtl* ctl = a.ctl;
        int ok = 1;
        const unsigned gen = ld_acquire(&ctl->bar_gen);
        __threadfence();
        if (atomicAdd(&ctl->bar_count, 1u) == gridDim.x - 1) {
            atomicExch(&ctl->bar_count, 0u);
            __threadfence();
            atomicAdd(&ctl->bar_gen, 1u);
        } else {
            const unsigned long long t0 = now_ns(), lim = (unsigned long long)a.wait_us * 1000ull;
            uint32_t polls = 0;
            while (ld_acquire(&ctl->bar_gen) == gen) {
                if ((++polls & 31u) == 0) {
                    if (ld_err(&ctl->err)) { ok = 0; break; }
                    if (now_ns() - t0 > lim) { record_error(ctl, kErrTimeout, ctl->hx.iters); ok = 0; break; }
                }
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

// One lane opens a window slot for large vertex v (d arcs, estimate e) in the
// frontier of parity q and queues its chunk tasks for sub-phase r+1.  coarse:
// the window covers [0, e] (iteration 1, where estimates fall far); otherwise
// it covers the 32 values at the top, where a drop usually stays.
__device__ void open_slot(const HxArgs& a, uint32_t q, uint32_t r, uint32_t v, uint32_t e, uint32_t d, bool coarse) {
    HxCtl* hx = &a.ctl->hx;
    const uint32_t s = atomicAdd(&hx->rl_n[q], 1u);
    if (s >= a.cap_l) { record_error(a.ctl, kErrOverflow, 0); return; }
    const uint32_t nch = (d + kHxChunk - 1) / kHxChunk;
    HxSlot sl;
    sl.v = v;
    sl.e = e;
    sl.hi = e;
    sl.lo = coarse ? 0u : (e >= 31u ? e - 31u : 0u);
    sl.sh = bin_shift(sl.lo, sl.hi);
    sl.done = 0;
    sl.nch = nch;
    sl.pad = 0;
    a.slots[q][s] = sl;
    uint4* b = reinterpret_cast<uint4*>(a.bins[q] + (size_t)s * kHxBinWords);
#pragma unroll
    for (int i = 0; i < (int)(kHxBinWords / 4); ++i) b[i] = make_uint4(0, 0, 0, 0);
    const uint32_t base = atomicAdd(&hx->cl_n[(r + 1) % 3], nch);
    if (base + nch > a.cap_cl) { record_error(a.ctl, kErrOverflow, 0); return; }
    unsigned long long* cl = a.cl[(r + 1) % 3];
    for (uint32_t c = 0; c < nch; ++c) cl[base + c] = ((unsigned long long)s << 32) | c;
}

// Largest h in [0, e] with at least h of the warp's values >= h (the values
// are x[k] of lane l for arc l + 32k < d), and the count at that h.
__device__ __forceinline__ uint32_t warp_hindex(const uint32_t (&x)[8], uint32_t d, uint32_t e, uint32_t* count) {
    const unsigned lane = lane_id();
    uint32_t lo = 0, hi = e;
    while (lo < hi) {   // warp-uniform
        const uint32_t mid = (lo + hi + 1) >> 1;
        uint32_t c = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) c += (lane + 32u * k < d && x[k] >= mid) ? 1u : 0u;
        c = __reduce_add_sync(kFull, c);
        if (c >= mid) lo = mid; else hi = mid - 1;
    }
    uint32_t c = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) c += (lane + 32u * k < d && x[k] >= lo) ? 1u : 0u;
    *count = __reduce_add_sync(kFull, c);
    return lo;
}

// Phase A for the warp frontier (vertices of at most kHxWarpArcs arcs), 32
// list entries per warp step.  The neighbours' estimates of as many whole
// vertices as fit kBatchVals values are gathered into shared memory with all
// loads in flight (the dependent load chain is paid once per batch, not once
// per vertex); then the warp finds each vertex's h-index from shared memory.
__device__ void warp_batch(const HxArgs& a, HxShared& sh, Stager& st, uint32_t p, const uint32_t* list, uint32_t n,
                           uint32_t wr, uint32_t nw) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    uint32_t* vals = sh.vals[wid];
    uint32_t* pref = sh.wbin[wid];   // 33 words: exclusive prefix of the degrees + total
    uint32_t* vs = sh.tstart[wid];
    uint32_t* es = sh.told[wid];
    uint32_t* ss = sh.tnew[wid];
    // entries per warp step: enough for every warp to get a share, at most 32
    const uint32_t B = min(32u, max(1u, (n + nw - 1) / nw));
    for (uint32_t i0 = wr * B; i0 < n; i0 += nw * B) {
        const uint32_t i = i0 + lane;
        uint32_t v = kFull, s0 = 0, d = 0, e = 0;
        if (lane < B && i < n) {
            v = __ldcg(list + i);
            if (v < a.V) {
                s0 = KC_LDG(a.off + v);
                d = min(KC_LDG(a.off + v + 1) - s0, kHxWarpArcs);
                e = __ldcg(a.est + v);
            } else {
                v = kFull;
            }
        }
        uint32_t total;
        const uint32_t ex = warp_excl_scan(d, &total);
        __syncwarp();
        vs[lane] = v;
        es[lane] = e;
        ss[lane] = s0;
        pref[lane] = ex;
        if (lane == 0) pref[32] = total;
        __syncwarp();
        uint32_t k0 = 0;
        while (k0 < 32) {   // warp-uniform
            // the batch: vertices k0..k1-1, the most whose arcs fit kBatchVals
            // (at least one: a degree is at most kHxWarpArcs <= kBatchVals)
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
                        u[j] = KC_LDG(a.nbr + ss[lo] + (qa - pref[lo]));
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t qi = q0 + 32u * j + lane;
                    if (qi < nv) vals[qi] = u[j] < a.V ? __ldcg(a.est + u[j]) : 0u;
                }
            }
            __syncwarp();
            for (uint32_t k = k0; k < k1; ++k) {   // warp-uniform
                const uint32_t vk = vs[k];
                const uint32_t dk = pref[k + 1] - pref[k];
                if (vk == kFull) continue;
                const uint32_t ek = es[k], ok = pref[k] - base;
                uint32_t x[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const uint32_t idx = lane + 32u * j;
                    x[j] = idx < dk ? vals[ok + idx] : 0u;
                }
                uint32_t c;
                const uint32_t h = warp_hindex(x, dk, ek, &c);
                if (lane == 0) {
                    a.cnt[vk] = c;
                    if (h < ek) {
                        a.old[vk] = ek;
                        a.est[vk] = h;
                    }
                }
                stage_bt(a, sh, st, p, h < ek ? 1u : 0u, (unsigned long long)vk << 32);
            }
            __syncwarp();
            k0 = k1;
        }
    }
}

// The warp that finished the last chunk of slot `s` reads the pass's bins.
__device__ void resolve_slot(const HxArgs& a, HxShared& sh, Stager& st, uint32_t p, uint32_t r, uint32_t s) {
    const unsigned lane = lane_id();
    HxSlot* sl = a.slots[p] + s;
    uint32_t* bins = a.bins[p] + (size_t)s * kHxBinWords;
    const uint32_t v = __ldcg(&sl->v), e = __ldcg(&sl->e), lo = __ldcg(&sl->lo), hi = __ldcg(&sl->hi);
    const uint32_t shft = __ldcg(&sl->sh), nch = __ldcg(&sl->nch);
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
    uint32_t nlo, nhi;
    if (ok) {
        const uint32_t bs = 31 - __clz(ok);
        const uint32_t Sb = __shfl_sync(kFull, S, bs);
        const uint32_t sb = lo + (bs << shft);
        if (shft == 0) {   // found: h = sb, counted Sb
            if (lane == 0) {
                a.cnt[v] = Sb;
                if (sb < e) {
                    a.old[v] = e;
                    a.est[v] = sb;
                }
            }
            if (sb < e) {
                // update tasks for every chunk of v
                HxCtl* hx = &a.ctl->hx;
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(&hx->bt_n[p], nch);
                base = __shfl_sync(kFull, base, 0);
                for (uint32_t c = lane; c < nch; c += 32) {
                    if (base + c < a.cap_bt) a.bt[p][base + c] = ((unsigned long long)v << 32) | c;
                    else record_error(a.ctl, kErrOverflow, 0);
                }
            }
            return;
        }
        nlo = sb;
        nhi = min(sb + (1u << shft) - 1u, hi);
    } else {   // h < lo (lo > 0 here: at lo = 0 bin 0 always qualifies)
        nlo = 0;
        nhi = lo - 1;
    }
    if (lane == 0) {
        sl->lo = nlo;
        sl->hi = nhi;
        sl->sh = bin_shift(nlo, nhi);
        sl->done = 0;
        atomicAdd(&a.ctl->hx.passes, 1u);
    }
    HxCtl* hx = &a.ctl->hx;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&hx->cl_n[(r + 1) % 3], nch);
    base = __shfl_sync(kFull, base, 0);
    if (base + nch > a.cap_cl) {
        if (lane == 0) record_error(a.ctl, kErrOverflow, 0);
        return;
    }
    for (uint32_t c = lane; c < nch; c += 32) a.cl[(r + 1) % 3][base + c] = ((unsigned long long)s << 32) | c;
}

// Phase A for one chunk task of a large vertex: bin its neighbours' estimates.
__device__ void chunk_task(const HxArgs& a, HxShared& sh, Stager& st, uint32_t p, uint32_t r,
                           unsigned long long task, bool degrees) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    const uint32_t s = (uint32_t)(task >> 32), c = (uint32_t)task;
    if (s >= a.cap_l) return;
    HxSlot* sl = a.slots[p] + s;
    const uint32_t v = __ldcg(&sl->v), lo = __ldcg(&sl->lo), hi = __ldcg(&sl->hi), shft = __ldcg(&sl->sh);
    const uint32_t nch = __ldcg(&sl->nch);
    if (v >= a.V) return;
    const uint32_t s0 = KC_LDG(a.off + v);
    const uint32_t d = KC_LDG(a.off + v + 1) - s0;
    const uint32_t b0 = c * kHxChunk;
    const uint32_t len = b0 < d ? min(kHxChunk, d - b0) : 0u;
    uint32_t bin[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint32_t i = lane + 32u * k;
        bin[k] = kNoBin;
        if (i < len) {
            const uint32_t u = KC_LDG(a.nbr + s0 + b0 + i);
            uint32_t x = 0;
            if (u < a.V) x = degrees ? KC_LDG(a.off + u + 1) - KC_LDG(a.off + u) : __ldcg(a.est + u);
            bin[k] = x > hi ? 32u : (x >= lo ? (x - lo) >> shft : kNoBin);
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
                             uint32_t wr, uint32_t nw) {
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
        if (lane < T && i64 < nbt) {
            const unsigned long long tk = __ldcg(a.bt[p] + i);
            const uint32_t u = (uint32_t)(tk >> 32), c = (uint32_t)tk;
            if (u < a.V) {
                const uint32_t s0 = KC_LDG(a.off + u);
                const uint32_t d = KC_LDG(a.off + u + 1) - s0;
                const uint32_t b0 = c * kHxChunk;
                len = b0 < d ? min(kHxChunk, d - b0) : 0u;
                s1 = s0 + b0;
                ol = __ldcg(a.old + u);
                nw_ = __ldcg(a.est + u);
            }
        }
        uint32_t total;
        const uint32_t ex = warp_excl_scan(len, &total);
        pref[lane] = ex;
        if (lane == 0) pref[32] = total;
        tstart[lane] = s1;
        told[lane] = ol;
        tnew[lane] = nw_;
        __syncwarp();
        uint32_t lo = 0;
        for (uint32_t q0 = 0; q0 < total; q0 += 128) {
            uint32_t wv[4], xv[4], kk[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t qi = q0 + 32u * j + lane;
                wv[j] = kFull;
                xv[j] = 0;
                kk[j] = 0;
                if (qi < total) {
                    uint32_t hi = 32;
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (pref[mid] <= qi) lo = mid; else hi = mid;
                    }
                    kk[j] = lo;
                    const uint32_t w = KC_LDG(a.nbr + tstart[lo] + (qi - pref[lo]));
                    if (w < a.V) {
                        wv[j] = w;
                        xv[j] = __ldcg(a.est + w);
                    }
                }
            }
            unsigned push_m = 0;
            uint32_t push_v = kFull;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                bool queue = false;
                if (wv[j] != kFull) {
                    const uint32_t x = xv[j];
                    if (tnew[kk[j]] < x && x <= told[kk[j]]) {
                        const uint32_t y = atomicSub(a.cnt + wv[j], 1u);
                        queue = (y == x);
                    }
                }
                // queue: small and mid-size vertices to the warp list, large ones to a slot
                uint32_t dq = 0;
                if (queue) dq = KC_LDG(a.off + wv[j] + 1) - KC_LDG(a.off + wv[j]);
                if (queue && dq > kHxWarpArcs) {
                    open_slot(a, q, r, wv[j], xv[j], dq, false);
                    queue = false;
                }
                push_m = __ballot_sync(kFull, queue);
                push_v = wv[j];
                stage_rm(a, sh, st, q, push_m, push_v);
            }
        }
        __syncwarp();
    }
    flush_rm(a, sh, st, q);
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
    Stager st;

    // Sub-phase 0: est = degree.
    for (uint32_t v = gw * 32 + lane; v < a.V; v += nw * 32) a.est[v] = KC_LDG(a.off + v + 1) - KC_LDG(a.off + v);
    if (!hx_barrier(a, sh)) return;

    // Iteration 1, first sweep (sub-phase 1): a lane per vertex of at most
    // kHxLaneArcs arcs; larger vertices are queued for phase A (parity 1).
    uint32_t r = 1;
    {
        for (uint32_t base = gw * 32; base < a.V; base += nw * 32) {
            const uint32_t v = base + lane;
            uint32_t s0 = 0, d = 0;
            if (v < a.V) {
                s0 = KC_LDG(a.off + v);
                d = KC_LDG(a.off + v + 1) - s0;
            }
            const bool small = v < a.V && d <= kHxLaneArcs;
            bool drop = false;
            if (small) {
                uint32_t x[kHxLaneArcs];
#pragma unroll
                for (uint32_t i = 0; i < kHxLaneArcs; ++i) {
                    x[i] = 0;
                    if (i < d) {
                        const uint32_t u = KC_LDG(a.nbr + s0 + i);
                        x[i] = u < a.V ? __ldcg(a.est + u) : 0u;
                    }
                }
                uint32_t lo = 0, hi = d;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    uint32_t c = 0;
#pragma unroll
                    for (uint32_t i = 0; i < kHxLaneArcs; ++i) c += (i < d && x[i] >= mid) ? 1u : 0u;
                    if (c >= mid) lo = mid; else hi = mid - 1;
                }
                uint32_t c = 0;
#pragma unroll
                for (uint32_t i = 0; i < kHxLaneArcs; ++i) c += (i < d && x[i] >= lo) ? 1u : 0u;
                a.cnt[v] = c;
                if (lo < d) {
                    a.old[v] = d;
                    a.est[v] = lo;
                    drop = true;
                }
            }
            stage_bt(a, sh, st, 1, __ballot_sync(kFull, drop), (unsigned long long)v << 32);
            const bool mid = v < a.V && d > kHxLaneArcs && d <= kHxWarpArcs;
            stage_rm(a, sh, st, 1, __ballot_sync(kFull, mid), v);
            if (v < a.V && d > kHxWarpArcs) open_slot(a, 1, 0, v, d, d, true);
        }
        flush_bt(a, sh, st, 1);
        flush_rm(a, sh, st, 1);
    }
    if (!hx_barrier(a, sh)) return;
    // (the first sweep queued chunk tasks into list (0 + 1) % 3 = 1, consumed at r = 1)

    uint32_t t = 1;
    for (;;) {
        const uint32_t p = t & 1u;
        // ---- phase A: window passes; the first also takes the warp frontier
        bool first = true;
        for (;;) {
            const uint32_t ncl = min(ld_relaxed(&hx->cl_n[r % 3]), a.cap_cl);
            const uint32_t nrm = first ? min(ld_relaxed(&hx->rm_n[p]), a.V) : 0u;
            if (ncl == 0 && nrm == 0) break;   // every CTA reads the same counts
            if (lead) hx->cl_n[(r + 2) % 3] = 0;
            if (nrm) warp_batch(a, sh, st, p, a.rm[p], nrm, wr, nw);
            for (uint32_t i = wr; i < ncl; i += nw) chunk_task(a, sh, st, p, r, __ldcg(a.cl[r % 3] + i), t == 1);
            flush_bt(a, sh, st, p);
            if (!hx_barrier(a, sh)) return;
            ++r;
            first = false;
        }
        // ---- phase B (sub-phase r)
        if (lead) {
            hx->cl_n[(r + 2) % 3] = 0;
            hx->bt_n[p ^ 1u] = 0;
            hx->rm_n[p] = 0;
            hx->rl_n[p] = 0;
        }
        const uint32_t nbt = min(ld_relaxed(&hx->bt_n[p]), a.cap_bt);
        update_tasks(a, sh, st, p, r, nbt, wr, nw);
        if (!hx_barrier(a, sh)) return;
        ++r;
        const uint32_t nm = ld_relaxed(&hx->rm_n[p ^ 1u]), nl = ld_relaxed(&hx->rl_n[p ^ 1u]);
        if (nm == 0 && nl == 0) break;
        ++t;
        if (t > a.max_iters) {   // the level peel takes over
            if (lead) hx->iters = t;
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
        ctl->iterations = t;
        hx->solved = 1;
    }
}

}  // namespace

const void* peel_hindex_fn() { return reinterpret_cast<const void*>(&peel_hindex_kernel); }

}  // namespace kc
