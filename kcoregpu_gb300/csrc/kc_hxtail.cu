// h-index tail of the single-graph peel for sm_103a: one cluster of kCl CTAs
// finishes the peel on the induced subgraph of the survivors that the
// persistent kernel built when it stopped (kc_peel_impl.cuh tail_handoff),
// by the h-index fixed point instead of level by level.
//
// The survivors of level L-1 all have core numbers >= L (each has more than
// L-1 surviving neighbours), and among them the core numbers equal those of
// the induced subgraph.  Starting from the induced degrees, each vertex's
// estimate is replaced by the largest h in [L, estimate] with at least h
// neighbours whose estimate is >= h; the fixed point is the core numbers
// (see kc_hindex.cu for the rule, the counts and the proof).  On the
// benchmark graphs the dense core that the one-CTA level tail (kc_tail.cu)
// peels in 50-148 levels and up to 637 dependent rounds converges in 34-60
// iterations here.
//
// GB300 shape: one 16-CTA cluster.  Every CTA keeps a copy of all estimates
// in its shared memory (up to kHoV = 24,576 vertices: 96 KB), so a
// neighbour's estimate is a local load and a drop is broadcast by 16 DSMEM
// stores; counts and frontier bitmaps live with their owner (local id v in
// CTA v % kCl, slot v / kCl), so a decrement is a DSMEM atomic; the two
// barriers of an iteration are hardware cluster barriers.  The induced
// adjacency (16-byte quads, pads 0xFFFFFFFF) is read from L2.  Per iteration:
//   phase A: each CTA recomputes its frontier vertices: up to kWVals arcs a
//            warp (vertices batched so that their gathers overlap), larger
//            ones the whole CTA, from values gathered into shared memory;
//   phase B: each vertex that dropped scans its adjacency and decrements the
//            counts its drop crossed; the decrement that takes a count below
//            its estimate queues that vertex.
// After max iterations without convergence the kernel leaves the survivors
// to the level tail kernel, launched after it, which returns at once when
// this kernel set HxCtl::tail_solved.
//
// The same kernel finishes the h-index peel (kc_hindex.cu try_handoff): there
// S is the set of vertices whose estimates are at or above a floor T that the
// h-index peel certified (every member has at least T neighbours in S), the
// induced CSR is built by that kernel, and the iteration continues from its
// estimates, counts and queued vertices.  After max iterations without
// convergence the level peel runs from the start instead.
#include <cooperative_groups.h>

#include "kc_device.cuh"
#include "kc_peel.cuh"

namespace cg = cooperative_groups;

namespace kc {
namespace {

constexpr int kCl = 16;                     // CTAs of the cluster (non-portable size)
constexpr int kClThreads = 512;
constexpr int kClWarps = kClThreads / 32;
constexpr uint32_t kPer = kHoV / kCl;       // vertices a CTA owns
constexpr uint32_t kWVals = 1024;           // values a warp gathers
constexpr uint32_t kCVals = kClWarps * kWVals;   // values the CTA gathers

struct ClSmem {
    uint32_t eall[kHoV];            // every vertex's estimate (a copy in each CTA)
    uint32_t cnt[kPer];
    uint32_t old[kPer];
    uint32_t sdeg[kPer];            // induced degree and first quad of each slot (read once from L2)
    uint32_t sfq[kPer];
    uint32_t front[2][kPer / 32];   // frontier bitmaps by iteration parity
    uint32_t work[kPer];            // phase A: slots of up to kWVals arcs; phase B: slots that dropped
    uint32_t big[kPer];             // slots the whole CTA handles
    uint32_t nwork, nbig, nchg;
    uint32_t chg[kPer];             // slots that dropped in this iteration
    uint32_t flag[3];               // (CTA 0) a vertex was queued in iteration t (index t % 3)
    uint32_t red[kClWarps];
    uint32_t kmax;
    uint32_t wpref[kClWarps][33];   // per-warp batch: prefix of the degrees
    uint32_t wqpref[kClWarps][33];  // and of the quads
    uint32_t wfq[kClWarps][32];     // their first quads
    uint32_t wnew[kClWarps][32];    // phase B: new and old estimates
    uint32_t wold[kClWarps][32];
    uint32_t wslot[kClWarps][32];   // its slots
    uint32_t bq[kPer + 1];          // big slots: prefix of their quads
    uint32_t bv[kPer + 1];          // and of their degrees
    uint32_t vals[kCVals];          // gathered estimates (per warp: kWVals each)
};

__device__ __forceinline__ uint32_t cl_sum(uint32_t x, ClSmem& sm) {
    const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
    x = __reduce_add_sync(kFull, x);
    __syncthreads();
    if (lane == 0) sm.red[wid] = x;
    __syncthreads();
    return __reduce_add_sync(kFull, lane < kClWarps ? sm.red[lane] : 0u);
}

// Largest h in [fl, e] with ge(h) >= h (ge non-increasing); fl when none is
// (cannot happen: every value read is at least fl, and so is the degree).
template <class Ge>
__device__ __forceinline__ uint32_t tail_gallop(Ge ge, uint32_t fl, uint32_t e) {
    uint32_t bad = e + 1, t = 1, lo = fl;
    for (;;) {
        const uint32_t cand = e - fl >= t - 1 ? e - (t - 1) : fl;
        if (ge(cand) >= cand) { lo = cand; break; }
        bad = cand;
        if (cand == fl) return fl;
        t <<= 1;
    }
    uint32_t hi = bad - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (ge(mid) >= mid) lo = mid; else hi = mid - 1;
    }
    return lo;
}

struct Tail {
    const PeelArgs& a;
    ClSmem& sm;
    cg::cluster_group& cl;
    uint32_t n, L, rank, nquads;
    const uint4* nbr4;

    __device__ uint32_t est_of(uint32_t w) const { return sm.eall[w]; }
    __device__ uint32_t vertex(uint32_t s) const { return rank + kCl * s; }
    __device__ uint32_t first_quad(uint32_t v) const { return __ldg(a.tail_off + v) >> 2; }
    __device__ uint32_t degree(uint32_t v) const { return __ldg(a.tail_cur + v) - __ldg(a.tail_off + v); }
    __device__ uint4 quad(uint32_t q) const {
        return q < nquads ? __ldg(nbr4 + q) : make_uint4(kFull, kFull, kFull, kFull);
    }

    // Estimates of the arcs [0, d) of the adjacency starting at quad q0 into
    // out[], for the quads t0, t0 + stride, ... of it: four quads (16 values)
    // in flight per thread.
    __device__ void gather(uint32_t q0, uint32_t d, uint32_t* out, uint32_t t0, uint32_t stride) const {
        const uint32_t nq = (d + 3) / 4;
        for (uint32_t qb = t0; qb < nq; qb += 4 * stride) {
            uint4 x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t qq = qb + u * stride;
                x[u] = qq < nq ? quad(q0 + qq) : make_uint4(kFull, kFull, kFull, kFull);
            }
            uint32_t val[16];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t ids[4] = {x[u].x, x[u].y, x[u].z, x[u].w};
#pragma unroll
                for (int j = 0; j < 4; ++j) val[4 * u + j] = ids[j] < n ? est_of(ids[j]) : 0u;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t idx = 4 * (qb + u * stride) + j;
                    if (qb + u * stride < nq && idx < d) out[idx] = val[4 * u + j];
                }
            }
        }
    }

    // Flattened over a warp's batch of k1 <= 32 vertices (qpref: exclusive
    // prefix of their quad counts, qpref[32] = total; fq: first quad; pref:
    // exclusive prefix of their degrees): lane takes quads lane, lane + 32, ...
    // of the concatenation, four in flight, and stores the estimates of the
    // real arcs at out[pref[k] + arc].
    __device__ void gather_batch(const uint32_t* qpref, const uint32_t* fq, const uint32_t* pref, uint32_t k1,
                                 uint32_t* out) const {
        const unsigned lane = lane_id();
        const uint32_t qt = qpref[k1];
        uint32_t lo = 0;
        for (uint32_t qb = lane; qb < qt; qb += 128) {
            uint4 x[4];
            uint32_t kk[4], qi[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t qf = qb + 32u * u;
                kk[u] = 0;
                qi[u] = 0;
                x[u] = make_uint4(kFull, kFull, kFull, kFull);
                if (qf < qt) {
                    uint32_t hi = k1;
                    while (hi - lo > 1) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (qpref[mid] <= qf) lo = mid; else hi = mid;
                    }
                    kk[u] = lo;
                    qi[u] = qf - qpref[lo];
                    x[u] = quad(fq[lo] + qi[u]);
                }
            }
            uint32_t val[16];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t ids[4] = {x[u].x, x[u].y, x[u].z, x[u].w};
#pragma unroll
                for (int j = 0; j < 4; ++j) val[4 * u + j] = ids[j] < n ? est_of(ids[j]) : 0u;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (qb + 32u * u >= qt) continue;
                const uint32_t dk = pref[kk[u] + 1] - pref[kk[u]];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t idx = 4 * qi[u] + j;
                    if (idx < dk) out[pref[kk[u]] + idx] = val[4 * u + j];
                }
            }
        }
    }

    // Records a recomputed slot: count, and on a drop the old value and the new
    // estimate in every CTA's copy (plain stores; the cluster barrier that ends
    // the phase makes them visible).
    __device__ void result(uint32_t s, uint32_t e, uint32_t h, uint32_t c) {
        sm.cnt[s] = c;
        if (h < e) {
            sm.old[s] = e;
            const uint32_t v = vertex(s);
#pragma unroll
            for (int r = 0; r < kCl; ++r) *cl.map_shared_rank(&sm.eall[v], r) = h;
            const uint32_t k = atomicAdd(&sm.nchg, 1u);
            if (k < kPer) sm.chg[k] = s;
        }
    }

    // Phase A, warp path: batches of consecutive work slots whose arcs fit
    // kWVals; their neighbours' estimates are gathered together, then the
    // warp finds each h-index from shared memory.
    __device__ void recompute_warps() {
        const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
        uint32_t* vals = sm.vals + wid * kWVals;
        uint32_t* pref = sm.wpref[wid];
        uint32_t* wsl = sm.wslot[wid];
        const uint32_t nw = sm.nwork;
        const uint32_t per = (nw + kClWarps - 1) / kClWarps;   // consecutive slots per warp
        const uint32_t i0 = wid * per, i1 = min(nw, i0 + per);
        for (uint32_t b = i0; b < i1;) {   // warp-uniform
            const uint32_t i = b + lane;
            uint32_t s = kFull, d = 0;
            if (i < i1) {
                s = sm.work[i];
                d = sm.sdeg[s];
            }
            uint32_t tot;
            const uint32_t ex = warp_excl_scan(d, &tot);
            // the batch: the most leading slots whose arcs fit kWVals (at least one)
            const unsigned fit = __ballot_sync(kFull, i < i1 && ex + d <= kWVals);
            const uint32_t k1 = max(1u, (uint32_t)__popc(fit));
            pref[lane] = ex;
            wsl[lane] = s;
            if (lane == 0) pref[32] = tot;
            __syncwarp();
            // gather, flattened over the batch's quads
            uint32_t* qpref = sm.wqpref[wid];
            uint32_t* fq = sm.wfq[wid];
            uint32_t qtot;
            const uint32_t qex = warp_excl_scan(lane < k1 ? (d + 3) / 4 : 0u, &qtot);
            qpref[lane] = qex;
            if (lane == 0) qpref[32] = qtot;
            fq[lane] = lane < k1 ? sm.sfq[s] : 0u;
            __syncwarp();
            gather_batch(qpref, fq, pref, k1, vals);
            __syncwarp();
            for (uint32_t k = 0; k < k1; ++k) {
                const uint32_t sk = wsl[k], dk = pref[k + 1] - pref[k];
                const uint32_t* xs = vals + pref[k];
                const uint32_t e = sm.eall[vertex(sk)];
                auto ge = [&](uint32_t h) {
                    uint32_t c = 0;
                    for (uint32_t j = lane; j < dk; j += 32) c += xs[j] >= h ? 1u : 0u;
                    return __reduce_add_sync(kFull, c);
                };
                const uint32_t h = tail_gallop(ge, L, e);
                const uint32_t c = ge(h);
                if (lane == 0) result(sk, e, h, c);
            }
            __syncwarp();
            b += k1;
        }
    }

    // The big slots of this phase as a concatenation: bq[i] = exclusive prefix
    // of their quad counts (bq[nbig] = total), bv[i] = prefix of their degrees.
    __device__ void big_prefix() {
        if (threadIdx.x == 0) {
            uint32_t q = 0, v = 0;
            for (uint32_t i = 0; i < sm.nbig; ++i) {
                const uint32_t d = sm.sdeg[sm.big[i]];
                sm.bq[i] = q;
                sm.bv[i] = v;
                q += (d + 3) / 4;
                v += d;
            }
            sm.bq[sm.nbig] = q;
            sm.bv[sm.nbig] = v;
        }
        __syncthreads();
    }

    // Owner of flattened quad qf among the big slots [0, nb).
    __device__ __forceinline__ uint32_t big_owner(uint32_t qf, uint32_t nb, uint32_t& lo) const {
        uint32_t hi = nb;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (sm.bq[mid] <= qf) lo = mid; else hi = mid;
        }
        return lo;
    }

    // Phase A for the big slots: their estimates gathered together (all
    // threads, four quads in flight each) while they fit kCVals values, then
    // the h-indexes, a warp each when the batch holds four or more slots,
    // else one after the other with CTA reductions; a slot above kCVals arcs
    // alone.
    __device__ void recompute_big() {
        big_prefix();
        const unsigned tid = threadIdx.x;
        uint32_t i0 = 0;
        while (i0 < sm.nbig) {   // CTA-uniform
            uint32_t i1 = i0 + 1;
            while (i1 < sm.nbig && sm.bv[i1 + 1] - sm.bv[i0] <= kCVals) ++i1;
            if (sm.bv[i0 + 1] - sm.bv[i0] > kCVals) {
                recompute_cta(sm.big[i0]);
                i0 = i1;
                continue;
            }
            const uint32_t q0 = sm.bq[i0], qt = sm.bq[i1] - q0, v0 = sm.bv[i0];
            uint32_t lo = i0;
            for (uint32_t qb = tid; qb < qt; qb += 4 * kClThreads) {
                uint4 x[4];
                uint32_t kk[4], qi[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t qf = qb + u * kClThreads;
                    kk[u] = i0;
                    qi[u] = 0;
                    x[u] = make_uint4(kFull, kFull, kFull, kFull);
                    if (qf < qt) {
                        kk[u] = big_owner(qf + q0, i1, lo);
                        qi[u] = qf + q0 - sm.bq[kk[u]];
                        x[u] = quad(sm.sfq[sm.big[kk[u]]] + qi[u]);
                    }
                }
                uint32_t val[16];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t ids[4] = {x[u].x, x[u].y, x[u].z, x[u].w};
#pragma unroll
                    for (int j = 0; j < 4; ++j) val[4 * u + j] = ids[j] < n ? est_of(ids[j]) : 0u;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (qb + u * kClThreads >= qt) continue;
                    const uint32_t dk = sm.bv[kk[u] + 1] - sm.bv[kk[u]];
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const uint32_t idx = 4 * qi[u] + j;
                        if (idx < dk) sm.vals[sm.bv[kk[u]] - v0 + idx] = val[4 * u + j];
                    }
                }
            }
            __syncthreads();
            if (i1 - i0 >= 4) {   // several slots: a warp each
                const unsigned lane = lane_id(), wid = tid >> 5;
                for (uint32_t i = i0 + wid; i < i1; i += kClWarps) {   // warp-uniform
                    const uint32_t sl = sm.big[i], d = sm.bv[i + 1] - sm.bv[i];
                    const uint32_t* xs = sm.vals + (sm.bv[i] - v0);
                    const uint32_t e = sm.eall[vertex(sl)];
                    auto ge = [&](uint32_t h) {
                        uint32_t c = 0;
                        for (uint32_t j = lane; j < d; j += 32) c += xs[j] >= h ? 1u : 0u;
                        return __reduce_add_sync(kFull, c);
                    };
                    const uint32_t h = tail_gallop(ge, L, e);
                    const uint32_t c = ge(h);
                    if (lane == 0) result(sl, e, h, c);
                }
            } else {
                for (uint32_t i = i0; i < i1; ++i) {
                    const uint32_t sl = sm.big[i], off = sm.bv[i] - v0, d = sm.bv[i + 1] - sm.bv[i];
                    const uint32_t e = sm.eall[vertex(sl)];
                    auto ge = [&](uint32_t h) {
                        uint32_t c = 0;
                        for (uint32_t j = tid; j < d; j += kClThreads) c += sm.vals[off + j] >= h ? 1u : 0u;
                        return cl_sum(c, sm);
                    };
                    const uint32_t h = tail_gallop(ge, L, e);
                    const uint32_t c = ge(h);
                    if (tid == 0) result(sl, e, h, c);
                }
            }
            __syncthreads();
            i0 = i1;
        }
    }

    // Phase B for the big slots: their quads flattened over all threads.
    __device__ void update_big(uint32_t p, uint32_t t) {
        big_prefix();
        const unsigned tid = threadIdx.x;
        const uint32_t nb = sm.nbig, qt = sm.bq[nb];
        uint32_t lo = 0;
        for (uint32_t qb = tid; qb < qt; qb += 4 * kClThreads) {
            uint4 x[4];
            uint32_t kk[4], qi[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t qf = qb + u * kClThreads;
                kk[u] = 0;
                qi[u] = 0;
                x[u] = make_uint4(kFull, kFull, kFull, kFull);
                if (qf < qt) {
                    kk[u] = big_owner(qf, nb, lo);
                    qi[u] = qf - sm.bq[kk[u]];
                    x[u] = quad(sm.sfq[sm.big[kk[u]]] + qi[u]);
                }
            }
            uint32_t id[16], xs[16];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t ids[4] = {x[u].x, x[u].y, x[u].z, x[u].w};
                const uint32_t dk = sm.bv[kk[u] + 1] - sm.bv[kk[u]];
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    id[4 * u + j] = (qb + u * kClThreads < qt && 4 * qi[u] + j < dk) ? ids[j] : kFull;
            }
#pragma unroll
            for (int k = 0; k < 16; ++k) xs[k] = id[k] < n ? est_of(id[k]) : 0u;
            uint32_t y[16];
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                y[k] = kFull;
                const uint32_t sl = sm.big[kk[k >> 2]];
                if (id[k] < n && sm.eall[vertex(sl)] < xs[k] && xs[k] <= sm.old[sl])
                    y[k] = atomicSub(cl.map_shared_rank(&sm.cnt[id[k] / kCl], id[k] % kCl), 1u);
            }
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                if (y[k] != kFull && y[k] == xs[k]) {
                    const uint32_t sw = id[k] / kCl, ow = id[k] % kCl;
                    atomicOr(cl.map_shared_rank(&sm.front[p ^ 1u][sw >> 5], ow), 1u << (sw & 31));
                    *reinterpret_cast<volatile uint32_t*>(cl.map_shared_rank(&sm.flag[t % 3], 0)) = 1u;
                }
            }
        }
    }

    // Phase A, CTA path: one slot of more than kWVals arcs, read whole.
    __device__ void recompute_cta(uint32_t s) {
        const unsigned tid = threadIdx.x;
        const uint32_t q0 = sm.sfq[s], d = sm.sdeg[s];
        const uint32_t e = sm.eall[vertex(s)];
        const uint32_t m = min(d, kCVals);
        gather(q0, m, sm.vals, tid, kClThreads);
        __syncthreads();
        // (a degree above kCVals, possible only with repeated arcs, re-reads
        // the rest of the adjacency at every probe)
        auto ge = [&](uint32_t h) {
            uint32_t c = 0;
            for (uint32_t j = tid; j < m; j += kClThreads) c += sm.vals[j] >= h ? 1u : 0u;
            for (uint32_t q = (m >> 2) + tid; q * 4 < d; q += kClThreads) {
                const uint4 x = quad(q0 + q);
                const uint32_t ids[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (4 * q + j < d && 4 * q + j >= m && ids[j] < n && est_of(ids[j]) >= h) ++c;
            }
            return cl_sum(c, sm);
        };
        const uint32_t h = tail_gallop(ge, L, e);
        const uint32_t c = ge(h);
        if (tid == 0) result(s, e, h, c);
        __syncthreads();
    }

    // Phase B, warp path: up to 32 dropped slots per warp step, their quads
    // flattened (four in flight per lane).
    __device__ void update_warps(uint32_t p, uint32_t t) {
        const unsigned lane = lane_id(), wid = threadIdx.x >> 5;
        uint32_t* qpref = sm.wqpref[wid];
        uint32_t* fq = sm.wfq[wid];
        uint32_t* dd = sm.wpref[wid];
        uint32_t* wn = sm.wnew[wid];
        uint32_t* wo = sm.wold[wid];
        const uint32_t nwk = sm.nwork;
        const uint32_t per = (nwk + kClWarps - 1) / kClWarps;
        const uint32_t i0 = wid * per, i1 = min(nwk, i0 + per);
        for (uint32_t b = i0; b < i1; b += 32) {   // warp-uniform
            const uint32_t i = b + lane;
            uint32_t nq = 0;
            if (i < i1) {
                const uint32_t s = sm.work[i], v = vertex(s);
                const uint32_t d = sm.sdeg[s];
                nq = (d + 3) / 4;
                fq[lane] = sm.sfq[s];
                dd[lane] = d;
                wn[lane] = sm.eall[v];
                wo[lane] = sm.old[s];
            }
            uint32_t qt;
            const uint32_t qex = warp_excl_scan(nq, &qt);
            qpref[lane] = qex;
            if (lane == 0) qpref[32] = qt;
            const uint32_t k1 = min(32u, i1 - b);
            __syncwarp();
            uint32_t lo = 0;
            for (uint32_t qb = lane; qb < qt; qb += 128) {
                uint4 x[4];
                uint32_t kk[4], qi[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t qf = qb + 32u * u;
                    kk[u] = 0;
                    qi[u] = 0;
                    x[u] = make_uint4(kFull, kFull, kFull, kFull);
                    if (qf < qt) {
                        uint32_t hi = k1;
                        while (hi - lo > 1) {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (qpref[mid] <= qf) lo = mid; else hi = mid;
                        }
                        kk[u] = lo;
                        qi[u] = qf - qpref[lo];
                        x[u] = quad(fq[lo] + qi[u]);
                    }
                }
                uint32_t id[16], xs[16];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t ids[4] = {x[u].x, x[u].y, x[u].z, x[u].w};
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const bool real = qb + 32u * u < qt && 4 * qi[u] + j < dd[kk[u]];
                        id[4 * u + j] = real ? ids[j] : kFull;
                    }
                }
#pragma unroll
                for (int k = 0; k < 16; ++k) xs[k] = id[k] < n ? est_of(id[k]) : 0u;
                uint32_t y[16];
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    y[k] = kFull;
                    const uint32_t nw = wn[kk[k >> 2]], ol = wo[kk[k >> 2]];
                    if (id[k] < n && nw < xs[k] && xs[k] <= ol)
                        y[k] = atomicSub(cl.map_shared_rank(&sm.cnt[id[k] / kCl], id[k] % kCl), 1u);
                }
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    if (y[k] != kFull && y[k] == xs[k]) {
                        const uint32_t sw = id[k] / kCl, ow = id[k] % kCl;
                        atomicOr(cl.map_shared_rank(&sm.front[p ^ 1u][sw >> 5], ow), 1u << (sw & 31));
                        *reinterpret_cast<volatile uint32_t*>(cl.map_shared_rank(&sm.flag[t % 3], 0)) = 1u;
                    }
                }
            }
            __syncwarp();
        }
    }

};

__global__ void __launch_bounds__(kClThreads, 1) peel_hxtail_kernel(const __grid_constant__ PeelArgs a) {
    extern __shared__ __align__(16) unsigned char cl_smem[];
    ClSmem& sm = *reinterpret_cast<ClSmem*>(cl_smem);
    cg::cluster_group cl = cg::this_cluster();
    PeelCtl* ctl = a.ctl;
    const unsigned tid = threadIdx.x;
    // every CTA of the cluster takes the same exit here, before any barrier
    const bool ho = a.tail_est != nullptr;   // the launch after the h-index peel (hand-off mode)
    if (ctl->err != 0 || a.tail_hx_iters == 0 || (ho && ctl->hx.handoff == 0)) return;
    const uint32_t n = ho ? ctl->hx.ho_n : ctl->tail_n;
    if (n == 0 || n > kHoV || (!ho && (n > a.tail_cap_v || n > kTailV))) return;
    Tail T{a, sm, cl, n, ho ? ctl->hx.ho_floor : ctl->tail_level, (uint32_t)cl.block_rank(), ctl->tail_arcs / 4u,
           reinterpret_cast<const uint4*>(a.tail_nbr)};
    const uint32_t own = n > T.rank ? (n - T.rank + kCl - 1) / kCl : 0u;
    // level tail: estimates from the induced degrees, every vertex in the first
    // frontier; hand-off: the h-index peel's estimates and counts, its queued
    // vertices (a count below the estimate) in the first frontier
    for (uint32_t v = tid; v < kHoV; v += kClThreads)
        sm.eall[v] = v < n ? (ho ? __ldcg(a.tail_est + v) : T.degree(v)) : 0u;
    for (uint32_t s = tid; s < kPer; s += kClThreads) {
        sm.cnt[s] = ho && s < own ? __ldcg(a.tail_cnt + T.vertex(s)) : 0u;
        sm.sdeg[s] = s < own ? T.degree(T.vertex(s)) : 0u;
        sm.sfq[s] = s < own ? T.first_quad(T.vertex(s)) : 0u;
    }
    for (uint32_t w = tid; w < 2 * (kPer / 32); w += kClThreads) (&sm.front[0][0])[w] = 0;
    if (tid == 0) {
        sm.flag[0] = sm.flag[1] = sm.flag[2] = 0;
        sm.kmax = 0;
    }
    __syncthreads();
    if (ho)
        for (uint32_t s = tid; s < own; s += kClThreads)
            if (sm.cnt[s] < sm.eall[T.vertex(s)]) atomicOr(&sm.front[1][s >> 5], 1u << (s & 31));
    cl.sync();

    bool solved = false;
    uint32_t t = 1;
    for (;;) {
        const uint32_t p = t & 1u;
        // ---- phase A: the frontier (iteration 1: every vertex)
        if (tid == 0) { sm.nwork = 0; sm.nbig = 0; sm.nchg = 0; }
        if (T.rank == 0 && tid == 0) sm.flag[(t + 1) % 3] = 0;
        __syncthreads();
        for (uint32_t s = tid; s < own; s += kClThreads) {
            const bool in = (t == 1 && !ho) || ((sm.front[p][s >> 5] >> (s & 31)) & 1u);
            if (!in) continue;
            if (sm.sdeg[s] <= kWVals) sm.work[atomicAdd(&sm.nwork, 1u)] = s;
            else sm.big[atomicAdd(&sm.nbig, 1u)] = s;
        }
        __syncthreads();
        for (uint32_t w = tid; w < kPer / 32; w += kClThreads) sm.front[p][w] = 0;   // consumed
        T.recompute_warps();
        __syncthreads();
        T.recompute_big();
        cl.sync();   // every estimate of this iteration is final
        // ---- phase B: the vertices that dropped
        if (tid == 0) { sm.nwork = 0; sm.nbig = 0; }
        __syncthreads();
        for (uint32_t i = tid; i < min(sm.nchg, kPer); i += kClThreads) {
            const uint32_t s = sm.chg[i];
            if (sm.sdeg[s] <= kWVals) sm.work[atomicAdd(&sm.nwork, 1u)] = s;
            else sm.big[atomicAdd(&sm.nbig, 1u)] = s;
        }
        __syncthreads();
        T.update_warps(p, t);
        __syncthreads();
        T.update_big(p, t);
        cl.sync();   // every count and frontier bit of this iteration is final
        const uint32_t any = *cl.map_shared_rank(&sm.flag[t % 3], 0);
        if (!any) { solved = true; break; }
        if (++t > a.tail_hx_iters) break;
    }
    if (solved) {
        uint32_t mx = 0;
        for (uint32_t s = tid; s < own; s += kClThreads) {
            const uint32_t v = T.vertex(s);
            const uint32_t g = __ldcg(a.tail_ids + v);
            if (g < a.V) a.core[g] = sm.eall[v];
            mx = max(mx, sm.eall[v]);
        }
        mx = __reduce_max_sync(kFull, mx);
        if (lane_id() == 0 && mx) atomicMax(cl.map_shared_rank(&sm.kmax, 0), mx);
    }
    cl.sync();
    if (solved && T.rank == 0 && tid == 0) {
        ctl->kmax = sm.kmax;
        ctl->levels = sm.kmax + 1;
        ctl->hx.tail_iters = t;
        if (ho) {   // the vertices outside S kept their final estimates
            ctl->iterations = ctl->hx.iters + t;
            ctl->hx.solved = 1;
        } else {
            ctl->iterations = ctl->tail_iter + t;
            ctl->hx.tail_solved = 1;
        }
    }
    cl.sync();   // no CTA leaves while another may still read its shared memory
}

}  // namespace

const void* peel_hxtail_fn() { return reinterpret_cast<const void*>(&peel_hxtail_kernel); }
size_t peel_hxtail_smem() { return sizeof(ClSmem); }
int peel_hxtail_cluster() { return kCl; }
int peel_hxtail_threads() { return kClThreads; }

}  // namespace kc
