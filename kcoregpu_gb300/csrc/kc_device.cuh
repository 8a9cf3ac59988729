// Device-side building blocks of the GB300 level-synchronous peel.
//
// Algorithm (same result as the reference's kcore(), src/ours.cc:117-160):
// for level = 0,1,2,... every vertex whose remaining degree equals `level` is
// peeled; peeling v decrements each neighbour u with deg[u] > level, and a
// neighbour whose degree falls to `level` is peeled in the same level
// (ours.cc:92-105).  When every vertex is peeled, the level at which a vertex
// was peeled is its core number and the last level is kmax (ours.cc:151).
//
// GB300 design (no reference counterpart):
//  * w[v] holds deg(v) + kBias.  Bit 31 (kClaim) marks a vertex as peeled
//    ("claimed").  A vertex is claimed exactly once, by one atomic that sees
//    the bit clear: the frontier scan's atomicOr (w == level+kBias), a
//    walker's atomicCAS(level+1 -> level | claim), which decrements and
//    claims at once, or the atomicOr of the walker whose atomicSub took w
//    from level+1 to level (ours.cc:96).  The bias keeps transient
//    over-decrements (decrements that raced below the level and are undone,
//    as in ours.cc:102-105) from ever borrowing into the claim bit.
//  * Because claims are exclusive, the scan and the neighbour walk of one
//    level run concurrently: scan hits are walked inline by the scanning warp,
//    cascades go to a warp-local list while it holds at most local_budget
//    arcs, and hubs (> kLocalArcs arcs), the rest of wide cascades and list
//    overflow go to a global queue of arc-range tasks.  There is no grid
//    barrier inside a level; a level ends when every CTA has finished its scan
//    slice and every queued task is done, which every CTA reads off one
//    packed counter of the level (LevelSlot::units_tail).
//  * Every wait is bounded in time (wait_us); on expiry the kernel records
//    KC_ERR_TIMEOUT and returns instead of trapping.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

// Loads of the read-only CSR.  A kernel that peels graphs whose memory may be
// reused while it runs (the serve kernel) defines KC_LDG as __ldcg, so that no
// stale line of an earlier graph can be served from the non-coherent L1 path.
#ifndef KC_LDG
#define KC_LDG(p) __ldg(p)
#endif

namespace kc {

constexpr uint32_t kBias = 1u << 30;
constexpr uint32_t kClaim = 1u << 31;
constexpr uint32_t kItemCap = 128;    // per-warp batch of arc ranges
constexpr uint32_t kLocalArcs = 256;  // default hub threshold: vertices with more arcs go to the task queue
constexpr uint32_t kChunk = 256;      // largest (and default) arcs per queued task (len-1 fits 8 bits)
constexpr uint32_t kMinChunk = 64;    // smallest arcs per queued task a launch may choose
constexpr uint32_t kLocalBudget = 128;   // arcs a warp's cascade list may hold; the rest is queued
constexpr uint32_t kFull = 0xFFFFFFFFu;

// Device status codes (mirrors of KC_ERR_*; 0 = ok).
constexpr int kErrOverflow = -4;
constexpr int kErrTimeout = -5;
constexpr int kErrCheck = -12;   // checked build: an index was out of bounds (access skipped)
constexpr int kErrInvalid = -8;  // malformed input found on the device (a neighbour id >= V)

// Counters of one level iteration.  A ring of 4 slots is reused: CTA 0 clears
// the slot of iteration i-2 when it starts iteration i, when no warp can still
// touch it.
//
// Level completion.  A level's work units are the participants' scans (one
// per CTA) and the tasks pushed to the queue.  `units_tail` packs the units
// finished in its high half with the tasks pushed in its low half, so one
// 64-bit word holds both sides of the test: the level is complete exactly
// when units == participants + tasks.  A push happens inside a unit that is
// not finished yet (a scan before its arrival, a task before its completion)
// and is ordered before the completion of the task it pushes (the claimer
// reads the entry written after the push), so no snapshot of the word shows
// the equality early.  Arrivals and completions are a release fence and one
// add; every poller sees the end from one load.
struct alignas(128) LevelSlot {
    unsigned long long units_tail;   // [63:32] units finished, [31:0] tasks pushed in this level
    unsigned int pad0[30];
    unsigned int head;               // tasks claimed
    unsigned int pad1[31];
    unsigned int peeled;             // vertices claimed in this level
    unsigned int arrived;            // participants arrived (traced runs only)
    unsigned int pad2[30];
    unsigned int alive_next;  // survivors appended to the next alive list
    unsigned int min_next;    // smallest survivor state seen by the scans (0xFFFFFFFF = none)
    unsigned long long arcs_next;   // sum of the survivor degrees seen by the scans (>= induced arcs)
    unsigned int pad3[28];
};

// Control words of the h-index peel (kc_hindex.cu).  Work lists come in
// rotating copies so that no counter is cleared while a producer of the same
// sub-phase may add to it: chunk-task lists by sub-phase mod 3, the others by
// iteration parity.  Each hot counter has its own 128-byte line.
struct alignas(128) HxCtl {
    unsigned int solved;       // 1: every core number is found (the peel kernels return at once)
    unsigned int iters;        // h-index iterations run
    unsigned int passes;       // window passes over large vertices (sub-phases of phase A)
    unsigned int pad0[29];
    unsigned int cl_n[3];      // chunk tasks of large vertices, by sub-phase mod 3
    unsigned int pad1[29];
    unsigned int bt_n[2];      // update tasks (vertices whose estimate dropped), by iteration parity
    unsigned int pad2[30];
    unsigned int rm_n[2];      // next frontier: vertices of at most kHxWarpArcs arcs
    unsigned int pad3[30];
    unsigned int rl_n[2];      // next frontier: larger vertices (window slots)
    unsigned int pad4[30];
    unsigned int bar;          // grid barrier: arrivals so far (barrier k completes at k * grid)
    unsigned int pad5[31];
    unsigned int rc_n[3];      // CTA entries (large vertices read whole by one CTA), by sub-phase mod 3
    unsigned int pad6[29];
    unsigned int tail_solved;  // 1: the cluster h-index tail found the survivors' core numbers
    unsigned int tail_iters;   // its iterations
    unsigned int pad7[30];
    unsigned int peel_done;    // 1: a level peel finished every level (later peel launches return at once)
    unsigned int stopped;      // 1: the level peel stopped early (PeelArgs::stop_alive) for the h-index
    unsigned int pad8[30];
    // Hand-off of the h-index peel to the cluster tail (kc_hindex.cu try_handoff)
    unsigned int handoff;      // 1: the set S below was handed over; the cluster tail finishes it
    unsigned int ho_floor;     // T: every vertex of S has at least T neighbours in S
    unsigned int ho_n;         // |S| (local ids 0 .. ho_n-1)
    unsigned int pad9[29];
    // counters of an attempt, by attempt parity (the lead clears the other
    // parity's during an attempt, so no attempt needs a barrier to reset them)
    unsigned int ho_min[2];      // smallest estimate of the frontier
    unsigned int ho_cnt[2][5];   // vertices at or above each candidate floor
    unsigned int ho_m[2];        // members given local ids
    unsigned int ho_fail[2];     // a member has fewer than T neighbours in S, or a buffer is too small
    unsigned int ho_tasks[2];    // chunk tasks over the members' sources
    unsigned long long ho_arcs[2];   // induced-CSR entries reserved (each member: its source length,
                                     // padded to quads; 64 bits, so that no sum wraps)
    unsigned int pad10[10];
};

struct alignas(128) PeelCtl {
    LevelSlot slot[4];
    unsigned int iters_done;   // level iterations completed (CTA 0 writes it; diagnostics)
    unsigned int pad0[31];
    unsigned int order_tail;   // next peel-order position
    unsigned int pad1[31];
    int err;                   // first error (0 = ok)
    unsigned int err_level;
    unsigned int kmax;
    unsigned int levels;       // kmax + 1, as the reference counts them
    unsigned long long tasks;  // tasks pushed (stats)
    unsigned int err_site;     // checked build: access site of the first violation
    unsigned int iterations;   // level iterations actually run (empty runs skipped)
    unsigned long long err_index;   // checked build: its index
    unsigned int bar_count;    // grid barrier of the tail hand-off: arrivals
    unsigned int bar_gen;      // and generation
    unsigned int tail_n;       // vertices handed to the tail peel (0 = none)
    unsigned int tail_level;   // first level of the tail peel
    unsigned int tail_peeled;  // vertices peeled before it
    unsigned int tail_iter;    // level iterations run before it
    unsigned int tail_items;   // fill work items of the induced CSR
    unsigned int tail_arcs;    // arcs of the induced CSR
    unsigned int maxdeg;       // maximum degree found by the device-side CSR validation
    unsigned int pad2[13];
    HxCtl hx;                  // h-index peel (zero when only the level peel runs)
};

// h-index peel of one graph (kc_hindex.cu).
constexpr uint32_t kHxLaneArcs = 16;    // iteration 1: one lane finds the h-index of a vertex this small
constexpr uint32_t kHxWarpArcs = 256;   // one warp, 8 values a lane; larger vertices are split in chunks
constexpr uint32_t kHxChunk = 256;      // arcs per chunk task
constexpr uint32_t kHxBinWords = 40;    // per window slot: 32 bins, the count above the window, padding
constexpr uint32_t kHxCtaVals = 8192;   // a CTA reads a large vertex whole up to this many entries

// Window state of a large vertex whose h-index is being searched.  Bin b
// counts the neighbour estimates in [lo + b*2^sh, lo + (b+1)*2^sh - 1]
// (clipped at hi); bin 32 counts those above hi.  A pass reads either the
// whole adjacency (mode 0; it also rebuilds the active list from the
// neighbours at or above lo) or the vertex's active list (mode 1).
struct HxSlot {
    uint32_t v;       // vertex
    uint32_t e;       // its estimate when the search started (upper bound of the new one)
    uint32_t lo, hi;  // window
    uint32_t sh;      // log2 of the bin width
    uint32_t done;    // chunk tasks finished in this pass
    uint32_t nch;     // chunk tasks per pass
    uint32_t mode;    // 0: adjacency, 1: active list
    uint32_t len;     // entries a pass reads
    uint32_t pad[3];
};

struct HxArgs {
    const uint32_t* off;
    const uint32_t* nbr;
    uint32_t* est;      // estimate per vertex; the core number once converged (the core output)
    uint32_t* cnt;      // neighbours counted at or above the estimate (a lower bound of the true count)
    uint32_t* old;      // estimate before the last drop
    // Active lists of large vertices: act[off[v] ...) holds alen[v] neighbours
    // of v, every one whose estimate is at or above alo[v] (and possibly some
    // that fell below since); alen[v] = 0xFFFFFFFF: no list.  Estimates only
    // fall, so once v's estimate is at or above alo[v] no other neighbour can
    // count towards its h-index or be crossed by its drops.
    uint32_t* act;
    uint32_t* alo;
    uint32_t* alen;
    uint32_t* rm[2];    // frontier lists of vertices with at most kHxWarpArcs arcs (V each)
    HxSlot* slots[2];   // frontier of larger vertices, cap_l each
    uint32_t* bins[2];  // kHxBinWords per slot
    unsigned long long* cl[3];   // chunk tasks: slot << 32 | chunk
    uint32_t* rc[3];             // CTA entries: vertex | 0x80000000 when read from its active list
    unsigned long long* bt[2];   // update tasks: vertex << 32 | chunk
    PeelCtl* ctl;
    uint32_t V;
    uint32_t E;
    uint32_t cap_l, cap_cl, cap_bt;
    uint32_t max_iters;   // give up (the level peel runs instead) after this many iterations
    uint32_t wait_us;
    uint32_t max_level;   // 0xFFFFFFFF: the CSR was validated on the device (return if that failed)
    // Start after a level peel that stopped early (HxCtl::stopped): w holds its
    // states (claim bit and remaining degree + kBias) and est the core numbers
    // of the peeled vertices; the survivors start from their remaining degree.
    const uint32_t* w;
    uint32_t after_peel;
    // Hand-off to the cluster tail (handoff != 0): the induced CSR of S with
    // local ids, in the tail buffers of the level peel (kTailV vertices), plus
    // S's estimates and counts by local id; lmap (V entries; may be `old`,
    // which holds nothing between iterations) maps a vertex to its local id.
    uint32_t handoff;
    uint32_t* lmap;
    uint32_t* tail_ids;
    uint32_t* tail_off;
    uint32_t* tail_cur;
    uint32_t* tail_nbr;
    uint32_t* tail_est;
    uint32_t* tail_cnt;
    uint32_t tail_cap_arcs;
    uint32_t ho_front;   // try the hand-off once the frontier holds at most this many vertices
    uint32_t ho_max;     // and S at most this many (<= kTailV)
};

struct PeelArgs {
    const uint32_t* off;        // V+1 arc offsets
    const uint32_t* nbr;        // arcs
    uint32_t* w;                // working state, roundup(V,128) entries, 16-B aligned
    uint32_t* core;             // out: core number per vertex
    uint32_t* order;            // optional out: vertices in peel order
    uint32_t* shells;           // optional out: k-shell offsets into order
    unsigned long long* tasks;  // task queue storage
    PeelCtl* ctl;
    unsigned long long task_cap;
    uint32_t V;
    uint32_t shell_cap;
    uint32_t max_level;         // max degree: no vertex survives past it (0xFFFFFFFF: the device
                                // validation found it, in ctl->maxdeg; the peel returns at once
                                // if that validation recorded an error)
    uint32_t epoch;             // 1..255, tags this run's task entries
    uint32_t wait_us;           // longest a warp waits for others before it gives up (KC_ERR_TIMEOUT)
    unsigned long long* trace;  // optional per-level timestamps (kTraceFields per level)
    uint32_t trace_cap;         // levels the trace buffer holds
    uint32_t* alive[2];         // optional alive-vertex lists (roundup(V,128) each); null = dense scans only
    uint32_t E;                 // arcs (= off[V])
    uint32_t zero_tasks;        // 1: the participants clear the task queue during level 0
                                // (for callers that cannot launch a memset while peeling)
    // Tail hand-off (zero caps = never): once at most tail_cap_v vertices
    // remain and their induced arcs fit tail_cap_arcs, the participants build
    // the induced CSR of the survivors (local ids) and stop; peel_tail_kernel
    // finishes the peel in one CTA with the states in shared memory.
    uint32_t tail_cap_v = 0;
    uint32_t tail_cap_arcs = 0;
    uint32_t* tail_ids = nullptr;              // tail_cap_v: global id of each local vertex
    uint32_t* tail_off = nullptr;              // tail_cap_v+1: induced CSR offsets
    uint32_t* tail_cur = nullptr;              // tail_cap_v: fill cursors
    uint32_t* tail_nbr = nullptr;              // tail_cap_arcs: induced CSR neighbours (local ids,
                                               // each adjacency padded to 4 entries with 0xFFFFFFFF)
    unsigned long long* tail_items = nullptr;  // fill work items: local id << 32 | arc chunk
    uint32_t tail_items_cap = 0;
    uint32_t local_budget = kLocalBudget;      // arcs a warp's cascade list may hold
    uint32_t claim_cas = 0;     // 1: the walk claims by CAS without reading the state first (one graph on
                                // the whole GPU: latency-bound); 0: it reads the state first (fewer atomics,
                                // for kernels that peel many graphs at once)
    uint32_t hub_arcs = kLocalArcs;   // vertices with more arcs are queued as tasks instead of walked inline
    uint32_t chunk_arcs = kChunk;     // arcs per queued task, kMinChunk..kChunk
    uint32_t tail_hx_iters = 0;       // > 0: the cluster h-index tail (kc_hxtail.cu) runs first, for at most
                                      // this many iterations; the level tail kernel finishes otherwise
    uint32_t stop_alive = 0;          // > 0: stop after the first level that leaves at most this many
                                      // survivors (HxCtl::stopped), for the h-index peel to finish
    uint32_t* tail_est = nullptr;     // h-index hand-off: estimates and counts of S by local id
    uint32_t* tail_cnt = nullptr;
};

// Tail peel: one CTA of kTailThreads threads, states in shared memory.
constexpr uint32_t kTailThreads = 1024;
constexpr uint32_t kTailWarps = kTailThreads / 32;
constexpr uint32_t kHoV = 24576;         // largest set the h-index peel hands to the cluster kernel
constexpr uint32_t kTailV = 16384;        // largest tail (shared-memory states)
constexpr uint32_t kTailHandoffV = 12288;  // default hand-off point (survivors); measured best of
                                           // 8,192 / 12,288 / 16,384 on the three single-graph workloads
constexpr uint32_t kTailItems = 2 * kTailThreads;   // queue entries walked per round (2 per thread)
constexpr uint32_t kTailArcs = 1u << 22;  // default largest induced CSR handed over
constexpr uint32_t kFillChunk = 256;      // raw arcs per fill work item

// Per-level trace words: level start (CTA 0), CTA 0 arrival, level announced
// complete, CTA 0 saw completion, vertices peeled so far, last CTA arrival,
// walk rounds and quads walked (tail kernel levels only).
constexpr int kTraceFields = 8;

// ---------------------------------------------------------------- memory ops
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_relaxed(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// Device wall clock (ns) for time-bounded waits: __nanosleep durations are only
// hints (observed far below the request), so limits are in time, not polls.
__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ int ld_err(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Task entry: [63:32] first arc | [31:24] len-1 | [23:8] level | [7:0] epoch.
__device__ __forceinline__ unsigned long long make_task(uint32_t start, uint32_t len, uint32_t level,
                                                        uint32_t epoch) {
    return ((unsigned long long)start << 32) | ((unsigned long long)(len - 1) << 24) |
           ((unsigned long long)(level & 0xFFFF) << 8) | (epoch & 0xFF);
}
__device__ __forceinline__ bool task_ready(unsigned long long e, uint32_t level, uint32_t epoch) {
    return (uint32_t)(e & 0xFFFFFF) == (((level & 0xFFFF) << 8) | (epoch & 0xFF));
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp-wide exclusive prefix sum; *total receives the sum.
__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t x, uint32_t* total) {
    const unsigned lane = lane_id();
    uint32_t inc = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, inc, d);
        if (lane >= (unsigned)d) inc += y;
    }
    *total = __shfl_sync(kFull, inc, 31);
    return inc - x;
}

__device__ __forceinline__ void record_error(PeelCtl* ctl, int code, uint32_t level) {
    if (atomicCAS(&ctl->err, 0, code) == 0) ctl->err_level = level;
}

// Bounds check of the checked build (compiled with KC_CHECKED): records the
// first out-of-bounds index with its access site and level, and tells the
// caller to skip the access.  In the normal build it is a constant true.
#ifdef KC_CHECKED
static __device__ __noinline__ bool kc_in_bounds_fail(PeelCtl* ctl, unsigned long long idx, int site, uint32_t level) {
    if (atomicCAS(&ctl->err, 0, kErrCheck) == 0) {
        ctl->err_level = level;
        ctl->err_site = (unsigned)site;
        ctl->err_index = idx;
    }
    return false;
}
#define KC_IN(ctl, idx, size, site, level)                                                          \
    (((unsigned long long)(idx) < (unsigned long long)(size)) ? true                                \
                                                                : kc_in_bounds_fail((ctl), (idx), (site), (level)))
#else
#define KC_IN(ctl, idx, size, site, level) true
#endif

}  // namespace kc
