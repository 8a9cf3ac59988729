// C ABI of the single-graph peel: device-resident graphs (kc_graph), the
// persistent cooperative launch, and the one-shot host-buffer entry point.
// Replaces the reference's kcore() host loop (src/ours.cc:117-160) and its
// device memory glue (src/gpu_memory_allocation.cu:4-22).
#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kc_internal.h"
#include "kc_peel.cuh"

using kc::PeelArgs;
using kc::PeelCtl;

namespace kc {

int cuda_fail(cudaError_t e, const char* what) {
    set_error_msg(std::string(what) + ": " + cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation) return KC_ERR_OOM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return KC_ERR_NODEV;
    return KC_ERR_CUDA;
}

#define KC_CUDA(call)                                       \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// The bounds-checked kernel variant is used when KC_CHECKED=1 is set.
static bool checked_mode() {
    static const bool on = [] {
        const char* e = std::getenv("KC_CHECKED");
        return e && e[0] == '1';
    }();
    return on;
}

static const void* peel_kernel() { return checked_mode() ? peel_persistent_fn_checked() : peel_persistent_fn(); }

const void* peel_kernel_selected() { return peel_kernel(); }

// Longest a device wait may last before the kernel gives up with
// KC_ERR_TIMEOUT: 2 s.  KC_WAIT_US (read once per process) shortens it for the
// tests that make a wait run out.
uint32_t wait_limit_us() {
    static uint32_t w = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        w = 2000000;
        if (const char* e = std::getenv("KC_WAIT_US")) {
            const long long x = std::atoll(e);
            if (x >= 1 && x <= 60000000) w = (uint32_t)x;
        }
    });
    return w;
}

// Persistent grid size per device: one CTA per SM (the kernel is compiled for
// one 512-thread CTA per SM, up to 128 registers a thread).  The late levels
// are short, and their cost grows with the participants that must arrive at
// each level's end: on GB300 one CTA per SM was fastest (R-MAT 2^20: 3.7 ms at
// 152 CTAs against 4.5 ms at 304, in a 64-register build that fit two).
static int persistent_grid(int dev) {
    static std::mutex mu;
    static std::vector<int> cache;
    std::lock_guard<std::mutex> lk(mu);
    if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
    if (cache[dev]) return cache[dev];
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, peel_kernel(), kPeelThreads, 0);
    if (per < 1) per = 1;
    cache[dev] = sms;
    // KC_PEEL_GRID=n runs the persistent peel on n CTAs (n <= the co-resident
    // maximum): the level protocol is the one gangs of the serve kernel use.
    if (const char* e = std::getenv("KC_PEEL_GRID")) {
        const int n = std::atoi(e);
        if (n > 0 && n <= sms * per) cache[dev] = n;
    }
    return cache[dev];
}

}  // namespace kc

using namespace kc;

struct kc_graph {
    kc_tuning tune{};       // settings the autotuner chose at upload
    int dev = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint32_t V = 0;
    uint64_t E = 0;
    uint32_t maxdeg = 0;
    uint32_t cap_V = 0;      // allocated vertex capacity
    uint64_t cap_E = 0;      // allocated arc capacity
    uint32_t* d_off = nullptr;
    uint32_t* d_nbr = nullptr;
    uint32_t* d_w = nullptr;
    uint32_t* d_core = nullptr;
    uint32_t* d_order = nullptr;
    uint32_t* d_shells = nullptr;
    unsigned long long* d_tasks = nullptr;
    unsigned long long task_cap = 0;
    PeelCtl* d_ctl = nullptr;
    PeelCtl* h_ctl = nullptr;   // pinned
    PeelCtl* h_ctl_init = nullptr;   // pinned initial image (slot minima = none)
    uint32_t epoch = 0;
    int grid = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool pending = false;
    bool ran = false;
    bool with_order = false;
    uint32_t shell_cap = 0;
    unsigned long long* d_trace = nullptr;
    uint32_t trace_cap = 0;
    uint32_t* d_alive[2] = {nullptr, nullptr};   // alive-vertex lists (scratch)
    // tail hand-off (induced CSR of the survivors, local ids)
    uint32_t tail_cap_v = 0;      // 0 = the persistent kernel peels every level
    uint32_t tail_cap_arcs = 0;
    uint32_t tail_items_cap = 0;
    uint32_t* d_tail_ids = nullptr;
    uint32_t* d_tail_off = nullptr;
    uint32_t* d_tail_cur = nullptr;
    uint32_t* d_tail_nbr = nullptr;
    unsigned long long* d_tail_items = nullptr;
    // h-index peel (kc_hindex.cu): counts, old estimates, window slots and bins
    // of large vertices, chunk-task and update-task lists
    uint32_t* d_hx_cnt = nullptr;
    uint32_t* d_hx_old = nullptr;
    uint32_t* d_hx_act = nullptr;   // active lists (E), their floors and lengths (V each)
    uint32_t* d_hx_alo = nullptr;
    uint32_t* d_hx_alen = nullptr;
    HxSlot* d_hx_slots[2] = {nullptr, nullptr};
    uint32_t* d_hx_bins[2] = {nullptr, nullptr};
    unsigned long long* d_hx_cl[3] = {nullptr, nullptr, nullptr};
    uint32_t* d_hx_rc[3] = {nullptr, nullptr, nullptr};
    unsigned long long* d_hx_bt[2] = {nullptr, nullptr};
    uint32_t* d_hx_tail = nullptr;  // hand-off to the cluster: ids, offsets (kHoV + 4), cursors,
                                    // estimates and counts of S (kHoV each)
    uint32_t* d_hx_tnbr = nullptr;  // and its induced adjacency (spans as long as each member's source)
    uint32_t hx_tnbr_cap = 0;
    uint32_t hx_cap_v = 0, hx_cap_l = 0, hx_cap_cl = 0, hx_cap_bt = 0;
    uint32_t method = KC_METHOD_AUTO;
};

namespace {

void release(kc_graph* g) {
    if (!g) return;
    cudaSetDevice(g->dev);
    if (g->stream) cudaStreamSynchronize(g->stream);
    cudaFree(g->d_off); cudaFree(g->d_nbr); cudaFree(g->d_w); cudaFree(g->d_core);
    cudaFree(g->d_order); cudaFree(g->d_shells); cudaFree(g->d_tasks); cudaFree(g->d_ctl);
    cudaFree(g->d_trace);
    cudaFree(g->d_alive[0]); cudaFree(g->d_alive[1]);
    cudaFree(g->d_tail_ids); cudaFree(g->d_tail_off); cudaFree(g->d_tail_cur); cudaFree(g->d_tail_nbr);
    cudaFree(g->d_tail_items);
    cudaFree(g->d_hx_tail);
    cudaFree(g->d_hx_tnbr);
    cudaFree(g->d_hx_cnt); cudaFree(g->d_hx_old);
    cudaFree(g->d_hx_act); cudaFree(g->d_hx_alo); cudaFree(g->d_hx_alen);
    for (int i = 0; i < 2; ++i) { cudaFree(g->d_hx_slots[i]); cudaFree(g->d_hx_bins[i]); cudaFree(g->d_hx_bt[i]); }
    for (int i = 0; i < 3; ++i) { cudaFree(g->d_hx_cl[i]); cudaFree(g->d_hx_rc[i]); }
    if (g->h_ctl) cudaFreeHost(g->h_ctl);
    if (g->h_ctl_init) cudaFreeHost(g->h_ctl_init);
    if (g->ev0) cudaEventDestroy(g->ev0);
    if (g->ev1) cudaEventDestroy(g->ev1);
    if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
}

// Task queue entries of a graph: every vertex once plus every hub chunk.
// KC_TASK_CAP (read once per process) caps it, for the tests that make the
// queue overflow.
uint64_t task_capacity(uint32_t V, uint64_t E) {
    static uint64_t cap = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        if (const char* e = std::getenv("KC_TASK_CAP")) {
            const long long x = std::atoll(e);
            if (x >= 1) cap = (uint64_t)x;
        }
    });
    const uint64_t need = (uint64_t)V + E / kMinChunk + 64;   // (the smallest chunk a launch may choose)
    return cap ? std::min(cap, need) : need;
}

// Walk mode of the one-graph peel: claim by CAS without reading the state
// first (KC_CLAIM_CAS, default 1).
uint32_t claim_cas() {
    static uint32_t c = 1;
    static std::once_flag once;
    std::call_once(once, [] {
        if (const char* e = std::getenv("KC_CLAIM_CAS")) c = std::atoi(e) != 0 ? 1u : 0u;
    });
    return c;
}

// Experiment overrides of the tuned settings, read once per process (unset:
// the autotuner decides).  None changes a result.
struct Overrides {
    long long hub_arcs = -1, chunk_arcs = -1, local_budget = -1, tail_v = -1, tail_arcs = -1;
};
const Overrides& overrides() {
    static Overrides o;
    static std::once_flag once;
    std::call_once(once, [] {
        auto rd = [](const char* k, long long lo, long long hi) -> long long {
            const char* e = std::getenv(k);
            if (!e) return -1;
            const long long x = std::atoll(e);
            return (x >= lo && x <= hi) ? x : -1;
        };
        o.hub_arcs = rd("KC_HUB_ARCS", 32, 1 << 20);
        o.chunk_arcs = rd("KC_CHUNK_ARCS", kMinChunk, kChunk);
        o.local_budget = rd("KC_LOCAL_BUDGET", 32, 1 << 20);
        o.tail_v = rd("KC_TAIL_V", 0, kTailV);
        o.tail_arcs = rd("KC_TAIL_ARCS", 1, 1ll << 30);
    });
    return o;
}

// Method of the single-graph peel when a graph asks for none: the h-index
// fixed point (kc_hindex.cu) with the level peel as its fallback, or, with
// KC_ALGO=peel (read once per process), the level peel.  On GB300 the h-index
// peel measured 1.94 / 2.09 / 2.01 ms on R-MAT 400K / 2^20 / Chung-Lu 2.4M
// against 1.99 / 2.27 / 2.33 ms for the level peel.
bool hindex_default() {
    static bool on = true;
    static std::once_flag once;
    std::call_once(once, [] {
        if (const char* e = std::getenv("KC_ALGO")) on = std::strcmp(e, "peel") != 0;
    });
    return on;
}

// Where the h-index peel starts (KC_HX_START=n, read once per process): 0 =
// from the degrees; n > 0 = after a level peel that stops at the first level
// leaving at most V/n survivors, from their remaining degrees.
uint32_t hindex_start() {
    static uint32_t n = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        if (const char* e = std::getenv("KC_HX_START")) {
            const long long x = std::atoll(e);
            if (x >= 0 && x <= (1 << 20)) n = (uint32_t)x;
        }
    });
    return n;
}

// Iterations after which the h-index peel gives the graph to the level peel
// (KC_HX_ITERS, default 256): paths and long chains converge one hop per
// iteration, where the level peel walks them in one level.
uint32_t hindex_max_iters() {
    static uint32_t n = 256;
    static std::once_flag once;
    std::call_once(once, [] {
        if (const char* e = std::getenv("KC_HX_ITERS")) {
            const long long x = std::atoll(e);
            if (x >= 1 && x <= (1 << 24)) n = (uint32_t)x;
        }
    });
    return n;
}

// Largest induced adjacency handed to the tail kernel (KC_TAIL_ARCS, default
// kTailArcs).
uint32_t tail_arcs_limit() {
    const long long x = overrides().tail_arcs;
    return x > 0 ? (uint32_t)x : kTailArcs;
}

// The autotuner: settings of the single-graph peel from the CSR's degree
// distribution, sampled from the host offsets in 32 runs of 32 consecutive
// vertices (a few KB of reads, so the one-shot call can afford it before its
// upload), plus V.  The rules come from one-at-a-time sweeps on GB300 over
// R-MAT (400K, 2^20, 2^22 vertices), Chung-Lu (gamma 2.1 and 2.5) and
// Erdos-Renyi graphs:
//  * task chunks of 64 arcs: hubs split finer cost nothing where there are
//    none and gained 1-13% where there are (R-MAT 2^22: 7.18 -> 6.27 ms);
//  * the cascade budget follows the spread of the degrees: near-uniform degrees
//    (coefficient of variation below 1) gain from long warp-local cascades
//    (512 arcs: Erdos-Renyi 1M -12%), skewed ones lose (R-MAT 400K +8%), and
//    skewed graphs above 2M vertices sit between (256);
//  * the one-CTA tail takes the last 16,384 survivors of a graph above 256K
//    vertices (-1.6% on R-MAT 400K, -0.8% on Chung-Lu 2.4M), 12,288 below;
//  * the hub threshold moved nothing by more than 1% between 128 and 1,024
//    arcs and stays 256.
// Experiment overrides win.
void autotune(const uint32_t* off, uint32_t V, kc_tuning* t) {
    t->hub_arcs = kLocalArcs;
    t->chunk_arcs = kMinChunk;
    t->local_budget = kLocalBudget;
    t->tail_v = kTailHandoffV;
    t->grid = 0;
    if (V && off) {
        constexpr uint32_t kRuns = 32, kRun = 32;
        double sum = 0, sq = 0;
        uint32_t cnt = 0;
        for (uint32_t r = 0; r < kRuns; ++r) {
            const uint64_t v0 = (uint64_t)V * r / kRuns;
            for (uint32_t i = 0; i < kRun && v0 + i < V; ++i) {
                const double d = (double)(off[v0 + i + 1] - off[v0 + i]);
                sum += d;
                sq += d * d;
                ++cnt;
            }
        }
        const double mean = sum / cnt;
        const double var = sq / cnt - mean * mean;
        const double cv = mean > 0 ? std::sqrt(var > 0 ? var : 0.0) / mean : 0.0;
        t->local_budget = cv < 1.0 ? 512u : (V >= (2u << 20) ? 256u : kLocalBudget);
        t->tail_v = V > (256u << 10) ? kTailV : kTailHandoffV;
    }
    const Overrides& o = overrides();
    if (o.hub_arcs > 0) t->hub_arcs = (uint32_t)o.hub_arcs;
    if (o.chunk_arcs > 0) t->chunk_arcs = (uint32_t)o.chunk_arcs;
    if (o.local_budget > 0) t->local_budget = (uint32_t)o.local_budget;
    if (o.tail_v >= 0) t->tail_v = (uint32_t)o.tail_v;
}

// Buffers of the tail hand-off for a graph of at most E arcs, sized for the
// largest tail (kTailV survivors); each launch hands over at the tuned point.
int reserve_tail(kc_graph* g, uint64_t E) {
    if (overrides().tail_v == 0) { g->tail_cap_v = 0; return KC_OK; }
    const uint32_t cap_v = kTailV;
    uint32_t cap_arcs = tail_arcs_limit();
    // room for the padding of every adjacency to a multiple of 4 entries
    cap_arcs = (uint32_t)(((std::min<uint64_t>(cap_arcs, std::max<uint64_t>(E, 1)) + 3ull * kTailV + 16) + 3) & ~3ull);
    const uint64_t items = 2ull * cap_v + E / kFillChunk + 64;
    if (items > 0xFFFFFFFFull) { g->tail_cap_v = 0; return KC_OK; }
    if (!g->d_tail_ids) {
        KC_CUDA(cudaMalloc(&g->d_tail_ids, sizeof(uint32_t) * kTailV));
        // (kTailV + 1 offsets, rounded up to whole 16-byte words for the tail's bulk copy)
        KC_CUDA(cudaMalloc(&g->d_tail_off, sizeof(uint32_t) * (kTailV + 4)));
        KC_CUDA(cudaMalloc(&g->d_tail_cur, sizeof(uint32_t) * kTailV));
    }
    if (cap_arcs > g->tail_cap_arcs || !g->d_tail_nbr) {
        cudaFree(g->d_tail_nbr);
        g->d_tail_nbr = nullptr;
        KC_CUDA(cudaMalloc(&g->d_tail_nbr, sizeof(uint32_t) * cap_arcs));
        g->tail_cap_arcs = cap_arcs;
    }
    if (items > g->tail_items_cap || !g->d_tail_items) {
        cudaFree(g->d_tail_items);
        g->d_tail_items = nullptr;
        KC_CUDA(cudaMalloc(&g->d_tail_items, sizeof(unsigned long long) * items));
        g->tail_items_cap = (uint32_t)items;
    }
    g->tail_cap_v = cap_v;
    return KC_OK;
}

// Buffers of the h-index peel for the graph's capacity.  Large vertices (more
// than kHxWarpArcs arcs) number at most E / (kHxWarpArcs + 1); a pass queues at
// most one chunk task per kHxChunk arcs of them plus one per vertex; update
// tasks are one per vertex plus one per further chunk; a large vertex's active
// list lives in its own adjacency's range of an E-word array.
int reserve_hx(kc_graph* g) {
    const uint64_t V = g->cap_V, E = g->cap_E;
    const uint64_t cap_l = E / (kHxWarpArcs + 1) + 1;
    const uint64_t cap_cl = E / kHxChunk + cap_l + 64;
    const uint64_t cap_bt = V + E / kHxChunk + 64;
    if (cap_l > 0xFFFFFFFFull || cap_cl > 0xFFFFFFFFull || cap_bt > 0xFFFFFFFFull) {
        set_error_msg("graph too large for the h-index peel");
        return KC_ERR_OVERFLOW;
    }
    if (!g->d_hx_tail) KC_CUDA(cudaMalloc(&g->d_hx_tail, sizeof(uint32_t) * (5 * kHoV + 4)));
    {   // the hand-off's adjacency spans: up to every arc of the graph (at most 2^26), plus the quad padding
        const uint64_t cap = ((std::min<uint64_t>(std::max<uint64_t>(E, 1), 1ull << 26) + 3ull * kHoV + 16) + 3) & ~3ull;
        if (cap > g->hx_tnbr_cap) {
            cudaFree(g->d_hx_tnbr);
            g->d_hx_tnbr = nullptr;
            g->hx_tnbr_cap = 0;
            KC_CUDA(cudaMalloc(&g->d_hx_tnbr, sizeof(uint32_t) * cap));
            g->hx_tnbr_cap = (uint32_t)cap;
        }
    }
    if (g->d_hx_cnt && g->hx_cap_v >= V && g->hx_cap_l >= cap_l && g->hx_cap_cl >= cap_cl && g->hx_cap_bt >= cap_bt)
        return KC_OK;
    cudaFree(g->d_hx_cnt); cudaFree(g->d_hx_old);
    cudaFree(g->d_hx_act); cudaFree(g->d_hx_alo); cudaFree(g->d_hx_alen);
    for (int i = 0; i < 2; ++i) { cudaFree(g->d_hx_slots[i]); cudaFree(g->d_hx_bins[i]); cudaFree(g->d_hx_bt[i]); }
    for (int i = 0; i < 3; ++i) { cudaFree(g->d_hx_cl[i]); cudaFree(g->d_hx_rc[i]); }
    g->d_hx_cnt = g->d_hx_old = g->d_hx_act = g->d_hx_alo = g->d_hx_alen = nullptr;
    for (int i = 0; i < 2; ++i) { g->d_hx_slots[i] = nullptr; g->d_hx_bins[i] = nullptr; g->d_hx_bt[i] = nullptr; }
    for (int i = 0; i < 3; ++i) { g->d_hx_cl[i] = nullptr; g->d_hx_rc[i] = nullptr; }
    g->hx_cap_v = 0;
    KC_CUDA(cudaMalloc(&g->d_hx_cnt, sizeof(uint32_t) * (V + 4)));
    KC_CUDA(cudaMalloc(&g->d_hx_old, sizeof(uint32_t) * (V + 4)));
    KC_CUDA(cudaMalloc(&g->d_hx_act, sizeof(uint32_t) * (E + 4)));
    KC_CUDA(cudaMalloc(&g->d_hx_alo, sizeof(uint32_t) * (V + 4)));
    KC_CUDA(cudaMalloc(&g->d_hx_alen, sizeof(uint32_t) * (V + 4)));
    for (int i = 0; i < 2; ++i) {
        KC_CUDA(cudaMalloc(&g->d_hx_slots[i], sizeof(HxSlot) * cap_l));
        KC_CUDA(cudaMalloc(&g->d_hx_bins[i], sizeof(uint32_t) * kHxBinWords * cap_l));
        KC_CUDA(cudaMalloc(&g->d_hx_bt[i], sizeof(unsigned long long) * cap_bt));
    }
    for (int i = 0; i < 3; ++i) {
        KC_CUDA(cudaMalloc(&g->d_hx_cl[i], sizeof(unsigned long long) * cap_cl));
        KC_CUDA(cudaMalloc(&g->d_hx_rc[i], sizeof(uint32_t) * cap_l));
    }
    g->hx_cap_v = (uint32_t)V;
    g->hx_cap_l = (uint32_t)cap_l;
    g->hx_cap_cl = (uint32_t)cap_cl;
    g->hx_cap_bt = (uint32_t)cap_bt;
    return KC_OK;
}

// The cluster h-index kernel (kc_hxtail.cu) on device `dev`: its
// shared-memory and 16-CTA cluster opt-ins set, or null where such a cluster
// cannot run.
const void* hxcluster_kernel(int dev) {
    static std::mutex mu;
    static std::vector<int> state;   // 0 unknown, 1 usable, 2 not
    std::lock_guard<std::mutex> lk(mu);
    if ((int)state.size() <= dev) state.resize(dev + 1, 0);
    if (state[dev] == 0) {
        const void* fn = peel_hxtail_fn();
        bool ok = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)peel_hxtail_smem()) ==
                      cudaSuccess &&
                  cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
        if (ok) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(peel_hxtail_cluster());
            cfg.blockDim = dim3(peel_hxtail_threads());
            cfg.dynamicSmemBytes = peel_hxtail_smem();
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = peel_hxtail_cluster();
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nc = 0;
            ok = cudaOccupancyMaxActiveClusters(&nc, fn, &cfg) == cudaSuccess && nc >= 1;
        }
        cudaGetLastError();   // (a refused opt-in is not an error of the next call)
        state[dev] = ok ? 1 : 2;
    }
    return state[dev] == 1 ? peel_hxtail_fn() : nullptr;
}

// The cluster kernel for the level peel's tails, or null: KC_TAIL=hindex
// (read once per process) sends the tails to it; by default every tail goes
// to the level tail, which measured faster on the benchmark graphs.
const void* hxtail_kernel(int dev) {
    static const bool on = [] {
        const char* e = std::getenv("KC_TAIL");
        return e && std::strcmp(e, "hindex") == 0;
    }();
    return on ? hxcluster_kernel(dev) : nullptr;
}

// The cluster kernel for the h-index peel's hand-off, or null: on by default,
// KC_HX_HANDOFF=0 (read once per process) leaves every iteration to the
// h-index kernel.
const void* hxhandoff_kernel(int dev) {
    static const bool on = [] {
        const char* e = std::getenv("KC_HX_HANDOFF");
        return !(e && std::strcmp(e, "0") == 0);
    }();
    return on ? hxcluster_kernel(dev) : nullptr;
}

// When the h-index peel tries the hand-off: once its frontier holds at most
// KC_HX_HO_FRONT vertices (default 256), with S of at most KC_HX_HO_N
// vertices (default and largest kHoV); read once per process.
void handoff_limits(uint32_t& front, uint32_t& nmax) {
    static uint32_t f = 256, m = kHoV;
    static std::once_flag once;
    std::call_once(once, [] {
        if (const char* e = std::getenv("KC_HX_HO_FRONT")) {
            const long long x = std::atoll(e);
            if (x >= 1 && x <= (1ll << 31)) f = (uint32_t)x;
        }
        if (const char* e = std::getenv("KC_HX_HO_N")) {
            const long long x = std::atoll(e);
            if (x >= 1 && x <= (long long)kHoV) m = (uint32_t)x;
        }
    });
    front = f;
    nmax = m;
}

// Launches the cluster kernel on the stream.
int launch_hxcluster(const void* fn, PeelArgs* a, cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(peel_hxtail_cluster());
    cfg.blockDim = dim3(peel_hxtail_threads());
    cfg.dynamicSmemBytes = peel_hxtail_smem();
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = peel_hxtail_cluster();
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    void* args[] = {a};
    KC_CUDA(cudaLaunchKernelExC(&cfg, fn, args));
    return KC_OK;
}

// Iterations after which the cluster h-index tail leaves the survivors to the
// level tail (KC_HX_TAIL_ITERS, default 512).
uint32_t hxtail_max_iters() {
    static uint32_t n = 512;
    static std::once_flag once;
    std::call_once(once, [] {
        if (const char* e = std::getenv("KC_HX_TAIL_ITERS")) {
            const long long x = std::atoll(e);
            if (x >= 1 && x <= (1 << 24)) n = (uint32_t)x;
        }
    });
    return n;
}

// The tail kernel with its shared-memory opt-in set on device `dev`.
const void* tail_kernel(int dev) {
    static std::mutex mu;
    static std::vector<char> done;
    std::lock_guard<std::mutex> lk(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, 0);
    if (!done[dev]) {
        cudaFuncSetAttribute(peel_tail_fn(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)peel_tail_smem());
        done[dev] = 1;
    }
    return peel_tail_fn();
}

// (Re)allocates device buffers for a graph of V vertices / E arcs.
int reserve(kc_graph* g, uint32_t V, uint64_t E) {
    const uint32_t Vpad = (V + 127u) / 128u * 128u;
    if (V > g->cap_V || !g->d_off) {
        cudaFree(g->d_off); cudaFree(g->d_w); cudaFree(g->d_core); cudaFree(g->d_order);
        cudaFree(g->d_shells); cudaFree(g->d_alive[0]); cudaFree(g->d_alive[1]);
        g->d_off = g->d_w = g->d_core = g->d_order = g->d_shells = nullptr;
        g->d_alive[0] = g->d_alive[1] = nullptr;
        KC_CUDA(cudaMalloc(&g->d_off, sizeof(uint32_t) * ((size_t)Vpad + 4)));
        KC_CUDA(cudaMalloc(&g->d_w, sizeof(uint32_t) * ((size_t)Vpad + 4)));
        KC_CUDA(cudaMalloc(&g->d_core, sizeof(uint32_t) * ((size_t)Vpad + 4)));
        KC_CUDA(cudaMalloc(&g->d_alive[0], sizeof(uint32_t) * ((size_t)Vpad + 4)));
        KC_CUDA(cudaMalloc(&g->d_alive[1], sizeof(uint32_t) * ((size_t)Vpad + 4)));
        g->cap_V = V;
    }
    if (E > g->cap_E || !g->d_nbr) {
        cudaFree(g->d_nbr);
        g->d_nbr = nullptr;
        KC_CUDA(cudaMalloc(&g->d_nbr, sizeof(uint32_t) * (E ? E : 1)));
        g->cap_E = E;
    }
    const unsigned long long tc = task_capacity(g->cap_V, g->cap_E);
    if (tc > g->task_cap || !g->d_tasks) {
        cudaFree(g->d_tasks);
        g->d_tasks = nullptr;
        KC_CUDA(cudaMalloc(&g->d_tasks, sizeof(unsigned long long) * tc));
        KC_CUDA(cudaMemsetAsync(g->d_tasks, 0, sizeof(unsigned long long) * tc, g->stream));
        g->task_cap = tc;
        g->epoch = 0;
    }
    return reserve_tail(g, g->cap_E);
}

int graph_create(kc_graph** out) {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        set_error_msg("no CUDA device is available");
        return KC_ERR_NODEV;
    }
    kc_graph* g = new kc_graph();
    KC_CUDA(cudaGetDevice(&g->dev));
    KC_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    g->own_stream = true;
    KC_CUDA(cudaEventCreate(&g->ev0));
    KC_CUDA(cudaEventCreate(&g->ev1));
    KC_CUDA(cudaMalloc(&g->d_ctl, sizeof(PeelCtl)));
    KC_CUDA(cudaMallocHost(&g->h_ctl, sizeof(PeelCtl)));
    std::memset(g->h_ctl, 0, sizeof(PeelCtl));
    KC_CUDA(cudaMallocHost(&g->h_ctl_init, sizeof(PeelCtl)));
    std::memset(g->h_ctl_init, 0, sizeof(PeelCtl));
    for (auto& sl : g->h_ctl_init->slot) sl.min_next = 0xFFFFFFFFu;
    g->grid = persistent_grid(g->dev);
    *out = g;
    return KC_OK;
}

// Uploads a host CSR.  With host_validate the offsets and neighbour ids are
// checked here (an invalid graph is refused at upload); without it the
// device checks them after the upload, before the next peel touches them
// (kc_validate.cu), and that peel reports KC_ERR_INVALID.
int graph_load(kc_graph* g, const uint32_t* off, const uint32_t* nbr, uint32_t V, bool host_validate = true) {
    const uint64_t E = V ? off[V] : 0;
    if (V && off[0] != 0) { set_error_msg("offsets[0] must be 0"); return KC_ERR_INVALID; }
    autotune(off, V, &g->tune);
    if (!host_validate) {
        int rc = reserve(g, V, E);
        if (rc) return rc;
        g->V = V;
        g->E = E;
        g->maxdeg = kFull;   // found by the device validation
        if (V) KC_CUDA(cudaMemcpyAsync(g->d_off, off, sizeof(uint32_t) * ((size_t)V + 1), cudaMemcpyHostToDevice, g->stream));
        if (E) KC_CUDA(cudaMemcpyAsync(g->d_nbr, nbr, sizeof(uint32_t) * E, cudaMemcpyHostToDevice, g->stream));
        g->ran = false;
        return KC_OK;
    }
    uint32_t maxdeg = 0;
    for (uint32_t v = 0; v < V; ++v) {
        if (off[v + 1] < off[v]) { set_error_msg("offsets must be non-decreasing"); return KC_ERR_INVALID; }
        maxdeg = std::max(maxdeg, off[v + 1] - off[v]);
    }
    if (maxdeg >= kBias) { set_error_msg("a degree above 2^30 is not supported"); return KC_ERR_INVALID; }
    // Every neighbour id must name a vertex: the kernels index the state array
    // with it.
    uint32_t bad = 0;
#pragma omp parallel for reduction(| : bad) schedule(static)
    for (int64_t j = 0; j < (int64_t)E; ++j) bad |= (nbr[j] >= V);
    if (bad) { set_error_msg("a neighbour id is >= V"); return KC_ERR_INVALID; }
    int rc = reserve(g, V, E);
    if (rc) return rc;
    g->V = V;
    g->E = E;
    g->maxdeg = maxdeg;
    if (V) KC_CUDA(cudaMemcpyAsync(g->d_off, off, sizeof(uint32_t) * ((size_t)V + 1), cudaMemcpyHostToDevice, g->stream));
    if (E) KC_CUDA(cudaMemcpyAsync(g->d_nbr, nbr, sizeof(uint32_t) * E, cudaMemcpyHostToDevice, g->stream));
    g->ran = false;
    return KC_OK;
}

int graph_launch(kc_graph* g, bool with_order, bool with_trace = false) {
    KC_CUDA(cudaSetDevice(g->dev));
    g->with_order = with_order;
    const bool device_validate = g->maxdeg == kFull;
    if (device_validate && (with_order || with_trace)) {
        set_error_msg("peel order and trace need a graph validated at upload");
        return KC_ERR_INVALID;
    }
    if (g->V == 0) {   // the reference loop never runs: kmax = level-1 = 0xFFFFFFFF
        std::memset(g->h_ctl, 0, sizeof(PeelCtl));
        g->h_ctl->kmax = 0xFFFFFFFFu;
        g->h_ctl->levels = 0;
        g->pending = false;
        g->ran = true;
        KC_CUDA(cudaEventRecord(g->ev0, g->stream));
        KC_CUDA(cudaEventRecord(g->ev1, g->stream));
        return KC_OK;
    }
    if (with_order) {
        const uint32_t sc = g->maxdeg + 2;
        if (!g->d_order || sc > g->shell_cap) {
            cudaFree(g->d_order); cudaFree(g->d_shells);
            g->d_order = g->d_shells = nullptr;
            KC_CUDA(cudaMalloc(&g->d_order, sizeof(uint32_t) * ((size_t)g->cap_V + 4)));
            KC_CUDA(cudaMalloc(&g->d_shells, sizeof(uint32_t) * sc));
            g->shell_cap = sc;
        }
    }
    if (with_trace) {
        const uint32_t tc = g->maxdeg + 2;
        if (!g->d_trace || tc > g->trace_cap) {
            cudaFree(g->d_trace);
            g->d_trace = nullptr;
            KC_CUDA(cudaMalloc(&g->d_trace, sizeof(unsigned long long) * kTraceFields * tc));
            g->trace_cap = tc;
        }
        KC_CUDA(cudaMemsetAsync(g->d_trace, 0, sizeof(unsigned long long) * kTraceFields * g->trace_cap, g->stream));
    }
    g->epoch = g->epoch % 255u + 1u;
    if (g->epoch == 1u)
        KC_CUDA(cudaMemsetAsync(g->d_tasks, 0, sizeof(unsigned long long) * g->task_cap, g->stream));
    KC_CUDA(cudaMemcpyAsync(g->d_ctl, g->h_ctl_init, sizeof(PeelCtl), cudaMemcpyHostToDevice, g->stream));
    KC_CUDA(cudaEventRecord(g->ev0, g->stream));
    if (device_validate && launch_validate_csr(g->d_off, g->d_nbr, g->V, g->E, g->d_ctl, g->stream)) {
        set_error_msg("CSR validation kernel launch failed");
        return KC_ERR_CUDA;
    }
    PeelArgs a;
    a.off = g->d_off;
    a.nbr = g->d_nbr;
    a.w = g->d_w;
    a.core = g->d_core;
    a.order = with_order ? g->d_order : nullptr;
    a.shells = with_order ? g->d_shells : nullptr;
    a.tasks = g->d_tasks;
    a.ctl = g->d_ctl;
    a.task_cap = g->task_cap;
    a.V = g->V;
    a.shell_cap = with_order ? g->shell_cap : 0;
    a.max_level = g->maxdeg;
    a.epoch = g->epoch;
    a.wait_us = wait_limit_us();
    a.E = (uint32_t)g->E;
    a.zero_tasks = 0;   // the queue is cleared by a memset when the tag epoch wraps
    a.alive[0] = g->d_alive[0];
    a.alive[1] = g->d_alive[1];
    a.trace = with_trace ? g->d_trace : nullptr;
    a.trace_cap = with_trace ? g->trace_cap : 0;
    a.local_budget = g->tune.local_budget;
    a.hub_arcs = g->tune.hub_arcs;
    a.chunk_arcs = g->tune.chunk_arcs;
    a.claim_cas = claim_cas();
    const bool tail = g->tail_cap_v != 0 && g->tune.tail_v != 0;
    if (tail) {
        a.tail_cap_v = std::min(g->tail_cap_v, g->tune.tail_v);
        a.tail_cap_arcs = g->tail_cap_arcs;
        a.tail_ids = g->d_tail_ids;
        a.tail_off = g->d_tail_off;
        a.tail_cur = g->d_tail_cur;
        a.tail_nbr = g->d_tail_nbr;
        a.tail_items = g->d_tail_items;
        a.tail_items_cap = g->tail_items_cap;
    }
    // The h-index peel first (not for the peel order, the per-level trace or the
    // bounds-checked build, which follow the level peel); the persistent kernel
    // returns at once when it solved the graph.
    const bool hindex = g->method == KC_METHOD_HINDEX || (g->method == KC_METHOD_AUTO && hindex_default());
    // (vertex ids below 2^31: the h-index frontier tags entries with the top bit)
    if (hindex && !with_order && !with_trace && !checked_mode() && g->V < 0x80000000u) {
        int rc = reserve_hx(g);
        if (rc) return rc;
        HxArgs h;
        h.off = g->d_off;
        h.nbr = g->d_nbr;
        h.est = g->d_core;
        h.cnt = g->d_hx_cnt;
        h.old = g->d_hx_old;
        h.act = g->d_hx_act;
        h.alo = g->d_hx_alo;
        h.alen = g->d_hx_alen;
        h.rm[0] = g->d_alive[0];
        h.rm[1] = g->d_alive[1];
        for (int i = 0; i < 2; ++i) { h.slots[i] = g->d_hx_slots[i]; h.bins[i] = g->d_hx_bins[i]; h.bt[i] = g->d_hx_bt[i]; }
        for (int i = 0; i < 3; ++i) { h.cl[i] = g->d_hx_cl[i]; h.rc[i] = g->d_hx_rc[i]; }
        h.ctl = g->d_ctl;
        h.V = g->V;
        h.E = (uint32_t)g->E;
        h.cap_l = g->hx_cap_l;
        h.cap_cl = g->hx_cap_cl;
        h.cap_bt = g->hx_cap_bt;
        h.max_iters = hindex_max_iters();
        h.wait_us = wait_limit_us();
        h.max_level = g->maxdeg;
        h.w = g->d_w;
        h.after_peel = 0;
        // the hand-off to the cluster kernel (not after a level peel, whose
        // peeled vertices keep no counts)
        const void* hof = !hindex_start() ? hxhandoff_kernel(g->dev) : nullptr;
        h.handoff = hof ? 1u : 0u;
        h.lmap = g->d_hx_old;
        // (buffers of its own, not the level tail's: KC_TAIL_V does not touch it)
        h.tail_ids = g->d_hx_tail + 2 * kHoV;
        h.tail_cur = g->d_hx_tail + 3 * kHoV;
        h.tail_off = g->d_hx_tail + 4 * kHoV;   // kHoV + 4 entries
        h.tail_nbr = g->d_hx_tnbr;
        h.tail_est = g->d_hx_tail;
        h.tail_cnt = g->d_hx_tail + kHoV;
        h.tail_cap_arcs = g->hx_tnbr_cap;
        handoff_limits(h.ho_front, h.ho_max);
        if (const uint32_t n = hindex_start()) {
            // The level peel's first levels, until at most V/n vertices survive
            // (no tail hand-off).  It tags its task entries with its own epoch,
            // so the fallback level peel below, which starts over, takes none
            // of them for its own.
            PeelArgs a0 = a;
            a0.stop_alive = std::max<uint32_t>(1u, g->V / n);
            a0.tail_cap_v = 0;
            a0.epoch = g->epoch;
            g->epoch = g->epoch % 255u + 1u;
            if (g->epoch == 1u)
                KC_CUDA(cudaMemsetAsync(g->d_tasks, 0, sizeof(unsigned long long) * g->task_cap, g->stream));
            a.epoch = g->epoch;
            void* a0args[] = {&a0};
            KC_CUDA(cudaLaunchCooperativeKernel(peel_kernel(), dim3(g->grid), dim3(kPeelThreads), a0args, 0, g->stream));
            h.after_peel = 1;
        }
        void* hargs[] = {&h};
        KC_CUDA(cudaLaunchCooperativeKernel(peel_hindex_fn(), dim3(g->grid), dim3(kPeelThreads), hargs, 0, g->stream));
        if (hof) {   // returns at once unless the h-index kernel handed over
            PeelArgs ah = a;
            ah.tail_est = h.tail_est;
            ah.tail_cnt = h.tail_cnt;
            ah.tail_nbr = h.tail_nbr;
            ah.tail_ids = h.tail_ids;
            ah.tail_off = h.tail_off;
            ah.tail_cur = h.tail_cur;
            ah.tail_hx_iters = hxtail_max_iters();
            const int rc = launch_hxcluster(hof, &ah, g->stream);
            if (rc) return rc;
        }
    }
    // The survivors handed over go to the cluster h-index tail first (not for
    // the peel order or the per-level trace, which follow the level tail);
    // the level tail kernel returns at once when it finished them.
    const void* hxt = (tail && !with_order && !with_trace) ? hxtail_kernel(g->dev) : nullptr;
    a.tail_hx_iters = hxt ? hxtail_max_iters() : 0u;
    void* args[] = {&a};
    KC_CUDA(cudaLaunchCooperativeKernel(peel_kernel(), dim3(g->grid), dim3(kPeelThreads), args, 0, g->stream));
    if (hxt) {
        const int rc = launch_hxcluster(hxt, &a, g->stream);
        if (rc) return rc;
    }
    if (tail)
        KC_CUDA(cudaLaunchKernel(tail_kernel(g->dev), dim3(1), dim3(kTailThreads), args, peel_tail_smem(), g->stream));
    KC_CUDA(cudaEventRecord(g->ev1, g->stream));
    KC_CUDA(cudaMemcpyAsync(g->h_ctl, g->d_ctl, sizeof(PeelCtl), cudaMemcpyDeviceToHost, g->stream));
    g->pending = true;
    g->ran = true;
    return KC_OK;
}

int graph_finish(kc_graph* g, kc_stats* st) {
    KC_CUDA(cudaSetDevice(g->dev));
    if (!g->ran) { set_error_msg("no peel has been run on this graph"); return KC_ERR_INVALID; }
    KC_CUDA(cudaStreamSynchronize(g->stream));
    g->pending = false;
    if (g->h_ctl->err == kErrInvalid) {
        set_error_msg("invalid CSR: offsets must start at 0 and not decrease, neighbour ids must be < V, "
                      "degrees below 2^30");
        return KC_ERR_INVALID;
    }
    if (g->h_ctl->err) {
        std::string m = std::string("device peel failed at level ") + std::to_string(g->h_ctl->err_level);
        if (g->h_ctl->err == kErrCheck)
            m += ": out-of-bounds index " + std::to_string(g->h_ctl->err_index) + " at access site " +
                 std::to_string(g->h_ctl->err_site) + " (skipped)";
        set_error_msg(m);
        return g->h_ctl->err == kErrCheck ? KC_ERR_OVERFLOW : g->h_ctl->err;
    }
    if (st) {
        float ms = 0;
        cudaEventElapsedTime(&ms, g->ev0, g->ev1);
        st->V = g->V;
        st->kmax = g->h_ctl->kmax;
        st->levels = g->h_ctl->hx.solved ? g->h_ctl->kmax + 1 : g->h_ctl->levels;
        st->iterations = g->h_ctl->iterations;
        st->blocks = (uint32_t)g->grid;
        st->arcs = g->E;
        st->tasks = g->h_ctl->tasks;
        st->method = g->h_ctl->hx.solved ? 1u : 0u;
        st->peel_ms = ms;
    }
    return KC_OK;
}

std::mutex g_oneshot_mu;
std::vector<kc_graph*> g_oneshot;   // per device

}  // namespace

extern "C" {

const char* kc_strerror(int code) {
    switch (code) {
        case KC_OK: return "ok";
        case KC_ERR_IO: return "i/o error";
        case KC_ERR_PARSE: return "parse error";
        case KC_ERR_OOM: return "out of memory";
        case KC_ERR_OVERFLOW: return "queue or size overflow";
        case KC_ERR_TIMEOUT: return "bounded device wait timed out";
        case KC_ERR_CUDA: return "CUDA error";
        case KC_ERR_BUDGET: return "request exceeds the HBM budget";
        case KC_ERR_INVALID: return "invalid argument";
        case KC_ERR_NODEV: return "no CUDA device";
        case KC_ERR_BUSY: return "busy / not ready";
        case KC_ERR_CLOSED: return "closed";
        default: return "unknown error";
    }
}

int kc_graph_upload(const uint32_t* off, const uint32_t* nbr, uint32_t V, kc_graph** out) {
    if (!out || (V && (!off || (off[V] && !nbr)))) { set_error_msg("null argument"); return KC_ERR_INVALID; }
    *out = nullptr;
    kc_graph* g = nullptr;
    int rc = graph_create(&g);
    if (rc) { if (g) { release(g); delete g; } return rc; }
    rc = graph_load(g, off, nbr, V);
    if (rc == KC_OK) {
        cudaError_t e = cudaStreamSynchronize(g->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "upload");
    }
    if (rc) { release(g); delete g; return rc; }
    *out = g;
    return KC_OK;
}

int kc_graph_set_method(kc_graph* g, uint32_t method) {
    if (!g || method > KC_METHOD_PEEL) { set_error_msg("unknown method"); return KC_ERR_INVALID; }
    g->method = method;
    return KC_OK;
}

int kc_graph_set_stream(kc_graph* g, void* stream) {
    if (!g) return KC_ERR_INVALID;
    cudaSetDevice(g->dev);
    if (g->stream) cudaStreamSynchronize(g->stream);
    if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
    if (stream) {
        g->stream = (cudaStream_t)stream;
        g->own_stream = false;
    } else {
        KC_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
        g->own_stream = true;
    }
    return KC_OK;
}

int kc_graph_peel_async(kc_graph* g) {
    if (!g) return KC_ERR_INVALID;
    return graph_launch(g, false);
}

int kc_graph_fetch(kc_graph* g, uint32_t* core_out, uint32_t* kmax, kc_stats* st) {
    if (!g) return KC_ERR_INVALID;
    int rc = graph_finish(g, st);
    if (rc) return rc;
    if (core_out && g->V)
        KC_CUDA(cudaMemcpy(core_out, g->d_core, sizeof(uint32_t) * g->V, cudaMemcpyDeviceToHost));
    if (kmax) *kmax = g->h_ctl->kmax;
    return KC_OK;
}

int kc_peel(kc_graph* g, uint32_t* core_out, uint32_t* kmax, kc_stats* st) {
    if (!g) return KC_ERR_INVALID;
    auto t0 = std::chrono::steady_clock::now();
    int rc = graph_launch(g, false);
    if (rc) return rc;
    rc = kc_graph_fetch(g, core_out, kmax, st);
    if (st) st->total_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int kc_degeneracy_order(kc_graph* g, uint32_t* order_out, uint32_t* shells_out, uint32_t shell_cap,
                        uint32_t* kmax) {
    if (!g) return KC_ERR_INVALID;
    int rc = graph_launch(g, true);
    if (rc) return rc;
    rc = graph_finish(g, nullptr);
    if (rc) return rc;
    const uint32_t km = g->h_ctl->kmax;
    if (kmax) *kmax = km;
    if (g->V == 0) {
        if (shells_out && shell_cap) shells_out[0] = 0;
        return KC_OK;
    }
    if (order_out) KC_CUDA(cudaMemcpy(order_out, g->d_order, sizeof(uint32_t) * g->V, cudaMemcpyDeviceToHost));
    if (shells_out) {
        const uint32_t need = km + 2;
        if (shell_cap < need) { set_error_msg("shell_offsets_out needs kmax+2 entries"); return KC_ERR_INVALID; }
        KC_CUDA(cudaMemcpy(shells_out, g->d_shells, sizeof(uint32_t) * need, cudaMemcpyDeviceToHost));
    }
    return KC_OK;
}

int kc_graph_trace(kc_graph* g, uint64_t* out, uint32_t level_cap, uint32_t* levels) {
    if (!g || !out) return KC_ERR_INVALID;
    int rc = graph_launch(g, false, true);
    if (rc) return rc;
    rc = graph_finish(g, nullptr);
    if (rc) return rc;
    const uint32_t lv = g->h_ctl->iterations;
    if (levels) *levels = lv;
    const uint32_t n = std::min(lv, level_cap);
    if (n) KC_CUDA(cudaMemcpy(out, g->d_trace, sizeof(uint64_t) * kTraceFields * n, cudaMemcpyDeviceToHost));
    return KC_OK;
}

int kc_graph_device_ptrs(kc_graph* g, const uint32_t** d_off, const uint32_t** d_nbr, uint32_t** d_core) {
    if (!g) return KC_ERR_INVALID;
    if (d_off) *d_off = g->d_off;
    if (d_nbr) *d_nbr = g->d_nbr;
    if (d_core) *d_core = g->d_core;
    return KC_OK;
}

void kc_graph_free(kc_graph* g) {
    if (!g) return;
    release(g);
    delete g;
}

int kc_peel_csr(const uint32_t* off, const uint32_t* nbr, uint32_t V, uint32_t* core_out, uint32_t* kmax) {
    if (V && (!off || !core_out || (off[V] && !nbr))) { set_error_msg("null argument"); return KC_ERR_INVALID; }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    std::lock_guard<std::mutex> lk(g_oneshot_mu);
    if ((int)g_oneshot.size() <= dev) g_oneshot.resize(dev + 1, nullptr);
    if (!g_oneshot[dev]) {
        int rc = graph_create(&g_oneshot[dev]);
        if (rc) return rc;
    }
    kc_graph* g = g_oneshot[dev];
    int rc = graph_load(g, off, nbr, V, /*host_validate=*/false);
    if (rc) return rc;
    rc = graph_launch(g, false);
    if (rc) return rc;
    rc = graph_finish(g, nullptr);
    if (rc) return rc;
    if (V) KC_CUDA(cudaMemcpyAsync(core_out, g->d_core, sizeof(uint32_t) * V, cudaMemcpyDeviceToHost, g->stream));
    KC_CUDA(cudaStreamSynchronize(g->stream));
    if (kmax) *kmax = g->h_ctl->kmax;
    return KC_OK;
}

int kc_autotune(const uint32_t* offsets, uint32_t V, kc_tuning* out) {
    if (!out || (V && !offsets)) { set_error_msg("null argument"); return KC_ERR_INVALID; }
    autotune(offsets, V, out);
    return KC_OK;
}

int kc_device_info(int* sms, int* grid, int* cc_major, int* cc_minor) {
    int dev = 0, n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { set_error_msg("no CUDA device"); return KC_ERR_NODEV; }
    KC_CUDA(cudaGetDevice(&dev));
    if (sms) cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
    if (cc_major) cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev);
    if (cc_minor) cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (grid) *grid = persistent_grid(dev);
    return KC_OK;
}

void* kc_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) return nullptr;
    return p;
}

void kc_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
