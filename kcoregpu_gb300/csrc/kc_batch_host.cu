// Host side of the batched peel: segmented CSR upload, the autotuner, the
// batched launch, the one-graph-per-launch baseline and the batch generator.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>
#include <omp.h>

#include "kc_batch.cuh"
#include "kc_internal.h"
#include "kc_peel.cuh"

using namespace kc;

namespace kc {
int cuda_fail(cudaError_t e, const char* what);
}

#define KC_CUDA(call)                                       \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// Per-graph plan chosen by the autotuner.
struct GraphPlan {
    uint32_t V;
    uint64_t E;
    uint32_t maxdeg;
    uint32_t hindex;   // h-index of the degree sequence: an upper bound on kmax
    double cost;       // estimated work (arcs walked + state reads over the levels)
};

struct kc_batch {
    int dev = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint32_t ngraphs = 0;
    uint64_t Vtot = 0, Etot = 0;
    std::vector<unsigned long long> vbase, abase;
    std::vector<GraphPlan> plan;
    std::vector<uint32_t> schedule;   // graphs for the batched kernel, largest first
    std::vector<uint32_t> giants;     // graphs run with the grid-wide peel instead
    uint32_t qcap = 0;                // queue entries per CTA (max V of the batched graphs)
    int grid = 0;                     // CTAs of the batched kernel
    uint32_t bits_cap = 0;            // vertices of the per-CTA peeled bitmap (shared memory)
    size_t bits_bytes = 0;            // its dynamic shared memory
    // device
    unsigned long long *d_vbase = nullptr, *d_abase = nullptr;
    uint32_t *d_off = nullptr, *d_nbr = nullptr, *d_core = nullptr, *d_kmax = nullptr, *d_levels = nullptr;
    uint32_t *d_sched = nullptr, *d_next = nullptr, *d_queues = nullptr;
    int* d_err = nullptr;
    // scratch of the grid-wide peel (giants and the per-graph baseline)
    uint32_t gV = 0;
    uint64_t gE = 0;
    uint32_t *d_gw = nullptr, *d_galive0 = nullptr, *d_galive1 = nullptr;
    unsigned long long* d_gtasks = nullptr;
    unsigned long long gtask_cap = 0;
    PeelCtl* d_gctl = nullptr;
    PeelCtl* h_gctl_init = nullptr;
    uint32_t gepoch = 0;
    int ggrid = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_ms = 0;
};

namespace {

uint32_t h_index(const uint32_t* off, uint32_t V) {
    // largest h such that at least h vertices have degree >= h
    std::vector<uint32_t> cnt(V + 2, 0);
    for (uint32_t v = 0; v < V; ++v) cnt[std::min(off[v + 1] - off[v], V + 1)]++;
    uint32_t acc = 0;
    for (uint32_t h = V + 1; h > 0; --h) {
        acc += cnt[h];
        if (acc >= h) return h;
    }
    return 0;
}

// The autotuner: from each graph's degree histogram (V, E, max degree,
// h-index) estimate its peel cost, order graphs largest first (LPT over the
// CTAs), route graphs too large for one CTA to the grid-wide peel, size the
// per-CTA queue for the largest remaining graph and pick CTAs per SM.
void autotune(kc_batch* b, int sms, int per_sm) {
    const size_t G = b->ngraphs;
    double total = 0;
    for (auto& p : b->plan) {
        // scans: one pass over V per level while many vertices remain, i.e. about
        // min(h, 32) passes; walks: every arc once
        p.cost = (double)p.E + (double)p.V * (double)std::min<uint32_t>(p.hindex + 1, 32) * 0.25;
        total += p.cost;
    }
    const int ctas = std::max(1, sms * per_sm);
    // a graph whose estimated cost exceeds eight times one CTA's even share of
    // the batch runs grid-wide (alone on one CTA it would dominate the tail)
    const double giant = std::max(4.0e6, 8.0 * total / ctas);
    std::vector<uint32_t> ids(G);
    std::iota(ids.begin(), ids.end(), 0u);
    std::stable_sort(ids.begin(), ids.end(), [&](uint32_t x, uint32_t y) { return b->plan[x].cost > b->plan[y].cost; });
    b->schedule.clear();
    b->giants.clear();
    b->qcap = 1;
    for (uint32_t g : ids) {
        if (b->plan[g].cost > giant && b->plan[g].V > 4096) b->giants.push_back(g);
        else {
            b->schedule.push_back(g);
            b->qcap = std::max(b->qcap, b->plan[g].V);
        }
    }
    // fewer graphs than CTA slots: one CTA per graph is enough
    b->grid = (int)std::min<size_t>((size_t)ctas, std::max<size_t>(1, b->schedule.size()));
}

void release(kc_batch* b) {
    if (!b) return;
    cudaSetDevice(b->dev);
    if (b->stream) cudaStreamSynchronize(b->stream);
    cudaFree(b->d_vbase); cudaFree(b->d_abase); cudaFree(b->d_off); cudaFree(b->d_nbr);
    cudaFree(b->d_core); cudaFree(b->d_kmax); cudaFree(b->d_levels); cudaFree(b->d_sched);
    cudaFree(b->d_next); cudaFree(b->d_queues); cudaFree(b->d_err);
    cudaFree(b->d_gw); cudaFree(b->d_galive0); cudaFree(b->d_galive1); cudaFree(b->d_gtasks);
    cudaFree(b->d_gctl);
    if (b->h_gctl_init) cudaFreeHost(b->h_gctl_init);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
}

// Scratch for running the grid-wide persistent peel on single graphs of the batch.
int reserve_grid_scratch(kc_batch* b, uint32_t V, uint64_t E) {
    if (V <= b->gV && E <= b->gE && b->d_gw) return KC_OK;
    b->gV = std::max(b->gV, V);
    b->gE = std::max(b->gE, E);
    const size_t Vpad = (size_t)(b->gV + 127) / 128 * 128 + 4;
    cudaFree(b->d_gw); cudaFree(b->d_galive0); cudaFree(b->d_galive1); cudaFree(b->d_gtasks);
    KC_CUDA(cudaMalloc(&b->d_gw, 4 * Vpad));
    KC_CUDA(cudaMalloc(&b->d_galive0, 4 * Vpad));
    KC_CUDA(cudaMalloc(&b->d_galive1, 4 * Vpad));
    b->gtask_cap = (unsigned long long)b->gV + b->gE / kChunk + 64;
    KC_CUDA(cudaMalloc(&b->d_gtasks, 8 * b->gtask_cap));
    KC_CUDA(cudaMemsetAsync(b->d_gtasks, 0, 8 * b->gtask_cap, b->stream));
    b->gepoch = 0;
    if (!b->d_gctl) {
        KC_CUDA(cudaMalloc(&b->d_gctl, sizeof(PeelCtl)));
        KC_CUDA(cudaMallocHost(&b->h_gctl_init, sizeof(PeelCtl)));
        std::memset(b->h_gctl_init, 0, sizeof(PeelCtl));
        for (auto& sl : b->h_gctl_init->slot) sl.min_next = 0xFFFFFFFFu;
    }
    return KC_OK;
}

// Stream-ordered grid-wide peel of graph g (core numbers into its output slice).
int launch_single(kc_batch* b, uint32_t g) {
    const GraphPlan& p = b->plan[g];
    uint32_t* core = b->d_core + b->vbase[g];
    if (p.V == 0) {   // kmax = level-1 = 0xFFFFFFFF, as the reference loop computes it
        KC_CUDA(cudaMemsetAsync(b->d_kmax + g, 0xFF, 4, b->stream));
        KC_CUDA(cudaMemsetAsync(b->d_levels + g, 0, 4, b->stream));
        return KC_OK;
    }
    b->gepoch = b->gepoch % 255u + 1u;
    if (b->gepoch == 1u) KC_CUDA(cudaMemsetAsync(b->d_gtasks, 0, 8 * b->gtask_cap, b->stream));
    KC_CUDA(cudaMemcpyAsync(b->d_gctl, b->h_gctl_init, sizeof(PeelCtl), cudaMemcpyHostToDevice, b->stream));
    PeelArgs a;
    std::memset(&a, 0, sizeof(a));
    a.local_budget = kLocalBudget;
    a.hub_arcs = kLocalArcs;
    a.chunk_arcs = kChunk;
    a.claim_cas = 1;   // one giant graph on the whole GPU
    a.off = b->d_off + b->vbase[g] + g;
    a.nbr = b->d_nbr + b->abase[g];
    a.w = b->d_gw;
    a.core = core;
    a.tasks = b->d_gtasks;
    a.ctl = b->d_gctl;
    a.task_cap = b->gtask_cap;
    a.V = p.V;
    a.max_level = p.maxdeg;
    a.epoch = b->gepoch;
    a.wait_us = 2000000;   // 2 s
    a.E = (uint32_t)p.E;
    a.alive[0] = b->d_galive0;
    a.alive[1] = b->d_galive1;
    void* args[] = {&a};
    KC_CUDA(cudaLaunchCooperativeKernel(peel_persistent_fn(), dim3(b->ggrid), dim3(kPeelThreads), args, 0, b->stream));
    // kmax of this graph -> the batch's kmax array (device to device)
    KC_CUDA(cudaMemcpyAsync(b->d_kmax + g, &b->d_gctl->kmax, 4, cudaMemcpyDeviceToDevice, b->stream));
    KC_CUDA(cudaMemcpyAsync(b->d_levels + g, &b->d_gctl->iterations, 4, cudaMemcpyDeviceToDevice, b->stream));
    return KC_OK;
}

}  // namespace

extern "C" {

int kc_batch_upload(const kc_segcsr* s, kc_batch** out) {
    if (!s || !out || (s->ngraphs && (!s->vbase || !s->abase || !s->offsets))) {
        set_error_msg("kc_batch_upload: null argument");
        return KC_ERR_INVALID;
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { set_error_msg("no CUDA device is available"); return KC_ERR_NODEV; }
    kc_batch* b = new kc_batch();
    auto fail = [&](int rc) { release(b); delete b; return rc; };
    const uint32_t G = s->ngraphs;
    b->ngraphs = G;
    b->vbase.assign(s->vbase, s->vbase + G + 1);
    b->abase.assign(s->abase, s->abase + G + 1);
    b->Vtot = b->vbase[G];
    b->Etot = b->abase[G];
    b->plan.resize(G);
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : bad)
    for (int64_t g = 0; g < (int64_t)G; ++g) {
        GraphPlan& p = b->plan[g];
        const uint32_t* off = s->offsets + b->vbase[g] + g;
        p.V = (uint32_t)(b->vbase[g + 1] - b->vbase[g]);
        p.E = b->abase[g + 1] - b->abase[g];
        if (off[0] != 0 || off[p.V] != p.E) { bad = 1; continue; }
        p.maxdeg = 0;
        for (uint32_t v = 0; v < p.V; ++v) {
            if (off[v + 1] < off[v]) bad = 1;
            p.maxdeg = std::max(p.maxdeg, off[v + 1] - off[v]);
        }
        const uint32_t* nb = s->neighbors + b->abase[g];
        for (uint64_t j = 0; j < p.E; ++j) if (nb[j] >= p.V) { bad = 1; break; }
        p.hindex = h_index(off, p.V);
    }
    if (bad) { set_error_msg("kc_batch_upload: inconsistent segmented CSR"); return fail(KC_ERR_INVALID); }
    cudaGetDevice(&b->dev);
    int sms = 0, per = 0, gper = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->dev);
    // the peeled-vertex bitmap covers the largest graph, up to kBatchBitsMax
    uint32_t vmax = 0;
    for (const auto& p : b->plan) vmax = std::max(vmax, p.V);
    b->bits_cap = std::min(vmax, kBatchBitsMax);
    b->bits_bytes = (size_t)((b->bits_cap + 31) / 32) * 4;
    // static plus dynamic shared memory may exceed the default 48 KB window
    if (cudaError_t ea = cudaFuncSetAttribute(peel_batch_fn(), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)b->bits_bytes))
        return fail(cuda_fail(ea, "cudaFuncSetAttribute(peel_batch_kernel)"));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, peel_batch_fn(), kBatchThreads, b->bits_bytes);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gper, peel_persistent_fn(), kPeelThreads, 0);
    b->ggrid = gper > 0 ? sms : 0;   // giants: one CTA per SM, as the single-graph peel
    autotune(b, sms, std::max(1, per));
    cudaError_t e;
#define KC_B(call) do { e = (call); if (e != cudaSuccess) return fail(cuda_fail(e, #call)); } while (0)
    KC_B(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    b->own_stream = true;
    KC_B(cudaEventCreate(&b->ev0));
    KC_B(cudaEventCreate(&b->ev1));
    const size_t offn = b->Vtot + G;
    KC_B(cudaMalloc(&b->d_vbase, 8 * (G + 1)));
    KC_B(cudaMalloc(&b->d_abase, 8 * (G + 1)));
    KC_B(cudaMalloc(&b->d_off, 4 * std::max<size_t>(offn, 1)));
    KC_B(cudaMalloc(&b->d_nbr, 4 * std::max<uint64_t>(b->Etot, 1)));
    KC_B(cudaMalloc(&b->d_core, 4 * std::max<uint64_t>(b->Vtot, 1)));
    KC_B(cudaMalloc(&b->d_kmax, 4 * std::max<uint32_t>(G, 1)));
    KC_B(cudaMalloc(&b->d_levels, 4 * std::max<uint32_t>(G, 1)));
    KC_B(cudaMalloc(&b->d_sched, 4 * std::max<size_t>(b->schedule.size(), 1)));
    KC_B(cudaMalloc(&b->d_next, 4));
    KC_B(cudaMalloc(&b->d_err, 4));
    KC_B(cudaMalloc(&b->d_queues, 4 * (size_t)kCtaScratch * b->qcap * b->grid));
    KC_B(cudaMemcpyAsync(b->d_vbase, b->vbase.data(), 8 * (G + 1), cudaMemcpyHostToDevice, b->stream));
    KC_B(cudaMemcpyAsync(b->d_abase, b->abase.data(), 8 * (G + 1), cudaMemcpyHostToDevice, b->stream));
    if (offn) KC_B(cudaMemcpyAsync(b->d_off, s->offsets, 4 * offn, cudaMemcpyHostToDevice, b->stream));
    if (b->Etot) KC_B(cudaMemcpyAsync(b->d_nbr, s->neighbors, 4 * b->Etot, cudaMemcpyHostToDevice, b->stream));
    if (!b->schedule.empty())
        KC_B(cudaMemcpyAsync(b->d_sched, b->schedule.data(), 4 * b->schedule.size(), cudaMemcpyHostToDevice, b->stream));
    if (!b->giants.empty()) {
        uint32_t gv = 0; uint64_t ge = 0;
        for (uint32_t g : b->giants) { gv = std::max(gv, b->plan[g].V); ge = std::max(ge, b->plan[g].E); }
        int rc = reserve_grid_scratch(b, gv, ge);
        if (rc) return fail(rc);
    }
    KC_B(cudaStreamSynchronize(b->stream));
#undef KC_B
    *out = b;
    return KC_OK;
}

int kc_batch_set_stream(kc_batch* b, void* stream) {
    if (!b) return KC_ERR_INVALID;
    cudaSetDevice(b->dev);
    cudaStreamSynchronize(b->stream);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    if (stream) { b->stream = (cudaStream_t)stream; b->own_stream = false; }
    else { KC_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)); b->own_stream = true; }
    return KC_OK;
}

int kc_batch_peel_async(kc_batch* b) {
    if (!b) return KC_ERR_INVALID;
    KC_CUDA(cudaSetDevice(b->dev));
    KC_CUDA(cudaEventRecord(b->ev0, b->stream));
    KC_CUDA(cudaMemsetAsync(b->d_next, 0, 4, b->stream));
    KC_CUDA(cudaMemsetAsync(b->d_err, 0, 4, b->stream));
    for (uint32_t g : b->giants) {
        int rc = launch_single(b, g);
        if (rc) return rc;
    }
    if (!b->schedule.empty()) {
        BatchArgs a;
        a.vbase = b->d_vbase;
        a.abase = b->d_abase;
        a.offsets = b->d_off;
        a.nbr = b->d_nbr;
        a.core = b->d_core;
        a.kmax = b->d_kmax;
        a.levels_run = b->d_levels;
        a.schedule = b->d_sched;
        a.next = b->d_next;
        a.queues = b->d_queues;
        a.err = b->d_err;
        a.ngraphs = (uint32_t)b->schedule.size();
        a.qcap = b->qcap;
        a.bits_cap = b->bits_cap;
        void* args[] = {&a};
        KC_CUDA(cudaLaunchKernel(peel_batch_fn(), dim3(b->grid), dim3(kBatchThreads), args, b->bits_bytes, b->stream));
    }
    KC_CUDA(cudaEventRecord(b->ev1, b->stream));
    return KC_OK;
}

int kc_batch_fetch(kc_batch* b, uint32_t* core_out, uint32_t* kmax_out, kc_batch_stats* st) {
    if (!b) return KC_ERR_INVALID;
    KC_CUDA(cudaSetDevice(b->dev));
    KC_CUDA(cudaStreamSynchronize(b->stream));
    int err = 0;
    KC_CUDA(cudaMemcpy(&err, b->d_err, 4, cudaMemcpyDeviceToHost));
    if (err) { set_error_msg("batched peel reported an error"); return err; }
    if (b->giants.size()) {
        PeelCtl c;
        KC_CUDA(cudaMemcpy(&c, b->d_gctl, sizeof(c), cudaMemcpyDeviceToHost));
        if (c.err) { set_error_msg("grid-wide peel of a large batch graph failed"); return c.err; }
    }
    if (core_out && b->Vtot) KC_CUDA(cudaMemcpy(core_out, b->d_core, 4 * b->Vtot, cudaMemcpyDeviceToHost));
    if (kmax_out && b->ngraphs) KC_CUDA(cudaMemcpy(kmax_out, b->d_kmax, 4 * b->ngraphs, cudaMemcpyDeviceToHost));
    float ms = 0;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    b->last_ms = ms;
    if (st) {
        st->ngraphs = b->ngraphs;
        st->giants = (uint32_t)b->giants.size();
        st->blocks = (uint32_t)b->grid;
        st->qcap = b->qcap;
        st->V_total = b->Vtot;
        st->arcs_total = b->Etot;
        st->peel_ms = ms;
    }
    return KC_OK;
}

int kc_batch_peel_per_graph(kc_batch* b, float* ms_out) {
    if (!b) return KC_ERR_INVALID;
    KC_CUDA(cudaSetDevice(b->dev));
    uint32_t gv = 0; uint64_t ge = 0;
    for (auto& p : b->plan) { gv = std::max(gv, p.V); ge = std::max(ge, p.E); }
    int rc = reserve_grid_scratch(b, gv, ge);
    if (rc) return rc;
    KC_CUDA(cudaMemsetAsync(b->d_err, 0, 4, b->stream));
    KC_CUDA(cudaEventRecord(b->ev0, b->stream));
    for (uint32_t g = 0; g < b->ngraphs; ++g) {
        rc = launch_single(b, g);
        if (rc) return rc;
    }
    KC_CUDA(cudaEventRecord(b->ev1, b->stream));
    KC_CUDA(cudaStreamSynchronize(b->stream));
    PeelCtl c;
    KC_CUDA(cudaMemcpy(&c, b->d_gctl, sizeof(c), cudaMemcpyDeviceToHost));
    if (c.err) { set_error_msg("one-graph-per-launch peel failed"); return c.err; }
    float ms = 0;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    if (ms_out) *ms_out = ms;
    return KC_OK;
}

int kc_batch_plan(kc_batch* b, uint32_t* schedule_out, uint32_t* ngiants, uint32_t* qcap, uint32_t* blocks) {
    if (!b) return KC_ERR_INVALID;
    if (schedule_out) {
        std::copy(b->giants.begin(), b->giants.end(), schedule_out);
        std::copy(b->schedule.begin(), b->schedule.end(), schedule_out + b->giants.size());
    }
    if (ngiants) *ngiants = (uint32_t)b->giants.size();
    if (qcap) *qcap = b->qcap;
    if (blocks) *blocks = (uint32_t)b->grid;
    return KC_OK;
}

void kc_batch_free(kc_batch* b) {
    if (!b) return;
    release(b);
    delete b;
}

int kc_batch_peel(const kc_segcsr* s, uint32_t* core_out, uint32_t* kmax_out, kc_batch_stats* st) {
    kc_batch* b = nullptr;
    int rc = kc_batch_upload(s, &b);
    if (rc) return rc;
    rc = kc_batch_peel_async(b);
    if (rc == KC_OK) rc = kc_batch_fetch(b, core_out, kmax_out, st);
    kc_batch_free(b);
    return rc;
}

void kc_segcsr_free(kc_segcsr_host* s) {
    if (!s) return;
    std::free(s->vbase); std::free(s->abase); std::free(s->offsets); std::free(s->neighbors);
    std::memset(s, 0, sizeof(*s));
}

int kc_gen_batch(uint32_t ngraphs, uint64_t seed_base, uint32_t nmin, uint32_t nmax, double dmin, double dmax,
                 double a, double bb, double c, kc_segcsr_host* out) {
    if (!out || ngraphs == 0 || nmin < 2 || nmax < nmin || dmin <= 0 || dmax < dmin) {
        set_error_msg("kc_gen_batch: bad argument");
        return KC_ERR_INVALID;
    }
    std::memset(out, 0, sizeof(*out));
    std::vector<kc_csr_host> gs(ngraphs);
    int bad = 0;
    const int nested = omp_get_max_active_levels();
    omp_set_max_active_levels(1);   // one thread per graph, generators run serially inside
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
    for (int64_t g = 0; g < (int64_t)ngraphs; ++g) {
        const uint64_t seed = seed_base + (uint64_t)g;
        // n ~ log-uniform[nmin, nmax], average degree 2m/n ~ U[dmin, dmax]
        const double u1 = rnd_unit(seed, 7, 0), u2 = rnd_unit(seed, 7, 1);
        const uint32_t n = (uint32_t)std::floor(std::exp(std::log((double)nmin) +
                                                         u1 * (std::log((double)nmax) - std::log((double)nmin))));
        const double d = dmin + u2 * (dmax - dmin);
        const uint64_t m = (uint64_t)std::llround((double)n * d / 2.0);
        std::vector<uint32_t> src(m), dst(m);
        int rc = (g % 2 == 0) ? kc_gen_er(n, m, seed, src.data(), dst.data())
                              : kc_gen_rmat(n, m, a, bb, c, seed, src.data(), dst.data());
        if (rc == KC_OK) rc = build_csr(src.data(), dst.data(), m, &gs[g]);
        if (rc) bad = 1;
    }
    omp_set_max_active_levels(nested);
    if (bad) {
        for (auto& x : gs) kc_csr_free(&x);
        set_error_msg("kc_gen_batch: generation failed");
        return KC_ERR_OOM;
    }
    out->ngraphs = ngraphs;
    out->vbase = (uint64_t*)std::malloc(8 * (size_t)(ngraphs + 1));
    out->abase = (uint64_t*)std::malloc(8 * (size_t)(ngraphs + 1));
    out->vbase[0] = out->abase[0] = 0;
    for (uint32_t g = 0; g < ngraphs; ++g) {
        out->vbase[g + 1] = out->vbase[g] + gs[g].V;
        out->abase[g + 1] = out->abase[g] + gs[g].E;
    }
    out->offsets = (uint32_t*)std::malloc(4 * (size_t)(out->vbase[ngraphs] + ngraphs));
    out->neighbors = (uint32_t*)std::malloc(4 * (size_t)std::max<uint64_t>(out->abase[ngraphs], 1));
    if (!out->vbase || !out->abase || !out->offsets || !out->neighbors) {
        for (auto& x : gs) kc_csr_free(&x);
        kc_segcsr_free(out);
        set_error_msg("kc_gen_batch: host allocation failed");
        return KC_ERR_OOM;
    }
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t g = 0; g < (int64_t)ngraphs; ++g) {
        std::memcpy(out->offsets + out->vbase[g] + g, gs[g].offsets, 4 * ((size_t)gs[g].V + 1));
        if (gs[g].E) std::memcpy(out->neighbors + out->abase[g], gs[g].neighbors, 4 * (size_t)gs[g].E);
        kc_csr_free(&gs[g]);
    }
    return KC_OK;
}

}  // extern "C"
