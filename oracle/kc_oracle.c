/*
 * kc_oracle.c - TEST INFRASTRUCTURE ONLY.  The parity oracle and the timed CPU
 * baseline for the k-core peel.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU legs may load this library; the product (libkcore_gb300.so)
 * never links or calls it.
 *
 * Two CPU restatements of the reference computation, both over the reference
 * CSR (offsets[V+1], neighbors[E], ascending, deduplicated, symmetric):
 *
 *   kco_levelsync : the reference's own algorithm, the level-synchronous peel of
 *                   kcore() (src/ours.cc:117-160): per level a scan for
 *                   deg==level (ours.cc:15-25), then a queue walk in which each
 *                   neighbour u with deg[u]>level is decremented; old==level+1
 *                   enqueues u in the same level (ours.cc:92-100) and
 *                   old<=level undoes the decrement (ours.cc:102-105).  The
 *                   loop runs while count<V and kmax = level-1 (ours.cc:138-151).
 *                   Runs on `nthreads` OpenMP threads with one shared queue.
 *   kco_bz        : Batagelj-Zaversnik O(n+m) bucket peel (single thread),
 *                   an independent algorithm with the same unique result.
 *
 * Core numbers are unique for a graph, so both must agree bit for bit with the
 * GPU peel and with networkx.core_number.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#define KCO_EMPTY 0xFFFFFFFFu

/* Batagelj & Zaversnik, "An O(m) Algorithm for Cores Decomposition of
 * Networks" (2003).  Returns kmax (0xFFFFFFFF when V == 0, as ours.cc:151
 * computes level-1 with level == 0). */
uint32_t kco_bz(uint32_t V, const uint32_t* off, const uint32_t* nbr, uint32_t* core) {
    if (V == 0) return 0xFFFFFFFFu;
    uint32_t md = 0;
    for (uint32_t v = 0; v < V; ++v) {
        core[v] = off[v + 1] - off[v];
        if (core[v] > md) md = core[v];
    }
    uint32_t* bin = (uint32_t*)calloc((size_t)md + 1, sizeof(uint32_t));
    uint32_t* pos = (uint32_t*)malloc(sizeof(uint32_t) * V);
    uint32_t* vert = (uint32_t*)malloc(sizeof(uint32_t) * V);
    for (uint32_t v = 0; v < V; ++v) bin[core[v]]++;
    uint32_t start = 0;
    for (uint32_t d = 0; d <= md; ++d) { uint32_t num = bin[d]; bin[d] = start; start += num; }
    for (uint32_t v = 0; v < V; ++v) { pos[v] = bin[core[v]]; vert[pos[v]] = v; bin[core[v]]++; }
    for (uint32_t d = md; d >= 1; --d) bin[d] = bin[d - 1];
    bin[0] = 0;
    for (uint32_t i = 0; i < V; ++i) {
        uint32_t v = vert[i];
        for (uint32_t j = off[v]; j < off[v + 1]; ++j) {
            uint32_t u = nbr[j];
            if (core[u] > core[v]) {
                uint32_t du = core[u], pu = pos[u], pw = bin[du], w = vert[pw];
                if (u != w) { pos[u] = pw; vert[pu] = w; pos[w] = pu; vert[pw] = u; }
                bin[du]++;
                core[u]--;
            }
        }
    }
    uint32_t kmax = 0;
    for (uint32_t v = 0; v < V; ++v) if (core[v] > kmax) kmax = core[v];
    free(bin); free(pos); free(vert);
    return kmax;
}

/* Level-synchronous peel (src/ours.cc:117-160) on the host.  `order` (V
 * entries, may be NULL) receives vertices in peel order and `shells`
 * (kmax+2 entries, may be NULL, capacity shell_cap) the k-shell offsets,
 * like the global-buffer prototype's glBuffer / cShellOffsets
 * (kcore-global-buffer/KCore.h:253-266).  Returns kmax; *levels_out = kmax+1. */
uint32_t kco_levelsync(uint32_t V, const uint32_t* off, const uint32_t* nbr, uint32_t* deg,
                       uint32_t* order, uint32_t* shells, uint32_t shell_cap, int nthreads,
                       uint32_t* levels_out) {
    if (nthreads < 1) nthreads = 1;
    uint32_t* q = order ? order : (uint32_t*)malloc(sizeof(uint32_t) * (V ? V : 1));
    for (uint32_t v = 0; v < V; ++v) { deg[v] = off[v + 1] - off[v]; q[v] = KCO_EMPTY; }
    uint32_t level = 0;
    uint64_t count = 0;        /* vertices peeled so far (global_count, ours.cc:111-113) */
    if (shells && shell_cap > 0) shells[0] = 0;
    while (count < V) {                                   /* ours.cc:138 */
        uint64_t lvl_start = count;
        uint64_t tail = count, head = count, done = count;
        /* scan: every vertex with deg == level joins the frontier (ours.cc:15-25) */
#pragma omp parallel num_threads(nthreads)
        {
            int nt = omp_get_num_threads(), id = omp_get_thread_num();
            uint64_t lo = (uint64_t)V * id / nt, hi = (uint64_t)V * (id + 1) / nt;
            for (uint64_t v = lo; v < hi; ++v)
                if (deg[v] == level) {
                    uint64_t p = __atomic_fetch_add(&tail, 1, __ATOMIC_RELAXED);
                    __atomic_store_n(&q[p], (uint32_t)v, __ATOMIC_RELEASE);
                }
        }
        /* process: walk the queue, including entries appended in this level
         * (ours.cc:60-107).  A worker that finds the queue empty waits until
         * every claimed entry is finished (done == tail). */
#pragma omp parallel num_threads(nthreads)
        {
            for (;;) {
                uint64_t i = __atomic_fetch_add(&head, 1, __ATOMIC_RELAXED);
                uint32_t v = KCO_EMPTY;
                for (;;) {
                    if (i < __atomic_load_n(&tail, __ATOMIC_ACQUIRE)) {
                        v = __atomic_load_n(&q[i], __ATOMIC_ACQUIRE);
                        if (v != KCO_EMPTY) break;
                        continue;
                    }
                    uint64_t d = __atomic_load_n(&done, __ATOMIC_ACQUIRE);
                    uint64_t t = __atomic_load_n(&tail, __ATOMIC_ACQUIRE);
                    if (d == t && i >= t) break;
                }
                if (v == KCO_EMPTY) break;
                for (uint32_t j = off[v]; j < off[v + 1]; ++j) {
                    uint32_t u = nbr[j];
                    /* Signed compare: a transient undershoot below zero reads as
                     * negative instead of wrapping to a huge unsigned value. */
                    if ((int32_t)__atomic_load_n(&deg[u], __ATOMIC_RELAXED) > (int32_t)level) {
                        uint32_t a = __atomic_fetch_sub(&deg[u], 1, __ATOMIC_ACQ_REL);
                        if (a == level + 1) {
                            uint64_t p = __atomic_fetch_add(&tail, 1, __ATOMIC_ACQ_REL);
                            __atomic_store_n(&q[p], u, __ATOMIC_RELEASE);
                        }
                        if ((int32_t)a <= (int32_t)level) __atomic_fetch_add(&deg[u], 1, __ATOMIC_ACQ_REL);
                    }
                }
                __atomic_fetch_add(&done, 1, __ATOMIC_ACQ_REL);
            }
        }
        (void)lvl_start;
        count = tail;
        ++level;
        if (shells && level < shell_cap) shells[level] = (uint32_t)count;
    }
    if (!order) free(q);
    if (levels_out) *levels_out = level;
    return level - 1u;   /* 0xFFFFFFFF for V == 0, as ours.cc:151 */
}

/* Many independent graphs (segmented CSR with 64-bit per-graph bases): one
 * BZ per graph in an OpenMP parallel-for over graphs on all host cores.
 * voff[g]..voff[g+1] index the concatenated vertex arrays, aoff[g] the first
 * arc of graph g; offsets are graph-local.  kmax_out[g] per graph. */
void kco_batch_bz(uint32_t ngraphs, const uint64_t* voff, const uint64_t* aoff,
                  const uint32_t* offsets, const uint32_t* nbr, uint32_t* core,
                  uint32_t* kmax_out, int nthreads) {
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int64_t g = 0; g < (int64_t)ngraphs; ++g) {
        uint32_t V = (uint32_t)(voff[g + 1] - voff[g]);
        const uint32_t* o = offsets + voff[g] + g;   /* V+1 entries per graph */
        kmax_out[g] = kco_bz(V, o, nbr + aoff[g], core + voff[g]);
    }
}

int kco_num_threads(void) { return omp_get_max_threads(); }
