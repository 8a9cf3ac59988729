// Batched peel: many independent graphs in one persistent launch.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace kc {

constexpr int kBatchThreads = 512;
constexpr int kBatchWarps = kBatchThreads / 32;
constexpr uint32_t kBatchChunk = kBatchThreads * 2;   // queue items per walk round
constexpr uint32_t kCtaScratch = 3;   // per-CTA scratch, in units of qcap: the queue and two alive lists
// Largest graph (vertices) whose peeled-vertex bitmap the batched kernel keeps
// in shared memory: 96 KB, so two CTAs still fit on one SM.
constexpr uint32_t kBatchBitsMax = 96u * 1024u * 8u;

struct BatchArgs {
    const unsigned long long* vbase;  // ngraphs+1: first vertex of each graph
    const unsigned long long* abase;  // ngraphs+1: first arc of each graph
    const uint32_t* offsets;          // graph g: V_g+1 graph-local offsets at vbase[g]+g
    const uint32_t* nbr;              // graph-local neighbour ids
    uint32_t* core;                   // working degrees -> core numbers (sum of V_g)
    uint32_t* kmax;                   // per graph
    uint32_t* levels_run;             // per graph: level iterations actually run
    const uint32_t* schedule;         // graph ids in the order CTAs take them
    uint32_t* next;                   // device work-queue counter (zeroed before launch)
    uint32_t* queues;                 // per CTA: kCtaScratch*qcap entries (peel order, two alive lists)
    int* err;                         // first error (0 = ok)
    uint32_t ngraphs;
    uint32_t qcap;                    // >= max V_g
    uint32_t bits_cap;                // vertices the dynamic shared-memory bitmap covers (0 = none)
};

const void* peel_batch_fn();

}  // namespace kc
