// Batched peel kernel for sm_103a: thousands of independent graphs in one
// persistent launch; each CTA takes the next graph from a device work counter
// (graphs ordered largest first by the host autotuner) and peels it alone
// (kc_batch_impl.cuh).
#include "kc_batch_impl.cuh"

namespace kc {
namespace {

__global__ void __launch_bounds__(kBatchThreads, 2) peel_batch_kernel(const __grid_constant__ BatchArgs a) {
    __shared__ BatchShared sh;
    extern __shared__ uint32_t peeled_bits[];   // (bits_cap + 31) / 32 words
    for (;;) {
        if (threadIdx.x == 0) sh.g = atomicAdd(a.next, 1u);
        __syncthreads();
        const uint32_t s = sh.g;
        __syncthreads();
        if (s >= a.ngraphs) return;
        const uint32_t g = a.schedule[s];
        const unsigned long long vb = a.vbase[g];
        uint32_t* scratch = a.queues + (size_t)blockIdx.x * kCtaScratch * a.qcap;
        peel_graph_cta(a.offsets + vb + g, a.nbr + a.abase[g], a.core + vb, (uint32_t)(a.vbase[g + 1] - vb),
                       scratch, scratch + a.qcap, a.qcap, a.err, a.kmax + g, a.levels_run + g, sh,
                       a.bits_cap ? peeled_bits : nullptr, a.bits_cap);
        __syncthreads();
    }
}

}  // namespace

const void* peel_batch_fn() { return reinterpret_cast<const void*>(&peel_batch_kernel); }

}  // namespace kc
