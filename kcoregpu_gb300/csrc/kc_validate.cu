// Device-side validation of a CSR before the peel: offsets start at 0, never
// decrease and end at E; every neighbour id is < V; every degree is below
// 2^30 (the state bias of the peel).  It also computes the maximum degree,
// which the peel kernels read from the control block when the caller did not
// pass one.  A one-shot peel of host arrays then validates at device
// bandwidth after the upload instead of in a host pass before it.  The peel
// kernels launched after it on the same stream return at once when it
// recorded kErrInvalid.
#include <algorithm>

#include "kc_device.cuh"
#include "kc_peel.cuh"

namespace kc {
namespace {

__global__ void __launch_bounds__(256) validate_csr_kernel(const uint32_t* __restrict__ off,
                                                            const uint32_t* __restrict__ nbr, uint32_t V,
                                                            uint64_t E, PeelCtl* ctl) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t first = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false;
    uint32_t md = 0;
    for (uint64_t v = first; v < V; v += stride) {
        const uint32_t a = __ldg(off + v), b = __ldg(off + v + 1);
        if (b < a) bad = true;
        else md = max(md, b - a);
    }
    if (first == 0 && (__ldg(off) != 0 || __ldg(off + V) != E)) bad = true;
    for (uint64_t j = first; j < E; j += stride)
        if (__ldg(nbr + j) >= V) bad = true;
    if (md >= kBias) bad = true;
    md = __reduce_max_sync(kFull, md);
    if ((threadIdx.x & 31) == 0 && md) atomicMax(&ctl->maxdeg, md);
    if (__any_sync(kFull, bad) && (threadIdx.x & 31) == 0) atomicCAS(&ctl->err, 0, kErrInvalid);
}

}  // namespace

int launch_validate_csr(const uint32_t* off, const uint32_t* nbr, uint32_t V, uint64_t E, PeelCtl* ctl,
                        cudaStream_t stream) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t work = std::max<uint64_t>((uint64_t)V, E);
    const uint64_t want = (work + 255) / 256;
    const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)std::max(1, sms) * 8));
    validate_csr_kernel<<<blocks, 256, 0, stream>>>(off, nbr, V, E, ctl);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace kc
