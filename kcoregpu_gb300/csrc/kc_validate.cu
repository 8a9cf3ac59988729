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

// One vertex's offset pair: b follows a (degree b - a, below the bias).
__device__ __forceinline__ void check_pair(uint32_t a, uint32_t b, bool& bad, uint32_t& md) {
    if (b < a) bad = true;
    else md = max(md, b - a);
}

// The CSR is read once, so the kernel is bound by DRAM: every thread keeps
// several 16-byte loads in flight (four offset words plus the next one, or
// four quads of neighbour ids).  Pointers that are not 16-byte aligned (the
// allocation-free entry takes the caller's) use 4-byte loads.
__global__ void __launch_bounds__(256) validate_csr_kernel(const uint32_t* __restrict__ off,
                                                            const uint32_t* __restrict__ nbr, uint32_t V,
                                                            uint64_t E, PeelCtl* ctl) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t first = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false;
    uint32_t md = 0;
    uint64_t vdone = 0;   // vertices covered by the vector loop
    if ((reinterpret_cast<uintptr_t>(off) & 15u) == 0) {
        const uint64_t nq = V / 4;   // quads of vertices: offsets 4q..4q+4 (4q+4 <= V)
        const uint4* o4 = reinterpret_cast<const uint4*>(off);
        for (uint64_t q = first; q < nq; q += stride) {
            const uint4 x = __ldg(o4 + q);
            const uint32_t e = __ldg(off + 4 * q + 4);
            check_pair(x.x, x.y, bad, md);
            check_pair(x.y, x.z, bad, md);
            check_pair(x.z, x.w, bad, md);
            check_pair(x.w, e, bad, md);
        }
        vdone = 4 * nq;
    }
    for (uint64_t v = vdone + first; v < V; v += stride) check_pair(__ldg(off + v), __ldg(off + v + 1), bad, md);
    if (first == 0 && (__ldg(off) != 0 || __ldg(off + V) != E)) bad = true;
    uint64_t adone = 0;   // arcs covered by the vector loop
    if ((reinterpret_cast<uintptr_t>(nbr) & 15u) == 0) {
        const uint64_t nq = E / 4;
        const uint4* n4 = reinterpret_cast<const uint4*>(nbr);
        for (uint64_t q = first; q < nq; q += 4 * stride) {
            uint4 x[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint64_t i = q + k * stride;
                x[k] = i < nq ? __ldg(n4 + i) : make_uint4(0, 0, 0, 0);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (x[k].x >= V || x[k].y >= V || x[k].z >= V || x[k].w >= V) bad = true;
        }
        adone = 4 * nq;
    }
    for (uint64_t j = adone + first; j < E; j += stride)
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
