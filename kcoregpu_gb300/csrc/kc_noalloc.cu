// Allocation-free variant of the single-graph peel (kc_peel_noalloc).
//
// Some callers cannot call cudaMalloc: a plugin whose host application owns
// all device memory through its own pool and hands out only the buffers it
// allocated, or a latency-critical serving loop where a cudaMalloc/cudaFree
// pair would add allocator latency and device-wide synchronisation.  They pass
// their own device buffers for the graph and the result; the peel's scratch
// (working degrees, task queue, alive lists, level counters) lives in the one
// file-scope device array below, sized for graphs of up to
// KC_NOALLOC_MAX_V vertices and KC_NOALLOC_MAX_ARCS arcs.  Every GPU that loads
// this library holds that array (about 10.3 MiB) until the process exits.
//
// The array is shared by every call on a device and keeps the last call's
// contents; what must start from zero (the level counters, the task queue's
// tags) is reset by each call.  Calls that overlap on the GPU race on it, so a
// caller must serialise them (one stream, or wait between calls); calls from
// several host threads on one device are serialised here, calls on different
// devices run independently.
#include <cstring>
#include <mutex>

#include "kc_internal.h"
#include "kc_peel.cuh"

namespace kc {
namespace {

constexpr size_t kNaVpad = (size_t)(KC_NOALLOC_MAX_V + 127u) / 128u * 128u + 4;
constexpr size_t kNaTaskCap = (size_t)KC_NOALLOC_MAX_V + (size_t)KC_NOALLOC_MAX_ARCS / kChunk + 64;
constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kOffCtl = 0;
constexpr size_t kOffW = kOffCtl + align256(sizeof(PeelCtl));
constexpr size_t kOffTasks = kOffW + align256(kNaVpad * sizeof(uint32_t));
constexpr size_t kOffAlive0 = kOffTasks + align256(kNaTaskCap * sizeof(unsigned long long));
constexpr size_t kOffAlive1 = kOffAlive0 + align256(kNaVpad * sizeof(uint32_t));
constexpr size_t kScratchBytes = kOffAlive1 + align256(kNaVpad * sizeof(uint32_t));

}  // namespace

// The scratch.  In host code this name is only a stand-in: its device address
// comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Resets the level counters (all zero, slot minima "none").
__global__ void noalloc_reset_ctl(PeelCtl* ctl) {
    unsigned int* words = reinterpret_cast<unsigned int*>(ctl);
    for (size_t i = threadIdx.x; i < sizeof(PeelCtl) / sizeof(unsigned int); i += blockDim.x) words[i] = 0;
    __syncthreads();
    if (threadIdx.x < 4) ctl->slot[threadIdx.x].min_next = 0xFFFFFFFFu;
}

namespace {

struct DeviceScratch {
    std::mutex mu;                   // serialises the calls on this device
    bool ready = false;
    unsigned char* base = nullptr;   // device address of g_noalloc_scratch
    uint32_t epoch = 0;              // task-tag epoch of the last call
    int grid = 0;
};

constexpr int kMaxDevices = 64;
DeviceScratch g_na[kMaxDevices];

// First call on a device: resolve the scratch address (with that device current).
int noalloc_setup(int dev, DeviceScratch& s) {
    if (s.ready) return KC_OK;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        set_error_msg(std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
        return KC_ERR_CUDA;
    }
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, peel_kernel_selected(), kPeelThreads, 0);
    if (e != cudaSuccess) {
        set_error_msg(std::string("occupancy query: ") + cudaGetErrorString(e));
        return KC_ERR_CUDA;
    }
    if (per < 1 || sms < 1) {   // the cooperative launch needs one resident CTA per SM
        set_error_msg("kc_peel_noalloc: the peel kernel cannot keep one CTA resident per SM on this device");
        return KC_ERR_CUDA;
    }
    s.base = static_cast<unsigned char*>(p);
    s.grid = sms;   // one CTA per SM, as the single-graph peel
    s.epoch = 0;
    s.ready = true;
    return KC_OK;
}

}  // namespace
}  // namespace kc

using namespace kc;

extern "C" int kc_peel_noalloc(const uint32_t* d_offsets, const uint32_t* d_neighbors, uint32_t V,
                               uint32_t n_arcs, uint32_t* d_core_out, uint32_t* kmax_out, void* stream) {
    if (V > KC_NOALLOC_MAX_V || n_arcs > KC_NOALLOC_MAX_ARCS) {
        set_error_msg("kc_peel_noalloc: graph exceeds the scratch limits (V <= " +
                      std::to_string(KC_NOALLOC_MAX_V) + ", arcs <= " + std::to_string(KC_NOALLOC_MAX_ARCS) + ")");
        return KC_ERR_INVALID;
    }
    if (V && (!d_offsets || !d_core_out || (n_arcs && !d_neighbors))) {
        set_error_msg("kc_peel_noalloc: null device pointer");
        return KC_ERR_INVALID;
    }
    if (V == 0) {   // the reference loop never runs: kmax = level-1 = 0xFFFFFFFF
        if (kmax_out) *kmax_out = 0xFFFFFFFFu;
        return KC_OK;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_error_msg("kc_peel_noalloc: no usable current device");
        return KC_ERR_NODEV;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DeviceScratch& s = g_na[dev];
    std::lock_guard<std::mutex> lk(s.mu);
    int rc = noalloc_setup(dev, s);
    if (rc) return rc;

    PeelCtl* ctl = reinterpret_cast<PeelCtl*>(s.base + kOffCtl);
    unsigned long long* tasks = reinterpret_cast<unsigned long long*>(s.base + kOffTasks);
    s.epoch = s.epoch % 255u + 1u;
    if (s.epoch == 1u) {   // first call, or the 8-bit tag wrapped: clear stale entries
        e = cudaMemsetAsync(tasks, 0, sizeof(unsigned long long) * kNaTaskCap, st);
        if (e != cudaSuccess) { set_error_msg(cudaGetErrorString(e)); return KC_ERR_CUDA; }
    }
    noalloc_reset_ctl<<<1, 256, 0, st>>>(ctl);
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_error_msg(std::string("counter reset: ") + cudaGetErrorString(e)); return KC_ERR_CUDA; }
    // The CSR is the caller's device memory: it is checked on the device
    // (offsets, neighbour ids, degrees) before the peel indexes with it.
    if (launch_validate_csr(d_offsets, d_neighbors, V, n_arcs, ctl, st)) {
        set_error_msg("kc_peel_noalloc: CSR validation launch failed");
        return KC_ERR_CUDA;
    }

    PeelArgs a;
    std::memset(&a, 0, sizeof(a));
    a.off = d_offsets;
    a.nbr = d_neighbors;
    a.w = reinterpret_cast<uint32_t*>(s.base + kOffW);
    a.core = d_core_out;
    a.tasks = tasks;
    a.ctl = ctl;
    a.task_cap = kNaTaskCap;
    a.V = V;
    a.max_level = kFull;   // from the device validation
    a.local_budget = kLocalBudget;
    a.hub_arcs = kLocalArcs;
    a.chunk_arcs = kChunk;
    a.claim_cas = 1;   // one graph on the whole GPU
    a.epoch = s.epoch;
    a.wait_us = wait_limit_us();
    a.E = n_arcs;
    a.alive[0] = reinterpret_cast<uint32_t*>(s.base + kOffAlive0);
    a.alive[1] = reinterpret_cast<uint32_t*>(s.base + kOffAlive1);
    void* args[] = {&a};
    e = cudaLaunchCooperativeKernel(peel_kernel_selected(), dim3(s.grid), dim3(kPeelThreads), args, 0, st);
    if (e != cudaSuccess) { set_error_msg(std::string("peel launch: ") + cudaGetErrorString(e)); return KC_ERR_CUDA; }
    int err = 0;
    uint32_t kmax = 0;
    e = cudaMemcpyAsync(&err, &ctl->err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&kmax, &ctl->kmax, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { set_error_msg(std::string("kc_peel_noalloc: ") + cudaGetErrorString(e)); return KC_ERR_CUDA; }
    if (err == kErrInvalid) {
        set_error_msg("kc_peel_noalloc: invalid CSR (offsets must start at 0 and not decrease, neighbour ids "
                      "must be < V)");
        return KC_ERR_INVALID;
    }
    if (err == kErrCheck) {   // bounds-checked kernel (KC_CHECKED=1): an index was out of bounds
        set_error_msg("kc_peel_noalloc: out-of-bounds index recorded by the checked kernel (access skipped)");
        return KC_ERR_OVERFLOW;
    }
    if (err) {
        set_error_msg("kc_peel_noalloc: device peel reported an error");
        return err;
    }
    if (kmax_out) *kmax_out = kmax;
    return KC_OK;
}
