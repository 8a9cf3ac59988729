// Served peel: continuous batching of k-core requests on one GPU.
//
// A C++ request loop (one host thread) admits submitted graphs against an HBM
// budget, uploads their CSR, and publishes a job descriptor to a device ring.
// A persistent serve kernel keeps running while requests flow: its CTAs take
// consecutive tickets, and each job owns a ticket range as wide as its gang.
// A small graph (gang 1) is peeled by one CTA alone (the batched peel's CTA
// routine); a large one by a gang of CTAs running the single-graph level
// protocol with the gang as its grid.  Jobs that arrive while others run are
// picked up by whichever CTAs free up first, so their work overlaps on the
// device.  Completions are written to host-mapped memory; the request loop
// copies the core numbers back, frees the job's memory and records latency.
//
// No reference counterpart: the reference peels one graph per process.
#define KC_PEEL_NO_KERNEL
#define KC_VNS serve_peel
#define KC_LDG(p) __ldcg(p)
#include "kc_peel_impl.cuh"
#include "kc_batch_impl.cuh"

#include <algorithm>
#include <cstdlib>
#include <unistd.h>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "kc_internal.h"

namespace kc {
int cuda_fail(cudaError_t e, const char* what);
using namespace KC_VNS;   // the gang peel (peel_body, CtaShared) compiled for this kernel

namespace {

// Job descriptor in the device ring (written by the host with cudaMemcpyAsync).
struct ServeJob {
    unsigned long long seq;      // job sequence number (ring slot = seq % cap)
    unsigned long long ticket0;  // first ticket of the job
    uint32_t gang;               // CTAs that peel it (1 = one CTA alone)
    uint32_t slot;               // completion slot in the host-mapped table
    uint32_t V, E, maxdeg, epoch;
    const uint32_t* off;
    const uint32_t* nbr;
    uint32_t* core;              // result
    uint32_t* w;                 // gang scratch: state, alive lists, tasks, counters
    uint32_t* alive0;
    uint32_t* alive1;
    unsigned long long* tasks;
    unsigned long long task_cap;
    PeelCtl* ctl;
    uint32_t* finished;          // gang members done
    uint32_t direct;             // 1: the gang copies the CSR in from, and the result out to, host memory
    uint32_t pad;
    const uint32_t* h_off;       // the request's host arrays (reached through the system page tables)
    const uint32_t* h_nbr;
    uint32_t* h_core;
};

static_assert(sizeof(ServeJob) % 8 == 0, "descriptors are copied in 8-byte words");

struct alignas(128) ServeCtl {
    unsigned long long ticket_head;  // next ticket handed to a CTA
    unsigned int pad0[30];
    unsigned int tail;               // jobs published (host writes it)
    unsigned int stop;               // host writes 1 to stop the kernel
    int err;                         // first error
    unsigned int idle_exits;         // CTAs that left after the idle limit
    unsigned int pad1[28];
};

// Completion record in host-mapped memory, one per ring slot.
struct ServeDone {
    unsigned long long seq_plus1;  // seq+1 of the job that completed in this slot
    uint32_t kmax;
    int err;
    uint32_t iters;
    uint32_t pad;
    unsigned long long t_start;    // device clock (ns): the job's first CTA started
    unsigned long long t_copied;   // the CSR was in device memory (all members)
    unsigned long long t_peeled;   // the peel was done (all members)
    unsigned long long t_out;      // the result was in host memory
};

struct ServeArgs {
    const ServeJob* ring;
    uint32_t ring_cap;
    ServeCtl* ctl;
    ServeDone* done;        // device pointer of the host-mapped table
    uint32_t* queues;       // per-CTA scratch for gang-1 jobs (kCtaScratch*qcap entries)
    uint32_t qcap;
    uint32_t bits_cap;      // vertices of the peeled bitmap of gang-1 jobs (dynamic shared memory)
    uint32_t wait_us;       // bounded waits inside a gang peel
    uint32_t idle_us;       // time a CTA waits on an empty ring before it leaves
    unsigned long long cursor0;   // oldest unfinished job when the kernel was launched
};

struct ServeShared {
    union {
        CtaShared peel;
        BatchShared batch;
    } u;
    ServeJob job;           // validated copy of this CTA's job descriptor
    unsigned long long ticket;
    int state;              // 1 = job found, 2 = stop, 3 = idle limit
    uint32_t kmax, iters;
    int err;                // this CTA's job error (one-CTA jobs)
    int bad;                // a neighbour id >= V was copied in
};

constexpr unsigned long long kNoSeq = ~0ull;

// Loads of words the host writes (through copies) while the kernel runs: system
// scope, so they are performed at the coherence point and never served from a
// stale line.
__device__ __forceinline__ unsigned long long ld_sys64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_sys32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Seqlock read of ring slot `pos`: copies the descriptor when its seq is `pos`
// before and after the copy (the host writes the body with seq = kNoSeq, then
// the seq, then the tail, as three ordered copies).
__device__ bool read_job(const ServeArgs& s, unsigned long long pos, ServeJob* out) {
    const ServeJob* j = s.ring + (pos % s.ring_cap);
    const unsigned long long s1 = ld_sys64(&j->seq);
    if (s1 != pos) return false;
    fence_acq_rel();
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(j);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(out);
    for (size_t i = 0; i < sizeof(ServeJob) / 8; ++i) dst[i] = ld_sys64(src + i);
    fence_acq_rel();
    const unsigned long long s2 = ld_sys64(&j->seq);
    return s2 == pos && out->seq == pos;
}

// Copies n 32-bit words from src to dst by the threads first, first+stride, ...
// (16-byte words when both pointers allow).  Used for the request's host
// arrays, which the device reads and writes through the system's page tables
// (pageable memory access) at the host link's rate.  With limit != 0 it also
// returns whether any word copied is >= limit (a neighbour id outside the
// graph: the job is refused instead of peeled).
__device__ bool copy_words(uint32_t* dst, const uint32_t* src, uint64_t n, uint64_t first, uint64_t stride,
                           uint32_t limit = 0) {
    bool bad = false;
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0) {
        const uint64_t n4 = n / 4;
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        uint4* d4 = reinterpret_cast<uint4*>(dst);
        for (uint64_t i = first; i < n4; i += stride) {
            const uint4 x = s4[i];
            if (limit) bad |= (x.x >= limit) | (x.y >= limit) | (x.z >= limit) | (x.w >= limit);
            d4[i] = x;
        }
        for (uint64_t i = n4 * 4 + first; i < n; i += stride) {
            const uint32_t x = src[i];
            if (limit) bad |= x >= limit;
            dst[i] = x;
        }
    } else {
        for (uint64_t i = first; i < n; i += stride) {
            const uint32_t x = src[i];
            if (limit) bad |= x >= limit;
            dst[i] = x;
        }
    }
    return bad;
}

__device__ void publish_done(const ServeArgs& s, const ServeJob& j, uint32_t kmax, int err, uint32_t iters) {
    ServeDone* d = s.done + j.slot;
    d->kmax = kmax;
    d->err = err;
    d->iters = iters;
    __threadfence_system();
    *(volatile unsigned long long*)&d->seq_plus1 = j.seq + 1;
    __threadfence_system();
}

__global__ void __launch_bounds__(kPeelThreads, 1) serve_kernel(const __grid_constant__ ServeArgs s) {
    extern __shared__ uint32_t serve_bits[];   // (bits_cap + 31) / 32 words
    __shared__ ServeShared sh;
    unsigned long long cursor = s.cursor0;   // ring position: jobs before it end below this CTA's tickets
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long t = atomicAdd(&s.ctl->ticket_head, 1ull);
            sh.ticket = t;
            int state = 0;
            uint32_t nap = 64;
            const unsigned long long since = now_ns();
            for (;;) {
                const unsigned tail = ld_sys32(&s.ctl->tail);
                while (cursor < tail) {
                    // A slot whose seq is not `cursor` (being rewritten, or reused by a
                    // later job) held a job that has retired: its tickets are behind t.
                    if (read_job(s, cursor, &sh.job) && t < sh.job.ticket0 + sh.job.gang) break;
                    ++cursor;
                }
                if (cursor < tail) { state = 1; break; }
                if (ld_sys32(&s.ctl->stop)) { state = 2; break; }
                if (now_ns() - since > (unsigned long long)s.idle_us * 1000ull) {
                    state = 3;
                    atomicAdd(&s.ctl->idle_exits, 1u);
                    break;
                }
                __nanosleep(nap);
                nap = min(nap * 2, 2048u);
            }
            sh.state = state;
        }
        __syncthreads();
        if (sh.state != 1) return;
        const ServeJob& j = sh.job;
        const unsigned long long t = sh.ticket;
        ServeDone* dn = s.done + j.slot;
        if (j.gang <= 1) {
            if (threadIdx.x == 0) { sh.err = 0; sh.kmax = 0; sh.iters = 0; dn->t_start = now_ns(); }
            bool bad = false;
            if (j.direct) {
                copy_words(const_cast<uint32_t*>(j.off), j.h_off, (uint64_t)j.V + 1, threadIdx.x, blockDim.x);
                bad = copy_words(const_cast<uint32_t*>(j.nbr), j.h_nbr, j.E, threadIdx.x, blockDim.x, j.V);
            }
            bad = __syncthreads_or(bad);
            if (threadIdx.x == 0) dn->t_copied = now_ns();
            if (bad) {
                if (threadIdx.x == 0) sh.err = kErrInvalid;
            } else {
                uint32_t* scratch = s.queues + (size_t)blockIdx.x * kCtaScratch * s.qcap;
                peel_graph_cta(j.off, j.nbr, j.core, j.V, scratch, scratch + s.qcap, s.qcap,
                               &sh.err, &sh.kmax, &sh.iters, sh.u.batch, s.bits_cap ? serve_bits : nullptr,
                               s.bits_cap);
            }
            __syncthreads();
            if (threadIdx.x == 0) dn->t_peeled = now_ns();
            if (j.direct && !sh.err) copy_words(j.h_core, j.core, j.V, threadIdx.x, blockDim.x);
            __syncthreads();
            if (threadIdx.x == 0) {
                dn->t_out = now_ns();
                publish_done(s, j, sh.kmax, sh.err, sh.iters);
            }
        } else {
            PeelArgs a;
            a.off = j.off;
            a.nbr = j.nbr;
            a.w = j.w;
            a.core = j.core;
            a.order = nullptr;
            a.shells = nullptr;
            a.tasks = j.tasks;
            a.ctl = j.ctl;
            a.task_cap = j.task_cap;
            a.V = j.V;
            a.shell_cap = 0;
            a.max_level = j.maxdeg;
            a.epoch = j.epoch;
            a.wait_us = s.wait_us;
            a.trace = nullptr;
            a.trace_cap = 0;
            a.alive[0] = j.alive0;
            a.alive[1] = j.alive1;
            a.E = j.E;
            a.zero_tasks = 1;
            const uint32_t part = (uint32_t)(t - j.ticket0);
            const uint64_t first = (uint64_t)part * blockDim.x + threadIdx.x;
            const uint64_t stride = (uint64_t)j.gang * blockDim.x;
            bool ok = true;
            if (part == 0 && threadIdx.x == 0) dn->t_start = now_ns();
            if (j.direct) {   // the gang copies the CSR in, then starts together
                copy_words(const_cast<uint32_t*>(j.off), j.h_off, (uint64_t)j.V + 1, first, stride);
                const bool bad = copy_words(const_cast<uint32_t*>(j.nbr), j.h_nbr, j.E, first, stride, j.V);
                if (__syncthreads_or(bad) && threadIdx.x == 0) record_error(j.ctl, kErrInvalid, 0);
                ok = part_barrier(a, sh.u.peel, j.gang, 0);
            }
            if (part == 0 && threadIdx.x == 0) dn->t_copied = now_ns();
            if (ok) peel_body(a, sh.u.peel, part, j.gang);
            // every member is done: the gang copies the result out
            const bool all_done = part_barrier(a, sh.u.peel, j.gang, 0);
            if (part == 0 && threadIdx.x == 0) dn->t_peeled = now_ns();
            if (j.direct && all_done && !ld_err(&j.ctl->err)) copy_words(j.h_core, j.core, j.V, first, stride);
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence_system();   // this member's result words before its count
                const unsigned fin = atomicAdd(j.finished, 1u) + 1u;
                if (fin == j.gang) {
                    __threadfence();
                    dn->t_out = now_ns();
                    publish_done(s, j, ld_relaxed(&j.ctl->kmax), ld_err(&j.ctl->err), ld_relaxed(&j.ctl->iterations));
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace
}  // namespace kc

using namespace kc;

#define KC_CUDA(call)                                       \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

namespace {

using clk = std::chrono::steady_clock;

struct Request {
    uint64_t id;
    const uint32_t* off;
    const uint32_t* nbr;
    uint32_t V;
    uint64_t E;
    uint32_t maxdeg;
    uint32_t* core_out;
    uint32_t gang;
    uint64_t bytes;          // device memory charged against the budget
    // device allocations
    uint32_t *d_off = nullptr, *d_nbr = nullptr, *d_core = nullptr, *d_w = nullptr, *d_a0 = nullptr, *d_a1 = nullptr;
    unsigned long long* d_tasks = nullptr;
    unsigned long long task_cap = 0;
    PeelCtl* d_ctl = nullptr;
    uint32_t* d_fin = nullptr;
    unsigned long long seq = 0;
    cudaEvent_t copied = nullptr;
    int state = 0;           // 0 pending, 1 uploading, 2 running, 3 copying back, 4 done
    int err = 0;
    uint32_t kmax = 0, iters = 0;
    double copy_in_us = 0, peel_us = 0, copy_out_us = 0;   // device clock
    clk::time_point t_submit, t_admit, t_publish, t_done;
};

}  // namespace

struct kc_server {
    kc_serve_cfg cfg{};
    int dev = 0;
    int grid = 0;
    uint32_t bits_cap = 0;   // vertices of the gang-1 jobs' peeled bitmap
    size_t bits_bytes = 0;   // its dynamic shared memory per CTA
    cudaStream_t ks = nullptr;     // serve kernel
    cudaStream_t cs = nullptr;     // copies, allocations, publication
    cudaMemPool_t pool = nullptr;  // the requests' device memory: keeps up to the budget mapped between requests
    ServeCtl* d_ctl = nullptr;
    ServeJob* d_ring = nullptr;
    ServeJob* h_ring = nullptr;    // pinned mirror (copy sources)
    unsigned* h_tails = nullptr;   // pinned copy sources for the tail, one per slot
    unsigned long long* h_seqs = nullptr;   // pinned copy sources for the seq, one per slot
    unsigned* h_stop = nullptr;
    ServeDone* h_done = nullptr;   // host-mapped completion table
    ServeDone* d_done = nullptr;
    uint32_t* d_queues = nullptr;
    PeelCtl* h_ctl_init = nullptr;
    // Pinned staging for every host<->device copy of request data: a copy from
    // or to pageable memory waits for the running serve kernel, so requests are
    // moved through two pinned halves (double buffered).
    unsigned char* stage = nullptr;
    size_t stage_half = 0;
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};
    int stage_next = 0;
    unsigned char* dbg = nullptr;   // pinned scratch of kc_serve_debug
    uint32_t* h_zero = nullptr;     // pinned zero words (copy source of counter resets)
    bool kernel_running = false;
    // The device reaches pageable host memory through the system page tables
    // (cudaDevAttrPageableMemoryAccess): each job's gang then copies the CSR in
    // and the result out itself, at the host link's rate and in parallel across
    // jobs, and the staging above is not used (KC_SERVE_STAGED=1 forces it).
    bool direct = false;
    bool big_inflight = false;   // a gang of more than half the CTAs is running alone
    unsigned long long next_ticket = 0;
    unsigned long long next_seq = 0;
    uint64_t in_use = 0;
    uint32_t epoch = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> pending;
    std::vector<Request*> inflight;
    std::unordered_map<uint64_t, Request*> all;
    uint64_t next_id = 1;
    bool closing = false;
    int fatal = 0;
    std::thread loop;
    clk::time_point last_activity;
    kc_serve_stats stats{};
};

namespace {

uint64_t align_up(uint64_t x) { return (x + 255) / 256 * 256; }

// Host memcpy split over the host cores (one core alone copies far below the
// host-device link rate).
void parallel_copy(unsigned char* dst, const unsigned char* src, size_t n) {
    if (n < (4u << 20)) { std::memcpy(dst, src, n); return; }
    const int64_t parts = 16;
#pragma omp parallel for schedule(static) num_threads(16)
    for (int64_t i = 0; i < parts; ++i) {
        const size_t a = n * (size_t)i / parts, b = n * (size_t)(i + 1) / parts;
        std::memcpy(dst + a, src + a, b - a);
    }
}

// Host -> device through the pinned staging halves, ordered on the copy stream.
int stage_h2d(kc_server* s, void* dst, const void* src, size_t bytes) {
    const unsigned char* p = static_cast<const unsigned char*>(src);
    for (size_t done = 0; done < bytes;) {
        const int k = s->stage_next;
        s->stage_next ^= 1;
        KC_CUDA(cudaEventSynchronize(s->stage_ev[k]));   // the half's previous copy has left
        const size_t n = std::min(bytes - done, s->stage_half);
        parallel_copy(s->stage + k * s->stage_half, p + done, n);
        KC_CUDA(cudaMemcpyAsync(static_cast<unsigned char*>(dst) + done, s->stage + k * s->stage_half, n,
                                cudaMemcpyHostToDevice, s->cs));
        KC_CUDA(cudaEventRecord(s->stage_ev[k], s->cs));
        done += n;
    }
    return KC_OK;
}

// Device -> host through the staging halves (returns when dst holds the data).
int stage_d2h(kc_server* s, void* dst, const void* src, size_t bytes) {
    unsigned char* p = static_cast<unsigned char*>(dst);
    for (size_t done = 0; done < bytes;) {
        const int k = s->stage_next;
        s->stage_next ^= 1;
        KC_CUDA(cudaEventSynchronize(s->stage_ev[k]));
        const size_t n = std::min(bytes - done, s->stage_half);
        KC_CUDA(cudaMemcpyAsync(s->stage + k * s->stage_half, static_cast<const unsigned char*>(src) + done, n,
                                cudaMemcpyDeviceToHost, s->cs));
        KC_CUDA(cudaEventRecord(s->stage_ev[k], s->cs));
        KC_CUDA(cudaEventSynchronize(s->stage_ev[k]));
        parallel_copy(p + done, s->stage + k * s->stage_half, n);
        done += n;
    }
    return KC_OK;
}

// Publishes the descriptor in h_ring[slot] behind the job's uploads on the copy
// stream: body with an invalid seq, then the seq, then the tail (seqlock order
// for the kernel's reader).  h_seqs keeps a pinned copy source per slot.
void publish(kc_server* s, uint32_t slot) {
    ServeJob& j = s->h_ring[slot];
    s->h_seqs[slot] = j.seq;
    j.seq = kNoSeq;
    cudaMemcpyAsync(s->d_ring + slot, &j, sizeof(j), cudaMemcpyHostToDevice, s->cs);
    cudaMemcpyAsync(&s->d_ring[slot].seq, &s->h_seqs[slot], 8, cudaMemcpyHostToDevice, s->cs);
    cudaMemcpyAsync(&s->d_ctl->tail, &s->h_tails[slot], 4, cudaMemcpyHostToDevice, s->cs);
}

void plan_request(kc_server* s, Request* r) {
    const uint64_t Vpad = (uint64_t)(r->V + 127) / 128 * 128 + 4;
    uint32_t gang = (uint32_t)std::min<uint64_t>((uint64_t)s->cfg.max_gang, std::max<uint64_t>(1, r->E / s->cfg.gang_arcs));
    if (r->V > s->cfg.small_vertices && gang < 2) gang = 2;   // the per-CTA queue holds small graphs only
    gang = std::min<uint32_t>(gang, (uint32_t)s->grid);
    r->gang = gang;
    uint64_t b = align_up(4 * ((uint64_t)r->V + 1)) + align_up(4 * std::max<uint64_t>(r->E, 1)) + align_up(4 * Vpad);
    if (gang > 1) {
        r->task_cap = (uint64_t)r->V + r->E / kChunk + 64;
        b += 3 * align_up(4 * Vpad) + align_up(8 * r->task_cap) + align_up(sizeof(PeelCtl)) + 256;
    }
    r->bytes = b;
}

int device_alloc(kc_server* s, Request* r) {
    const uint64_t Vpad = (uint64_t)(r->V + 127) / 128 * 128 + 4;
    KC_CUDA(cudaMallocFromPoolAsync(&r->d_off, 4 * ((size_t)r->V + 1), s->pool, s->cs));
    KC_CUDA(cudaMallocFromPoolAsync(&r->d_nbr, 4 * std::max<uint64_t>(r->E, 1), s->pool, s->cs));
    KC_CUDA(cudaMallocFromPoolAsync(&r->d_core, 4 * Vpad, s->pool, s->cs));
    if (r->gang > 1) {
        KC_CUDA(cudaMallocFromPoolAsync(&r->d_w, 4 * Vpad, s->pool, s->cs));
        KC_CUDA(cudaMallocFromPoolAsync(&r->d_a0, 4 * Vpad, s->pool, s->cs));
        KC_CUDA(cudaMallocFromPoolAsync(&r->d_a1, 4 * Vpad, s->pool, s->cs));
        KC_CUDA(cudaMallocFromPoolAsync(&r->d_tasks, 8 * r->task_cap, s->pool, s->cs));
        KC_CUDA(cudaMallocFromPoolAsync(&r->d_ctl, sizeof(PeelCtl), s->pool, s->cs));
        KC_CUDA(cudaMallocFromPoolAsync(&r->d_fin, 256, s->pool, s->cs));
        // Resets are copies, never memsets: a memset runs as a kernel and would
        // wait for SM room the serve kernel does not leave.  The task queue is
        // cleared by the gang itself during level 0 (zero_tasks).
        KC_CUDA(cudaMemcpyAsync(r->d_ctl, s->h_ctl_init, sizeof(PeelCtl), cudaMemcpyHostToDevice, s->cs));
        KC_CUDA(cudaMemcpyAsync(r->d_fin, s->h_zero, 4, cudaMemcpyHostToDevice, s->cs));
    }
    if (s->direct) return KC_OK;   // the gang copies the CSR in
    int rc = stage_h2d(s, r->d_off, r->off, 4 * ((size_t)r->V + 1));
    if (rc == KC_OK && r->E) rc = stage_h2d(s, r->d_nbr, r->nbr, 4 * r->E);
    return rc;
}

void device_free(kc_server* s, Request* r) {
    for (void* p : {(void*)r->d_off, (void*)r->d_nbr, (void*)r->d_core, (void*)r->d_w, (void*)r->d_a0,
                    (void*)r->d_a1, (void*)r->d_tasks, (void*)r->d_ctl, (void*)r->d_fin})
        if (p) cudaFreeAsync(p, s->cs);
    r->d_off = r->d_nbr = r->d_core = r->d_w = r->d_a0 = r->d_a1 = nullptr;
    r->d_tasks = nullptr;
    r->d_ctl = nullptr;
    r->d_fin = nullptr;
}

int launch_kernel(kc_server* s) {
    ServeArgs a;
    a.ring = s->d_ring;
    a.ring_cap = s->cfg.ring_slots;
    a.ctl = s->d_ctl;
    a.done = s->d_done;
    a.queues = s->d_queues;
    a.qcap = s->cfg.small_vertices;
    a.bits_cap = s->bits_cap;
    a.wait_us = 2000000;    // 2 s
    a.idle_us = 10000000;   // 10 s safety net: the request loop stops an idle kernel after 100 ms itself
    // ring position where the new kernel's CTAs start looking: the oldest job
    // not yet finished (every earlier job is done)
    // (only the request-loop thread changes `inflight`, and this runs on it)
    unsigned long long c0 = s->next_seq;
    for (Request* r : s->inflight)
        if (r->state == 2) c0 = std::min(c0, r->seq);
    a.cursor0 = c0;
    void* args[] = {&a};
    KC_CUDA(cudaLaunchCooperativeKernel((const void*)serve_kernel, dim3(s->grid), dim3(kPeelThreads), args, s->bits_bytes,
                                        s->ks));
    s->kernel_running = true;
    return KC_OK;
}

// Waits for the serve kernel to leave (stop flag or idle limit) and resumes the
// ticket count where the kernel left it (tickets held by leaving CTAs are skipped).
int drain_kernel(kc_server* s, bool stop) {
    if (!s->kernel_running) return KC_OK;
    if (stop) {
        *s->h_stop = 1;
        KC_CUDA(cudaMemcpyAsync(&s->d_ctl->stop, s->h_stop, 4, cudaMemcpyHostToDevice, s->cs));
    }
    KC_CUDA(cudaStreamSynchronize(s->ks));
    s->kernel_running = false;
    KC_CUDA(cudaStreamSynchronize(s->cs));
    unsigned long long th = 0;
    KC_CUDA(cudaMemcpy(&th, &s->d_ctl->ticket_head, 8, cudaMemcpyDeviceToHost));
    s->next_ticket = th;
    *s->h_stop = 0;
    KC_CUDA(cudaMemcpy(&s->d_ctl->stop, s->h_stop, 4, cudaMemcpyHostToDevice));
    return KC_OK;
}

// One pass of the request loop; returns true when it made progress.
bool loop_once(kc_server* s) {
    bool progress = false;
    std::vector<Request*> admit;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        // Admission, first come first served: stop at the first request that
        // does not fit the budget or the ring.  A big gang (more than half the
        // CTAs) runs alone: it is admitted once nothing else is in flight, and
        // nothing is admitted beside it -- its level chain waits for every
        // member at every level, and members that share an SM with other jobs
        // slowed it several-fold when it co-ran.
        while (!s->pending.empty()) {
            Request* r = s->pending.front();
            if (s->big_inflight) break;
            const bool big = 2 * r->gang > (uint32_t)s->grid;
            if (big && !(s->inflight.empty() && admit.empty())) break;
            if (s->in_use + r->bytes > s->cfg.hbm_budget_bytes) break;
            if (s->inflight.size() + admit.size() >= s->cfg.ring_slots) break;
            s->pending.pop_front();
            if (big) s->big_inflight = true;
            s->in_use += r->bytes;
            admit.push_back(r);
        }
        s->stats.peak_in_use = std::max<uint64_t>(s->stats.peak_in_use, s->in_use);
    }
    for (Request* r : admit) {
        r->t_admit = clk::now();
        int rc = device_alloc(s, r);
        if (rc) {   // the request fails alone; its budget share and a big gang's exclusivity are released
            device_free(s, r);
            std::lock_guard<std::mutex> lk(s->mu);
            s->in_use -= r->bytes;
            if (2 * r->gang > (uint32_t)s->grid) s->big_inflight = false;
            r->err = rc;
            r->t_done = clk::now();
            r->state = 4;
            s->stats.completed++;
            s->cv.notify_all();
            continue;
        }
        r->seq = s->next_seq++;
        const uint32_t slot = (uint32_t)(r->seq % s->cfg.ring_slots);
        ServeJob& j = s->h_ring[slot];
        std::memset(&j, 0, sizeof(j));
        j.seq = r->seq;
        j.ticket0 = s->next_ticket;
        j.gang = r->gang;
        j.slot = slot;
        j.V = r->V;
        j.E = (uint32_t)r->E;
        j.maxdeg = r->maxdeg;
        j.epoch = 1;
        j.off = r->d_off;
        j.nbr = r->d_nbr;
        j.core = r->d_core;
        j.w = r->d_w;
        j.alive0 = r->d_a0;
        j.alive1 = r->d_a1;
        j.tasks = r->d_tasks;
        j.task_cap = r->task_cap;
        j.ctl = r->d_ctl;
        j.finished = r->d_fin;
        j.direct = s->direct ? 1u : 0u;
        j.h_off = r->off;
        j.h_nbr = r->nbr;
        j.h_core = r->core_out;
        s->next_ticket += r->gang;
        s->h_tails[slot] = (unsigned)(r->seq + 1);
        publish(s, slot);
        r->t_publish = clk::now();
        r->state = 2;
        std::lock_guard<std::mutex> lk(s->mu);
        s->inflight.push_back(r);
        progress = true;
    }
    if (!admit.empty() && !s->kernel_running) {
        if (launch_kernel(s)) { s->fatal = KC_ERR_CUDA; }
    }
    // completions
    std::vector<Request*> finished;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (Request* r : s->inflight) {
            if (r->state != 2) continue;
            const ServeDone& d = s->h_done[r->seq % s->cfg.ring_slots];
            const unsigned long long sp = *(volatile const unsigned long long*)&d.seq_plus1;
            if (sp == r->seq + 1) {
                std::atomic_thread_fence(std::memory_order_acquire);
                r->kmax = d.kmax;
                r->err = d.err;
                r->iters = d.iters;
                r->copy_in_us = (d.t_copied - d.t_start) * 1e-3;
                r->peel_us = (d.t_peeled - d.t_copied) * 1e-3;
                r->copy_out_us = (d.t_out - d.t_peeled) * 1e-3;
                r->state = 3;
                finished.push_back(r);
            }
        }
    }
    for (Request* r : finished) {
        if (r->V && !s->direct) {
            const int rc = stage_d2h(s, r->core_out, r->d_core, 4 * (size_t)r->V);
            if (rc && !r->err) r->err = rc;
        }
        device_free(s, r);
        r->t_done = clk::now();
        std::lock_guard<std::mutex> lk(s->mu);
        s->in_use -= r->bytes;
        s->inflight.erase(std::find(s->inflight.begin(), s->inflight.end(), r));
        if (2 * r->gang > (uint32_t)s->grid) s->big_inflight = false;
        r->state = 4;
        s->stats.completed++;
        progress = true;
    }
    if (!finished.empty()) s->cv.notify_all();
    // the kernel leaves by itself after an idle stretch; relaunch when needed
    if (s->kernel_running && cudaStreamQuery(s->ks) == cudaSuccess) {
        drain_kernel(s, false);
        std::lock_guard<std::mutex> lk(s->mu);
        // Jobs published to a kernel that had already decided to leave (its
        // idle safety net) get new tickets; a gang job that some members had
        // started is reset first, so it reruns from a clean state.
        for (Request* r : s->inflight)
            if (r->state == 2) {
                const ServeDone& d = s->h_done[r->seq % s->cfg.ring_slots];
                if (*(volatile const unsigned long long*)&d.seq_plus1 == r->seq + 1) continue;   // finished
                const uint32_t slot = (uint32_t)(r->seq % s->cfg.ring_slots);
                if (r->gang > 1) {   // (the rerun clears its task queue in level 0)
                    cudaMemcpyAsync(r->d_ctl, s->h_ctl_init, sizeof(PeelCtl), cudaMemcpyHostToDevice, s->cs);
                    cudaMemcpyAsync(r->d_fin, s->h_zero, 4, cudaMemcpyHostToDevice, s->cs);
                }
                s->h_ring[slot].seq = r->seq;
                s->h_ring[slot].ticket0 = s->next_ticket;
                s->next_ticket += r->gang;
                publish(s, slot);
            }
        if (!s->inflight.empty()) {
            cudaStreamSynchronize(s->cs);
            if (launch_kernel(s)) s->fatal = KC_ERR_CUDA;
        }
    }
    if (progress) s->last_activity = clk::now();
    // Nothing queued or in flight for 100 ms: stop the kernel (it is relaunched
    // by the next admission), so CTAs do not poll an empty ring for long.
    if (s->kernel_running && clk::now() - s->last_activity > std::chrono::milliseconds(100)) {
        bool idle;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            idle = s->pending.empty() && s->inflight.empty();
        }
        if (idle) drain_kernel(s, true);
    }
    return progress;
}

void request_loop(kc_server* s) {
    cudaSetDevice(s->dev);
    for (;;) {
        const bool progress = loop_once(s);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->closing && s->pending.empty() && s->inflight.empty()) break;
            if (s->fatal) break;
        }
        if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    drain_kernel(s, true);
    s->cv.notify_all();
}

}  // namespace

extern "C" {

int kc_serve_open(const kc_serve_cfg* cfg, kc_server** out) {
    if (!out) return KC_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { set_error_msg("no CUDA device is available"); return KC_ERR_NODEV; }
    kc_server* s = new kc_server();
    if (cfg) s->cfg = *cfg;
    if (!s->cfg.hbm_budget_bytes) s->cfg.hbm_budget_bytes = 64ull << 30;
    if (!s->cfg.ring_slots) s->cfg.ring_slots = 1024;
    if (!s->cfg.gang_arcs) s->cfg.gang_arcs = 1u << 19;
    if (!s->cfg.small_vertices) s->cfg.small_vertices = 1u << 18;
    cudaGetDevice(&s->dev);
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->dev);
    // gang-1 jobs (at most small_vertices vertices) keep a bitmap of their
    // queued vertices in shared memory, up to kBatchBitsMax vertices
    s->bits_cap = std::min(s->cfg.small_vertices, kBatchBitsMax);
    s->bits_bytes = (size_t)((s->bits_cap + 31) / 32) * 4;
    // static plus dynamic shared memory exceeds the default 48 KB window
    if (cudaError_t ea = cudaFuncSetAttribute((const void*)serve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)s->bits_bytes)) {
        const int rc = cuda_fail(ea, "cudaFuncSetAttribute(serve_kernel)");
        delete s;
        return rc;
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)serve_kernel, kPeelThreads, s->bits_bytes);
    s->grid = sms * std::max(1, per);
    if (!s->cfg.max_gang || s->cfg.max_gang > (uint32_t)s->grid) s->cfg.max_gang = (uint32_t)s->grid;
    int pageable = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, s->dev);
    const char* staged = std::getenv("KC_SERVE_STAGED");
    s->direct = pageable == 1 && !(staged && std::atoi(staged) != 0);
    auto fail = [&](cudaError_t e, const char* w) { int rc = cuda_fail(e, w); delete s; return rc; };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&s->ks, cudaStreamNonBlocking))) return fail(e, "stream");
    if ((e = cudaStreamCreateWithFlags(&s->cs, cudaStreamNonBlocking))) return fail(e, "stream");
    {   // A pool of its own that keeps up to the HBM budget mapped: with the
        // default pool's release threshold of 0, memory freed by one stretch of
        // requests went back to the system at the next synchronisation, and the
        // next stretch paid to map it again (a slower first pass).
        cudaMemPoolProps pp{};
        pp.allocType = cudaMemAllocationTypePinned;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = s->dev;
        if ((e = cudaMemPoolCreate(&s->pool, &pp))) return fail(e, "memory pool");
        uint64_t keep = s->cfg.hbm_budget_bytes;
        if ((e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep))) return fail(e, "memory pool");
    }
    if ((e = cudaMalloc(&s->d_ctl, sizeof(ServeCtl)))) return fail(e, "ctl");
    if ((e = cudaMemset(s->d_ctl, 0, sizeof(ServeCtl)))) return fail(e, "ctl");
    if ((e = cudaMalloc(&s->d_ring, sizeof(ServeJob) * s->cfg.ring_slots))) return fail(e, "ring");
    if ((e = cudaMemset(s->d_ring, 0xFF, sizeof(ServeJob) * s->cfg.ring_slots))) return fail(e, "ring");
    if ((e = cudaMallocHost(&s->h_ring, sizeof(ServeJob) * s->cfg.ring_slots))) return fail(e, "ring");
    if ((e = cudaMallocHost(&s->h_tails, 4 * s->cfg.ring_slots))) return fail(e, "tails");
    if ((e = cudaMallocHost(&s->h_seqs, 8 * s->cfg.ring_slots))) return fail(e, "seqs");
    if ((e = cudaMallocHost(&s->h_stop, 4))) return fail(e, "stop");
    *s->h_stop = 0;
    if ((e = cudaHostAlloc(&s->h_done, sizeof(ServeDone) * s->cfg.ring_slots, cudaHostAllocMapped))) return fail(e, "done");
    std::memset(s->h_done, 0, sizeof(ServeDone) * s->cfg.ring_slots);
    if ((e = cudaHostGetDevicePointer(&s->d_done, s->h_done, 0))) return fail(e, "done");
    if ((e = cudaMalloc(&s->d_queues, 4ull * kCtaScratch * s->cfg.small_vertices * s->grid))) return fail(e, "queues");
    if ((e = cudaMallocHost(&s->h_ctl_init, sizeof(PeelCtl)))) return fail(e, "ctl init");
    std::memset(s->h_ctl_init, 0, sizeof(PeelCtl));
    for (auto& sl : s->h_ctl_init->slot) sl.min_next = 0xFFFFFFFFu;
    s->stage_half = 32ull << 20;
    if ((e = cudaMallocHost(&s->stage, 2 * s->stage_half))) return fail(e, "staging");
    if ((e = cudaMallocHost(&s->dbg, 8192))) return fail(e, "debug scratch");
    if ((e = cudaMallocHost(&s->h_zero, 256))) return fail(e, "zero words");
    std::memset(s->h_zero, 0, 256);
    for (auto& ev : s->stage_ev) {
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming))) return fail(e, "staging event");
        if ((e = cudaEventRecord(ev, s->cs))) return fail(e, "staging event");
    }
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, s->dev) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    s->last_activity = clk::now();
    s->loop = std::thread(request_loop, s);
    *out = s;
    return KC_OK;
}

int kc_serve_submit(kc_server* s, const uint32_t* offsets, const uint32_t* neighbors, uint32_t V,
                    uint32_t* core_out, uint64_t* request_id) {
    if (!s || !request_id || (V && (!offsets || !core_out))) return KC_ERR_INVALID;
    Request* r = new Request();
    r->off = offsets;
    r->nbr = neighbors;
    r->V = V;
    r->E = V ? offsets[V] : 0;
    if (r->E && !neighbors) { delete r; return KC_ERR_INVALID; }
    // Offsets must start at 0 and never decrease (the kernels trust arc
    // ranges); with pinned staging the neighbour ids are checked here too,
    // otherwise while the gang copies them in.
    uint32_t md = 0;
    int bad = V && offsets[0] != 0;
#pragma omp parallel for reduction(max : md) reduction(| : bad) schedule(static)
    for (int64_t v = 0; v < (int64_t)V; ++v) {
        if (offsets[v + 1] < offsets[v]) bad = 1;
        else md = std::max(md, offsets[v + 1] - offsets[v]);
    }
    if (!bad && !s->direct) {
#pragma omp parallel for reduction(| : bad) schedule(static)
        for (int64_t e = 0; e < (int64_t)r->E; ++e) bad |= (neighbors[e] >= V);
    }
    if (bad || md >= (1u << 30)) {
        delete r;
        set_error_msg("invalid CSR: offsets must start at 0 and not decrease, neighbour ids must be < V, "
                      "degrees below 2^30");
        return KC_ERR_INVALID;
    }
    r->maxdeg = md;
    r->core_out = core_out;
    if (s->direct && V) {
        // The device writes the result straight into core_out; a page the host
        // never touched would be faulted in one device write at a time (about
        // 5 GB/s measured), so every page is touched once here, in parallel.
        const long ps = sysconf(_SC_PAGESIZE);
        const size_t step = ps > 0 ? (size_t)ps / sizeof(uint32_t) : 1024;
        const int64_t pages = (int64_t)(((size_t)V + step - 1) / step);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < pages; ++i) core_out[(size_t)i * step] = 0;
    }
    plan_request(s, r);
    if (r->bytes > s->cfg.hbm_budget_bytes) {
        delete r;
        set_error_msg("request needs more device memory than the server's HBM budget");
        return KC_ERR_BUDGET;
    }
    cudaSetDevice(s->dev);
    if (cudaEventCreateWithFlags(&r->copied, cudaEventDisableTiming) != cudaSuccess) { delete r; return KC_ERR_CUDA; }
    r->t_submit = clk::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->closing) { cudaEventDestroy(r->copied); delete r; return KC_ERR_CLOSED; }
    r->id = s->next_id++;
    if (V == 0) {   // nothing to peel: kmax = level-1 = 0xFFFFFFFF
        r->kmax = 0xFFFFFFFFu;
        r->state = 4;
        r->t_admit = r->t_publish = r->t_done = r->t_submit;
        s->stats.completed++;
    } else {
        s->pending.push_back(r);
    }
    s->all[r->id] = r;
    s->stats.submitted++;
    *request_id = r->id;
    return KC_OK;
}

static void fill_timing(const Request* r, kc_serve_timing* t) {
    if (!t) return;
    auto us = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double, std::micro>(b - a).count(); };
    t->queue_us = us(r->t_submit, r->t_admit);
    t->latency_us = us(r->t_submit, r->t_done);
    t->gang = r->gang;
    t->iterations = r->iters;
    t->copy_in_us = r->copy_in_us;
    t->peel_us = r->peel_us;
    t->copy_out_us = r->copy_out_us;
}

int kc_serve_poll(kc_server* s, uint64_t id, uint32_t* kmax, kc_serve_timing* timing) {
    if (!s) return KC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return KC_ERR_INVALID;
    Request* r = it->second;
    if (r->state != 4) return s->fatal ? s->fatal : KC_ERR_BUSY;
    if (kmax) *kmax = r->kmax;
    fill_timing(r, timing);
    const int err = r->err;
    cudaEventDestroy(r->copied);
    s->all.erase(it);
    delete r;
    return err;
}

int kc_serve_wait(kc_server* s, uint64_t id, uint32_t* kmax, kc_serve_timing* timing, double timeout_s) {
    if (!s) return KC_ERR_INVALID;
    const auto deadline = clk::now() + std::chrono::duration_cast<clk::duration>(std::chrono::duration<double>(timeout_s));
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        auto it = s->all.find(id);
        if (it == s->all.end()) return KC_ERR_INVALID;
        if (it->second->state == 4) break;
        if (s->fatal) return s->fatal;
        if (s->cv.wait_until(lk, deadline) == std::cv_status::timeout) return KC_ERR_BUSY;
    }
    lk.unlock();
    return kc_serve_poll(s, id, kmax, timing);
}

// Diagnostic snapshot (read-only): out[0..9] = ticket_head, tail, stop, err,
// idle_exits, kernel running, next ticket, next seq, bytes in use, requests in
// flight; then 8 words per in-flight request: seq, gang, ticket0, state, its
// gang counters' iterations done, error, members finished, kmax.
int kc_serve_debug(kc_server* s, uint64_t* out, uint32_t n) {
    if (!s || !out || n < 10) return KC_ERR_INVALID;
    cudaSetDevice(s->dev);
    cudaStream_t ds;
    KC_CUDA(cudaStreamCreateWithFlags(&ds, cudaStreamNonBlocking));
    // pinned scratch: a copy into pageable memory would wait for the serve kernel
    ServeCtl& c = *reinterpret_cast<ServeCtl*>(s->dbg);
    PeelCtl& pc = *reinterpret_cast<PeelCtl*>(s->dbg + 2048);
    uint32_t& fin = *reinterpret_cast<uint32_t*>(s->dbg + 6144);
    cudaMemcpyAsync(&c, s->d_ctl, sizeof(c), cudaMemcpyDeviceToHost, ds);
    cudaStreamSynchronize(ds);
    std::lock_guard<std::mutex> lk(s->mu);
    out[0] = c.ticket_head; out[1] = c.tail; out[2] = c.stop; out[3] = (uint64_t)(int64_t)c.err;
    out[4] = c.idle_exits; out[5] = s->kernel_running; out[6] = s->next_ticket; out[7] = s->next_seq;
    out[8] = s->in_use; out[9] = s->inflight.size();
    uint32_t k = 10;
    for (Request* r : s->inflight) {
        if (k + 8 > n) break;
        const ServeJob& j = s->h_ring[r->seq % s->cfg.ring_slots];
        std::memset(&pc, 0, sizeof(pc));
        fin = 0;
        if (r->d_ctl) cudaMemcpyAsync(&pc, r->d_ctl, sizeof(pc), cudaMemcpyDeviceToHost, ds);
        if (r->d_fin) cudaMemcpyAsync(&fin, r->d_fin, 4, cudaMemcpyDeviceToHost, ds);
        cudaStreamSynchronize(ds);
        out[k++] = r->seq; out[k++] = r->gang; out[k++] = j.ticket0; out[k++] = (uint64_t)r->state;
        out[k++] = pc.iters_done; out[k++] = (uint64_t)(int64_t)pc.err; out[k++] = fin; out[k++] = pc.kmax;
    }
    cudaStreamDestroy(ds);
    return KC_OK;
}

int kc_serve_stats_get(kc_server* s, kc_serve_stats* st) {
    if (!s || !st) return KC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *st = s->stats;
    st->in_use = s->in_use;
    st->pending = (uint32_t)s->pending.size();
    st->inflight = (uint32_t)s->inflight.size();
    st->blocks = (uint32_t)s->grid;
    st->direct = s->direct ? 1u : 0u;
    return KC_OK;
}

int kc_serve_close(kc_server* s) {
    if (!s) return KC_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->closing = true;
    }
    if (s->loop.joinable()) s->loop.join();
    const int fatal = s->fatal;
    cudaSetDevice(s->dev);
    for (auto& kv : s->all) {
        device_free(s, kv.second);
        if (kv.second->copied) cudaEventDestroy(kv.second->copied);
        delete kv.second;
    }
    cudaStreamSynchronize(s->cs);
    cudaFree(s->d_ctl); cudaFree(s->d_ring); cudaFree(s->d_queues);
    cudaFreeHost(s->h_ring); cudaFreeHost(s->h_tails); cudaFreeHost(s->h_seqs); cudaFreeHost(s->h_stop); cudaFreeHost(s->h_done);
    cudaFreeHost(s->h_ctl_init);
    cudaFreeHost(s->stage);
    cudaFreeHost(s->dbg);
    cudaFreeHost(s->h_zero);
    for (auto& ev : s->stage_ev) if (ev) cudaEventDestroy(ev);
    cudaStreamDestroy(s->ks);
    cudaStreamDestroy(s->cs);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return fatal;
}

}  // extern "C"
