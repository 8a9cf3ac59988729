// TEST INFRASTRUCTURE ONLY.  Runs the reference's own GPU peel
// (selectNodesAtLevel1 / processNodes1 from src/ours.cc, compiled unmodified
// into oracle/_ref/ref_peel.cubin by oracle/build_ref.sh) and replays its host
// loop, kcore() (src/ours.cc:117-160), through the CUDA driver API; then copies
// the degree array back (get_results_from_gpu, src/gpu_memory_allocation.cu:14-16),
// which holds the core numbers.
//
//   ref_peel_driver <cubin> <csr.bin> <core_out.bin>
// csr.bin: uint32 V, uint32 E, offsets[V+1], neighbors[E] (little endian).
// Prints "kmax <k> levels <L> ms <t>".
//
// Safety: the reference kernels assert() when a per-block queue passes
// GLBUFFER_SIZE = 1e6 entries (src/buffer.cc:2, inc/common.h:12), which would
// trap the GPU context.  A level can only put its own frontier into the queues,
// so the driver first computes every level's size on the host (bucket peel) and
// refuses (exit 3) any graph with a level of 1e6 vertices or more.
#include <cuda.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static const unsigned kBlocks = 56, kThreads = 1024;   // inc/common.h:4-5
static const size_t kQueue = 1000000;                  // inc/common.h:12

#define CK(x)                                                                  \
    do {                                                                       \
        CUresult r_ = (x);                                                     \
        if (r_ != CUDA_SUCCESS) {                                              \
            const char* s_ = nullptr;                                          \
            cuGetErrorString(r_, &s_);                                         \
            std::fprintf(stderr, "%s failed: %s\n", #x, s_ ? s_ : "?");        \
            return 4;                                                          \
        }                                                                      \
    } while (0)

struct GPointers {   // layout of G_pointers (inc/common.h:45-50)
    CUdeviceptr neighbors;
    CUdeviceptr neighbors_offset;
    CUdeviceptr degrees;
    unsigned int V;
};

// Largest k-shell (vertices peeled in one level), by a bucket peel.
static size_t max_shell(uint32_t V, const std::vector<uint32_t>& off, const std::vector<uint32_t>& nbr) {
    std::vector<uint32_t> d(V), bin, pos(V), vert(V);
    uint32_t md = 0;
    for (uint32_t v = 0; v < V; ++v) { d[v] = off[v + 1] - off[v]; md = std::max(md, d[v]); }
    bin.assign(md + 1, 0);
    for (uint32_t v = 0; v < V; ++v) bin[d[v]]++;
    uint32_t s = 0;
    for (uint32_t k = 0; k <= md; ++k) { uint32_t n = bin[k]; bin[k] = s; s += n; }
    for (uint32_t v = 0; v < V; ++v) { pos[v] = bin[d[v]]; vert[pos[v]] = v; bin[d[v]]++; }
    for (uint32_t k = md; k >= 1; --k) bin[k] = bin[k - 1];
    if (md + 1 > 0) bin[0] = 0;
    for (uint32_t i = 0; i < V; ++i) {
        uint32_t v = vert[i];
        for (uint32_t j = off[v]; j < off[v + 1]; ++j) {
            uint32_t u = nbr[j];
            if (d[u] > d[v]) {
                uint32_t du = d[u], pu = pos[u], pw = bin[du], w = vert[pw];
                if (u != w) { pos[u] = pw; vert[pu] = w; pos[w] = pu; vert[pw] = u; }
                bin[du]++;
                d[u]--;
            }
        }
    }
    std::vector<size_t> cnt(md + 2, 0);
    size_t best = 0;
    for (uint32_t v = 0; v < V; ++v) best = std::max(best, ++cnt[d[v]]);
    return best;
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: ref_peel_driver <cubin> <csr.bin> <core_out.bin>\n");
        return 2;
    }
    FILE* f = std::fopen(argv[2], "rb");
    if (!f) { std::perror("csr"); return 2; }
    uint32_t V = 0, E = 0;
    if (std::fread(&V, 4, 1, f) != 1 || std::fread(&E, 4, 1, f) != 1) return 2;
    std::vector<uint32_t> off((size_t)V + 1), nbr(E ? E : 1);
    if (std::fread(off.data(), 4, (size_t)V + 1, f) != (size_t)V + 1) return 2;
    if (E && std::fread(nbr.data(), 4, E, f) != E) return 2;
    std::fclose(f);
    if (V == 0 || V > 0x7FFFFFFFu) { std::fprintf(stderr, "unsupported V\n"); return 3; }
    size_t ms = max_shell(V, off, nbr);
    if (ms >= kQueue) {
        std::fprintf(stderr, "refused: a level holds %zu vertices >= per-block queue %zu\n", ms, kQueue);
        return 3;
    }

    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CUmodule mod;
    CK(cuModuleLoad(&mod, argv[1]));
    unsigned nf = 0;
    CK(cuModuleGetFunctionCount(&nf, mod));
    std::vector<CUfunction> fns(nf);
    CK(cuModuleEnumerateFunctions(fns.data(), nf, mod));
    CUfunction fsel = nullptr, fproc = nullptr;
    for (CUfunction fn : fns) {
        const char* name = nullptr;
        CK(cuFuncGetName(&name, fn));
        if (std::strstr(name, "selectNodesAtLevel1")) fsel = fn;
        if (std::strstr(name, "processNodes1")) fproc = fn;
    }
    if (!fsel || !fproc) { std::fprintf(stderr, "kernels not found in cubin\n"); return 4; }

    GPointers p{};
    p.V = V;
    CUdeviceptr global_count, bufTails, glBuffers;
    CK(cuMemAlloc(&p.neighbors, sizeof(uint32_t) * (E ? E : 1)));
    CK(cuMemAlloc(&p.neighbors_offset, sizeof(uint32_t) * ((size_t)V + 1)));
    CK(cuMemAlloc(&p.degrees, sizeof(uint32_t) * V));
    if (E) CK(cuMemcpyHtoD(p.neighbors, nbr.data(), sizeof(uint32_t) * E));
    CK(cuMemcpyHtoD(p.neighbors_offset, off.data(), sizeof(uint32_t) * ((size_t)V + 1)));
    std::vector<uint32_t> deg(V);
    for (uint32_t v = 0; v < V; ++v) deg[v] = off[v + 1] - off[v];
    CK(cuMemcpyHtoD(p.degrees, deg.data(), sizeof(uint32_t) * V));
    CK(cuMemAlloc(&global_count, sizeof(uint32_t)));
    CK(cuMemAlloc(&bufTails, sizeof(uint32_t) * kBlocks));
    CK(cuMemAlloc(&glBuffers, sizeof(uint32_t) * kBlocks * kQueue));
    CK(cuMemsetD32(global_count, 0, 1));

    uint32_t maxdeg = 0;
    for (uint32_t v = 0; v < V; ++v) maxdeg = std::max(maxdeg, deg[v]);
    unsigned int level = 0, count = 0;
    auto t0 = std::chrono::steady_clock::now();
    while (count < V) {                                            // ours.cc:138
        CK(cuMemsetD32(bufTails, 0, kBlocks));                     // ours.cc:139
        unsigned int V_u = V;
        void* a1[] = {&p.degrees, &level, &V_u, &bufTails, &glBuffers};
        CK(cuLaunchKernel(fsel, kBlocks, 1, 1, kThreads, 1, 1, 0, nullptr, a1, nullptr));   // ours.cc:141
        int level_i = (int)level, V_i = (int)V;
        void* a2[] = {&p, &level_i, &V_i, &bufTails, &glBuffers, &global_count};
        CK(cuLaunchKernel(fproc, kBlocks, 1, 1, kThreads, 1, 1, 0, nullptr, a2, nullptr));  // ours.cc:144
        CK(cuMemcpyDtoH(&count, global_count, sizeof(uint32_t)));                          // ours.cc:147
        level++;
        if (level > maxdeg + 1) {   // every vertex is peeled by level maxdeg
            std::fprintf(stderr, "reference loop did not converge (count %u of %u)\n", count, V);
            return 5;
        }
    }
    unsigned int kmax = level - 1;                                 // ours.cc:151
    double msec = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    CK(cuMemcpyDtoH(deg.data(), p.degrees, sizeof(uint32_t) * V));
    FILE* o = std::fopen(argv[3], "wb");
    if (!o) { std::perror("out"); return 2; }
    std::fwrite(deg.data(), 4, V, o);
    std::fclose(o);
    std::printf("kmax %u levels %u ms %.3f\n", kmax, level, msec);
    cuMemFree(glBuffers); cuMemFree(bufTails); cuMemFree(global_count);
    cuMemFree(p.degrees); cuMemFree(p.neighbors_offset); cuMemFree(p.neighbors);
    cuModuleUnload(mod);
    cuDevicePrimaryCtxRelease(dev);
    return 0;
}
