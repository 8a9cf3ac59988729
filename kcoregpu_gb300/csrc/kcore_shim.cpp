// Reference-side shim: the driver signature `int kcore(Graph&)` of
// src/ours.cc:117 on top of the C ABI, so that a main.cu-style driver
// (main.cu:20-30, 60-61: repSimulation(kcore, g)) links against
// libkcore_gb300.so instead of compiling src/ours.cc.
//
// Build it with the caller's own graph.h on the include path:
//   g++ -O2 -c kcore_shim.cpp -I<reference>/inc -I<repo>/include
//   ... link: -L<repo>/kcoregpu_gb300 -lkcore_gb300
// and replace `#include "./src/ours.cc"` in main.cu by `int kcore(Graph&);`.
//
// Contract kept from the reference (src/ours.cc:117-160,
// src/gpu_memory_allocation.cu:4-22):
//   * g.degrees is only read (it is uploaded as the starting degrees in the
//     reference); the eight other variants of main.cu:64-88 re-upload it, so
//     the shim never writes it.  Core numbers go to a separate buffer
//     (kcore_into), never into the Graph.
//   * g.kmax is set to the last level, as ours.cc:151 sets level-1.
//   * The return value is the peel's elapsed milliseconds, measured like
//     ours.cc:136-153 (after the upload, until the last level is done).
//   * A failure prints the library's message and exits with -1, as chkerr
//     does (inc/gpu_memory_allocation.h:9-16).
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <iostream>
#include <vector>

#include "graph.h"
#include "kcore.h"

namespace {

[[noreturn]] void shim_fail(const char* what, int rc) {
    std::cout << what << ": " << kc_strerror(rc) << " (" << kc_last_error() << ")" << std::endl;
    std::exit(-1);
}

}  // namespace

// Peels g and writes the core number of every vertex to core_out (g.V
// entries; may be NULL).  Leaves every array of g untouched; sets g.kmax.
// Returns the peel's milliseconds.
int kcore_into(Graph& g, unsigned int* core_out) {
    kc_graph* dg = nullptr;
    int rc = kc_graph_upload(g.neighbors_offset, g.neighbors, g.V, &dg);
    if (rc != KC_OK) shim_fail("kc_graph_upload", rc);
    uint32_t kmax = 0;
    auto start = std::chrono::steady_clock::now();
    rc = kc_graph_peel_async(dg);
    if (rc == KC_OK) rc = kc_graph_fetch(dg, nullptr, &kmax, nullptr);
    auto end = std::chrono::steady_clock::now();
    if (rc == KC_OK && core_out) rc = kc_graph_fetch(dg, core_out, nullptr, nullptr);
    kc_graph_free(dg);
    if (rc != KC_OK) shim_fail("kcore", rc);
    g.kmax = kmax;
    return (int)std::chrono::duration_cast<std::chrono::milliseconds>(end - start).count();
}

int kcore(Graph& g) { return kcore_into(g, nullptr); }
