// `kcore <edgelist>`: drop-in for the reference CLI (main.cu:44-91) on the
// GB300 peel.  Prints the reference's lines for the one variant it runs
// ("Ours"), including the loader's (graph.cpp:13,28,145-152) and the Graph
// destructor's (graph.cpp:157):
//
//   Graph loading Started...
//   Reading serialized file...                    (cache hit), or
//   serialized-<file> : File couldn't open        (cache miss)
//   Reading normal file...
//   [serialized-<file> : File couldn't open]      (the cache could not be written)
//   File Loaded in: <ms>
//   ******************  <file> ******************
//   V: <V>
//   E: <arcs>
//   Ours: <ms>
//   Kmax: <kmax>
//   Deallocated...
//
// A text file that cannot be opened prints "load graph file failed " and exits
// with status 255, like graph.cpp:63-66's exit(-1).
//
// Options (after the file): --cache-dir DIR (default ./output/, the reference's
// OUTPUT_LOC), --parse reference|snap, --json (writes DIR/pkc-kcore-<file>,
// graph.cpp:126-140), --txt FILE ("id core" lines), --order FILE (peel order and
// k-shell offsets), --stats (one JSON line with device timing).
#include <chrono>
#include <cstdio>
#include <sys/stat.h>
#include <cstring>
#include <string>
#include <vector>

#include "kcore.h"

static int die(const char* what, int rc) {
    std::fprintf(stderr, "%s: %s (%s)\n", what, kc_strerror(rc), kc_last_error());
    return 1;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::printf("Please provide data file\n");   // main.cu:45-47
        return 255;
    }
    std::string ds = argv[1];
    std::string cache = "./output/", txt, order_file;
    int mode = KC_PARSE_SNAP;
    bool json = false, stats = false;
    for (int i = 2; i < argc; ++i) {
        std::string a = argv[i];
        if (a == "--cache-dir" && i + 1 < argc) cache = argv[++i];
        else if (a == "--parse" && i + 1 < argc) mode = std::strcmp(argv[++i], "reference") == 0 ? KC_PARSE_REFERENCE : KC_PARSE_SNAP;
        else if (a == "--json") json = true;
        else if (a == "--txt" && i + 1 < argc) txt = argv[++i];
        else if (a == "--order" && i + 1 < argc) order_file = argv[++i];
        else if (a == "--stats") stats = true;
        else { std::fprintf(stderr, "unknown option %s\n", a.c_str()); return 2; }
    }
    std::printf("Graph loading Started... \n");
    const std::string base = ds.substr(ds.find_last_of('/') + 1);
    std::string cdir = cache;
    if (!cdir.empty() && cdir.back() != '/') cdir.push_back('/');
    kc_csr_host g{};
    int from_cache = 0;
    auto t0 = std::chrono::steady_clock::now();
    int rc = kc_load_graph(ds.c_str(), cache.c_str(), mode, &g, &from_cache);
    if (rc == KC_ERR_IO) {   // graph.cpp:13, 145, 63-66
        std::printf("serialized-%s : File couldn't open\n", base.c_str());
        std::printf("Reading normal file... \n");
        std::printf("load graph file failed \n");
        return 255;
    }
    if (rc) return die("load", rc);
    if (from_cache) {
        std::printf("Reading serialized file... \n");   // graph.cpp:13
    } else {
        std::printf("serialized-%s : File couldn't open\n", base.c_str());   // graph.cpp:28
        std::printf("Reading normal file... \n");                           // graph.cpp:145
        struct stat sb;
        if (stat((cdir + "serialized-" + base).c_str(), &sb) != 0)          // graph.cpp:52 (cache not written)
            std::printf("serialized-%s : File couldn't open\n", base.c_str());
        std::printf("File Loaded in: %lld\n", (long long)std::chrono::duration_cast<std::chrono::milliseconds>(
                                                  std::chrono::steady_clock::now() - t0).count());
    }
    std::printf("******************  %s ****************** \n", ds.c_str());
    std::printf("V: %u\n", g.V);
    std::printf("E: %u\n", g.E);

    kc_graph* dg = nullptr;
    rc = kc_graph_upload(g.offsets, g.neighbors, g.V, &dg);
    if (rc) return die("upload", rc);
    std::vector<uint32_t> core(g.V ? g.V : 1);
    uint32_t kmax = 0;
    kc_stats st{};
    auto t1 = std::chrono::steady_clock::now();
    rc = kc_peel(dg, core.data(), &kmax, &st);
    auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t1).count();
    if (rc) return die("peel", rc);
    std::printf("Ours: %lld \n", (long long)ms);
    std::printf("Kmax: %u\n", kmax);
    if (stats)
        std::printf("{\"V\": %u, \"arcs\": %llu, \"kmax\": %u, \"levels\": %u, \"peel_ms\": %.4f, \"blocks\": %u}\n",
                    g.V, (unsigned long long)st.arcs, st.kmax, st.levels, st.peel_ms, st.blocks);
    if (json) {
        rc = kc_write_core_json((cdir + "pkc-kcore-" + base).c_str(), core.data(), g.V);
        if (rc) return die("json", rc);
    }
    if (!txt.empty() && (rc = kc_write_core_txt(txt.c_str(), core.data(), g.V))) return die("txt", rc);
    if (!order_file.empty()) {
        std::vector<uint32_t> order(g.V ? g.V : 1), shells(kmax + 2 > 1 ? kmax + 2 : 2);
        uint32_t k2 = 0;
        rc = kc_degeneracy_order(dg, order.data(), shells.data(), (uint32_t)shells.size(), &k2);
        if (rc) return die("order", rc);
        FILE* f = std::fopen(order_file.c_str(), "w");
        if (!f) return die("order file", KC_ERR_IO);
        for (uint32_t k = 0; k + 1 < shells.size() && g.V; ++k) {
            std::fprintf(f, "shell %u:", k);
            for (uint32_t i = shells[k]; i < shells[k + 1]; ++i) std::fprintf(f, " %u", order[i]);
            std::fprintf(f, "\n");
        }
        std::fclose(f);
    }
    kc_graph_free(dg);
    kc_csr_free(&g);
    std::printf("Deallocated... \n");   // ~Graph, graph.cpp:157
    return 0;
}
