// Test driver of kcore_shim.cpp in the shape of the reference's main.cu
// (main.cu:20-30, 60-61): loads a binary CSR ("V E" as uint32, then offsets
// and neighbours), fills a Graph, and calls kcore(g) twice through
// repSimulation's signature.  Checks that g.degrees is unchanged by both calls
// and that both set the same kmax; writes the core numbers of a third call
// (kcore_into) to argv[2] and prints "kmax <k>".  Exit 0 on success.
#include <cstdio>
#include <cstring>
#include <iostream>
#include <vector>

#include "graph.h"

int kcore(Graph& g);
int kcore_into(Graph& g, unsigned int* core_out);

template <class T>
void repSimulation(int (*kern)(T), Graph& g) {
    unsigned int t = (*kern)(g);
    std::cout << t << " " << std::endl;
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    unsigned int hdr[2];
    if (std::fread(hdr, 4, 2, f) != 2) return 2;
    Graph g;
    g.V = hdr[0];
    g.E = hdr[1];
    std::vector<unsigned int> off(g.V + 1), nbr(g.E ? g.E : 1), deg(g.V ? g.V : 1);
    if (std::fread(off.data(), 4, g.V + 1, f) != g.V + 1) return 2;
    if (g.E && std::fread(nbr.data(), 4, g.E, f) != g.E) return 2;
    std::fclose(f);
    for (unsigned int v = 0; v < g.V; ++v) deg[v] = off[v + 1] - off[v];
    const std::vector<unsigned int> deg0 = deg;
    g.neighbors_offset = off.data();
    g.neighbors = nbr.data();
    g.degrees = deg.data();
    g.kmax = 0xDEADBEEFu;
    std::cout << "Ours: ";
    repSimulation(kcore, g);
    const unsigned int k1 = g.kmax;
    if (deg != deg0) { std::cout << "degrees changed by the first call" << std::endl; return 1; }
    if (k1 == 0xDEADBEEFu) { std::cout << "kmax not set" << std::endl; return 1; }
    g.kmax = 0xDEADBEEFu;
    std::cout << "Ours: ";
    repSimulation(kcore, g);
    if (deg != deg0) { std::cout << "degrees changed by the second call" << std::endl; return 1; }
    if (g.kmax != k1) { std::cout << "kmax differs between calls" << std::endl; return 1; }
    std::vector<unsigned int> core(g.V ? g.V : 1);
    kcore_into(g, core.data());
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    std::fwrite(core.data(), 4, g.V, o);
    std::fclose(o);
    std::cout << "kmax " << g.kmax << std::endl;
    return 0;
}
