// TEST INFRASTRUCTURE ONLY.  Driver around the reference's own loader
// (src/graph.cpp, compiled unmodified by oracle/build_ref.sh) used to make
// golden fixtures for the loader, the serialized cache and the JSON writer.
//
//   ref_loader load <edgelist>            Graph(path): writes ./output/serialized-<basename>
//   ref_loader json <edgelist> <corefile> Graph(path) (cache hit), degrees := the
//                                         whitespace-separated values of <corefile>,
//                                         writeKCoreToDisk(<basename>)
// Run it from a scratch directory that contains ./output/.
#include <fstream>
#include <iostream>
#include <string>

#include "graph.h"

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cerr << "usage: ref_loader load <edgelist> | json <edgelist> <corefile>\n";
        return 2;
    }
    std::string mode = argv[1];
    std::string path = argv[2];
    Graph g(path);
    std::cout << "V: " << g.V << "\nE: " << g.E << std::endl;
    if (mode == "json") {
        if (argc < 4) return 2;
        std::ifstream f(argv[3]);
        for (unsigned int i = 0; i < g.V; ++i) f >> g.degrees[i];
        std::string base = path.substr(path.find_last_of('/') + 1);
        g.writeKCoreToDisk(base);
    }
    return 0;
}
