// Test stand-in for the reference's Graph class (inc/graph.h:5-22): the same
// data members, in the same order and of the same types, which is all that
// kcore_shim.cpp reads or writes.  The shim's GPU test builds against this
// header on hosts without the reference sources; a CPU test builds the shim
// against the reference's own inc/graph.h and src/graph.cpp.
#ifndef KC_TEST_GRAPH_H
#define KC_TEST_GRAPH_H
class Graph {
public:
    unsigned int V;
    unsigned int E;
    unsigned int AVG_DEGREE = 0;
    unsigned int* neighbors;
    unsigned int* neighbors_offset;
    unsigned int* degrees;
    unsigned int kmax, dmax;
};
#endif
