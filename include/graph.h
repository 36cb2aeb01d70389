/* Graph<T>: host CSR in the reference's layout (LIB/include/graph.h:13-43).
 *
 * Header-only shim over libddp_gb300: same members, signatures and text
 * format as the reference, so code written against LIB/include builds
 * unchanged (LIB/main.cpp does).  N offsets (no sentinel); row u ends at
 * offsets[u+1], the last row at E.  Arrays are malloc-owned by the Graph. */
#ifndef DDP_LIB_GRAPH_H
#define DDP_LIB_GRAPH_H

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <unordered_map>

template <class DataType>
class Graph {
   public:
    unsigned int N;  // nodes 0 .. N-1
    unsigned int E;
    int *offsets;
    int *edges;
    DataType *weights;
    std::unordered_map<long, int> vertex_map;  // kept for interface parity

    Graph() : N(0), E(0), offsets(nullptr), edges(nullptr), weights(nullptr) {}

    void __alloc__(int n, int e) {
        N = (unsigned)n;
        E = (unsigned)e;
        offsets = (int *)std::malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
        edges = (int *)std::malloc(sizeof(int) * (size_t)(e > 0 ? e : 1));
        weights = (DataType *)std::malloc(sizeof(DataType) * (size_t)(e > 0 ? e : 1));
    }

    int get_num_nodes() { return (int)N; }
    int get_num_edges() { return (int)E; }
    int *get_offsets() { return offsets; }
    int *get_edges() { return edges; }
    DataType *get_weights() { return weights; }

    /* Text format: "N E", E heads, N offsets, E weights (whitespace
     * separated).  A missing file prints the reference's message and exits. */
    void read_graph(std::string filename) {
        std::ifstream in(filename);
        if (!in) {
            std::cout << "[ERROR] Couldn't open graph file\n";
            std::exit(1);
        }
        int n = 0, e = 0;
        in >> n >> e;
        __alloc__(n, e);
        for (int i = 0; i < e; i++) in >> edges[i];
        for (int i = 0; i < n; i++) in >> offsets[i];
        for (int i = 0; i < e; i++) in >> weights[i];
    }

    void free() {
        std::free(offsets);
        std::free(edges);
        std::free(weights);
        offsets = edges = nullptr;
        weights = nullptr;
    }
};

#endif
