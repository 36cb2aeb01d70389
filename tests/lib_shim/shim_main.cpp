// Exercises the header-only LIB shim (include/graph.h, a_star.h, and with
// nvcc graph.cuh, a_star.cuh) the way a caller of the reference's LIB
// classes does: read a graph file, run A_Star and GPU_A_Star with h = 0 (or
// without h), print each path on one line.
//   shim_main <graph file> <start> <end> [K]
#include <cstdio>
#include <cstdlib>
#include <string>

#include "include/a_star.h"
#include "include/dynamic_graph.h"
#include "include/graph.h"
#ifdef __NVCC__
#include "include/a_star.cuh"
#include "include/graph.cuh"
#endif

static void print_path(const char *tag, const std::vector<int> &p) {
    std::printf("%s", tag);
    for (size_t i = 0; i < p.size(); i++) std::printf(" %d", p[i]);
    std::printf("\n");
}

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s graph start end [K]\n", argv[0]);
        return 2;
    }
    const unsigned s = (unsigned)std::atoi(argv[2]), t = (unsigned)std::atoi(argv[3]);
    const unsigned K = argc > 4 ? (unsigned)std::atoi(argv[4]) : 1u;
    Graph<unsigned int> graph;
    graph.read_graph(std::string(argv[1]));
    Dynamic_Graph<unsigned int> dgraph(&graph);
    int *hx = (int *)std::calloc((size_t)graph.get_num_nodes(), sizeof(int));

    A_Star<unsigned int, int> unset(&dgraph, s, t, K);
    print_path("cpu_class_unset:", unset.get_path());
    A_Star<unsigned int, int> algo(&dgraph, s, t, K);
    algo.set_huiristics(hx);
    print_path("cpu_class:", algo.get_path());
#ifdef __NVCC__
    GPU_Graph<unsigned int> g(&graph);
    GPU_Dynamic_Graph<unsigned int> dg(&g);
    GPU_A_Star<unsigned int, int> galgo(&dg, s, t, K);
    galgo.set_huiristics(hx);
    print_path("gpu_class:", galgo.get_path());
    print_path("gpu_class_again:", galgo.get_path());
    g.__gpu_free();
#endif
    std::free(hx);
    graph.free();
    return 0;
}
