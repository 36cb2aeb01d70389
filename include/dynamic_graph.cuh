/* GPU_Dynamic_Graph<T> (LIB/include/dynamic_graph.cuh:8-26): a GPU_Graph
 * plus an optional GPU_Diff_Graph; get_graph() returns the GPU_Graph by
 * value (a shallow copy sharing its device arrays and engine graph). */
#ifndef DDP_LIB_DYNAMIC_GRAPH_CUH
#define DDP_LIB_DYNAMIC_GRAPH_CUH

#include "diff_graph.cuh"

template <class T>
class GPU_Dynamic_Graph {
   private:
    GPU_Graph<T> *graph = nullptr;
    GPU_Diff_Graph<T> *diff = nullptr;
    bool is_diff = false;

   public:
    GPU_Dynamic_Graph() {}
    GPU_Dynamic_Graph(GPU_Graph<T> *g, GPU_Diff_Graph<T> *d) : graph(g), diff(d), is_diff(true) {}
    GPU_Dynamic_Graph(GPU_Graph<T> *g) : graph(g) {}

    GPU_Graph<T> get_graph() { return *graph; }
    GPU_Diff_Graph<T> get_diff_graph() { return *diff; }
};

#endif
