/* GPU_Diff_Graph<T> (LIB/include/diff_graph.cuh:9-20): declared by the
 * reference for device-side update batches; kept for interface parity. */
#ifndef DDP_LIB_DIFF_GRAPH_CUH
#define DDP_LIB_DIFF_GRAPH_CUH

#include "graph.cuh"

template <class T = unsigned int>
class GPU_Diff_Graph : GPU_Graph<T> {
   private:
    int id = 0;

   public:
    GPU_Diff_Graph() {}
    GPU_Diff_Graph(int i) : id(i) {}
};

#endif
