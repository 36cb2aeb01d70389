/* GPU_A_Star<T, U> (LIB/include/a_star.cuh:12-52): A_Star on the
 * GPU_Graph's resident device graph.  Same conventions as A_Star ({-1}
 * without a heuristic, {} when unreachable, else start..end).  Unlike the
 * reference, get_path() can be called again (the reference re-allocates
 * and does not reset its costs); free_gpu(), declared there without a
 * definition, is a no-op here (the engine frees per-query state itself). */
#ifndef DDP_LIB_A_STAR_CUH
#define DDP_LIB_A_STAR_CUH

#include "a_star.h"
#include "dynamic_graph.cuh"

template <class T, class U>
class GPU_A_Star {
   private:
    GPU_Dynamic_Graph<T> *graph;
    U *Hx = nullptr;
    unsigned int start_node, end_node, num_pq;
    bool is_set_hx = false;

   public:
    GPU_A_Star(GPU_Dynamic_Graph<T> *g, unsigned int start, unsigned int end, unsigned int K)
        : graph(g), start_node(start), end_node(end), num_pq(K) {}

    void set_huiristics(U *hx) {
        Hx = hx;
        is_set_hx = true;
    }

    std::vector<int> get_path() {
        if (!is_set_hx) return std::vector<int>(1, -1);
        GPU_Graph<T> g = graph->get_graph();
        return ddp_lib::solve(g.ddp_handle(), g.get_num_nodes(), Hx, start_node, end_node);
    }

    void free_gpu() {}
};

#endif
