/* A_Star<T, U> (LIB/include/a_star.h:13-51, :191-275): one (start, end)
 * query with a caller-supplied heuristic.
 *
 * Same constructor, set_huiristics and get_path as the reference:
 * get_path() returns {-1} when no heuristic was set, {} when end cannot be
 * reached, else the path start..end.  The reference runs a serial CPU A*
 * here; the shim runs the same query through the GPU engine (ddp_solve),
 * which returns the same cost (ties may pick another equal-cost path).  K,
 * the reference's queue count, is accepted and not needed: the engine's
 * bucket width sets its parallelism.  The graph is uploaded per call, as
 * the reference re-reads it per call; GPU_A_Star keeps it resident. */
#ifndef DDP_LIB_A_STAR_H
#define DDP_LIB_A_STAR_H

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ddp_lib_detail.h"
#include "dynamic_graph.h"

template <class T, class U>
class A_Star {
   private:
    Dynamic_Graph<T> *graph;
    U *Hx = nullptr;
    unsigned int start_node, end_node, num_pq;
    bool is_set_hx = false;

   public:
    A_Star(Dynamic_Graph<T> *g, unsigned int start, unsigned int end, unsigned int K)
        : graph(g), start_node(start), end_node(end), num_pq(K) {}

    void set_huiristics(U *hx) {  // borrows the pointer, as the reference does
        Hx = hx;
        is_set_hx = true;
    }

    std::vector<int> get_path() {
        if (!is_set_hx) return std::vector<int>(1, -1);
        Graph<T> g = graph->get_graph();
        ddp_graph *dg = ddp_lib::upload(g.get_num_nodes(), g.get_num_edges(), g.get_offsets(), g.get_edges(),
                                        g.get_weights());
        std::vector<int> p = ddp_lib::solve(dg, g.get_num_nodes(), Hx, start_node, end_node);
        ddp_graph_free(dg);
        return p;
    }
};

#endif
