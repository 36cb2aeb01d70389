/* Dynamic_Graph<T> (LIB/include/dynamic_graph.h:7-29): a Graph plus an
 * optional Diff_Graph.  get_graph() returns the graph by value (a shallow
 * copy: the arrays stay shared), as in the reference.  merge / make_diff /
 * update_Del are declared without definitions there; they stay declared
 * only (the engine's update path is ddp_dyn_update). */
#ifndef DDP_LIB_DYNAMIC_GRAPH_H
#define DDP_LIB_DYNAMIC_GRAPH_H

#include "diff_graph.h"

template <class T = unsigned int>
class Dynamic_Graph {
   private:
    Graph<T> *graph;
    Diff_Graph<T> *diff;
    bool is_diff = false;

   public:
    Dynamic_Graph() : graph(new Graph<T>()), diff(new Diff_Graph<T>(0)), is_diff(true) {}
    Dynamic_Graph(Graph<T> *g, Diff_Graph<T> *d) : graph(g), diff(d), is_diff(true) {}
    Dynamic_Graph(Graph<T> *g) : graph(g), diff(nullptr), is_diff(false) {}

    Graph<T> get_graph() { return *graph; }
    Diff_Graph<T> get_diff_graph() { return *diff; }

    void merge();
    void make_diff();
    void update_Del();
};

#endif
