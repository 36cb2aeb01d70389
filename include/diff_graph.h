/* Diff_Graph<T> (LIB/include/diff_graph.h:6-20): a Graph with an id.  The
 * reference declares it for update batches but never fills it; updates go
 * through ddp_dyn_update here. */
#ifndef DDP_LIB_DIFF_GRAPH_H
#define DDP_LIB_DIFF_GRAPH_H

#include "graph.h"

template <class T = unsigned int>
class Diff_Graph : public Graph<T> {
   private:
    int id = 0;

   public:
    Diff_Graph() {}
    Diff_Graph(int i) : id(i) {}
};

#endif
