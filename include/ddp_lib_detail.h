/* Shared helpers of the header-only C++ shim (graph.h, a_star.h, graph.cuh,
 * a_star.cuh) that re-declares the reference's LIB/include classes on top of
 * the libddp_gb300 C ABI.  Not part of the reference's interface. */
#ifndef DDP_LIB_DETAIL_H
#define DDP_LIB_DETAIL_H

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "ddp_gb300.h"

namespace ddp_lib {

/* The reference stops the process on any CUDA error (gpuErrchk -> exit);
 * the shim does the same with the library's status code and message. */
inline void check(int rc) {
    if (rc != DDP_OK) {
        std::fprintf(stderr, "[ddp] error %d: %s\n", rc, ddp_last_error());
        std::exit(rc);
    }
}

/* Device graph from the reference's host CSR (N offsets, no sentinel). */
template <class T>
inline ddp_graph *upload(int n, int e, const int *offsets, const int *edges, const T *weights) {
    static_assert(std::is_integral<T>::value, "the engine is integer-exact: integral weights only");
    std::vector<uint32_t> w((size_t)(e > 0 ? e : 1));
    for (int i = 0; i < e; i++) w[(size_t)i] = (uint32_t)weights[i];
    ddp_graph *g = nullptr;
    check(ddp_graph_from_csr(n, e, offsets, n, edges, w.data(), &g));
    return g;
}

/* One query on a device graph with the caller's h (A_Star::set_huiristics):
 * {} when t is unreachable, else the path s..t.  h < 0 marks a node that
 * cannot reach t (it is pruned). */
template <class U>
inline std::vector<int> solve(ddp_graph *g, int n, const U *hx, unsigned s, unsigned t) {
    std::vector<int32_t> h((size_t)n);
    for (int i = 0; i < n; i++) h[(size_t)i] = (int32_t)hx[i];
    ddp_heuristic *hh = nullptr;
    check(ddp_heuristic_build(g, (int32_t)t, DDP_H_USER, h.data(), nullptr, &hh));
    ddp_query *q = nullptr;
    check(ddp_solve(g, hh, (int32_t)s, (int32_t)t, nullptr, &q));
    int32_t cost = 0, len = 0;
    check(ddp_query_cost(q, &cost));
    check(ddp_path_read(q, nullptr, 0, &len));
    std::vector<int> path;
    if (cost != DDP_INF && len > 0) {
        path.resize((size_t)len);
        check(ddp_path_read(q, path.data(), len, &len));
    }
    ddp_query_free(q);
    ddp_heuristic_free(hh);
    return path;
}

}  // namespace ddp_lib

#endif
