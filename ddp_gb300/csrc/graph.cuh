// Host-side handle types shared by the translation units of libddp_gb300.
#pragma once

#include <mutex>
#include <vector>

#include "common.cuh"

struct DynMirror;

struct ddp_graph {
    std::mutex mu;
    int device = 0;
    cudaStream_t stream = nullptr;
    int32_t n = 0;
    int64_t e = 0;      // arcs in the main CSR (dead ones included)
    int64_t e_rev = 0;  // arcs in the reverse CSR
    uint32_t wmin = 0, wmax = 0;
    uint32_t rho_fp = 0;  // Euclidean heuristic scale (16.16)
    int32_t *d_off = nullptr;
    uint2 *d_arc = nullptr;
    int32_t *d_roff = nullptr;
    uint2 *d_rarc = nullptr;
    int32_t *d_xy = nullptr;
    std::vector<int32_t> h_xy;
    // arcs inserted by dynamic updates (second CSR), null when none
    int32_t *d_doff = nullptr;
    uint2 *d_darc = nullptr;
    int32_t *d_droff = nullptr;
    uint2 *d_drarc = nullptr;
    // dynamic layout (rows with explicit ends), set by ddp_dyn_create
    int32_t *d_oend = nullptr;
    int32_t *d_roend = nullptr;
    DynMirror *dyn = nullptr;  // host mirror of a dynamic graph
    bool dyn_active = false;          // a ddp_dyn search owns the graph's updates
    // single-query workspace, allocated on first use
    struct Workspace *ws = nullptr;
};

namespace ddp {
DevGraph graph_view(const ddp_graph *g);
int ensure_device();
void workspace_release(ddp_graph *g);
void dyn_mirror_free(DynMirror *m);
int dyn_read_csr(const ddp_graph *g, int32_t *offsets, int32_t *cols, uint32_t *weights);
int64_t dyn_live_arcs(const ddp_graph *g);
int dyn_upload(ddp_graph *g);
int dyn_graph_prepare(ddp_graph *g);
}  // namespace ddp
