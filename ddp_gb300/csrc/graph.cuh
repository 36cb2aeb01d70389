// Host-side handle types shared by the translation units of libddp_gb300.
#pragma once

#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"

struct DynMirror;

// Runs a scatter of dynamic-graph changes into device arrays without a
// kernel launch of its own (a serving kernel that holds every SM runs it in
// place).  kind 0: arcs, dst0[list[i]] = vals[i] with list long long and
// vals uint2; kind 1: row bounds, for r = list[i] (int4 {row, begin, end}):
// dst0[r.x] = r.y, dst1[r.x] = r.z.  list and vals are host memory.
// Returns DDP_OK when done, SCATTER_LAUNCH when the caller must run the
// scatter itself, or an error code.
constexpr int SCATTER_LAUNCH = -1;
struct ScatterHook {
    int (*fn)(void *ctx, int kind, void *dst0, void *dst1, const void *list, const void *vals,
              int64_t k) = nullptr;
    void *ctx = nullptr;
};

struct ddp_graph {
    std::mutex mu;
    // the handle plus every object that keeps a pointer to the graph
    // (heuristics, batches, dynamic searches, servers); the last one frees it
    std::atomic<int> refs{1};
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
    // set while a serving kernel runs on the graph: scatters go through the
    // hook, and device frees (which would wait for that kernel) are deferred
    ScatterHook hook;
    bool defer_free = false;
    int64_t layout_gen = 0;  // bumps when the whole dynamic layout is uploaded again
    std::vector<void *> deferred;
    int64_t update_count = 0;  // update batches applied (dynamic graphs)
    // landmark distances for the ALT heuristic (DevGraph::lm), built for
    // the graph as it was at update_count == lm_stamp
    uint2 *d_lm = nullptr;
    int32_t lm_L = 0;
    int32_t lm_scale = 1;
    int32_t lm_bits = 16;
    int64_t lm_stamp = -1;
    std::vector<int32_t> lm_ids;
    // single-query workspace, allocated on first use
    struct Workspace *ws = nullptr;
};

namespace ddp {
DevGraph graph_view(const ddp_graph *g);
int ensure_device();
void workspace_release(ddp_graph *g);
void dyn_mirror_free(DynMirror *m);
int dyn_read_csr(ddp_graph *g, int32_t *offsets, int32_t *cols, uint32_t *weights);
int64_t dyn_live_arcs(ddp_graph *g);  // -1 on a CUDA error
int dyn_mirror_sync(ddp_graph *g);
int dyn_upload(ddp_graph *g, bool sync = true);
int dyn_graph_prepare(ddp_graph *g);
// cudaFree now, or later (graph_flush_frees) while g->defer_free is set
void graph_free_dev(ddp_graph *g, void *p);
void graph_ref(ddp_graph *g);
void graph_unref(ddp_graph *g);
void graph_flush_frees(ddp_graph *g);
}  // namespace ddp
