// Library plumbing and the device-resident graph.
//
// Replaces LIB/include/graph.h:93-118 (Graph<T>::read_graph), graph.cuh:62-72
// (GPU_Graph<T>::__gpu_alloc) and DA_star/genOpCSR.cpp:31-53 (reverse CSR,
// built here in memory instead of written to graph_op.txt).
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "graph.cuh"

namespace ddp {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}

bool trace_on() {
    static const bool on = [] {
        const char *v = std::getenv("DDP_TRACE");
        return v && v[0] == '1';
    }();
    return on;
}

void trace(const char *fmt, ...) {
    if (!trace_on()) return;
    const auto t = std::chrono::steady_clock::now().time_since_epoch();
    std::fprintf(stderr, "[ddp %.6f] ", std::chrono::duration<double>(t).count());
    va_list ap;
    va_start(ap, fmt);
    std::vfprintf(stderr, fmt, ap);
    va_end(ap);
    std::fputc('\n', stderr);
}

int cuda_fail(cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    set_error(m);
    return (e == cudaErrorMemoryAllocation) ? DDP_ERR_OOM
           : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? DDP_ERR_NO_DEVICE
                                                                          : DDP_ERR_CUDA;
}

DevGraph graph_view(const ddp_graph *g) {
    DevGraph d;
    d.n = g->n;
    d.e = g->e;
    d.off = g->d_off;
    d.arc = g->d_arc;
    d.roff = g->d_roff;
    d.rarc = g->d_rarc;
    d.xy = g->d_xy;
    d.wmin = g->wmin;
    d.rho_fp = g->rho_fp;
    d.doff = g->d_doff;
    d.darc = g->d_darc;
    d.droff = g->d_droff;
    d.drarc = g->d_drarc;
    d.oend = g->d_oend;
    d.roend = g->d_roend;
    const bool lm_ok = g->d_lm && g->lm_stamp == g->update_count;
    d.lm = lm_ok ? g->d_lm : nullptr;
    d.lm_L = lm_ok ? g->lm_L : 0;
    d.lm_scale = lm_ok ? g->lm_scale : 1;
    d.lm_bits = lm_ok ? g->lm_bits : 16;
    return d;
}

int ensure_device() {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        (void)cudaGetLastError();
        return fail(DDP_ERR_NO_DEVICE, "no CUDA device available");
    }
    return DDP_OK;
}

// Builds the interleaved forward arcs and the reverse CSR on the host, then
// uploads both.  off has n+1 entries.
static int upload_csr(ddp_graph *g, const int32_t *off, const int32_t *col, const uint32_t *w) {
    const int32_t n = g->n;
    const int64_t e = g->e;
    std::vector<uint2> arc((size_t)e);
    std::vector<int32_t> roff((size_t)n + 1, 0);
    uint32_t wmin = 0xFFFFFFFFu, wmax = 0;
    for (int32_t u = 0; u < n; u++) {
        for (int64_t j = off[u]; j < off[u + 1]; j++) {
            int32_t v = col[j];
            arc[(size_t)j] = make_uint2((uint32_t)v, w[j]);
            if (v >= 0) {
                roff[(size_t)v + 1]++;
                if (w[j] < wmin) wmin = w[j];
                if (w[j] > wmax) wmax = w[j];
            }
        }
    }
    for (int32_t v = 0; v < n; v++) roff[(size_t)v + 1] += roff[(size_t)v];
    const int64_t live = roff[(size_t)n];
    std::vector<uint2> rarc((size_t)(live > 0 ? live : 1));
    std::vector<int32_t> fill(roff.begin(), roff.end() - 1);
    for (int32_t u = 0; u < n; u++)
        for (int64_t j = off[u]; j < off[u + 1]; j++) {
            int32_t v = col[j];
            if (v < 0) continue;
            rarc[(size_t)fill[(size_t)v]++] = make_uint2((uint32_t)u, w[j]);
        }
    g->wmin = (wmin == 0xFFFFFFFFu) ? 0 : wmin;
    g->wmax = wmax;
    g->e_rev = live;
    DDP_CUDA(cudaMalloc(&g->d_off, sizeof(int32_t) * ((size_t)n + 1)));
    DDP_CUDA(cudaMalloc(&g->d_roff, sizeof(int32_t) * ((size_t)n + 1)));
    DDP_CUDA(cudaMalloc(&g->d_arc, sizeof(uint2) * (size_t)(e > 0 ? e : 1)));
    DDP_CUDA(cudaMalloc(&g->d_rarc, sizeof(uint2) * (size_t)(live > 0 ? live : 1)));
    DDP_CUDA(cudaMemcpy(g->d_off, off, sizeof(int32_t) * ((size_t)n + 1), cudaMemcpyHostToDevice));
    DDP_CUDA(cudaMemcpy(g->d_roff, roff.data(), sizeof(int32_t) * ((size_t)n + 1),
                        cudaMemcpyHostToDevice));
    if (e > 0)
        DDP_CUDA(cudaMemcpy(g->d_arc, arc.data(), sizeof(uint2) * (size_t)e, cudaMemcpyHostToDevice));
    if (live > 0)
        DDP_CUDA(cudaMemcpy(g->d_rarc, rarc.data(), sizeof(uint2) * (size_t)live,
                            cudaMemcpyHostToDevice));
    return DDP_OK;
}

void graph_free_dev(ddp_graph *g, void *p) {
    if (!p) return;
    if (g->defer_free)
        g->deferred.push_back(p);
    else
        cudaFree(p);
}

void graph_flush_frees(ddp_graph *g) {
    for (void *p : g->deferred) cudaFree(p);
    g->deferred.clear();
}

void graph_release(ddp_graph *g) {
    if (!g) return;
    graph_flush_frees(g);
    workspace_release(g);
    cudaFree(g->d_off);
    cudaFree(g->d_arc);
    cudaFree(g->d_roff);
    cudaFree(g->d_rarc);
    cudaFree(g->d_xy);
    cudaFree(g->d_doff);
    cudaFree(g->d_darc);
    cudaFree(g->d_droff);
    cudaFree(g->d_drarc);
    cudaFree(g->d_oend);
    cudaFree(g->d_roend);
    cudaFree(g->d_lm);
    dyn_mirror_free(g->dyn);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

void graph_ref(ddp_graph *g) { g->refs.fetch_add(1); }

void graph_unref(ddp_graph *g) {
    if (g && g->refs.fetch_sub(1) == 1) graph_release(g);
}

}  // namespace ddp

using namespace ddp;

extern "C" {

const char *ddp_last_error(void) { return g_last_error.c_str(); }

int ddp_version(void) { return 10000; }

int ddp_device_count(void) {
    int c = 0;
    if (cudaGetDeviceCount(&c) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    return c;
}

int ddp_graph_from_csr(int32_t n, int64_t e, const int32_t *offsets, int32_t offsets_len,
                       const int32_t *cols, const uint32_t *weights, ddp_graph **out) {
    if (!out) return fail(DDP_ERR_INVALID, "out is null");
    *out = nullptr;
    if (n < 1 || e < 0 || e > INT32_MAX || !offsets || (e > 0 && (!cols || !weights)))
        return fail(DDP_ERR_INVALID, "bad graph arguments");
    if (offsets_len != n && offsets_len != n + 1)
        return fail(DDP_ERR_INVALID, "offsets_len must be n or n+1");
    // validate and normalise to n+1 offsets
    std::vector<int32_t> off((size_t)n + 1);
    for (int32_t i = 0; i < n; i++) off[(size_t)i] = offsets[i];
    off[(size_t)n] = (offsets_len == n + 1) ? offsets[n] : (int32_t)e;
    if (off[0] != 0 || off[(size_t)n] != e)
        return fail(DDP_ERR_INVALID, "offsets must start at 0 and end at e");
    for (int32_t i = 0; i < n; i++)
        if (off[(size_t)i + 1] < off[(size_t)i])
            return fail(DDP_ERR_INVALID, "offsets must be non-decreasing");
    for (int64_t j = 0; j < e; j++)
        if (cols[j] >= n) return fail(DDP_ERR_INVALID, "arc head out of range");
    int rc = ensure_device();
    if (rc) return rc;
    ddp_graph *g = new ddp_graph();
    g->n = n;
    g->e = e;
    cudaGetDevice(&g->device);
    cudaError_t ce = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        graph_release(g);
        return cuda_fail(ce, "cudaStreamCreate");
    }
    rc = upload_csr(g, off.data(), cols, weights);
    if (rc) {
        graph_release(g);
        return rc;
    }
    *out = g;
    return DDP_OK;
}

int ddp_graph_load_text(const char *path, ddp_graph **out) {
    if (!out) return fail(DDP_ERR_INVALID, "out is null");
    int32_t n;
    int64_t e;
    int32_t *off, *col;
    uint32_t *w;
    int rc = ddp_io_read_graph_text(path, &n, &e, &off, &col, &w);
    if (rc) return fail(rc, std::string("cannot read graph file ") + (path ? path : "(null)"));
    rc = ddp_graph_from_csr(n, e, off, n + 1, col, w, out);
    ddp_free(off);
    ddp_free(col);
    ddp_free(w);
    return rc;
}

int ddp_graph_set_coords(ddp_graph *g, const int32_t *xy) {
    if (!g || !xy) return fail(DDP_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(g->mu);
    if (!g->d_xy) DDP_CUDA(cudaMalloc(&g->d_xy, sizeof(int32_t) * 2 * (size_t)g->n));
    DDP_CUDA(cudaMemcpy(g->d_xy, xy, sizeof(int32_t) * 2 * (size_t)g->n, cudaMemcpyHostToDevice));
    g->h_xy.assign(xy, xy + 2 * (size_t)g->n);
    return DDP_OK;
}

int ddp_graph_set_euclid(ddp_graph *g, uint32_t rho_fp) {
    if (!g) return fail(DDP_ERR_INVALID, "null graph");
    std::lock_guard<std::mutex> lk(g->mu);
    g->rho_fp = rho_fp;
    return DDP_OK;
}

int ddp_graph_info(const ddp_graph *g, int32_t *n, int64_t *e, uint32_t *wmin, uint32_t *wmax) {
    if (!g) return fail(DDP_ERR_INVALID, "null graph");
    std::lock_guard<std::mutex> lk(const_cast<ddp_graph *>(g)->mu);
    if (n) *n = g->n;
    if (e) {
        *e = g->dyn ? dyn_live_arcs(const_cast<ddp_graph *>(g)) : g->e;
        if (*e < 0) return fail(DDP_ERR_CUDA, "reading the dynamic graph back");
    }
    if (wmin) *wmin = g->wmin;
    if (wmax) *wmax = g->wmax;
    return DDP_OK;
}

int ddp_graph_read_csr(const ddp_graph *g, int32_t *offsets, int32_t *cols, uint32_t *weights) {
    if (!g) return fail(DDP_ERR_INVALID, "null graph");
    std::lock_guard<std::mutex> lk(const_cast<ddp_graph *>(g)->mu);
    if (g->dyn) return dyn_read_csr(const_cast<ddp_graph *>(g), offsets, cols, weights);
    if (offsets)
        DDP_CUDA(cudaMemcpy(offsets, g->d_off, sizeof(int32_t) * ((size_t)g->n + 1),
                            cudaMemcpyDeviceToHost));
    if ((cols || weights) && g->e > 0) {
        std::vector<uint2> arc((size_t)g->e);
        DDP_CUDA(cudaMemcpy(arc.data(), g->d_arc, sizeof(uint2) * (size_t)g->e,
                            cudaMemcpyDeviceToHost));
        for (int64_t j = 0; j < g->e; j++) {
            if (cols) cols[j] = (int32_t)arc[(size_t)j].x;
            if (weights) weights[j] = arc[(size_t)j].y;
        }
    }
    return DDP_OK;
}

int ddp_graph_free(ddp_graph *g) {
    graph_unref(g);  // objects built on the graph keep it until they are freed
    return DDP_OK;
}

}  // extern "C"
