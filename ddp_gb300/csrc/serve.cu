// Serving: continuous batching of A* requests on a resident graph, with
// edge-update batches interleaved.
//
// No reference counterpart (the reference answers one (s,t) per process).
// Requests are written to a ring in pinned host memory that the device reads
// directly (cudaHostAllocMapped); publishing a request is a store of the
// published count.  The persistent slot kernel (k_batch in serving mode) keeps
// one search per CTA: a slot that finishes claims the next published request
// at once, so requests that arrive while others run start as soon as a slot
// (and its pre-allocated queue and state memory) frees up.  Results come back
// the same way (cost, graph version, done flag) and are collected by polling.
// Slots leave after a bounded idle period; submit and poll relaunch the
// kernel when requests are pending and it is not running.
//
// Admission by memory: every slot owns a fixed footprint (state n x 8 B,
// touched-log n x 4 B, four queues); the number of slots is what fits in the
// memory budget, and a request waits in the ring until a slot is free.  A
// request whose search outgrows its slot is re-run on the single-query engine
// (which grows its queues) when it is polled.
//
// Updates: ddp_serve_update pauses claiming, waits for the slots to drain
// (every request runs on one consistent graph version), applies the batch
// with the dynamic-graph semantics, lowers the Euclidean scale if a lighter
// arc appeared, bumps the version and resumes.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "engine.cuh"
#include "graph.cuh"
#include "solve.cuh"

namespace ddp {
int dyn_graph_apply(ddp_graph *g, int32_t nupd, const int32_t *flag, const int32_t *u, const int32_t *v,
                    const uint32_t *w, std::vector<int4> &ups);
}

using namespace ddp;

static int64_t now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct ddp_server {
    std::mutex mu;
    ddp_graph *g = nullptr;
    int hkind = DDP_H_ZERO;
    ddp_opts o{};
    cudaStream_t stream = nullptr;
    int block = 512;
    SlotArrays sa;
    int64_t cap = 0;
    // mapped host memory (h_ = host view, d_ = device view)
    int32_t *h_S = nullptr, *h_T = nullptr, *h_cost = nullptr, *h_ver = nullptr;
    int *h_done = nullptr, *h_ctl = nullptr;  // ctl[0] = published count, ctl[1] = pause
    int32_t *d_S = nullptr, *d_T = nullptr, *d_cost = nullptr, *d_ver = nullptr;
    int *d_done = nullptr, *d_ctl = nullptr;
    int *d_work = nullptr;  // claim counter (device)
    int32_t *d_plen = nullptr, *d_paths = nullptr;
    int64_t submitted = 0, scan_lo = 0, completed = 0;
    std::vector<int64_t> t_sub;
    std::vector<char> reported;
    int version = 0;
    int launches = 0;
    int fallbacks = 0;
    bool running = false;
};

namespace {

bool kernel_running(ddp_server *s) {
    if (!s->running) return false;
    cudaError_t e = cudaStreamQuery(s->stream);
    if (e == cudaErrorNotReady) return true;
    (void)cudaGetLastError();
    s->running = false;
    return false;
}

int launch(ddp_server *s) {
    BatchArgs A;
    std::memset(&A, 0, sizeof(A));
    A.S = s->d_S;
    A.T = s->d_T;
    A.nq = INT32_MAX;  // slots stop by pause / idle, not by count
    A.cost = s->d_cost;
    A.plen = s->d_plen;
    A.paths = nullptr;
    A.path_cap = 0;
    A.work = s->d_work;
    A.status = s->d_work + 1;
    A.delta = s->o.delta > 0 ? (uint32_t)s->o.delta : auto_delta(s->g);
    A.K = s->o.K;
    A.bfs_budget = s->hkind == DDP_H_BFS_CAPPED ? bfs_budget(s->g->n) : 0;
    A.group = 1;
    A.sync_engine = (s->o.flags & DDP_OPT_SYNC) != 0;
    A.serve = 1;
    A.pub = s->d_ctl;
    A.pause = s->d_ctl + 1;
    A.idle_limit = 2000;  // ~2 ms of empty polls
    A.done = s->d_done;
    A.ver = s->d_ver;
    A.version = s->version;
    DDP_CUDA(cudaMemsetAsync(s->sa.ctl, 0, sizeof(SearchCtl) * (size_t)s->sa.nslots, s->stream));
    cudaError_t e = launch_slots(s->hkind, s->sa.nslots, s->block, false, graph_view(s->g), s->sa, A, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "serving kernel launch");
    s->running = true;
    s->launches++;
    return DDP_OK;
}

int ensure_running(ddp_server *s) {
    std::atomic_thread_fence(std::memory_order_seq_cst);
    const int pub = __atomic_load_n(&s->h_ctl[0], __ATOMIC_ACQUIRE);
    if (s->completed >= pub) return DDP_OK;
    if (kernel_running(s)) return DDP_OK;
    return launch(s);
}

}  // namespace

extern "C" {

int ddp_serve_create(ddp_graph *g, int32_t hkind, const ddp_opts *opts, int64_t max_requests, ddp_server **out) {
    if (!g || !out || max_requests < 1 || max_requests > INT32_MAX / 2)
        return fail(DDP_ERR_INVALID, "bad serving arguments");
    *out = nullptr;
    if (hkind != DDP_H_ZERO && hkind != DDP_H_BFS_HOPS && hkind != DDP_H_BFS_CAPPED && hkind != DDP_H_MANHATTAN &&
        hkind != DDP_H_EUCLID)
        return fail(DDP_ERR_INVALID, "unsupported heuristic kind for serving");
    if ((hkind == DDP_H_MANHATTAN || hkind == DDP_H_EUCLID) && !g->d_xy)
        return fail(DDP_ERR_INVALID, "graph has no coordinates (ddp_graph_set_coords)");
    ddp_server *s = new ddp_server();
    s->g = g;
    s->hkind = hkind;
    if (opts) s->o = *opts;
    s->block = s->o.block > 0 ? std::min(s->o.block, 512) : 256;
    s->cap = max_requests;
    auto bail = [&](int rc) {
        ddp_serve_free(s);
        return rc;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
    // slots: occupancy, then the memory budget (half of free memory)
    const int per_sm = std::max(1, slots_per_sm(hkind, s->block));
    int nslots = per_sm * device_sms();
    if (s->o.grid > 0) nslots = std::min(nslots, s->o.grid);
    const int64_t capq = s->o.queue_cap > 0 ? s->o.queue_cap : std::max<int64_t>(1 << 16, g->n / 8);
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    const bool hops = hkind == DDP_H_BFS_HOPS || hkind == DDP_H_BFS_CAPPED;
    const size_t per = slot_bytes(g->n, capq, capq, hops);
    if ((size_t)nslots * per > freeb / 2) nslots = (int)std::max<size_t>(1, (freeb / 2) / per);
    int rc = slots_alloc(s->sa, g->n, nslots, capq, capq, hops, s->stream);
    if (rc) return bail(rc);
    const size_t R = (size_t)max_requests;
    unsigned flags = cudaHostAllocMapped;
    e = cudaHostAlloc(&s->h_S, sizeof(int32_t) * R, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_T, sizeof(int32_t) * R, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_cost, sizeof(int32_t) * R, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_ver, sizeof(int32_t) * R, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_done, sizeof(int) * R, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_ctl, sizeof(int) * 4, flags);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaHostAlloc(request ring)"));
    std::memset(s->h_done, 0, sizeof(int) * R);
    std::memset(s->h_ctl, 0, sizeof(int) * 4);
    e = cudaHostGetDevicePointer((void **)&s->d_S, s->h_S, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_T, s->h_T, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_cost, s->h_cost, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_ver, s->h_ver, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_done, s->h_done, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_ctl, s->h_ctl, 0);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaHostGetDevicePointer"));
    e = cudaMalloc(&s->d_work, sizeof(int) * 2);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_plen, sizeof(int32_t) * R);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(serving state)"));
    DDP_CUDA(cudaMemsetAsync(s->d_work, 0, sizeof(int) * 2, s->stream));
    DDP_CUDA(cudaStreamSynchronize(s->stream));
    s->t_sub.assign(R, 0);
    s->reported.assign(R, 0);
    *out = s;
    return DDP_OK;
}

int ddp_serve_submit(ddp_server *s, int32_t n, const int32_t *src, const int32_t *dst, int64_t *first_id) {
    if (!s || n < 0 || (n > 0 && (!src || !dst))) return fail(DDP_ERR_INVALID, "bad submit arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->submitted + n > s->cap) return fail(DDP_ERR_QUEUE_OVERFLOW, "request ring full");
    const int64_t base = s->submitted;
    const int64_t t = now_ns();
    for (int32_t i = 0; i < n; i++) {
        s->h_S[base + i] = src[i];
        s->h_T[base + i] = dst[i];
        s->t_sub[(size_t)(base + i)] = t;
    }
    s->submitted += n;
    __atomic_store_n(&s->h_ctl[0], (int)s->submitted, __ATOMIC_RELEASE);
    if (first_id) *first_id = base;
    return ensure_running(s);
}

int ddp_serve_poll(ddp_server *s, int32_t max, int64_t *ids, int32_t *costs, int64_t *latency_ns,
                   int32_t *versions, int32_t *nout) {
    if (!s || !nout || max < 0) return fail(DDP_ERR_INVALID, "bad poll arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    int32_t k = 0;
    const int64_t t = now_ns();
    for (int64_t i = s->scan_lo; i < s->submitted && k < max; i++) {
        if (s->reported[(size_t)i]) continue;
        if (!__atomic_load_n(&s->h_done[i], __ATOMIC_ACQUIRE)) continue;
        int32_t c = s->h_cost[i];
        if (c == -1) {
            // the search outgrew its slot: re-run it on the single-query engine
            ddp_heuristic *h = nullptr;
            const int hk = s->hkind;
            int rc = ddp_heuristic_build(s->g, s->h_T[i], hk, nullptr, nullptr, &h);
            if (rc) return rc;
            ddp_query *q = nullptr;
            ddp_opts so = s->o;
            so.queue_cap = 0;
            so.grid = 0;
            rc = ddp_solve(s->g, h, s->h_S[i], s->h_T[i], &so, &q);
            ddp_heuristic_free(h);
            if (rc) return rc;
            ddp_query_cost(q, &c);
            ddp_query_free(q);
            s->fallbacks++;
        }
        s->reported[(size_t)i] = 1;
        s->completed++;
        if (ids) ids[k] = i;
        if (costs) costs[k] = c;
        if (latency_ns) latency_ns[k] = t - s->t_sub[(size_t)i];
        if (versions) versions[k] = s->h_ver[i];
        k++;
    }
    while (s->scan_lo < s->submitted && s->reported[(size_t)s->scan_lo]) s->scan_lo++;
    *nout = k;
    return ensure_running(s);
}

int ddp_serve_update(ddp_server *s, int32_t n, const int32_t *flag, const int32_t *u, const int32_t *v,
                     const uint32_t *w) {
    if (!s) return fail(DDP_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    // drain: stop claiming, wait for the slots to finish their searches
    __atomic_store_n(&s->h_ctl[1], 1, __ATOMIC_RELEASE);
    DDP_CUDA(cudaStreamSynchronize(s->stream));
    s->running = false;
    ddp_graph *g = s->g;
    std::vector<int4> ups;
    int rc;
    {
        std::lock_guard<std::mutex> glk(g->mu);
        rc = dyn_graph_apply(g, n, flag, u, v, w, ups);
    }
    if (rc == DDP_OK && s->hkind == DDP_H_EUCLID && !g->h_xy.empty()) {
        // keep rho_fp a lower bound of w / length: only lighter or new arcs
        // can lower it
        uint64_t rho = g->rho_fp;
        for (const int4 &x : ups) {
            if (x.x != 1 && x.x != 3) continue;  // insert or lighter arc
            const double dx = (double)g->h_xy[2 * (size_t)x.z] - g->h_xy[2 * (size_t)x.y];
            const double dy = (double)g->h_xy[2 * (size_t)x.z + 1] - g->h_xy[2 * (size_t)x.y + 1];
            const double len = std::sqrt(dx * dx + dy * dy);
            if (len <= 0) continue;
            const double r = std::floor((double)(uint32_t)x.w * 65536.0 / len) - 1.0;
            if (r < (double)rho) rho = r > 0 ? (uint64_t)r : 0;
        }
        g->rho_fp = (uint32_t)rho;
    }
    s->version++;
    __atomic_store_n(&s->h_ctl[1], 0, __ATOMIC_RELEASE);
    if (rc) return rc;
    return ensure_running(s);
}

int ddp_serve_stats(const ddp_server *s, int64_t *stats6) {
    if (!s || !stats6) return fail(DDP_ERR_INVALID, "null argument");
    stats6[0] = s->submitted;
    stats6[1] = s->completed;
    stats6[2] = s->sa.nslots;
    stats6[3] = s->launches;
    stats6[4] = s->version;
    stats6[5] = s->fallbacks;
    return DDP_OK;
}

int ddp_serve_free(ddp_server *s) {
    if (!s) return DDP_OK;
    if (s->h_ctl) __atomic_store_n(&s->h_ctl[1], 1, __ATOMIC_RELEASE);
    if (s->stream) cudaStreamSynchronize(s->stream);
    slots_free(s->sa);
    cudaFreeHost(s->h_S);
    cudaFreeHost(s->h_T);
    cudaFreeHost(s->h_cost);
    cudaFreeHost(s->h_ver);
    cudaFreeHost(s->h_done);
    cudaFreeHost(s->h_ctl);
    cudaFree(s->d_work);
    cudaFree(s->d_plen);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return DDP_OK;
}

}  // extern "C"
