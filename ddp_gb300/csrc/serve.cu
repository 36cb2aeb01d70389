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
// A slot with no work for ~2 ms votes to leave and keeps polling; the slots
// leave together once all have voted, so a launch never thins out while
// requests keep coming.  Submit and poll relaunch the kernel when requests
// are pending and it is not running.
//
// Admission by memory: every slot owns a fixed footprint (state n x 8 B,
// touched-log n x 4 B, four queues); the number of slots is what fits in the
// memory budget, and a request waits in the ring until a slot is free.  A
// request whose search outgrows its slot is re-run on the single-query engine
// (which grows its queues) when it is polled.
//
// Updates never drain the GPU.  The graph is kept in versions: version v
// lives in buffer v % K of a ring of K device copies.  An update is applied
// to the master copy (the graph handle's arrays in the dynamic layout, with
// its host mirror); the next ring buffer, once no search runs on it, is
// brought up to date by copying only the arc slots and row bounds that the
// batches since its last version changed, and the version is published.
// While the slot kernel holds every SM, these scatters and gathers run on
// its service CTA (one CTA of the launch that serves no requests); lists
// travel in mapped host memory, so an update needs neither a kernel launch
// nor a copy engine.  A slot pins the latest version when it claims a
// request (it counts itself on the buffer, then re-reads the version), so
// every search sees one consistent graph and searches on older versions
// finish undisturbed.  The Euclidean scale is kept per version: lighter or
// new arcs lower it.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.cuh"
#include "graph.cuh"
#include "solve.cuh"

namespace ddp {
int dyn_graph_apply(ddp_graph *g, int32_t nupd, const int32_t *flag, const int32_t *u, const int32_t *v,
                    const uint32_t *w, std::vector<int4> &ups, bool sync = true);
}

// One graph version on the device (dynamic layout: row begin/end arrays).
struct VBuf {
    int32_t *off = nullptr, *oend = nullptr, *roff = nullptr, *roend = nullptr;
    uint2 *arc = nullptr, *rarc = nullptr;
    int64_t arc_cap = 0, rarc_cap = 0;
    int held = -1;  // version the buffer holds, -1 none
};

// What one update batch changed in the master copy.
struct Delta {
    int ver = 0;
    bool full = false;  // the whole layout was uploaded again
    std::vector<long long> arc, rarc;
    std::vector<int32_t> row, rrow;
};

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
    int hk = 0;  // k_batch instance (heuristic kind and record layout)
    ddp_opts o{};
    cudaStream_t stream = nullptr;
    int block = 512;
    SlotArrays sa;
    int64_t cap = 0;
    // mapped host memory (h_ = host view, d_ = device view)
    int32_t *h_S = nullptr, *h_T = nullptr, *h_cost = nullptr, *h_ver = nullptr;
    int *h_done = nullptr, *h_ctl = nullptr;  // ctl: [0] published count, [1] pause, [2] graph version
    int32_t *d_S = nullptr, *d_T = nullptr, *d_cost = nullptr, *d_ver = nullptr;
    int *d_done = nullptr, *d_ctl = nullptr;
    int *d_work = nullptr;  // claim counter (device)
    int32_t *d_plen = nullptr;
    // paths (ddp_serve_record_paths): path_cap node ids per request in mapped
    // host memory, written by the slot before the request's done flag;
    // requests re-run on the host keep theirs in host_paths
    int32_t path_cap = 0;
    int32_t *h_paths = nullptr, *d_paths = nullptr;
    int32_t *h_plen = nullptr;  // with paths: d_plen is the device view of this
    std::unordered_map<int64_t, std::vector<int32_t>> host_paths;
    int64_t submitted = 0, scan_lo = 0, completed = 0;
    std::vector<int64_t> t_sub;
    std::vector<char> reported;
    int version = 0;
    int launches = 0;
    int fallbacks = 0;
    bool running = false;
    // graph versions (table and counts in mapped host memory)
    int nver = 0;
    std::vector<VBuf> vb;
    DevGraph *h_vtab = nullptr, *d_vtab = nullptr;
    int *h_inflight = nullptr, *d_inflight = nullptr;
    std::deque<Delta> deltas;
    Delta cur;  // being recorded by the scatter hook
    cudaStream_t cstream = nullptr;  // maintenance launches while no slot kernel runs
    // service CTA job and its list staging (mapped host memory)
    SvcJob *h_svc = nullptr, *d_svc = nullptr;
    int svc_seq = 0;
    char *h_stage = nullptr, *d_stage = nullptr;
    size_t stage_cap = 0;
    std::vector<void *> stage_old;  // pinned buffers to free when no kernel runs
    // update timings (ns): apply to master, wait for the buffer, patch it
    int64_t t_apply = 0, t_wait = 0, t_patch = 0;
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

// Staging for maintenance lists: bytes of mapped host memory, reused by
// every job (one job runs at a time).
int stage_reserve(ddp_server *s, size_t bytes) {
    if (bytes <= s->stage_cap) return DDP_OK;
    size_t cap = std::max<size_t>(bytes + bytes / 2, 4u << 20);
    char *h = nullptr;
    DDP_CUDA(cudaHostAlloc(&h, cap, cudaHostAllocMapped | cudaHostAllocPortable));
    char *d = nullptr;
    cudaError_t e = cudaHostGetDevicePointer((void **)&d, h, 0);
    if (e != cudaSuccess) {
        cudaFreeHost(h);
        return cuda_fail(e, "cudaHostGetDevicePointer(staging)");
    }
    if (s->h_stage) s->stage_old.push_back(s->h_stage);
    s->h_stage = h;
    s->d_stage = d;
    s->stage_cap = cap;
    return DDP_OK;
}

// Runs maintenance subs: on the service CTA of the running slot kernel, or
// with ordinary launches when none runs.
int svc_run(ddp_server *s, const SvcSub *subs, int nsub) {
    if (kernel_running(s) && s->sa.nslots >= 2) {
        SvcJob *j = s->h_svc;
        const int id = ++s->svc_seq;
        j->nsub = nsub;
        for (int i = 0; i < nsub; i++) j->sub[i] = subs[i];
        __atomic_store_n(&j->seq, id, __ATOMIC_RELEASE);
        const int64_t t0 = now_ns();
        for (;;) {
            if (__atomic_load_n(&j->done, __ATOMIC_ACQUIRE) == id) return DDP_OK;
            if (!kernel_running(s)) {
                // the kernel left: it ran the job before leaving, or never took it
                if (__atomic_load_n(&j->done, __ATOMIC_ACQUIRE) == id) return DDP_OK;
                __atomic_store_n(&j->done, id, __ATOMIC_RELEASE);  // retire it; run it here
                break;
            }
            if (now_ns() - t0 > 30000000000LL)
                return fail(DDP_ERR_TIMEOUT, "service CTA did not run the graph maintenance job");
            std::this_thread::sleep_for(std::chrono::microseconds(2));
        }
    }
    cudaError_t e = svc_run_direct(subs, nsub, s->cstream);
    if (e != cudaSuccess) return cuda_fail(e, "graph maintenance launch");
    return DDP_OK;
}

SvcSub sub_of(int kind, long long k, const void *p0, const void *p1, const void *p2, const void *p3) {
    SvcSub x;
    x.kind = kind;
    x.pad = 0;
    x.k = k;
    x.p0 = (unsigned long long)(uintptr_t)p0;
    x.p1 = (unsigned long long)(uintptr_t)p1;
    x.p2 = (unsigned long long)(uintptr_t)p2;
    x.p3 = (unsigned long long)(uintptr_t)p3;
    return x;
}

// Scatter hook of the served graph: records what changed (for the version
// buffers) and runs the scatter on the service CTA while the kernel runs.
int svc_scatter(void *ctx, int kind, void *dst0, void *dst1, const void *list, const void *vals, int64_t k) {
    ddp_server *s = static_cast<ddp_server *>(ctx);
    ddp_graph *g = s->g;
    if (kind == 0) {
        const long long *sl = static_cast<const long long *>(list);
        std::vector<long long> &rec = (dst0 == (void *)g->d_arc) ? s->cur.arc : s->cur.rarc;
        rec.insert(rec.end(), sl, sl + k);
    } else {
        const int4 *r = static_cast<const int4 *>(list);
        std::vector<int32_t> &rec = (dst0 == (void *)g->d_off) ? s->cur.row : s->cur.rrow;
        for (int64_t i = 0; i < k; i++) rec.push_back(r[i].x);
    }
    if (!kernel_running(s) || s->sa.nslots < 2) return SCATTER_LAUNCH;
    SvcSub x;
    if (kind == 0) {
        const size_t a = sizeof(long long) * (size_t)k, b = sizeof(uint2) * (size_t)k;
        int rc = stage_reserve(s, a + b);
        if (rc) return rc;
        std::memcpy(s->h_stage, list, a);
        std::memcpy(s->h_stage + a, vals, b);
        x = sub_of(SVC_SCATTER_ARCS, k, dst0, nullptr, s->d_stage, s->d_stage + a);
    } else {
        const size_t a = sizeof(int4) * (size_t)k;
        int rc = stage_reserve(s, a);
        if (rc) return rc;
        std::memcpy(s->h_stage, list, a);
        x = sub_of(SVC_SCATTER_ROWS, k, dst0, dst1, s->d_stage, nullptr);
    }
    return svc_run(s, &x, 1);
}

// Brings ring buffer k to version v (the master copy), once no search runs
// on it: a patch of the entries the batches since its version changed, or a
// full copy.
int fill_buffer(ddp_server *s, int k, int v) {
    ddp_graph *g = s->g;
    const int64_t t0 = now_ns();
    // the release store of the previous version and this read of the count
    // pair with the slots' count-then-re-read (both sides fenced)
    __atomic_thread_fence(__ATOMIC_SEQ_CST);
    while (__atomic_load_n(&s->h_inflight[k], __ATOMIC_ACQUIRE) != 0) {
        if (now_ns() - t0 > 30000000000LL) return fail(DDP_ERR_TIMEOUT, "graph version buffer stayed busy");
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    const int64_t t1 = now_ns();
    VBuf &b = s->vb[(size_t)k];
    const int32_t n = g->n;
    bool full = b.held < 0 || b.arc_cap < g->e || b.rarc_cap < g->e_rev;
    if (!full) {
        // every batch after the buffer's version must be on record, none a
        // whole new layout
        int want = b.held + 1;
        for (const Delta &d : s->deltas) {
            if (d.ver <= b.held) continue;
            if (d.ver != want || d.full) {
                full = true;
                break;
            }
            want++;
        }
        if (want != v + 1) full = true;
    }
    if (!b.off) {
        DDP_CUDA(cudaMalloc(&b.off, sizeof(int32_t) * ((size_t)n + 1)));
        DDP_CUDA(cudaMalloc(&b.oend, sizeof(int32_t) * (size_t)n));
        DDP_CUDA(cudaMalloc(&b.roff, sizeof(int32_t) * ((size_t)n + 1)));
        DDP_CUDA(cudaMalloc(&b.roend, sizeof(int32_t) * (size_t)n));
    }
    if (b.arc_cap < g->e) {
        graph_free_dev(g, b.arc);
        b.arc = nullptr;
        DDP_CUDA(cudaMalloc(&b.arc, sizeof(uint2) * (size_t)g->e));
        b.arc_cap = g->e;
    }
    if (b.rarc_cap < g->e_rev) {
        graph_free_dev(g, b.rarc);
        b.rarc = nullptr;
        DDP_CUDA(cudaMalloc(&b.rarc, sizeof(uint2) * (size_t)g->e_rev));
        b.rarc_cap = g->e_rev;
    }
    SvcSub subs[6];
    int ns = 0;
    size_t patched = 0;
    if (full) {
        subs[ns++] = sub_of(SVC_COPY_WORDS, n, b.off, g->d_off, nullptr, nullptr);
        subs[ns++] = sub_of(SVC_COPY_WORDS, n, b.oend, g->d_oend, nullptr, nullptr);
        subs[ns++] = sub_of(SVC_COPY_WORDS, n, b.roff, g->d_roff, nullptr, nullptr);
        subs[ns++] = sub_of(SVC_COPY_WORDS, n, b.roend, g->d_roend, nullptr, nullptr);
        subs[ns++] = sub_of(SVC_COPY_WORDS, 2 * g->e, b.arc, g->d_arc, nullptr, nullptr);
        subs[ns++] = sub_of(SVC_COPY_WORDS, 2 * g->e_rev, b.rarc, g->d_rarc, nullptr, nullptr);
    } else {
        std::vector<long long> arc, rarc;
        std::vector<int32_t> row, rrow;
        for (const Delta &d : s->deltas) {
            if (d.ver <= b.held) continue;
            arc.insert(arc.end(), d.arc.begin(), d.arc.end());
            rarc.insert(rarc.end(), d.rarc.begin(), d.rarc.end());
            row.insert(row.end(), d.row.begin(), d.row.end());
            rrow.insert(rrow.end(), d.rrow.begin(), d.rrow.end());
        }
        auto uniq = [](auto &x) {
            std::sort(x.begin(), x.end());
            x.erase(std::unique(x.begin(), x.end()), x.end());
        };
        uniq(arc);
        uniq(rarc);
        uniq(row);
        uniq(rrow);
        auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
        const size_t o1 = al(8 * arc.size()), o2 = o1 + al(8 * rarc.size()), o3 = o2 + al(4 * row.size());
        const size_t tot = o3 + al(4 * rrow.size());
        int rc = stage_reserve(s, tot);
        if (rc) return rc;
        std::memcpy(s->h_stage, arc.data(), 8 * arc.size());
        std::memcpy(s->h_stage + o1, rarc.data(), 8 * rarc.size());
        std::memcpy(s->h_stage + o2, row.data(), 4 * row.size());
        std::memcpy(s->h_stage + o3, rrow.data(), 4 * rrow.size());
        char *d = s->d_stage;
        subs[ns++] = sub_of(SVC_GATHER_ARCS, (long long)arc.size(), b.arc, g->d_arc, d, nullptr);
        subs[ns++] = sub_of(SVC_GATHER_ARCS, (long long)rarc.size(), b.rarc, g->d_rarc, d + o1, nullptr);
        subs[ns++] = sub_of(SVC_GATHER_INTS, (long long)row.size(), b.off, g->d_off, d + o2, nullptr);
        subs[ns++] = sub_of(SVC_GATHER_INTS, (long long)row.size(), b.oend, g->d_oend, d + o2, nullptr);
        subs[ns++] = sub_of(SVC_GATHER_INTS, (long long)rrow.size(), b.roff, g->d_roff, d + o3, nullptr);
        subs[ns++] = sub_of(SVC_GATHER_INTS, (long long)rrow.size(), b.roend, g->d_roend, d + o3, nullptr);
        patched = arc.size() + rarc.size() + row.size() + rrow.size();
    }
    int rc = svc_run(s, subs, ns);
    if (rc) return rc;
    b.held = v;
    const int64_t t2 = now_ns();
    s->t_wait += t1 - t0;
    s->t_patch += t2 - t1;
    trace("serve: version %d in buffer %d: %s (%zu entries), wait %.3f ms, patch %.3f ms", v, k,
          full ? "full copy" : "patch", patched, (t1 - t0) / 1e6, (t2 - t1) / 1e6);
    return DDP_OK;
}

// Brings ring buffer v % K to version v and publishes it.
int publish(ddp_server *s, int v) {
    ddp_graph *g = s->g;
    const int k = v % s->nver;
    int rc = fill_buffer(s, k, v);
    if (rc) return rc;
    const VBuf &b = s->vb[(size_t)k];
    DevGraph view = graph_view(g);
    view.off = b.off;
    view.oend = b.oend;
    view.roff = b.roff;
    view.roend = b.roend;
    view.arc = b.arc;
    view.rarc = b.rarc;
    s->h_vtab[k] = view;
    __atomic_store_n(&s->h_ctl[2], v, __ATOMIC_RELEASE);
    // drop the records every buffer has seen (a buffer with no version
    // takes a full copy anyway)
    int oldest = v;
    for (const VBuf &x : s->vb)
        if (x.held >= 0) oldest = std::min(oldest, x.held);
    while (!s->deltas.empty() && s->deltas.front().ver <= oldest) s->deltas.pop_front();
    return DDP_OK;
}

// Applies an update batch to the master copy (running searches read their
// own version) and publishes it as the next version.
int apply_and_publish(ddp_server *s, int32_t n, const int32_t *flag, const int32_t *u, const int32_t *v,
                      const uint32_t *w) {
    ddp_graph *g = s->g;
    std::vector<int4> ups;
    std::lock_guard<std::mutex> glk(g->mu);
    const int64_t t0 = now_ns();
    const int64_t gen = g->layout_gen;
    s->cur = Delta();
    s->cur.ver = s->version + 1;
    int rc = dyn_graph_apply(g, n, flag, u, v, w, ups);
    if (rc) {
        // the master may hold part of the batch: no buffer may be patched
        // from records that miss it
        s->cur.full = true;
        s->deltas.push_back(std::move(s->cur));
        return rc;
    }
    s->cur.full = g->layout_gen != gen;
    s->deltas.push_back(std::move(s->cur));
    if (s->hkind == DDP_H_EUCLID && !g->h_xy.empty()) {
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
    s->t_apply += now_ns() - t0;
    trace("serve: batch of %d applied to the master in %.3f ms", n, (now_ns() - t0) / 1e6);
    return publish(s, s->version + 1);
}

int launch(ddp_server *s) {
    BatchArgs A;
    std::memset(&A, 0, sizeof(A));
    A.S = s->d_S;
    A.T = s->d_T;
    A.nq = INT32_MAX;  // slots stop by pause / idle, not by count
    A.cost = s->d_cost;
    A.plen = s->d_plen;
    A.paths = s->d_paths;  // null unless paths are recorded
    A.path_cap = s->path_cap;
    A.work = s->d_work;
    A.status = s->d_work + 1;
    A.delta = s->o.delta > 0                ? (uint32_t)s->o.delta
              : is_bidir_kind(s->hkind) ? auto_delta_bidir(s->g)
                                        : auto_delta(s->g);
    A.K = s->o.K;
    A.bfs_budget = s->hkind == DDP_H_BFS_CAPPED ? bfs_budget(s->g->n) : 0;
    A.group = 1;
    A.sync_engine = (s->o.flags & DDP_OPT_SYNC) != 0;
    A.serve = 1;
    A.pub = s->d_ctl;
    A.pause = s->d_ctl + 1;
    A.idle_limit = 2000;  // ~2 ms of empty polls
    A.idle_votes = s->d_work + 2;
    A.closing = s->d_work + 3;
    // with two or more slots the last CTA is the service CTA
    A.serve_slots = s->sa.nslots >= 2 ? s->sa.nslots - 1 : s->sa.nslots;
    A.svc = s->sa.nslots >= 2 ? s->d_svc : nullptr;
    {
        // nothing runs: retire any job and release deferred frees
        std::lock_guard<std::mutex> glk(s->g->mu);
        __atomic_store_n(&s->h_svc->done, s->h_svc->seq, __ATOMIC_RELEASE);
        graph_flush_frees(s->g);
        for (void *p : s->stage_old) cudaFreeHost(p);
        s->stage_old.clear();
    }
    trace("serve: launch %d (%d slots, version %d, %lld requests pending)", s->launches + 1, s->sa.nslots,
          s->version, (long long)(__atomic_load_n(&s->h_ctl[0], __ATOMIC_ACQUIRE) - s->completed));
    A.done = s->d_done;
    A.ver = s->d_ver;
    A.version = s->version;
    A.vtab = s->d_vtab;
    A.nver = s->nver;
    A.cur_ver = s->d_ctl + 2;
    A.inflight = s->d_inflight;
    DDP_CUDA(cudaMemsetAsync(s->sa.ctl, 0, sizeof(SearchCtl) * (size_t)s->sa.nslots, s->stream));
    DDP_CUDA(cudaMemsetAsync(s->d_work + 2, 0, sizeof(int) * 2, s->stream));
    cudaError_t e = launch_slots(s->hk, s->sa.nslots, s->block, false, graph_view(s->g), s->sa, A, s->stream);
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

int ddp_serve_create(ddp_graph *g, int32_t hkind, const ddp_opts *opts, int64_t max_requests, int32_t versions,
                     ddp_server **out) {
    if (!g || !out || max_requests < 1 || max_requests > INT32_MAX / 2 || versions < 2 || versions > 64)
        return fail(DDP_ERR_INVALID, "bad serving arguments");
    *out = nullptr;
    if (hkind != DDP_H_ZERO && hkind != DDP_H_BFS_HOPS && hkind != DDP_H_BFS_CAPPED && hkind != DDP_H_MANHATTAN &&
        hkind != DDP_H_EUCLID && hkind != DDP_H_LANDMARK && !is_bidir_kind(hkind))
        return fail(DDP_ERR_INVALID, "unsupported heuristic kind for serving");
    if (hkind == DDP_H_LANDMARK && !graph_view(g).lm)
        return fail(DDP_ERR_INVALID, "no current landmark table (ddp_landmarks_build)");
    if ((hkind == DDP_H_MANHATTAN || hkind == DDP_H_EUCLID || hkind == DDP_H_BIDIR_EUCLID ||
         hkind == DDP_H_BIDIR_MANHATTAN) && !g->d_xy)
        return fail(DDP_ERR_INVALID, "graph has no coordinates (ddp_graph_set_coords)");
    ddp_server *s = new ddp_server();
    s->g = g;
    graph_ref(g);
    s->hkind = hkind;
    if (opts) s->o = *opts;
    s->block = s->o.block > 0 ? std::min(s->o.block, 512) : 512;  // wider slots: lower latency, more per-query parallelism
    s->cap = max_requests;
    auto bail = [&](int rc) {
        ddp_serve_free(s);
        return rc;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
    // slots: occupancy, then the memory budget (half of free memory)
    s->hk = kernel_hk(hkind, g->d_xy != nullptr, false);
    const int per_sm = std::max(1, slots_per_sm(s->hk, s->block));
    int nslots = per_sm * device_sms();
    if (s->o.grid > 0) nslots = std::min(nslots, s->o.grid);
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    const int hops = hk_slot_kind(s->hk);  // slot layout
    // queue capacities: what each slot's share of half the free memory
    // holds after its state, up to the batch engine's sizes (n + 4096 near,
    // 2n + 4096 far); at least 64k.  A request that still outgrows its slot
    // is re-run on the single-query engine when it is polled.
    int64_t capq = s->o.queue_cap, capf = s->o.queue_cap;
    if (capq <= 0) {
        const size_t fixed = slot_bytes(g->n, 0, 0, hops);
        const size_t share = (freeb / 2) / (size_t)std::max(1, nslots);
        const size_t per_entry = 2 * sizeof(uint2) + 2 * 2 * sizeof(uint4);  // q0/q1 + two far piles of 2x
        const int64_t fit = share > fixed ? (int64_t)((share - fixed) / per_entry) : 0;
        capq = std::min<int64_t>((int64_t)g->n + 4096, std::max<int64_t>(1 << 16, fit));
        capf = std::min<int64_t>(2 * (int64_t)g->n + 4096, 2 * capq);
    }
    const size_t per = slot_bytes(g->n, capq, capf, hops);
    if ((size_t)nslots * per > freeb / 2) nslots = (int)std::max<size_t>(1, (freeb / 2) / per);
    int rc = slots_alloc(s->sa, g->n, nslots, capq, capf, hops, s->stream);
    if (rc) return bail(rc);
    const size_t R = (size_t)max_requests;
    unsigned flags = cudaHostAllocMapped;
    e = cudaHostAlloc(&s->h_S, sizeof(int32_t) * R, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_T, sizeof(int32_t) * R, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_cost, sizeof(int32_t) * R, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_ver, sizeof(int32_t) * R, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_done, sizeof(int) * R, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_ctl, sizeof(int) * 4, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_svc, sizeof(SvcJob), flags);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaHostAlloc(request ring)"));
    std::memset(s->h_done, 0, sizeof(int) * R);
    std::memset(s->h_ctl, 0, sizeof(int) * 4);
    std::memset(s->h_svc, 0, sizeof(SvcJob));
    e = cudaHostGetDevicePointer((void **)&s->d_S, s->h_S, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_T, s->h_T, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_cost, s->h_cost, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_ver, s->h_ver, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_done, s->h_done, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_ctl, s->h_ctl, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_svc, s->h_svc, 0);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaHostGetDevicePointer"));
    e = cudaMalloc(&s->d_work, sizeof(int) * 4);  // claim counter, status, idle votes, closing
    if (e == cudaSuccess) e = cudaMalloc(&s->d_plen, sizeof(int32_t) * R);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(serving state)"));
    DDP_CUDA(cudaMemsetAsync(s->d_work, 0, sizeof(int) * 4, s->stream));
    DDP_CUDA(cudaStreamSynchronize(s->stream));
    s->t_sub.assign(R, 0);
    s->reported.assign(R, 0);
    // graph versions: the graph moves to the dynamic layout (master copy),
    // version 0 is published into the ring
    e = cudaStreamCreateWithFlags(&s->cstream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
    s->nver = versions;
    s->vb.assign((size_t)versions, VBuf());
    e = cudaHostAlloc(&s->h_vtab, sizeof(DevGraph) * (size_t)versions, flags);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_inflight, sizeof(int) * (size_t)versions, flags);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_vtab, s->h_vtab, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_inflight, s->h_inflight, 0);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaHostAlloc(graph versions)"));
    std::memset((void *)s->h_vtab, 0, sizeof(DevGraph) * (size_t)versions);
    std::memset(s->h_inflight, 0, sizeof(int) * (size_t)versions);
    {
        std::lock_guard<std::mutex> glk(g->mu);
        if (g->hook.fn) {
            rc = fail(DDP_ERR_INVALID, "graph is already served");
        } else {
            rc = dyn_graph_prepare(g);
            // every buffer starts at version 0, so later versions are patches
            for (int k = 1; !rc && k < versions; k++) rc = fill_buffer(s, k, 0);
            if (!rc) rc = publish(s, 0);
            if (!rc) {
                g->hook.fn = svc_scatter;
                g->hook.ctx = s;
                g->defer_free = true;
            }
        }
    }
    if (rc) return bail(rc);
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
        int32_t ver = s->h_ver[i];
        if (c == -1) {
            // the search outgrew its slot: re-run it on the single-query engine
            // over the master copy, which is the latest version
            ddp_heuristic *h = nullptr;
            // (the bidirectional kind has no single-query form: Dijkstra
            // order gives the same cost)
            const int hk = is_bidir_kind(s->hkind) ? DDP_H_ZERO : s->hkind;
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
            if (s->path_cap > 0) {
                int32_t l = 0;
                rc = ddp_path_read(q, nullptr, 0, &l);
                std::vector<int32_t> p((size_t)std::max(l, 0));
                if (!rc && l > 0) rc = ddp_path_read(q, p.data(), l, &l);
                if (rc) {
                    ddp_query_free(q);
                    return rc;
                }
                s->host_paths[i] = std::move(p);
            }
            ddp_query_free(q);
            s->fallbacks++;
            ver = s->version;
        }
        s->reported[(size_t)i] = 1;
        s->completed++;
        if (ids) ids[k] = i;
        if (costs) costs[k] = c;
        if (latency_ns) latency_ns[k] = t - s->t_sub[(size_t)i];
        if (versions) versions[k] = ver;
        k++;
    }
    while (s->scan_lo < s->submitted && s->reported[(size_t)s->scan_lo]) s->scan_lo++;
    *nout = k;
    return ensure_running(s);
}

int ddp_serve_update(ddp_server *s, int32_t n, const int32_t *flag, const int32_t *u, const int32_t *v,
                     const uint32_t *w) {
    if (!s) return fail(DDP_ERR_INVALID, "null server");
    if (s->hkind == DDP_H_LANDMARK)
        return fail(DDP_ERR_INVALID, "a landmark server serves a fixed graph (updates would void the landmark bounds)");
    std::lock_guard<std::mutex> lk(s->mu);
    int rc = apply_and_publish(s, n, flag, u, v, w);
    if (rc) return rc;
    s->version++;
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

int ddp_serve_record_paths(ddp_server *s, int32_t path_cap) {
    if (!s || path_cap <= 0) return fail(DDP_ERR_INVALID, "bad path capacity");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->submitted > 0 || s->h_paths) return fail(DDP_ERR_INVALID, "paths must be set up before the first request");
    // no slot kernel runs before the first request: the lengths move to
    // mapped host memory too, so reading them never waits for that kernel
    const size_t bytes = sizeof(int32_t) * (size_t)s->cap * (size_t)path_cap;
    int32_t *dl = nullptr;
    cudaError_t e = cudaHostAlloc(&s->h_paths, bytes, cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&s->d_paths, s->h_paths, 0);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->h_plen, sizeof(int32_t) * (size_t)s->cap, cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&dl, s->h_plen, 0);
    if (e != cudaSuccess) {
        cudaFreeHost(s->h_paths);
        cudaFreeHost(s->h_plen);
        s->h_paths = s->d_paths = s->h_plen = nullptr;
        return cuda_fail(e, "cudaHostAlloc(paths)");
    }
    cudaFree(s->d_plen);
    s->d_plen = dl;
    s->path_cap = path_cap;
    return DDP_OK;
}

int ddp_serve_path(ddp_server *s, int64_t id, int32_t *buf, int32_t cap, int32_t *len) {
    if (!s || !len || cap < 0 || (cap > 0 && !buf)) return fail(DDP_ERR_INVALID, "bad path arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->h_paths) return fail(DDP_ERR_INVALID, "paths are not recorded (ddp_serve_record_paths)");
    if (id < 0 || id >= s->submitted || !s->reported[(size_t)id])
        return fail(DDP_ERR_INVALID, "request not completed (poll it first)");
    const auto it = s->host_paths.find(id);
    if (it != s->host_paths.end()) {
        *len = (int32_t)it->second.size();
        std::memcpy(buf, it->second.data(), sizeof(int32_t) * (size_t)std::min(cap, *len));
        return DDP_OK;
    }
    // written before the request's done flag, which poll has seen
    const int32_t l = s->h_plen[id];
    *len = l;
    if (l > s->path_cap) return fail(DDP_ERR_INVALID, "path longer than the recorded capacity (*len holds its length)");
    if (l > 0) std::memcpy(buf, s->h_paths + (size_t)id * s->path_cap, sizeof(int32_t) * (size_t)std::min(cap, l));
    return DDP_OK;
}

int ddp_serve_free(ddp_server *s) {
    if (!s) return DDP_OK;
    trace("serve: free (kernel %s)", s->running ? "launched" : "not running");
    if (s->h_ctl) __atomic_store_n(&s->h_ctl[1], 1, __ATOMIC_RELEASE);
    if (s->stream) cudaStreamSynchronize(s->stream);
    trace("serve: free: slots left");
    if (s->g) {
        std::lock_guard<std::mutex> glk(s->g->mu);
        if (s->g->hook.ctx == s) {
            s->g->hook = ScatterHook();
            s->g->defer_free = false;
            graph_flush_frees(s->g);
        }
    }
    trace("serve: free: graph released");
    slots_free(s->sa);
    for (VBuf &b : s->vb) {
        cudaFree(b.off);
        cudaFree(b.oend);
        cudaFree(b.roff);
        cudaFree(b.roend);
        cudaFree(b.arc);
        cudaFree(b.rarc);
    }
    cudaFreeHost(s->h_vtab);
    cudaFreeHost(s->h_inflight);
    cudaFreeHost(s->h_stage);
    for (void *p : s->stage_old) cudaFreeHost(p);
    if (s->cstream) cudaStreamDestroy(s->cstream);
    cudaFreeHost(s->h_S);
    cudaFreeHost(s->h_T);
    cudaFreeHost(s->h_cost);
    cudaFreeHost(s->h_ver);
    cudaFreeHost(s->h_done);
    cudaFreeHost(s->h_ctl);
    cudaFreeHost(s->h_svc);
    cudaFree(s->d_work);
    if (s->h_plen) cudaFreeHost(s->h_plen);
    else cudaFree(s->d_plen);
    cudaFreeHost(s->h_paths);
    if (s->stream) cudaStreamDestroy(s->stream);
    graph_unref(s->g);
    delete s;
    trace("serve: free: done");
    return DDP_OK;
}

}  // extern "C"
