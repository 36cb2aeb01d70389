// Autotuner for the batch engine: picks CTAs per slot (group), threads per
// CTA (block), the bucket width (delta) and the per-iteration expansion cap
// (K) by timing the engine on a caller-supplied sample of queries.
//
// No reference counterpart (the reference hard-codes K per run and has no
// batched form).  Search: the (group, block) grid first, since it decides
// how many queries run at once and dominates throughput; then delta around
// the automatic choice, walking on in the direction that wins; then K for multi-CTA slots (one-CTA slots run the
// asynchronous engine, which has no K); then the queue capacity per slot.  Every trial must return the same
// costs as the first one: a mismatch is reported as an error, never tuned
// around.
#include <chrono>
#include <cstring>
#include <vector>

#include "graph.cuh"
#include "solve.cuh"

using namespace ddp;

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Queries/s of one configuration on the sample (one warm-up pass over the
// whole sample, so that every slot has run before the timing, then one
// timed pass); costs into `cost`.
int trial(ddp_graph *g, int32_t hkind, const ddp_opts &o, int32_t n, const int32_t *S, const int32_t *T,
          std::vector<int32_t> &cost, double *qps) {
    ddp_batch *b = nullptr;
    int rc = ddp_batch_create(g, hkind, &o, &b);
    if (rc) return rc;
    std::vector<int32_t> plen((size_t)n);
    cost.assign((size_t)n, 0);
    rc = ddp_batch_solve(b, n, S, T, cost.data(), plen.data());
    if (!rc) {
        const double t0 = now_s();
        rc = ddp_batch_solve(b, n, S, T, cost.data(), plen.data());
        const double dt = now_s() - t0;
        *qps = dt > 0 ? n / dt : 0.0;
    }
    ddp_batch_free(b);
    return rc;
}

}  // namespace

extern "C" {

int ddp_batch_tune(ddp_graph *g, int32_t hkind, int32_t n, const int32_t *sources, const int32_t *targets,
                   const ddp_opts *base, ddp_opts *best, double *best_qps, int32_t *trials) {
    if (!g || !sources || !targets || !best || n < 1) return fail(DDP_ERR_INVALID, "bad tuning arguments");
    ddp_opts b0 = base ? *base : ddp_opts{};
    std::vector<int32_t> ref, cost;
    double top = -1.0;
    ddp_opts top_o = b0;
    int count = 0;
    auto run = [&](const ddp_opts &o) -> int {
        double q = 0.0;
        int rc = trial(g, hkind, o, n, sources, targets, ref.empty() ? ref : cost, &q);
        if (rc) return rc;
        count++;
        if (count > 1 && cost != ref)
            return fail(DDP_ERR_CUDA, "autotuner: two configurations returned different costs");
        if (q > top) {
            top = q;
            top_o = o;
        }
        return DDP_OK;
    };
    // 1. slot shape (bidirectional slots are one CTA)
    const int shapes[][2] = {{1, 512}, {1, 256}, {2, 512}, {4, 512}, {8, 512}, {19, 512}};
    const int nshapes = is_bidir_kind(hkind) ? 2 : 6;
    for (int si = 0; si < nshapes; si++) {
        const auto &sh = shapes[si];
        ddp_opts o = b0;
        o.group = sh[0];
        o.block = sh[1];
        o.K = 0;
        o.delta = 0;
        int rc = run(o);
        if (rc) return rc;
    }
    // 2. bucket width: half and twice the automatic one, then further steps
    //    of 2/3 (or 3/2) while the winning direction keeps winning
    const uint32_t d0 = is_bidir_kind(hkind) ? auto_delta_bidir(g) : auto_delta(g);
    const ddp_opts shape = top_o;
    uint32_t best_d = d0;
    for (uint32_t dv : {d0 / 2, d0 * 2}) {
        if (dv < 1 || dv == d0) continue;
        ddp_opts o = shape;
        o.delta = (int32_t)dv;
        const double before = top;
        int rc = run(o);
        if (rc) return rc;
        if (top > before) best_d = dv;
    }
    for (int step = 0; step < 3 && best_d != d0; step++) {
        const uint32_t nd = best_d < d0 ? best_d * 2 / 3 : best_d * 3 / 2;
        if (nd < 1 || nd == best_d) break;
        ddp_opts o = shape;
        o.delta = (int32_t)nd;
        const double before = top;
        int rc = run(o);
        if (rc) return rc;
        if (top <= before) break;
        best_d = nd;
    }
    // 3. expansion cap per iteration (phase-synchronous groups only)
    if (top_o.group > 1) {
        const ddp_opts shaped = top_o;
        for (int32_t k : {1024, 8192}) {
            ddp_opts o = shaped;
            o.K = k;
            int rc = run(o);
            if (rc) return rc;
        }
    }
    // 4. queue capacity per slot: smaller queues leave memory for more
    //    slots where memory, not occupancy, limits them; a query that
    //    outgrows its slot is re-run on the single-query engine, so a cap
    //    that is too small loses on time and is not taken
    {
        const ddp_opts capped = top_o;
        for (int64_t div : {4, 16}) {
            ddp_opts o = capped;
            o.queue_cap = (int64_t)g->n / div + 4096;
            const double before = top;
            int rc = run(o);
            if (rc) return rc;
            if (top <= before) break;
        }
    }
    *best = top_o;
    if (best_qps) *best_qps = top;
    if (trials) *trials = count;
    return DDP_OK;
}

}  // extern "C"
