// GA* search engine: device code shared by the single-query (whole grid)
// and batched (one CTA per query slot) kernels.
//
// What it replaces (lkoshale/DDP, LIB/include/kernels/a_star_kernels.cu):
//   extractMin  (:7-61)   K threads pop K heap tops
//   A_star_expand (:67-133) one thread per node, spin lock per child
//   keepHeapPQ + setNV + insertPQ (:138-237) heap repair, O(N) flag scan,
//                                           round-robin re-insert
//   checkMIN (:243-254)   stop when no heap top has f < f(t)
//
// How it works here:
//   * Open list = threshold buckets on f (near-far): `near` holds entries
//     with f < T, `far` the rest.  One iteration expands up to K entries of
//     near (all of it when K = 0); improved children go to `next` when
//     f < T, else to `far`.  When near and next are empty the far pile is
//     split at T' = T + delta (or at its smallest f + delta): f < T' moves to
//     near, the rest is compacted.  Stale entries (g changed since the push)
//     and entries with f >= f(t) are dropped at every pop and split.
//   * Termination (the GA* test of checkMIN, made exact): the search ends
//     when near, next and far are all empty after pruning, i.e. no open
//     node has f < f(t).  With an admissible heuristic g(t) is then optimal.
//   * Expansion is warp-cooperative: 32 popped nodes per warp, their rows are
//     concatenated by a warp prefix sum and walked 32 arcs at a time, so arc
//     loads are 8-byte {head, w} reads of consecutive row slices.
//   * Relaxation is lock-free: one 64-bit word per node packs (g << 32 |
//     parent); a plain L2 read filters the (common) non-improving arcs, then
//     a CAS loop installs strictly smaller g.  No spin locks (the reference's
//     `while(!leaveLoop)` lock with __syncthreads inside divergent code is
//     gone).
//   * Pushes are warp-aggregated: one atomic per warp per target queue.
//   * Every loop bound is data-driven; the only wait is the group barrier,
//     which is bounded (common.cuh).
#pragma once

#include "common.cuh"

namespace ddp {

constexpr unsigned FULL = 0xffffffffu;

// Control block of one search slot (global memory).  Push counters rotate
// over 4 phases so that a counter is reset two phases before it is used
// again, with a single barrier per phase.
struct SearchCtl {
    int nq[4];            // pushes into near/next (or BFS frontier) this phase
    int fq[4];            // pushes into far this phase
    unsigned int mf[4];   // min f kept in far during a split phase
    int err[4];           // ST_* raised during the phase (read after its barrier)
    int ck[4];            // chunks of 32 entries claimed so far in the phase
    int touched;          // nodes whose state left the initial value
    int status;           // ST_* bits
    int iters;            // phases run
    int pad;
    unsigned long long expanded, scanned, relaxed, pad2;
    unsigned long long bfs_reached, bfs_scanned;  // heuristic BFS work
    unsigned long long far_scanned;               // far entries read by splits
    unsigned int tag;     // hop-array tag of the current query (batch)
    unsigned int hcap;    // hop cap of the last BFS
    int cur_q;            // query the slot is working on (batch)
    int far_n, far_sel;   // far pile left by the last run (dynamic resume)
    int cur_ver;          // graph version of the current search (serving)
    unsigned int bar_count, bar_gen;  // grid barrier (single-query form)
    int cold_n;           // entries in the far pile's cold tier (keep mode)
};

// Buffers of one slot.
struct SlotBufs {
    unsigned long long *state;  // n, (g << 32) | parent; all-ones = unreached
    uint2 *q0, *q1;             // near / next ping-pong, cap_q entries {node, g}
    uint4 *f0, *f1;             // far ping-pong, cap_f entries {node, g, f, 0}
    int32_t *touched;           // n: nodes whose state must be reset
    uint32_t *hops;             // n: per-target hop heuristic (may be null)
    SearchCtl *ctl;
    int64_t cap_q, cap_f;
    int64_t swords;  // 64-bit words of the state array
    int hbits;       // hashed records: log2 of the table size (0: one record per node)
};

// ---- groups ------------------------------------------------------------------
struct CtaGroup {
    int *status;
    __device__ int rank() const { return threadIdx.x; }
    __device__ int size() const { return blockDim.x; }
    __device__ int warp() const { return threadIdx.x >> 5; }
    __device__ int nwarps() const { return blockDim.x >> 5; }
    __device__ void sync() const { __syncthreads(); }
};

struct GridGroup {
    GridBarrier bar;
    int *status;
    __device__ int rank() const { return blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ int size() const { return gridDim.x * blockDim.x; }
    __device__ int warp() const { return (blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
    __device__ int nwarps() const { return (gridDim.x * blockDim.x) >> 5; }
    __device__ void sync() const { grid_sync(bar, gridDim.x, status); }
};

// G consecutive CTAs of a cooperative launch working on one query.
struct SubGridGroup {
    GridBarrier bar;
    int *status;
    int G;
    __device__ int rank() const { return (blockIdx.x % G) * blockDim.x + threadIdx.x; }
    __device__ int size() const { return G * blockDim.x; }
    __device__ int warp() const { return rank() >> 5; }
    __device__ int nwarps() const { return size() >> 5; }
    __device__ void sync() const { grid_sync(bar, (unsigned)G, status); }
};

// ---- heuristics (h(v) as uint32, INF_G = "cannot reach the target") -------
struct HeurZero {
    __device__ uint32_t operator()(int32_t) const { return 0; }
};

struct HeurHops {  // reverse-BFS hop count x scale (GA_star/bfs_hx.cu)
    const uint32_t *hops;
    uint32_t scale;
    uint32_t cap;  // hops assumed for unreached nodes (HOPS_INF = cannot reach t)
    uint32_t tag;  // 0: plain levels; else epoch-tagged words (run_bfs_hops)
    __device__ uint32_t operator()(int32_t v) const {
        const uint32_t x = __ldcg(hops + v);
        uint32_t hv;
        if (tag) hv = ((x & 0xFFFFFF00u) == tag) ? (x & 0xFFu) : cap;
        else hv = (x == HOPS_INF) ? cap : x;
        if (hv == HOPS_INF) return INF_G;
        unsigned long long p = (unsigned long long)hv * scale;
        return p >= INF_G ? INF_G : (uint32_t)p;
    }
};

struct HeurArray {  // caller-supplied h; negative = cannot reach the target
    const int32_t *h;
    __device__ uint32_t operator()(int32_t v) const {
        int32_t x = __ldg(h + v);
        return x < 0 ? INF_G : (uint32_t)x;
    }
};

struct HeurManhattan {
    const int32_t *xy;
    int32_t tx, ty;
    uint32_t scale;
    __device__ uint32_t operator()(int32_t v) const {
        int2 p = __ldg(reinterpret_cast<const int2 *>(xy) + v);
        unsigned long long d = (unsigned long long)(abs(p.x - tx)) + (unsigned long long)(abs(p.y - ty));
        d *= scale;
        return d >= INF_G ? INF_G : (uint32_t)d;
    }
};

// ALT lower bound: max over landmarks L of d(L,t) - d(L,v) and d(v,L) - d(t,L)
// (triangle inequality, so admissible, and consistent when s = 1).  The
// table holds q = floor(d / s); d(a) - d(b) >= s (q_a - q_b) - (s - 1),
// which is the exact difference when s = 1.  The engines need
// admissibility only: a node reached again with a smaller g is re-expanded.  A landmark that reaches v but not t, or is
// reached from t but not from v, proves that v cannot reach t.
// unroll factor of the landmark row loops (row loads issued ahead of use)
#ifndef DDP_ALT_UNROLL
#define DDP_ALT_UNROLL 8
#endif
constexpr int ALT_UNROLL = DDP_ALT_UNROLL;
struct HeurALT {
    const uint2 *tab;  // DevGraph::lm: rows of 2L entries
    int32_t L;         // landmarks, a multiple of 4 (16-bit) or 8 (8-bit)
    int32_t s;         // DevGraph::lm_scale
    int32_t t;
    int32_t bits;      // DevGraph::lm_bits: 16 or 8
    // One packed word of B-bit entries, a from the row that must be larger:
    // the lanes' a - b, saturated at 0 and zeroed where either side is the
    // unreachable marker, fold into the lane-wise maximum m; lanes where a
    // is the marker and b is not (the landmark relates v and t one way
    // only, so v cannot reach t) fold into the cut mask cm.  Since s >= 1,
    // the maximum over terms of s (a - b) - (s - 1), floored at 0, is
    // s max(a - b) - (s - 1) when that maximum is positive, else 0.
    template <int B>
    __device__ __forceinline__ void word(uint32_t a, uint32_t b, uint32_t &m, uint32_t &cm) const {
        if (B == 8) {
            const uint32_t ea = __vcmpeq4(a, 0xFFFFFFFFu), eb = __vcmpeq4(b, 0xFFFFFFFFu);
            cm |= ea & ~eb;
            m = __vmaxu4(m, __vsubus4(a, b) & ~(ea | eb));
        } else {
            const uint32_t ea = __vcmpeq2(a, 0xFFFFFFFFu), eb = __vcmpeq2(b, 0xFFFFFFFFu);
            cm |= ea & ~eb;
            m = __vmaxu2(m, __vsubus2(a, b) & ~(ea | eb));
        }
    }
    template <int B>
    __device__ __forceinline__ void terms(uint2 a, uint2 b, uint32_t &m, uint32_t &cm) const {
        word<B>(a.x, b.x, m, cm);
        word<B>(a.y, b.y, m, cm);
    }
    template <int B>
    __device__ __forceinline__ uint32_t eval(int32_t v) const {
        const int W = L / (64 / B);  // 8-byte words per half row
        const uint2 *rv = tab + (size_t)v * (2 * W);
        const uint2 *rt = tab + (size_t)t * (2 * W);
        uint32_t m = 0, cm = 0;
        if ((W & 1) == 0) {
            // both halves start on a 16-byte boundary: 16-byte loads
            const uint4 *qv = reinterpret_cast<const uint4 *>(rv), *qt = reinterpret_cast<const uint4 *>(rt);
            const int W2 = W >> 1;
#pragma unroll ALT_UNROLL
            for (int i = 0; i < W2; i++) {
                const uint4 fv = __ldg(qv + i), ft = __ldg(qt + i);
                terms<B>(make_uint2(ft.x, ft.y), make_uint2(fv.x, fv.y), m, cm);
                terms<B>(make_uint2(ft.z, ft.w), make_uint2(fv.z, fv.w), m, cm);
            }
#pragma unroll ALT_UNROLL
            for (int i = W2; i < 2 * W2; i++) {
                const uint4 bv = __ldg(qv + i), bt = __ldg(qt + i);
                terms<B>(make_uint2(bv.x, bv.y), make_uint2(bt.x, bt.y), m, cm);
                terms<B>(make_uint2(bv.z, bv.w), make_uint2(bt.z, bt.w), m, cm);
            }
        } else {
            for (int i = 0; i < W; i++) {
                const uint2 fv = __ldg(rv + i), ft = __ldg(rt + i);
                const uint2 bv = __ldg(rv + W + i), bt = __ldg(rt + W + i);
                terms<B>(ft, fv, m, cm);
                terms<B>(bv, bt, m, cm);
            }
        }
        if (cm) return INF_G;
        const uint32_t mx = B == 8 ? max(max(m & 0xFFu, (m >> 8) & 0xFFu), max((m >> 16) & 0xFFu, m >> 24))
                                   : max(m & 0xFFFFu, m >> 16);
        // mx s <= q s <= the largest table distance, below INF_G
        return mx ? mx * (uint32_t)s - (uint32_t)(s - 1) : 0u;
    }
    __device__ uint32_t operator()(int32_t v) const { return bits == 8 ? eval<8>(v) : eval<16>(v); }
};

// floor(sqrt(x)) for x < 2^62, exact: a float estimate, then integer fix-up
__host__ __device__ __forceinline__ uint64_t isqrt_floor(uint64_t x) {
    uint64_t r = (uint64_t)sqrt((double)x);
    while (r * r > x) r--;
    while ((r + 1) * (r + 1) <= x) r++;
    return r;
}

struct HeurEuclid {  // floor(rho * floor(dist)), rho <= w / length on every arc
    const int32_t *xy;
    int32_t tx, ty;
    uint32_t rho_fp;  // 16.16
    __device__ uint32_t operator()(int32_t v) const {
        int2 p = __ldg(reinterpret_cast<const int2 *>(xy) + v);
        const int64_t dx = (int64_t)p.x - tx, dy = (int64_t)p.y - ty;
        const uint64_t r = isqrt_floor((uint64_t)(dx * dx + dy * dy));
        const uint64_t h = (r * rho_fp) >> 16;
        return h >= INF_G ? INF_G - 1 : (uint32_t)h;
    }
};

// Heuristics computed from registers and one small load (coordinates): the
// one-CTA engine evaluates them speculatively, beside the relaxation's
// atomic, instead of after it.  Table heuristics (hops, landmarks, arrays)
// are read only for relaxations that improve g.
template <class H>
struct heur_cheap {
    static constexpr bool value = false;
};
template <>
struct heur_cheap<HeurZero> {
    static constexpr bool value = true;
};
template <>
struct heur_cheap<HeurManhattan> {
    static constexpr bool value = true;
};
template <>
struct heur_cheap<HeurEuclid> {
    static constexpr bool value = true;
};

// ---- warp helpers ----------------------------------------------------------
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// Returns this lane's slot in a warp-aggregated append (or -1 when !pred).
__device__ __forceinline__ int warp_append(bool pred, int *counter) {
    unsigned m = __ballot_sync(FULL, pred);
    if (m == 0) return -1;
    int lane = lane_id();
    int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(FULL, base, leader);
    return pred ? base + __popc(m & ((1u << lane) - 1u)) : -1;
}

__device__ __forceinline__ int warp_excl_scan(int x, int *total) {
    int lane = lane_id();
    int v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += y;
    }
    *total = __shfl_sync(FULL, v, 31);
    return v - x;
}

// Claims the next chunk of a phase for this warp (dynamic balance: warps
// that finish early take more chunks).  Returns the chunk index.
__device__ __forceinline__ int64_t claim_chunk(int *counter) {
    int c = 0;
    if ((threadIdx.x & 31) == 0) c = atomicAdd(counter, 1);
    return (int64_t)__shfl_sync(0xffffffffu, c, 0);
}

// Records an error for phase `ph` (consistent control flow after the
// barrier) and in the sticky status word (reporting).
__device__ __forceinline__ void raise_err(SearchCtl *ctl, int ph, int bit) {
    atomicOr(&ctl->err[ph], bit);
    atomicOr(&ctl->status, bit);
}

__device__ __forceinline__ uint32_t sat_add(uint32_t a, uint32_t b) {
    uint32_t c = a + b;
    return c < a ? 0xFFFFFFFFu : c;
}

// Per-warp shared memory: staging of 32 popped rows, and staging buffers
// for queue pushes (flushed with one atomic per >= 32 entries, so the L2
// round trip of a queue reservation is paid once per flush instead of once
// per 32 arcs, and the stores are coalesced).
struct WarpRows {
    int excl[32];
    int rb[32];      // first arc of the base row
    int bdeg[32];    // base-row length (diff arcs follow)
    int drb[32];     // first arc of the diff row
    uint32_t g[32];
    int u[32];
    uint2 sn[64];    // staged near/next pushes
    int2 snr[64];    // one-CTA engine: row bounds of the staged own children
    uint4 sf[64];    // staged far pushes
    int st[64];      // staged first touches / BFS frontier pushes
};

// Copies a warp's staged entries to dst[base + reserved ..] (all lanes).
template <class T>
__device__ __forceinline__ void stage_flush(T *buf, int &cnt, int *counter, T *dst, int64_t base,
                                            int64_t cap, SearchCtl *ctl, int ph);

template <class T>
__device__ __forceinline__ void stage_push(bool pred, T val, T *buf, int &cnt, int *counter, T *dst,
                                           int64_t base, int64_t cap, SearchCtl *ctl, int ph) {
    const unsigned m = __ballot_sync(FULL, pred);
    if (pred) buf[cnt + __popc(m & ((1u << (threadIdx.x & 31)) - 1u))] = val;
    cnt += __popc(m);
    if (cnt >= 32) stage_flush(buf, cnt, counter, dst, base, cap, ctl, ph);
}

template <class T>
__device__ __forceinline__ void stage_flush(T *buf, int &cnt, int *counter, T *dst, int64_t base,
                                            int64_t cap, SearchCtl *ctl, int ph) {
    if (cnt == 0) return;  // warp-uniform
    __syncwarp();
    int b = 0;
    if ((threadIdx.x & 31) == 0) b = atomicAdd(counter, cnt);
    b = __shfl_sync(FULL, b, 0);
    for (int i = threadIdx.x & 31; i < cnt; i += 32) {
        const int64_t pos = base + b + i;
        if (pos < cap) dst[pos] = buf[i];
        else raise_err(ctl, ph, ST_OVERFLOW);
    }
    __syncwarp();
    cnt = 0;
}

__device__ __forceinline__ int row_owner(const WarpRows &wr, int k) {
    int o = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1)
        if (wr.excl[o + step] <= k) o += step;
    return o;
}

__device__ __forceinline__ uint2 row_arc(const DevGraph &G, const WarpRows &wr, int o, int k,
                                         bool fwd) {
    int j = k - wr.excl[o];
    if (j < wr.bdeg[o]) {
        if (G.oend) return fwd ? __ldcg(G.arc + wr.rb[o] + j) : __ldcg(G.rarc + wr.rb[o] + j);
        return fwd ? __ldg(G.arc + wr.rb[o] + j) : __ldg(G.rarc + wr.rb[o] + j);
    }
    j -= wr.bdeg[o];
    return fwd ? __ldcg(G.darc + wr.drb[o] + j) : __ldcg(G.drarc + wr.drb[o] + j);
}

// ---- search parameters -------------------------------------------------------
struct SearchParams {
    int32_t s, t;
    uint32_t delta;
    int32_t K;     // 0 = whole near bucket per iteration
    int keep;      // keep every generated node open (no f(t) pruning): the
                   // state stays resumable after graph updates
    int resume;    // continue from the slot's far pile instead of starting at s
    int no_touch_log;  // do not log first touches (slots that are never reset)
    // t < 0: no target, the search settles everything reachable from s
    // Keep mode, resumed searches: cold tier of the far pile.  The first
    // split moves live entries with g >= cold_x (their f is at least g) to
    // `cold` unexamined; later splits scan the rest until min(f(t),
    // threshold) passes cold_x, when one split takes the cold entries back.
    // They rejoin the far pile when the search ends.  cold_x = 0xFFFFFFFF:
    // no cold tier.
    uint2 *cold = nullptr;
    int64_t cold_cap = 0;
    uint32_t cold_x = 0xFFFFFFFFu;
};

struct SearchResult {
    uint32_t cost;  // g(t) + h(t), >= INF_G when unreachable
    int iters;
};

// One A* run on one slot, executed collectively by every thread of `grp`.
// Precondition: slot state is all-ones (unreached) for every node.
template <class Grp, class Heur>
__device__ SearchResult run_search(const Grp &grp, const DevGraph &G, const SlotBufs &B,
                                   const Heur &H, const SearchParams &P, WarpRows *wrows) {
    SearchCtl *ctl = B.ctl;
    const int lane = lane_id();
    WarpRows &wr = wrows[threadIdx.x >> 5];
    const bool has_diff = G.doff != nullptr;

    if (grp.rank() == 0) {
        for (int i = 0; i < 4; i++) {
            ctl->nq[i] = 0;
            ctl->fq[i] = 0;
            ctl->mf[i] = 0xFFFFFFFFu;
            ctl->err[i] = 0;
            ctl->ck[i] = 0;
        }
        ctl->iters = 0;
        ctl->expanded = ctl->scanned = ctl->relaxed = 0;
        ctl->far_scanned = 0;
        ctl->cold_n = 0;
        if (!P.resume) {
            ctl->touched = 1;
            B.state[P.s] = st_make(0, -1);
            B.touched[0] = P.s;
            B.q0[0] = make_uint2((uint32_t)P.s, 0u);
        }
    }
    const int64_t far_resume = P.resume ? (int64_t)(*(volatile int *)&ctl->far_n) : 0;
    const bool far_in_f1 = P.resume && (*(volatile int *)&ctl->far_sel) != 0;
    grp.sync();

    uint2 *qcur = B.q0, *qnxt = B.q1;
    uint4 *fcur = far_in_f1 ? B.f1 : B.f0, *falt = far_in_f1 ? B.f0 : B.f1;
    int64_t nnear = P.resume ? 0 : 1, head = 0, nnext = 0, nfar = far_resume;
    const uint32_t hs = H(P.s);
    uint32_t T = sat_add(hs, P.delta);
    uint32_t Tsplit = T;
    bool splitting = P.resume != 0;
    if (P.resume) {
        T = 0;
        Tsplit = 0;  // the first split only measures the far pile's minimum f
    }
    // compaction: a split pass at the current T that only drops stale and
    // pruned far entries, run when the far pile fills up between splits
    bool compacting = false;
    int64_t far_after_compact = 0;
    unsigned long long n_exp = 0, n_scan = 0, n_rel = 0;
    int it = 0;
    int status = 0;
    const int64_t max_phases = 4 * (int64_t)G.n + (1 << 22);
    // cold tier (keep mode, resumed): made by the first split
    uint32_t cold_x = (P.keep && P.resume && P.cold) ? P.cold_x : 0xFFFFFFFFu;
    bool cold_pass = cold_x != 0xFFFFFFFFu;
    int64_t ncold = 0;
    uint2 *cold_stage = reinterpret_cast<uint2 *>(wr.snr);

    for (;;) {
        const int PH = (it + 1) & 3, RS = (it + 3) & 3;
        // f(t) snapshot: only decreases, so a stale value only prunes less.
        const uint64_t st_t = P.t >= 0 ? __ldcg(B.state + P.t) : ~0ull;
        const uint32_t ht = P.t >= 0 ? H(P.t) : 0u;
        const uint64_t ft64 = (uint64_t)st_g(st_t) + ht;
        const uint32_t ft = ft64 >= 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)ft64;
        int64_t end = 0;
        if (!splitting) {
            end = (P.K > 0) ? min(nnear, head + (int64_t)P.K) : nnear;
            int c_n = 0, c_f = 0, c_t = 0;  // staged pushes of this warp
            // chunk claims are prefetched one ahead to hide their round trip
            int64_t cnext = claim_chunk(&ctl->ck[PH]);
            for (int64_t base = head + 32 * cnext; base < end; base = head + 32 * cnext) {
                cnext = claim_chunk(&ctl->ck[PH]);
                const int64_t idx = base + lane;
                int u = -1, rb = 0, bdeg = 0, drb = 0, deg = 0;
                uint32_t gu = 0;
                bool requeue = false;
                if (idx < end) {
                    const uint2 en = __ldcg(qcur + idx);
                    u = (int)en.x;
                    gu = en.y;
                    // independent loads issued together (speculatively for
                    // entries that turn out stale)
                    const uint64_t su = __ldcg(B.state + u);
                    // every near entry was pushed with f = g + h(u) < T
                    // (relaxations, split and compaction moves alike; T only
                    // grows), so while f(t) >= T the pop test f < f(t)
                    // passes without reading h again; keep mode re-derives it
                    const uint32_t hu = (ft < T || (P.keep && ft != 0xFFFFFFFFu)) ? H(u) : 0u;
                    const int r0 = row_begin(G.off, G.oend, u), r1 = row_end(G.off, G.oend, u);
                    int d0 = 0, d1 = 0;
                    if (has_diff) {
                        d0 = __ldcg(G.doff + u);
                        d1 = __ldcg(G.doff + u + 1);
                    }
                    if (st_g(su) == gu && u != P.t) {
                        if ((uint64_t)gu + hu < ft) {
                            rb = r0;
                            bdeg = r1 - r0;
                            drb = d0;
                            deg = bdeg + (d1 - d0);
                            n_exp++;
                        } else if (P.keep) {
                            requeue = true;  // stays open beyond f(t)
                        }
                    }
                }
                stage_push(requeue, make_uint4((uint32_t)u, gu, 0u, 0u), wr.sf, c_f, &ctl->fq[PH],  // keep mode: f re-derived
                           fcur, nfar, B.cap_f, ctl, PH);
                int total;
                int ex = warp_excl_scan(deg, &total);
                wr.excl[lane] = ex;
                wr.rb[lane] = rb;
                wr.bdeg[lane] = bdeg;
                wr.drb[lane] = drb;
                wr.g[lane] = gu;
                wr.u[lane] = u;
                __syncwarp();
                n_scan += (lane == 0) ? (unsigned long long)total : 0ull;
                // ARCS arcs per lane per step; every stage issues all of its
                // loads / atomics before consuming any result
#ifndef DDP_ARCS
#define DDP_ARCS 2
#endif
                constexpr int ARCS = DDP_ARCS;
                for (int kb = 0; kb < total; kb += 32 * ARCS) {
                    int v[ARCS], o[ARCS];
                    uint32_t ng[ARCS], hv[ARCS];
                    uint64_t sv[ARCS], prev[ARCS];
                    bool live[ARCS], go[ARCS];
#pragma unroll
                    for (int r = 0; r < ARCS; r++) {
                        const int k = kb + 32 * r + lane;
                        live[r] = false;
                        v[r] = 0;
                        ng[r] = 0;
                        o[r] = 0;
                        if (k < total) {
                            o[r] = row_owner(wr, k);
                            const uint2 a = row_arc(G, wr, o[r], k, true);
                            v[r] = (int)a.x;
                            const uint64_t ng64 = (uint64_t)wr.g[o[r]] + a.y;
                            live[r] = v[r] >= 0 && ng64 < INF_G;
                            ng[r] = (uint32_t)ng64;
                        }
                    }
#pragma unroll
                    for (int r = 0; r < ARCS; r++) sv[r] = live[r] ? __ldcg(B.state + v[r]) : 0ull;
#pragma unroll
                    for (int r = 0; r < ARCS; r++) {
                        live[r] = live[r] && ng[r] < st_g(sv[r]);
                        hv[r] = live[r] ? H(v[r]) : 0u;
                    }
#pragma unroll
                    for (int r = 0; r < ARCS; r++) {
                        go[r] = live[r] && (P.keep ? hv[r] < INF_G : (uint64_t)ng[r] + hv[r] < ft);
                        prev[r] = go[r] ? atomicCAS(B.state + v[r], sv[r], st_make(ng[r], wr.u[o[r]])) : sv[r];
                    }
#pragma unroll
                    for (int r = 0; r < ARCS; r++) {
                        bool to_near = false, to_far = false, first = false;
                        if (go[r]) {
                            uint64_t cur = sv[r];
                            uint64_t got = prev[r];
                            // retry only when another relaxation got in between
                            while (got != cur) {
                                cur = got;
                                if (ng[r] >= st_g(cur)) break;
                                got = atomicCAS(B.state + v[r], cur, st_make(ng[r], wr.u[o[r]]));
                            }
                            if (got == cur) {
                                first = !P.no_touch_log && st_g(cur) >= INF_G;
                                const uint64_t fv = (uint64_t)ng[r] + hv[r];
                                if (fv < T) to_near = true;
                                else to_far = true;
                            }
                        }
                        if (to_near || to_far) n_rel++;
                        const uint2 en = make_uint2((uint32_t)v[r], ng[r]);
                        stage_push(to_near, en, wr.sn, c_n, &ctl->nq[PH], qnxt, nnext, B.cap_q, ctl, PH);
                        stage_push(to_far, make_uint4(en.x, en.y, sat_add(ng[r], hv[r]), 0u), wr.sf, c_f,
                                   &ctl->fq[PH], fcur, nfar, B.cap_f, ctl, PH);
                        // at most n first touches: the touched log never overflows
                        stage_push(first, v[r], wr.st, c_t, &ctl->touched, B.touched, 0, (int64_t)G.n, ctl, PH);
                    }
                }
                __syncwarp();
            }
            stage_flush(wr.sn, c_n, &ctl->nq[PH], qnxt, nnext, B.cap_q, ctl, PH);
            stage_flush(wr.sf, c_f, &ctl->fq[PH], fcur, nfar, B.cap_f, ctl, PH);
            stage_flush(wr.st, c_t, &ctl->touched, B.touched, 0, (int64_t)G.n, ctl, PH);
        } else {
            // split the far pile at Tsplit (or compact it at T).  Entries
            // carry f from their push: a split reads no node state, stale
            // entries are dropped when they are popped.  Keep mode (h may
            // have changed since the push) and compaction (which must drop
            // stale entries) re-check the state and h.
            const uint32_t thr = compacting ? T : Tsplit;
            const bool recheck = P.keep || compacting;
            // cold tier: made here (first split of a resumed search), or
            // scanned with the pile once min(f(t), threshold) passes cold_x
            const bool to_cold = cold_pass && !compacting;
            const bool merge_cold = !compacting && ncold > 0 && min(ft, thr) > cold_x;
            const int64_t nscan = nfar + (merge_cold ? ncold : 0);
            if (grp.rank() == 0) ctl->far_scanned += (unsigned long long)nscan;
            uint2 *dst = compacting ? qnxt : qcur;
            const int64_t dbase = compacting ? nnext : 0;
            unsigned int local_min = 0xFFFFFFFFu;
            int c_n = 0, c_f = 0, c_c = 0;
            for (int64_t base = 32 * claim_chunk(&ctl->ck[PH]); base < nscan;
                 base = 32 * claim_chunk(&ctl->ck[PH])) {
                const int64_t idx = base + lane;
                bool to_near = false, keep = false, cold = false;
                uint4 en = make_uint4(0u, 0u, 0u, 0u);
                if (idx < nscan) {
                    if (idx < nfar) {
                        en = __ldcg(fcur + idx);
                    } else {
                        const uint2 c = __ldcg(P.cold + (idx - nfar));
                        en = make_uint4(c.x, c.y, 0u, 0u);  // f re-derived below (keep mode)
                    }
                    bool live = true;
                    uint64_t f = en.z;
                    if (recheck) {
                        live = st_g(__ldcg(B.state + en.x)) == en.y;
                        if (live && to_cold && en.y >= cold_x) {
                            cold = true;  // f >= g >= cold_x: h is not read
                            live = false;
                        } else {
                            f = (uint64_t)en.y + H((int)en.x);
                            en.z = f >= 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)f;
                        }
                    }
                    if (live) {
                        if (f < ft && f < thr) {
                            to_near = true;
                        } else if (f < ft || (P.keep && f < INF_G)) {
                            keep = true;
                            local_min = min(local_min, (uint32_t)f);
                        }
                    }
                }
                stage_push(to_near, make_uint2(en.x, en.y), wr.sn, c_n, &ctl->nq[PH], dst, dbase, B.cap_q, ctl, PH);
                // compaction never grows the pile
                stage_push(keep, en, wr.sf, c_f, &ctl->fq[PH], falt, 0, B.cap_f, ctl, PH);
                if (to_cold)
                    stage_push(cold, make_uint2(en.x, en.y), cold_stage, c_c, &ctl->cold_n, P.cold, 0, P.cold_cap,
                               ctl, PH);
            }
            stage_flush(wr.sn, c_n, &ctl->nq[PH], dst, dbase, B.cap_q, ctl, PH);
            stage_flush(wr.sf, c_f, &ctl->fq[PH], falt, 0, B.cap_f, ctl, PH);
            if (to_cold) stage_flush(cold_stage, c_c, &ctl->cold_n, P.cold, 0, P.cold_cap, ctl, PH);
            if (merge_cold) {
                ncold = 0;  // every cold entry was examined: none is left
                cold_x = 0xFFFFFFFFu;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) local_min = min(local_min, __shfl_xor_sync(FULL, local_min, o));
            if (lane == 0 && local_min != 0xFFFFFFFFu) atomicMin(&ctl->mf[PH], local_min);
        }

        grp.sync();
        if (grp.rank() == 0) {
            ctl->nq[RS] = 0;
            ctl->fq[RS] = 0;
            ctl->mf[RS] = 0xFFFFFFFFu;
            ctl->err[RS] = 0;
            ctl->ck[RS] = 0;
        }
        const int a = *(volatile int *)&ctl->nq[PH];
        const int b = *(volatile int *)&ctl->fq[PH];
        const unsigned int m = *(volatile unsigned int *)&ctl->mf[PH];
        const int perr = *(volatile int *)&ctl->err[PH];
        status = *(volatile int *)&ctl->status;
        it++;
        if ((perr & ST_OVERFLOW) || (status & ST_TIMEOUT)) break;
        if (it > max_phases) {
            // a search never needs this many phases; stop instead of spinning
            if (grp.rank() == 0) atomicOr(&ctl->status, ST_TIMEOUT);
            break;
        }
        if (compacting) {
            uint4 *t2 = fcur;
            fcur = falt;
            falt = t2;
            nfar = b;
            nnext += a;
            far_after_compact = nfar;
            compacting = false;
            splitting = false;
        } else if (!splitting) {
            nnext += a;
            nfar += b;
            head = end;
            if (head >= nnear) {
                uint2 *t2 = qcur;
                qcur = qnxt;
                qnxt = t2;
                nnear = nnext;
                nnext = 0;
                head = 0;
                if (nnear == 0) {
                    splitting = true;
                    Tsplit = sat_add(T, P.delta);
                }
            }
            if (!splitting && nfar > B.cap_f / 2 && nfar - far_after_compact > B.cap_f / 8) {
                compacting = true;
                splitting = true;  // the split code path runs the compaction
            }
        } else {
            uint4 *t2 = fcur;
            fcur = falt;
            falt = t2;
            nfar = b;
            nnear = a;
            head = 0;
            nnext = 0;
            if (cold_pass) {
                // pushes past the buffer raised an overflow (the loop ends below)
                ncold = min((int64_t)*(volatile int *)&ctl->cold_n, P.cold_cap);
                cold_pass = false;
            }
            // cold entries have f >= cold_x
            const uint32_t mall = ncold > 0 ? min(m, cold_x) : m;
            if (nnear > 0) {
                T = Tsplit;
                splitting = false;
            } else if ((nfar == 0 && ncold == 0) || mall >= ft) {
                break;  // no open node with f < f(t): done
            } else {
                Tsplit = sat_add(mall, P.delta);
            }
        }
        if (nnear > B.cap_q || nfar > B.cap_f) {
            if (grp.rank() == 0) atomicOr(&ctl->status, ST_OVERFLOW);
            break;  // uniform: every thread computed the same counts
        }
    }

    // fold per-thread counters
    if (lane == 0 && n_scan) atomicAdd(&ctl->scanned, n_scan);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        n_exp += __shfl_xor_sync(FULL, n_exp, o);
        n_rel += __shfl_xor_sync(FULL, n_rel, o);
    }
    if (lane == 0) {
        if (n_exp) atomicAdd(&ctl->expanded, n_exp);
        if (n_rel) atomicAdd(&ctl->relaxed, n_rel);
    }
    if (ncold > 0) {
        // the cold tier rejoins the far pile (f re-derived by the next split)
        for (int64_t i = grp.rank(); i < ncold; i += grp.size()) {
            const uint2 c = __ldcg(P.cold + i);
            if (nfar + i < B.cap_f) fcur[nfar + i] = make_uint4(c.x, c.y, 0u, 0u);
            else atomicOr(&ctl->status, ST_OVERFLOW);
        }
        nfar = min(nfar + ncold, B.cap_f);
    }
    if (grp.rank() == 0) {
        ctl->far_n = (int)nfar;
        ctl->far_sel = fcur == B.f1 ? 1 : 0;
    }
    grp.sync();
    SearchResult r;
    const uint64_t st_t = P.t >= 0 ? __ldcg(B.state + P.t) : ~0ull;
    const uint64_t c = (uint64_t)st_g(st_t) + (P.t >= 0 ? H(P.t) : 0u);
    r.cost = (st_g(st_t) >= INF_G || c >= INF_G) ? 0xFFFFFFFFu : (uint32_t)c;
    r.iters = it;
    if (grp.rank() == 0) ctl->iters = it;
    return r;
}

// Reverse BFS from `t` (hop counts to t), executed collectively by `grp`.
// Replaces GA_star/bfs_hx.cu: the level loop runs on the device (no per-level
// D2H of the frontier size), frontier expansion is warp-cooperative over
// reverse-CSR rows, and each node is claimed once with a CAS.
//
// tag == 0: hops[] is first filled with HOPS_INF and then holds plain levels.
// tag != 0: hops[] is not cleared; a word is valid for this run when its high
//   24 bits equal tag >> 8, its low 8 bits hold the level (so levels stop at
//   254).  This lets a batch slot reuse the array per query without a fill.
// budget > 0: the BFS stops after the first level at which it has reached
//   `budget` nodes.  Returns the cap for unreached nodes in hop units:
//   HOPS_INF when the BFS ran to completion (unreached = cannot reach t),
//   else L+1 with L the last level claimed (unreached nodes are at least
//   L+1 hops away), so min(hops, cap) x wmin stays admissible and consistent.
template <class Grp>
__device__ uint32_t run_bfs_hops(const Grp &grp, const DevGraph &G, const SlotBufs &B, int32_t t,
                                 WarpRows *wrows, uint32_t tag, int64_t budget, bool spare_q0 = false) {
    SearchCtl *ctl = B.ctl;
    const int lane = lane_id();
    WarpRows &wr = wrows[threadIdx.x >> 5];
    const bool has_diff = G.doff != nullptr;
    // frontier ping-pong: the two near queues, or (when q0 is the
    // asynchronous ring that must stay clean) q1 and the second far pile
    int *fa = spare_q0 ? reinterpret_cast<int *>(B.f1) : reinterpret_cast<int *>(B.q0);
    int *fb = reinterpret_cast<int *>(B.q1);
    const int64_t capf = 2 * (spare_q0 ? min(B.cap_q, B.cap_f) : B.cap_q);  // uint2 slots reused as ints
    const uint32_t max_lvl = tag ? 254u : 0xFFFFFFF0u;

    if (!tag)
        for (int64_t i = grp.rank(); i < G.n; i += grp.size()) B.hops[i] = HOPS_INF;
    if (grp.rank() == 0) {
        for (int i = 0; i < 4; i++) {
            ctl->nq[i] = 0;
            ctl->err[i] = 0;
            ctl->ck[i] = 0;
        }
        ctl->bfs_scanned = 0;
        ctl->bfs_reached = 0;
    }
    grp.sync();
    if (grp.rank() == 0) {
        B.hops[t] = tag;  // level 0
        fa[0] = t;
    }
    grp.sync();
    int64_t nf = 1;
    uint32_t lvl = 0;
    int it = 0;
    unsigned long long b_reached = 1, b_scanned = 0;
    bool complete = true;
    while (nf > 0) {
        if (lvl >= max_lvl || (budget > 0 && (int64_t)b_reached >= budget)) {
            complete = false;
            break;
        }
        const int PH = (it + 1) & 3, RS = (it + 3) & 3;
        const uint32_t claim_val = tag | (lvl + 1);
        int c_b = 0;
        for (int64_t base = 32 * claim_chunk(&ctl->ck[PH]); base < nf; base = 32 * claim_chunk(&ctl->ck[PH])) {
            const int64_t idx = base + lane;
            int rb = 0, bdeg = 0, drb = 0, deg = 0;
            if (idx < nf) {
                int u = __ldcg(fa + idx);
                rb = row_begin(G.roff, G.roend, u);
                bdeg = row_end(G.roff, G.roend, u) - rb;
                deg = bdeg;
                if (has_diff) {
                    drb = __ldcg(G.droff + u);
                    deg += __ldcg(G.droff + u + 1) - drb;
                }
            }
            int total;
            int ex = warp_excl_scan(deg, &total);
            wr.excl[lane] = ex;
            wr.rb[lane] = rb;
            wr.bdeg[lane] = bdeg;
            wr.drb[lane] = drb;
            __syncwarp();
            if (lane == 0) b_scanned += (unsigned long long)total;
            for (int kb = 0; kb < total; kb += 32) {
                const int k = kb + lane;
                bool claim = false;
                int p = -1;
                if (k < total) {
                    const int o = row_owner(wr, k);
                    p = (int)row_arc(G, wr, o, k, false).x;
                    if (p >= 0) {
                        const uint32_t x = __ldcg(B.hops + p);
                        const bool seen = tag ? ((x & 0xFFFFFF00u) == tag) : (x != HOPS_INF);
                        if (!seen) claim = atomicCAS(B.hops + p, x, claim_val) == x;
                    }
                }
                stage_push(claim, p, wr.st, c_b, &ctl->nq[PH], fb, 0, capf, ctl, PH);
            }
            __syncwarp();
        }
        stage_flush(wr.st, c_b, &ctl->nq[PH], fb, 0, capf, ctl, PH);
        grp.sync();
        if (grp.rank() == 0) {
            ctl->nq[RS] = 0;
            ctl->err[RS] = 0;
            ctl->ck[RS] = 0;
        }
        nf = *(volatile int *)&ctl->nq[PH];
        b_reached += (unsigned long long)nf;
        const int perr = *(volatile int *)&ctl->err[PH];
        const int status = *(volatile int *)&ctl->status;
        it++;
        lvl++;
        int *tmp = fa;
        fa = fb;
        fb = tmp;
        if ((perr & ST_OVERFLOW) || (status & ST_TIMEOUT)) break;
    }
    if (lane == 0 && b_scanned) atomicAdd(&ctl->bfs_scanned, b_scanned);
    if (grp.rank() == 0) ctl->bfs_reached = b_reached;
    grp.sync();
    return complete ? HOPS_INF : lvl + 1;
}

// Parent walk t -> s into path[0..cap) in s..t order; returns the length
// (0 when unreachable).  One thread.
__device__ inline int32_t write_path(const SlotBufs &B, int32_t s, int32_t t, int32_t *path,
                                     int32_t cap, int32_t n, int *status) {
    uint64_t st = __ldcg(B.state + t);
    if (st_g(st) >= INF_G) return 0;
    int32_t len = 0;
    int32_t c = t;
    while (c >= 0 && len <= n) {
        if (len < cap) path[len] = c;
        len++;
        if (c == s) break;
        c = st_parent(__ldcg(B.state + c));
    }
    if (len <= cap) {
        for (int32_t i = 0, j = len - 1; i < j; i++, j--) {
            int32_t x = path[i];
            path[i] = path[j];
            path[j] = x;
        }
    } else {
        // too long: second walk keeps the first `cap` ids in s..t order
        atomicOr(status, ST_PATH_TRUNC);
        c = t;
        for (int32_t i = len - 1; i >= 0 && c >= 0; i--) {
            if (i < cap) path[i] = c;
            c = st_parent(__ldcg(B.state + c));
        }
    }
    return len;
}

}  // namespace ddp
