// Bidirectional one-CTA search: a forward search from s over the CSR and a
// reverse search from t over the reverse CSR, run together by one CTA until
// they meet.  No per-graph table: the plain kind keys both searches by g,
// so on graphs of small hop diameter two balls of half the radius replace
// one ball of the full radius (orders of magnitude fewer nodes on random
// digraphs); on graphs with coordinates the searches may key by g plus the
// average of two coordinate potentials (bidirectional A*, section
// "potentials" below).
//
// Labels: each node has a record of two units, forward then reverse, each a
// (g, parent) label (reverse: successor toward t).  Loading v's record gives
// the label being relaxed and the other side's label for the meeting test;
// a label changes by one compare-and-swap of its unit.  Three layouts
// (section "record layouts" below):
//   RecDense   32 bytes per node (one DRAM sector), 16-byte units
//              {epoch, g, parent, 0}.  A unit whose epoch is not the current
//              query's reads as unreached, so a slot is never reset between
//              queries: each query only advances the slot's epoch.
//   RecPair16  16 bytes per node, a 64-bit (g << 32 | parent) word per
//              direction; two nodes share a sector, which pays where node
//              ids have spatial locality.  Needs a touched log and a reset.
//   RecHash    an open-addressing table of epoch-tagged records sized to the
//              touched set instead of n.
// Entries carry their direction in the top bit of the node id: ring and far
// entries are {v | dir << 31, key}.  The ring holds one bucket; when it is
// full, entries stay in the far pile.
//
// Work distribution is the asynchronous engine's (engine_async.cuh): the
// current bucket (keys below the thresholds) is a pool that warps drain
// concurrently, chasing their own children first and spilling to the ring;
// a `pending` count in shared memory ends the bucket.  Between buckets the
// far pile is split at each advancing direction's threshold + delta.
//
// Meeting: relaxing arc (u, v) in direction dir with v's other-side label
// finite offers mu = g(u) + w + g_other(v), kept with the arc's forward-side
// tail x (u forward, v reverse) in one 64-bit atomicMin (mu << 32 | x).
// Labels only decrease, so at the end some arc (x, y) of x's forward row
// has g_f(x) + w + g_r(y) == mu, and the path is s .. x (forward parents),
// y .. t (reverse successors).
//
// Balance: each direction keeps its own threshold T_d, and a split advances
// direction d only while its open set is at most twice the other's (plus a
// little), so the search grows the smaller ball, as bidirectional Dijkstra
// expands the side with the smaller queue.  A query whose source has only
// heavy out-arcs then advances the forward side alone instead of letting the
// reverse ball grow far past the meeting radius.
//
// Stop rule (bidirectional Dijkstra; stated here for keys equal to g, and
// with 2 mu in place of mu for potential keys): after a bucket is drained,
// every node with a forward distance below the smallest open forward key a
// is final and expanded, and likewise below b in reverse.  When
// a + b >= mu, a shorter s-t path P would hold an arc (x, y) with d_s(x) < a and
// d_t(y) < b; both ends were expanded with final labels, and whichever
// expansion read the other's word second saw it final (labels are
// installed by an atomic that completes before the entry is pushed, and
// the pair is read from L2), so mu <= len(P): no shorter path exists.  An
// empty direction (a or b infinite) also ends the search.  Relaxations and
// far entries with g >= mu are dropped: no path through them is shorter.
#pragma once

#include "engine_async.cuh"

namespace ddp {

// Longest sleep (ns) of an idle warp's poll for bucket work.  With 64 ns
// polls, idle warps executed half of all instructions of a batch; backing
// off to 1 us halves the instruction count and costs no time.
#ifndef DDP_BIDIR_SPIN_CAP
#define DDP_BIDIR_SPIN_CAP 1024
#endif

// Fewest ring entries a warp claims at once (at most 32).  A warp claims
// ceil(available / warps) entries, clamped to [DDP_BIDIR_CLAIM_MIN, 32]:
// a bucket of a few hundred entries then keeps every warp busy instead of
// queueing 32-entry chunks (8 dependent rounds of arcs each) on a few.
#ifndef DDP_BIDIR_CLAIM_MIN
#define DDP_BIDIR_CLAIM_MIN 4
#endif

// Far entries a lane loads at once when a split scans the far pile.
#ifndef DDP_BIDIR_SPLIT_UNROLL
#define DDP_BIDIR_SPLIT_UNROLL 4
#endif

constexpr uint32_t DIR_BIT = 0x80000000u;
constexpr uint32_t NODE_MASK = 0x7FFFFFFFu;

struct BiQ {
    int head, tail;     // ring positions of the current bucket
    int pending;        // entries pushed to the bucket and not yet retired
    int far_cnt;        // far pushes appended this bucket
    int alt_cnt;        // split: far entries kept
    int status;
    unsigned int minkey[2];  // split: smallest key left open, per direction
    int open_dir[2];         // far entries per direction (kept by the last split + pushed since)
    int moved_dir[2];        // split: entries moved to the ring, per direction
    unsigned long long mu;   // (best s-t length << 32) | forward-side tail of its arc
};

// Reserves k ring slots (lane 0 only); returns the first position or -1 when
// the ring would overflow (the caller then sends the entries to far).
__device__ __forceinline__ int bi_ring_reserve(BiQ *sq, int k, int cap) {
    for (;;) {
        const int t = *(volatile int *)&sq->tail;
        if (t + k > cap) return -1;
        if (atomicCAS(&sq->tail, t, t + k) == t) return t;
    }
}

// Flushes a warp's staged split entries to the ring; entries past the
// ring's capacity go to the far pile `falt` instead, where they stay open
// (the stop rule reads its keys) and move at the next split.
__device__ __forceinline__ void flush_ring_or_far(uint2 *buf, int &cnt, BiQ *sq, uint2 *ring, int cap, uint2 *falt,
                                                  int64_t cap_f, SearchCtl *ctl) {
    if (cnt == 0) return;  // warp-uniform
    __syncwarp();
    const int lane = threadIdx.x & 31;
    int b = 0;
    if (lane == 0) b = atomicAdd(&sq->tail, cnt);
    b = __shfl_sync(FULL, b, 0);
    const int over = min(cnt, max(0, b + cnt - cap));
    int fb = 0;
    if (over > 0 && lane == 0) fb = atomicAdd(&sq->alt_cnt, over);
    fb = __shfl_sync(FULL, fb, 0);
    const int first_over = max(b, cap);
    for (int i = lane; i < cnt; i += 32) {
        const int pos = b + i;
        if (pos < cap) {
            ring[pos] = buf[i];
        } else {
            const int64_t p2 = (int64_t)fb + (pos - first_over);
            if (p2 < cap_f) falt[p2] = buf[i];
            else raise_err(ctl, 0, ST_OVERFLOW);
        }
    }
    __syncwarp();
    cnt = 0;
}

// Unit of node v in direction dir of a paired slot's records.
__device__ __forceinline__ uint4 *unit_ptr(unsigned long long *st, int v, uint32_t dir) {
    return reinterpret_cast<uint4 *>(st) + 2 * (size_t)v + dir;
}

// g of a unit, or INF_G when it belongs to another query.
__device__ __forceinline__ uint32_t unit_g(const uint4 &u, uint32_t ep) { return u.x == ep ? u.y : INF_G; }

__device__ __forceinline__ bool unit_eq(const uint4 &a, const uint4 &b) {
    return a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
}

// 128-bit compare-and-swap (PTX atom.cas.b128, sm_90 and later) on a
// 16-byte aligned unit; returns the unit's old value.  The first 64-bit
// operand of each pair is the low half ({x, y}), the second the high half.
__device__ __forceinline__ uint4 cas_unit(uint4 *addr, const uint4 &cmp, const uint4 &val) {
    const unsigned long long c0 = ((unsigned long long)cmp.y << 32) | cmp.x;
    const unsigned long long c1 = ((unsigned long long)cmp.w << 32) | cmp.z;
    const unsigned long long v0 = ((unsigned long long)val.y << 32) | val.x;
    const unsigned long long v1 = ((unsigned long long)val.w << 32) | val.z;
    unsigned long long o0, o1;
    asm volatile(
        "{\n\t.reg .b128 cc, vv, oo;\n\t"
        "mov.b128 cc, {%2, %3};\n\t"
        "mov.b128 vv, {%4, %5};\n\t"
        "atom.global.cas.b128 oo, [%6], cc, vv;\n\t"
        "mov.b128 {%0, %1}, oo;\n\t}"
        : "=l"(o0), "=l"(o1)
        : "l"(c0), "l"(c1), "l"(v0), "l"(v1), "l"(addr)
        : "memory");
    return make_uint4((uint32_t)o0, (uint32_t)(o0 >> 32), (uint32_t)o1, (uint32_t)(o1 >> 32));
}

// ---- record layouts ----------------------------------------------------------
// A layout maps node v to its record (two units, forward then reverse).
// find(v) returns the record or null when v has none this query; claim(v)
// returns it, creating it if needed (null when the table is full).
// keyw(v) is the forward unit's w field: 0 for dense records, the node id
// for hashed ones.

// Unit operations shared by the epoch-tagged layouts (16-byte units).
struct UnitOps16 {
    using U = uint4;
    static constexpr bool logs = false;  // no touched log: epochs retire the records
    __device__ static U ld(const U *p) { return __ldcg(p); }
    __device__ static uint32_t g(const U &u, uint32_t ep) { return unit_g(u, ep); }
    __device__ static int32_t link(const U &u) { return (int32_t)u.z; }
    __device__ static U make(uint32_t ep, uint32_t g, uint32_t parent, uint32_t keyw) {
        return make_uint4(ep, g, parent, keyw);
    }
    __device__ static U cas(U *p, const U &cmp, const U &val) { return cas_unit(p, cmp, val); }
    __device__ static bool eq(const U &a, const U &b) { return unit_eq(a, b); }
};

// One record per node, at index v (the slot's state array holds n).
struct RecDense : UnitOps16 {
    static constexpr bool hashed = false;
    unsigned long long *st;
    __device__ uint4 *find(int v, uint32_t) const { return unit_ptr(st, v, 0); }
    __device__ uint4 *claim(int v, uint32_t) const { return unit_ptr(st, v, 0); }
    __device__ uint32_t keyw(int) const { return 0u; }
};

// One 16-byte pair per node: a 64-bit (g << 32 | parent) word per direction,
// all-ones = unreached.  Two nodes share a 32-byte sector, which pays where
// node ids have spatial locality (grids in row order, points in Morton
// order): a search's neighbours are then often in the same sector.  The
// price is a touched log and a reset pass after each query (full-sector
// stores of the logged nodes' sectors).
struct RecPair16 {
    using U = unsigned long long;
    static constexpr bool hashed = false;
    static constexpr bool logs = true;
    unsigned long long *st;
    __device__ U *find(int v, uint32_t) const { return st + 2 * (size_t)v; }
    __device__ U *claim(int v, uint32_t) const { return st + 2 * (size_t)v; }
    __device__ uint32_t keyw(int) const { return 0u; }
    __device__ static U ld(const U *p) { return __ldcg(p); }
    __device__ static uint32_t g(const U &u, uint32_t) { return min(st_g(u), INF_G); }
    __device__ static int32_t link(const U &u) { return st_parent(u); }
    __device__ static U make(uint32_t, uint32_t g, uint32_t parent, uint32_t) {
        return st_make(g, (int32_t)parent);
    }
    __device__ static U cas(U *p, const U &cmp, const U &val) { return atomicCAS(p, cmp, val); }
    __device__ static bool eq(const U &a, const U &b) { return a == b; }
};

// Open addressing: 2^bits records, multiplicative hashing, linear probing.
// A record belongs to this query when its forward unit carries the epoch,
// and to node v when that unit's w field is v; records of other epochs are
// free.  A record is claimed by one 128-bit CAS of its forward unit to
// {epoch, unreached, no parent, v}; within a query records are never freed,
// so a probe for v ends at v's record or at the first free one.  This is the
// closed set of a search that touches far fewer nodes than the graph holds:
// the table is sized to the touched set, not to n.
constexpr int HASH_PROBES = 256;  // probe limit before the table counts as full
struct RecHash : UnitOps16 {
    static constexpr bool hashed = true;
    unsigned long long *st;
    uint32_t mask;
    int shift;  // 32 - bits
    __device__ uint32_t home(int v) const { return ((uint32_t)v * 0x9E3779B1u) >> shift; }
    __device__ uint4 *rec(uint32_t i) const { return unit_ptr(st, (int)i, 0); }
    __device__ uint4 *find(int v, uint32_t ep) const {
        uint32_t i = home(v);
        for (int k = 0; k < HASH_PROBES; k++, i = (i + 1) & mask) {
            const uint4 f = __ldcg(rec(i));
            if (f.x != ep) return nullptr;
            if (f.w == (uint32_t)v) return rec(i);
        }
        return nullptr;
    }
    __device__ uint4 *claim(int v, uint32_t ep) const {
        uint32_t i = home(v);
        for (int k = 0; k < HASH_PROBES; k++, i = (i + 1) & mask) {
            uint4 f = __ldcg(rec(i));
            if (f.x != ep) {
                const uint4 got = cas_unit(rec(i), f, make_uint4(ep, INF_G, 0xFFFFFFFFu, (uint32_t)v));
                if (unit_eq(got, f)) return rec(i);
                f = got;  // another thread claimed it meanwhile
            }
            if (f.x == ep && f.w == (uint32_t)v) return rec(i);
        }
        return nullptr;
    }
    __device__ uint32_t keyw(int v) const { return (uint32_t)v; }
};

// Path s..t from the meeting word; returns its length (0 when no path).
template <class Rec>
__device__ inline int32_t write_path_bidir(const DevGraph &G, const Rec &R, uint32_t ep, int32_t s, int32_t t,
                                           unsigned long long mu, int32_t *path, int32_t cap, int *status) {
    const uint32_t cost = uint32_t(mu >> 32);
    if (cost >= INF_G) return 0;
    if (s == t) {
        if (cap > 0) path[0] = s;
        return 1;
    }
    // label of node v in direction dir (unit absent: unreached) and its
    // parent / successor
    auto lab = [&](int v, uint32_t dir, int32_t *link) -> uint32_t {
        const typename Rec::U *r = R.find(v, ep);
        if (!r) {
            *link = -1;
            return INF_G;
        }
        const typename Rec::U u = Rec::ld(r + dir);
        *link = Rec::link(u);
        return Rec::g(u, ep);
    };
    const int32_t x = int32_t(uint32_t(mu));
    int32_t lk;
    const uint32_t gx = lab(x, 0, &lk);
    int32_t y = -1;
    const int r1 = row_end(G.off, G.oend, x);
    for (int k = row_begin(G.off, G.oend, x); k < r1 && y < 0; k++) {
        const uint2 a = G.oend ? __ldcg(G.arc + k) : __ldg(G.arc + k);
        if ((int)a.x < 0) continue;
        const uint32_t gr = lab((int)a.x, 1, &lk);
        if (gr < INF_G && (uint64_t)gx + a.y + gr == cost) y = (int32_t)a.x;
    }
    if (y < 0) {
        atomicOr(status, ST_TIMEOUT);  // no meeting arc: report the query failed
        return 0;
    }
    // lengths of s..x (forward parents) and y..t (reverse successors)
    int32_t lf = 0, lr = 0;
    for (int32_t c = x; c >= 0 && lf <= G.n;) {
        lf++;
        if (c == s) break;
        lab(c, 0, &lk);
        c = lk;
    }
    for (int32_t c = y; c >= 0 && lr <= G.n;) {
        lr++;
        if (c == t) break;
        lab(c, 1, &lk);
        c = lk;
    }
    const int32_t len = lf + lr;
    if (len > cap) atomicOr(status, ST_PATH_TRUNC);
    int32_t i = lf - 1;
    for (int32_t c = x; c >= 0 && i >= 0; i--) {
        if (i < cap) path[i] = c;
        lab(c, 0, &lk);
        c = lk;
    }
    i = lf;
    for (int32_t c = y; c >= 0 && i < len; i++) {
        if (i < cap) path[i] = c;
        lab(c, 1, &lk);
        c = lk;
    }
    return len;
}

// ---- potentials (bidirectional A*) ------------------------------------------
// A potential pair gives, for node v, lower bounds pt(v) <= d(v, t) and
// ps(v) <= d(s, v), each consistent (|p(u) - p(v)| <= w(u, v) on every arc).
// The searches key their buckets by K_f(v) = 2 g_f(v) + pt(v) - ps(v) and
// K_r(v) = 2 g_r(v) + ps(v) - pt(v) (the average potentials, doubled to stay
// integral): both are non-negative and grow along arcs, so every proof of
// the plain engine holds on the keys, with the stop rule a + b >= 2 mu and
// pruning of a label g at v when g + pt(v) >= mu (forward) or
// g + ps(v) >= mu (reverse).  PotNone keeps the keys equal to g.
struct PotNone {
    static constexpr bool on = false;
    __device__ uint2 at(int) const { return make_uint2(0u, 0u); }
};

// floor(rho * |v - p|) in double precision: rho (16.16 fixed point, below
// min w / length over live arcs) makes the exact real potential consistent,
// and the rounding error (far below 1) cannot push a floor difference past
// an integer weight.
struct PotEuclid {
    static constexpr bool on = true;
    const int32_t *xy;
    int2 s, t;
    double rho;  // rho_fp / 65536
    __device__ uint32_t d1(const int2 &q, const int2 &p) const {
        const double dx = (double)q.x - p.x, dy = (double)q.y - p.y;
        const double h = floor(rho * sqrt(dx * dx + dy * dy));
        return h >= (double)(INF_G - 1) ? INF_G - 1 : (uint32_t)h;
    }
    __device__ uint2 at(int v) const {  // {pt(v), ps(v)}
        const int2 q = __ldg(reinterpret_cast<const int2 *>(xy) + v);
        return make_uint2(d1(q, t), d1(q, s));
    }
};

// wmin x Manhattan distance: consistent on grids whose arcs join
// 4-neighbours (length 1) with weights >= wmin.
struct PotManhattan {
    static constexpr bool on = true;
    const int32_t *xy;
    int2 s, t;
    uint32_t wmin;
    __device__ uint32_t d1(const int2 &q, const int2 &p) const {
        const uint64_t h = (uint64_t)wmin * (uint64_t)(abs(q.x - p.x) + abs(q.y - p.y));
        return h >= INF_G - 1 ? INF_G - 1 : (uint32_t)h;
    }
    __device__ uint2 at(int v) const {
        const int2 q = __ldg(reinterpret_cast<const int2 *>(xy) + v);
        return make_uint2(d1(q, t), d1(q, s));
    }
};

// Bucket key of label g in direction dir, with pot = {pt(v), ps(v)}.
template <class Pot>
__device__ __forceinline__ uint32_t bi_key(uint32_t g, uint32_t dir, uint2 pot) {
    if constexpr (!Pot::on) {
        return g;
    } else {
        const int64_t k = 2 * (int64_t)g + (dir ? (int64_t)pot.y - (int64_t)pot.x : (int64_t)pot.x - (int64_t)pot.y);
        return k <= 0 ? 0u : k >= 0xFFFFFFFFll ? 0xFFFFFFFFu : (uint32_t)k;
    }
}

// The key every open key must stay below to matter (keys of labels at or
// above mu's bound cannot lead to a shorter path).
template <class Pot>
__device__ __forceinline__ uint64_t bi_key_bound(uint32_t mu) {
    return Pot::on ? 2 * (uint64_t)mu : (uint64_t)mu;
}

// ep: the slot's epoch for this query (never 0; units of other epochs read
// as unreached).
template <class Pot, class Rec>
__device__ SearchResult run_bidir_cta(const DevGraph &G, const SlotBufs &B, const SearchParams &P, uint32_t ep,
                                      WarpRows *wrows, BiQ *sq, const Pot &pot, const Rec &R) {
    SearchCtl *ctl = B.ctl;
    const int lane = lane_id();
    const int warp = threadIdx.x >> 5;
    const int nw = (int)(blockDim.x >> 5);
    WarpRows &wr = wrows[warp];
    uint2 *ring = B.q0;
    const int cap = (int)min(B.cap_q, (int64_t)0x3FFFFFFF);

    if (threadIdx.x == 0) {
        ctl->iters = 0;
        ctl->expanded = ctl->scanned = ctl->relaxed = 0;
        ctl->far_scanned = 0;
        sq->head = 0;
        sq->tail = 0;
        sq->pending = 0;
        sq->far_cnt = 0;
        sq->alt_cnt = 0;
        sq->status = 0;
        sq->minkey[0] = sq->minkey[1] = 0xFFFFFFFFu;
        sq->open_dir[0] = sq->open_dir[1] = 0;
        sq->moved_dir[0] = sq->moved_dir[1] = 0;
        if (P.s == P.t) {
            sq->mu = (unsigned long long)(uint32_t)P.s;  // length 0
            ctl->touched = 0;
        } else {
            sq->mu = ~0ull;
            // the endpoints' records (a fresh slot's table has room for two)
            typename Rec::U *rs = R.claim(P.s, ep);
            typename Rec::U *rt = R.claim(P.t, ep);
            rs[0] = Rec::make(ep, 0u, 0xFFFFFFFFu, R.keyw(P.s));
            rt[1] = Rec::make(ep, 0u, 0xFFFFFFFFu, 0u);
            if constexpr (Rec::logs) {
                B.touched[0] = P.s;
                B.touched[1] = P.t;
            }
            ctl->touched = 2;
            ring[0] = make_uint2((uint32_t)P.s, bi_key<Pot>(0u, 0u, pot.at(P.s)));
            ring[1] = make_uint2((uint32_t)P.t | DIR_BIT, bi_key<Pot>(0u, 1u, pot.at(P.t)));
            sq->tail = 2;
            sq->pending = 2;
        }
    }
    __syncthreads();
    if (P.s == P.t) {
        SearchResult r0;
        r0.cost = 0;
        r0.iters = 0;
        return r0;
    }

    // ring and far entries hold {v | dir << 31, key}
    uint2 *fcur = reinterpret_cast<uint2 *>(B.f0), *falt = reinterpret_cast<uint2 *>(B.f1);
    uint2 *sf2 = reinterpret_cast<uint2 *>(wr.sf);  // staged far pushes
    int64_t nfar = 0;
    // the current bucket holds keys < T0 (forward) and < T1 (reverse); lo_d
    // is a lower bound of direction d's open keys when its last advance
    // moved nothing (the next advance jumps there)
    // keys are doubled with potentials: so is the bucket width
    const uint32_t dk = Pot::on ? 2 * P.delta : P.delta;
    uint32_t T0 = sat_add(bi_key<Pot>(0u, 0u, pot.at(P.s)), dk), T1 = sat_add(bi_key<Pot>(0u, 1u, pot.at(P.t)), dk);
    uint32_t lo0 = 0, lo1 = 0;
    bool do_expand = true;
    unsigned long long n_exp = 0, n_scan = 0, n_rel = 0, n_first = 0;
    int phases = 0;
    const int64_t max_phases = 4 * (int64_t)G.n + (1 << 22);

    for (;;) {
        if (do_expand) {
            int c_f = 0, c_loc = 0, c_t = 0;  // staged far pushes, own children, touches
            int nf0 = 0, nf1 = 0;             // far pushes per direction (this lane)
            for (;;) {
                const uint32_t mu = uint32_t(*(volatile unsigned long long *)&sq->mu >> 32);
                // 1. take work: own children first, else claim from the ring
                int n = 0;
                uint2 en = make_uint2(RING_EMPTY, 0u);
                if (c_loc > 0) {
                    n = min(32, c_loc);
                    if (lane < n) en = wr.sn[c_loc - n + lane];
                    c_loc -= n;
                    __syncwarp();
                } else {
                    int h0 = 0;
                    if (lane == 0) {
                        n = -1;
                        // an idle warp backs off exponentially (up to
                        // DDP_BIDIR_SPIN_CAP ns): its polls would otherwise
                        // take issue slots from the warps that have work
                        unsigned int ns = 32;
                        for (uint32_t spins = 0;; spins++) {
                            const int h = *(volatile int *)&sq->head, t = *(volatile int *)&sq->tail;
                            if (h < t) {
                                // a small bucket is spread over the CTA's
                                // warps instead of going to the first few
                                const int k = min(t - h, min(32, max(DDP_BIDIR_CLAIM_MIN, (t - h + nw - 1) / nw)));
                                if (atomicCAS(&sq->head, h, h + k) == h) {
                                    n = k;
                                    h0 = h;
                                    break;
                                }
                                continue;
                            }
                            if (*(volatile int *)&sq->pending == 0) break;  // bucket done
                            if (spins > SPIN_LIMIT) {
                                atomicOr(&sq->status, ST_TIMEOUT);
                                break;
                            }
                            __nanosleep(ns);
                            if (ns < DDP_BIDIR_SPIN_CAP) ns <<= 1;
                        }
                    }
                    n = __shfl_sync(FULL, n, 0);
                    h0 = __shfl_sync(FULL, h0, 0);
                    if (n < 0) break;
                    if (lane < n) {
                        volatile uint2 *slot = reinterpret_cast<volatile uint2 *>(ring + h0 + lane);
                        uint2 x = make_uint2(slot->x, slot->y);
                        for (uint32_t spins = 0; x.x == RING_EMPTY; spins++) {
                            // reserved by a producer that has not written yet
                            if (spins > SPIN_LIMIT) {
                                atomicOr(&sq->status, ST_TIMEOUT);
                                break;
                            }
                            __nanosleep(32);
                            x = make_uint2(slot->x, slot->y);
                        }
                        en = x;
                        slot->x = RING_EMPTY;  // clean for the next bucket
                    }
                }
                // 2. entry stage: live entries below mu expand
                int rb = 0, deg = 0;
                uint32_t gu = 0, ud = 0;
                if (lane < n && en.x != RING_EMPTY) {
                    ud = en.x;
                    gu = en.y;  // the entry's key
                    const int u = (int)(ud & NODE_MASK);
                    const uint32_t dir = ud >> 31;
                    // the row bounds load beside the record (used only when
                    // the entry turns out current): one round trip less
                    const int r0 = dir ? row_begin(G.roff, G.roend, u) : row_begin(G.off, G.oend, u);
                    const int r1 = dir ? row_end(G.roff, G.roend, u) : row_end(G.off, G.oend, u);
                    const typename Rec::U *ru = R.find(u, ep);
                    const uint32_t gl = ru ? Rec::g(Rec::ld(ru + dir), ep) : INF_G;
                    bool cur = false;
                    if constexpr (Pot::on) {
                        // the entry is current when its key is the label's key
                        cur = gl < INF_G && bi_key<Pot>(gl, dir, pot.at(u)) == gu &&
                              (uint64_t)gu < bi_key_bound<Pot>(mu);
                        gu = gl;
                    } else {
                        cur = gl == gu && gu < mu;
                    }
                    if (cur) {
                        rb = r0;
                        deg = r1 - r0;
                        n_exp++;
                    }
                }
                int total;
                const int ex = warp_excl_scan(deg, &total);
                wr.excl[lane] = ex;
                wr.rb[lane] = rb;
                wr.bdeg[lane] = deg;
                wr.drb[lane] = 0;
                wr.g[lane] = gu;
                wr.u[lane] = (int)ud;
                __syncwarp();
                n_scan += (lane == 0) ? (unsigned long long)total : 0ull;
                for (int kb = 0; kb < total; kb += 32) {
                    const int k = kb + lane;
                    bool live = false, first = false;
                    uint2 pv = make_uint2(0u, 0u);  // {pt(v), ps(v)}
                    typename Rec::U *rv = nullptr;  // v's record
                    int v = 0;
                    uint32_t ng = 0, dir = 0;
                    uint32_t uo = 0;
                    typename Rec::U uf{}, ur{};
                    if (k < total) {
                        const int o = row_owner(wr, k);
                        uo = (uint32_t)wr.u[o];
                        dir = uo >> 31;
                        const uint2 a = row_arc(G, wr, o, k, dir == 0);
                        v = (int)a.x;
                        const uint64_t ng64 = (uint64_t)wr.g[o] + a.y;
                        live = v >= 0 && ng64 < (uint64_t)min(mu, INF_G);
                        ng = (uint32_t)ng64;
                        // a layout whose records need no claim (dense,
                        // 16-byte pairs) loads v's record beside v's
                        // potentials, before the pruning test needs them: one
                        // dependent round trip less per generation of a long
                        // chain (a record loaded for a pruned v is not used)
                        constexpr bool early = Pot::on && !Rec::hashed;
                        if constexpr (early) {
                            if (live) {
                                rv = R.claim(v, ep);
                                uf = Rec::ld(rv);
                                ur = Rec::ld(rv + 1);
                            }
                        }
                        if constexpr (Pot::on) {
                            if (live) {
                                // a path through v is at least g + the
                                // bound of the other side
                                pv = pot.at(v);
                                live = ng64 + (dir ? pv.y : pv.x) < (uint64_t)mu;
                            }
                        }
                        if (live && !early) {
                            // the node's record: both units, one sector
                            rv = R.claim(v, ep);
                            if (rv) {
                                uf = Rec::ld(rv);
                                ur = Rec::ld(rv + 1);
                            } else {
                                atomicOr(&sq->status, ST_OVERFLOW);  // the slot's table is full
                                live = false;
                            }
                        }
                    }
                    if (live) {
                        const typename Rec::U mine = dir ? ur : uf;
                        const uint32_t go = Rec::g(dir ? uf : ur, ep);
                        if (go < INF_G) {
                            // the two searches meet over this arc
                            const uint64_t c = (uint64_t)ng + go;
                            if (c < mu) {
                                const uint32_t x = dir ? (uint32_t)v : (uo & NODE_MASK);
                                atomicMin(&sq->mu, (c << 32) | x);
                            }
                        }
                        live = ng < Rec::g(mine, ep);
                        if (live) {
                            const typename Rec::U nv = Rec::make(ep, ng, uo & NODE_MASK, dir ? 0u : R.keyw(v));
                            typename Rec::U *w = rv + dir;
                            typename Rec::U c0 = mine;
                            live = false;
                            // bounded: contention on one unit comes from at
                            // most the CTA's own threads
                            for (int tries = 0;; tries++) {
                                if (tries == 4096) {
                                    atomicOr(&sq->status, ST_TIMEOUT);
                                    break;
                                }
                                const typename Rec::U got = Rec::cas(w, c0, nv);
                                if (Rec::eq(got, c0)) {
                                    live = true;
                                    first = Rec::g(c0, ep) >= INF_G;
                                    break;
                                }
                                c0 = got;
                                if (ng >= Rec::g(c0, ep)) break;
                            }
                        }
                    }
                    const uint32_t nk = bi_key<Pot>(ng, dir, pv);
                    bool to_near = live && nk < (dir ? T1 : T0);
                    bool to_far = live && !to_near;
                    if (live) n_rel++;
                    const uint32_t vd = (uint32_t)v | (dir << 31);
                    // near pushes: counted in `pending` first, then kept as
                    // this warp's own work, or spilled to the ring when full
                    const unsigned mn = __ballot_sync(FULL, to_near);
                    if (mn) {
                        const int kn = __popc(mn);
                        const int rank_in = __popc(mn & ((1u << lane) - 1u));
                        if (lane == 0) atomicAdd(&sq->pending, kn);
                        __syncwarp();
                        if (c_loc + kn <= 64) {
                            if (to_near) wr.sn[c_loc + rank_in] = make_uint2(vd, nk);
                            c_loc += kn;
                        } else {
                            int p0 = 0;
                            if (lane == 0) p0 = bi_ring_reserve(sq, kn, cap);
                            p0 = __shfl_sync(FULL, p0, 0);
                            if (p0 >= 0) {
                                if (to_near) {
                                    volatile unsigned long long *slot =
                                        reinterpret_cast<volatile unsigned long long *>(ring + p0 + rank_in);
                                    *slot = ((unsigned long long)nk << 32) | vd;
                                }
                            } else {
                                if (lane == 0) atomicSub(&sq->pending, kn);
                                to_far = to_far || to_near;
                            }
                        }
                        __syncwarp();
                    }
                    if (to_far) {
                        if (dir) nf1++;
                        else nf0++;
                    }
                    stage_push(to_far, make_uint2(vd, nk), sf2, c_f, &sq->far_cnt, fcur, nfar, B.cap_f,
                               ctl, 0);
                    if constexpr (Rec::logs) {
                        // first touches of either direction (a node may be
                        // logged twice; the reset takes it twice)
                        stage_push(first, v, wr.st, c_t, &ctl->touched, B.touched, 0, 2 * (int64_t)G.n, ctl, 0);
                    } else if (first) {
                        n_first++;
                    }
                }
                __syncwarp();
                // 3. retire the chunk (its children are already counted)
                if (lane == 0 && n > 0) atomicSub(&sq->pending, n);
                if (*(volatile int *)&sq->status & ST_TIMEOUT) break;
            }
            stage_flush(sf2, c_f, &sq->far_cnt, fcur, nfar, B.cap_f, ctl, 0);
            if constexpr (Rec::logs) stage_flush(wr.st, c_t, &ctl->touched, B.touched, 0, 2 * (int64_t)G.n, ctl, 0);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                nf0 += __shfl_xor_sync(FULL, nf0, o);
                nf1 += __shfl_xor_sync(FULL, nf1, o);
            }
            if (lane == 0) {
                if (nf0) atomicAdd(&sq->open_dir[0], nf0);
                if (nf1) atomicAdd(&sq->open_dir[1], nf1);
            }
            __syncthreads();
            phases++;
            nfar += *(volatile int *)&sq->far_cnt;
            const int st = *(volatile int *)&sq->status | *(volatile int *)&ctl->status;
            __syncthreads();
            if (threadIdx.x == 0) {
                sq->far_cnt = 0;
                sq->head = 0;
                sq->tail = 0;
                sq->pending = 0;
            }
            if (st & (ST_OVERFLOW | ST_TIMEOUT)) {
                if (threadIdx.x == 0) atomicOr(&ctl->status, st & (ST_OVERFLOW | ST_TIMEOUT));
                break;
            }
            if (nfar > B.cap_f) {
                if (threadIdx.x == 0) atomicOr(&ctl->status, ST_OVERFLOW);
                break;
            }
            __syncthreads();
        }
        // ---- split the far pile, and the stop test -------------------------
        {
            const uint32_t mu = uint32_t(*(volatile unsigned long long *)&sq->mu >> 32);
            // advance the direction(s) whose open set is not much larger
            const int o0 = *(volatile int *)&sq->open_dir[0], o1 = *(volatile int *)&sq->open_dir[1];
            const bool adv0 = (int64_t)o0 <= 2 * (int64_t)o1 + 64;
            const bool adv1 = (int64_t)o1 <= 2 * (int64_t)o0 + 64;
            const uint32_t Ts0 = adv0 ? sat_add(max(T0, lo0), dk) : T0;
            const uint32_t Ts1 = adv1 ? sat_add(max(T1, lo1), dk) : T1;
            const uint64_t kb = bi_key_bound<Pot>(mu);
            unsigned int kmin0 = 0xFFFFFFFFu, kmin1 = 0xFFFFFFFFu;
            int kp0 = 0, kp1 = 0, mv0 = 0, mv1 = 0;  // kept / moved per direction (this lane)
            int c_n = 0, c_f = 0;
            if (threadIdx.x == 0) ctl->far_scanned += (unsigned long long)nfar;
            // DDP_BIDIR_SPLIT_UNROLL entries per lane per step: their loads
            // are issued together, then consumed one by one
            constexpr int SU = DDP_BIDIR_SPLIT_UNROLL;
            for (int64_t base0 = (int64_t)warp * 32 * SU; base0 < nfar; base0 += (int64_t)nw * 32 * SU) {
                uint2 ens[SU];
#pragma unroll
                for (int k = 0; k < SU; k++) {
                    const int64_t idx = base0 + 32 * k + lane;
                    ens[k] = idx < nfar ? __ldcg(fcur + idx) : make_uint2(0u, 0u);
                }
#pragma unroll
                for (int k = 0; k < SU; k++) {
                    const int64_t idx = base0 + 32 * k + lane;
                    bool to_near = false, keep = false;
                    uint2 en = make_uint2(0u, 0u);
                    if (idx < nfar) {
                        en = ens[k];
                        if ((uint64_t)en.y < kb) {
                            const bool rev = (en.x >> 31) != 0;
                            if (en.y < (rev ? Ts1 : Ts0)) to_near = true;
                            else keep = true;
                            if (rev) {
                                kmin1 = min(kmin1, en.y);
                                if (to_near) mv1++;
                                else kp1++;
                            } else {
                                kmin0 = min(kmin0, en.y);
                                if (to_near) mv0++;
                                else kp0++;
                            }
                        }
                    }
                    {
                        const unsigned m = __ballot_sync(FULL, to_near);
                        if (to_near) wr.sn[c_n + __popc(m & ((1u << lane) - 1u))] = en;
                        c_n += __popc(m);
                        if (c_n >= 32) flush_ring_or_far(wr.sn, c_n, sq, ring, cap, falt, B.cap_f, ctl);
                    }
                    stage_push(keep, en, sf2, c_f, &sq->alt_cnt, falt, 0, B.cap_f, ctl, 0);
                }
            }
            flush_ring_or_far(wr.sn, c_n, sq, ring, cap, falt, B.cap_f, ctl);
            stage_flush(sf2, c_f, &sq->alt_cnt, falt, 0, B.cap_f, ctl, 0);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                kmin0 = min(kmin0, __shfl_xor_sync(FULL, kmin0, o));
                kmin1 = min(kmin1, __shfl_xor_sync(FULL, kmin1, o));
                kp0 += __shfl_xor_sync(FULL, kp0, o);
                kp1 += __shfl_xor_sync(FULL, kp1, o);
                mv0 += __shfl_xor_sync(FULL, mv0, o);
                mv1 += __shfl_xor_sync(FULL, mv1, o);
            }
            __syncthreads();  // every thread has read open_dir
            if (threadIdx.x == 0) sq->open_dir[0] = sq->open_dir[1] = 0;
            __syncthreads();
            if (lane == 0) {
                if (kmin0 != 0xFFFFFFFFu) atomicMin(&sq->minkey[0], kmin0);
                if (kmin1 != 0xFFFFFFFFu) atomicMin(&sq->minkey[1], kmin1);
                if (kp0) atomicAdd(&sq->open_dir[0], kp0);
                if (kp1) atomicAdd(&sq->open_dir[1], kp1);
                if (mv0) atomicAdd(&sq->moved_dir[0], mv0);
                if (mv1) atomicAdd(&sq->moved_dir[1], mv1);
            }
            __syncthreads();
            const int m = min(*(volatile int *)&sq->tail, cap);
            const int kept = *(volatile int *)&sq->alt_cnt;
            const unsigned int a = *(volatile unsigned int *)&sq->minkey[0];
            const unsigned int b = *(volatile unsigned int *)&sq->minkey[1];
            const int moved0 = *(volatile int *)&sq->moved_dir[0], moved1 = *(volatile int *)&sq->moved_dir[1];
            const uint32_t mu2 = uint32_t(*(volatile unsigned long long *)&sq->mu >> 32);
            const int st = *(volatile int *)&ctl->status;
            phases++;
            __syncthreads();
            if (threadIdx.x == 0) {
                sq->alt_cnt = 0;
                sq->minkey[0] = sq->minkey[1] = 0xFFFFFFFFu;
                sq->moved_dir[0] = sq->moved_dir[1] = 0;
                sq->head = 0;
                sq->tail = m;  // entries past the ring's capacity stayed in far
                sq->pending = m;
            }
            uint2 *t2 = fcur;
            fcur = falt;
            falt = t2;
            nfar = kept;
            if (st & (ST_OVERFLOW | ST_TIMEOUT)) break;
            if (phases > max_phases) {
                if (threadIdx.x == 0) atomicOr(&ctl->status, ST_TIMEOUT);
                break;
            }
            // an empty direction, or a + b >= mu: mu is the distance.  The
            // ring entries just moved hold the direction minima too.
            if (a == 0xFFFFFFFFu || b == 0xFFFFFFFFu || (uint64_t)a + b >= bi_key_bound<Pot>(mu2)) {
                // the ring may hold moved entries nobody will pop: clear it
                for (int i = threadIdx.x; i < m; i += blockDim.x) ring[i].x = RING_EMPTY;
                break;
            }
            // a direction that advanced without moving anything jumps to its
            // smallest open key next time
            lo0 = (adv0 && moved0 == 0) ? a : 0u;
            lo1 = (adv1 && moved1 == 0) ? b : 0u;
            T0 = Ts0;
            T1 = Ts1;
            do_expand = m > 0;
            __syncthreads();
        }
    }

    if (lane == 0 && n_scan) atomicAdd(&ctl->scanned, n_scan);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        n_exp += __shfl_xor_sync(FULL, n_exp, o);
        n_rel += __shfl_xor_sync(FULL, n_rel, o);
        n_first += __shfl_xor_sync(FULL, n_first, o);
    }
    if (lane == 0) {
        if (n_exp) atomicAdd(&ctl->expanded, n_exp);
        if (n_rel) atomicAdd(&ctl->relaxed, n_rel);
        if (n_first) atomicAdd(&ctl->touched, (int)n_first);
    }
    if (threadIdx.x == 0) ctl->iters = phases;
    __syncthreads();
    SearchResult r;
    const unsigned long long mw = *(volatile unsigned long long *)&sq->mu;
    r.cost = uint32_t(mw >> 32) >= INF_G ? 0xFFFFFFFFu : uint32_t(mw >> 32);
    r.iters = phases;
    return r;
}

}  // namespace ddp
