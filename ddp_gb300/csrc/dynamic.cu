// Dynamic A*: edge insert / delete / weight-change batches with incremental
// repair of a resident search.
//
// Replaces DA_star/DA_dyn_cpu.cu (lkoshale/DDP): per batch the reference
// builds a diff CSR on the host (insertDiff/createDiffGraph :1928-2005),
// propagates inserts over all N nodes (propogateAdd :488-556,
// insert_propagate :558-648), marks deleted arcs on the host
// (removeDelEdges :2008-2043), re-parents nodes under spin locks with an
// ancestor walk to refuse cycles (propogateDel :378-486, delete_propagate
// :650-904), repairs remaining parent cycles on the host between rounds
// (check_remove_cycle :2138-2254, 4 N-array transfers per round), optionally
// re-runs GA* (:1642-1793), and folds the diff into a new CSR on the host
// (mergeDiff :2080-2128).
//
// Here, per batch:
//   host: the batch is resolved on a host mirror of the graph with the
//         reference's semantics (deletes and weight changes hit the first
//         live u->v arc of the pre-batch graph; inserts are appended to
//         their row), and only the touched arc slots / row bounds are
//         scattered to the device.  Rows carry slack and move to the end of
//         the arc array when full, so there is no per-batch merge.
//   device, one cooperative kernel:
//     A. heuristic repair: an inserted arc can shorten hop distances to the
//        target; hops are lowered by decrease propagation over the reverse
//        graph, so h stays admissible and consistent;
//     B. invalidation: a deleted (or heavier) arc that is the parent arc of
//        its head invalidates the head's subtree of the shortest-path tree
//        (found by walking child arcs whose head names the node as parent);
//     C. re-seeding: every invalidated node takes the best g over its live
//        in-arcs from valid nodes (reads first, then writes), and is queued;
//     D. inserted (and lighter) arcs relax their head from a reached tail;
//     E. the A* resumes from the retained open list (it runs in keep mode:
//        nodes beyond f(t) stay open), and stops when no open node has
//        f < f(t).
// No parent cycles can arise: parents always point to strictly earlier
// relaxations, and invalidated subtrees are rebuilt from valid nodes only.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <type_traits>
#include <vector>

#include "engine.cuh"
#include "graph.cuh"
#include "solve.cuh"

enum { UPD_INS = 1, UPD_TREE = 2, UPD_LIGHTER = 3 };

// Arcs a repair thread loads at once when it walks a row: the loads of a
// chunk (and then of its heads' words) are in flight together instead of
// one dependent pair per arc.
#ifndef DYN_ROW_UNROLL
#define DYN_ROW_UNROLL 8
#endif

// Host mirror of a dynamic graph: rows with explicit [beg, end) and a
// capacity, forward and reverse.
struct DynMirror {
    int32_t n = 0;
    std::vector<int32_t> beg, end, cap;
    std::vector<uint2> arc;
    std::vector<int32_t> rbeg, rend, rcap;
    std::vector<uint2> rarc;
    int64_t tail = 0, rtail = 0;  // first unused slot
    std::vector<int64_t> dirty_arc, dirty_rarc;
    std::vector<int32_t> dirty_row, dirty_rrow;
    bool full = true;  // next upload sends everything
    // device side: capacities of the arc arrays and scatter staging buffers
    int64_t arc_cap = 0, rarc_cap = 0;
    // Batches applied on the device (k_apply) leave the device arrays
    // authoritative: `stale` says the host copy is behind them (it is read
    // back on demand), `dev_meta` that the device row capacities and tails
    // match the host copy (host-side changes clear it).
    bool stale = false;
    bool dev_meta = false;
    int32_t *d_cap = nullptr, *d_rcap = nullptr;  // row capacities, n each
    long long *d_tails = nullptr;                 // first unused slot: forward, reverse
    int4 *h_ops = nullptr, *d_ops = nullptr;      // one batch {flag, u, v, w}
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // DDP_TRACE: around k_apply and k_dyn
    // staging of a batch's scatter lists: pinned host memory (the copy is
    // asynchronous; the buffer is reused once the graph's stream has been
    // synchronised, which every update path does) and its device twin
    char *h_stage = nullptr;
    char *d_stage = nullptr;
    int64_t stage_cap = 0;
    ~DynMirror() {
        cudaFree(d_stage);
        cudaFreeHost(h_stage);
        cudaFree(d_cap);
        cudaFree(d_rcap);
        cudaFree(d_tails);
        cudaFreeHost(h_ops);
        cudaFree(d_ops);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
};

namespace ddp {
namespace {

// Lays rows out with slack: capacity = used + max(2, used / 4); reserves
// room for relocations at the end.
// extra: arcs still to be appended right after the layout (the reserve
// holds them even if every one moves its row)
void mirror_layout(const std::vector<int32_t> &used_b, const std::vector<int32_t> &used_e,
                   const std::vector<uint2> &src, std::vector<int32_t> &beg, std::vector<int32_t> &end,
                   std::vector<int32_t> &cap, std::vector<uint2> &dst, int64_t &tail, int64_t extra = 0) {
    const size_t n = used_b.size();
    std::vector<int32_t> nb(n), ne(n), nc(n);
    int64_t total = 0;
    for (size_t u = 0; u < n; u++) {
        int32_t live = 0;
        for (int32_t j = used_b[u]; j < used_e[u]; j++)
            if ((int32_t)src[(size_t)j].x >= 0) live++;
        nc[u] = live + std::max(2, live / 4);
        total += nc[u];
    }
    const int64_t reserve = std::max<int64_t>({(int64_t)1 << 16, total / 4, 4 * extra + 1024});
    std::vector<uint2> out((size_t)(total + reserve), make_uint2(0xFFFFFFFFu, 0u));
    int64_t k = 0;
    for (size_t u = 0; u < n; u++) {
        nb[u] = (int32_t)k;
        int64_t p = k;
        for (int32_t j = used_b[u]; j < used_e[u]; j++)
            if ((int32_t)src[(size_t)j].x >= 0) out[(size_t)p++] = src[(size_t)j];
        ne[u] = (int32_t)p;
        k += nc[u];
    }
    beg.swap(nb);
    end.swap(ne);
    cap.swap(nc);
    dst.swap(out);
    tail = k;
}

// Whether mirror_append(u) would succeed (room in the row or at the end).
bool mirror_can_append(const std::vector<int32_t> &beg, const std::vector<int32_t> &end,
                       const std::vector<int32_t> &cap, const std::vector<uint2> &arc, int64_t tail, int32_t u) {
    if (end[(size_t)u] - beg[(size_t)u] < cap[(size_t)u]) return true;
    const int32_t ncap = std::max(4, 2 * cap[(size_t)u]);
    return tail + ncap <= (int64_t)arc.size() && tail + ncap <= INT32_MAX;
}

// Appends an arc to row u; moves the row to the end when it is full.
// Returns false when the arc array has no room left (caller re-lays out).
bool mirror_append(std::vector<int32_t> &beg, std::vector<int32_t> &end, std::vector<int32_t> &cap,
                   std::vector<uint2> &arc, int64_t &tail, int32_t u, uint2 a,
                   std::vector<int64_t> &dirty, std::vector<int32_t> &drow) {
    if (end[(size_t)u] - beg[(size_t)u] >= cap[(size_t)u]) {
        const int32_t used = end[(size_t)u] - beg[(size_t)u];
        const int32_t ncap = std::max(4, 2 * cap[(size_t)u]);
        if (tail + ncap > (int64_t)arc.size() || tail + ncap > INT32_MAX) return false;
        for (int32_t j = 0; j < used; j++) {
            arc[(size_t)(tail + j)] = arc[(size_t)(beg[(size_t)u] + j)];
            dirty.push_back(tail + j);
        }
        beg[(size_t)u] = (int32_t)tail;
        end[(size_t)u] = (int32_t)(tail + used);
        cap[(size_t)u] = ncap;
        tail += ncap;
    }
    const int32_t j = end[(size_t)u]++;
    arc[(size_t)j] = a;
    dirty.push_back(j);
    drow.push_back(u);
    return true;
}

// All of a batch's graph changes in one launch: thread i writes row bound
// i of the forward rows, then of the reverse rows, then arc slot i of the
// forward arcs, then of the reverse arcs.
struct ScatterAll {
    uint2 *arc, *rarc;
    int32_t *off, *oend, *roff, *roend;
    const int4 *rows;         // kr forward then krr reverse {row, begin, end}
    const long long *slots;   // ka forward then kra reverse arc slots
    const uint2 *vals;        // their values
    int64_t ka, kra, kr, krr;
};

__global__ void k_scatter_all(ScatterAll j) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < j.kr + j.krr) {
        const int4 r = j.rows[i];
        if (i < j.kr) {
            j.off[r.x] = r.y;
            j.oend[r.x] = r.z;
        } else {
            j.roff[r.x] = r.y;
            j.roend[r.x] = r.z;
        }
        return;
    }
    i -= j.kr + j.krr;
    if (i < j.ka) j.arc[j.slots[i]] = j.vals[i];
    else if (i < j.ka + j.kra) j.rarc[j.slots[i]] = j.vals[i];
}

// ---- update batches applied on the device ----------------------------------
// One CTA resolves and applies a batch of at most APPLY_MAX updates with the
// host path's semantics (the reference's: deletes and weight changes first,
// each on the first live u->v arc of the graph as the earlier updates left
// it; inserts appended to their rows in batch order), and writes the repair
// records.  Ops are sorted by (tail, index) and inserts also by (head,
// index), so each row's updates run in batch order on one thread (the
// row's leader) while different rows run in parallel.  A first pass checks
// that the rows that outgrow their capacity fit at the arrays' tails; if
// not, nothing is changed and the status asks for the host path (which lays
// the arrays out again).
constexpr int APPLY_MAX = 4096;
constexpr int DYN_OUT_APPLY = 12;  // words of the dyn output block k_apply writes (of 16)
constexpr int APPLY_THREADS = 1024;
enum { APPLY_NO_ROOM = 1 };

struct ApplyArgs {
    const int4 *ops;  // {flag, u, v, w}, batch order
    int nops;
    int32_t n;
    uint2 *arc, *rarc;
    int32_t *off, *oend, *cap, *roff, *roend, *rcap;
    long long *tails;           // first unused slot: forward, reverse
    long long arc_lim, rarc_lim;  // slots of the laid-out arrays
    int4 *ups;                  // repair records {kind, u, v, w}
    int *res;                   // [0] records written, [1] status
    // words the repair kernel that follows wants zeroed (its counters,
    // barrier and status): cleared here instead of by separate memsets
    uint32_t *zero[3];
    int zero_n[3];
};

__device__ __forceinline__ bool apply_valid(const int4 &o, int32_t n) {
    return o.x >= 0 && o.x <= 2 && o.y >= 0 && o.y < n && o.z >= 0 && o.z < n;
}

// Capacity of a row that holds `used` slots and receives `add` more:
// unchanged when they fit, else doubled (at least 4) until they do.
__device__ __forceinline__ long long grown_cap(int32_t used, int32_t cap, int32_t add) {
    if ((long long)used + add <= cap) return cap;
    long long c = max(4LL, 2LL * cap);
    while (c < (long long)used + add) c *= 2;
    return c;
}

// Sorts a and b (P = power of two entries each) ascending, bitonic.
__device__ void apply_sort2(unsigned long long *a, unsigned long long *b, int P) {
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    unsigned long long x = a[i], y = a[l];
                    if ((x > y) == up) {
                        a[i] = y;
                        a[l] = x;
                    }
                    x = b[i];
                    y = b[l];
                    if ((x > y) == up) {
                        b[i] = y;
                        b[l] = x;
                    }
                }
            }
            __syncthreads();
        }
}

// First slot in [b, e) whose arc has head x (and weight wt when `weighted`),
// -1 if none.  Eight loads are in flight per step: the rows are scanned by
// one thread, and a dependent load per arc would make the scan a chain of
// memory latencies.
__device__ __forceinline__ int apply_find(const uint2 *arc, int b, int e, uint32_t x, uint32_t wt, bool weighted) {
    for (int j0 = b; j0 < e; j0 += 8) {
        uint2 c[8];
#pragma unroll
        for (int k = 0; k < 8; k++) c[k] = j0 + k < e ? arc[j0 + k] : make_uint2(0xFFFFFFFFu, 0u);
#pragma unroll
        for (int k = 0; k < 8; k++)
            if (c[k].x == x && (!weighted || c[k].y == wt) && j0 + k < e) return j0 + k;
    }
    return -1;
}

// Moves row r (slots [beg, end)) to a fresh region of ncap slots at the
// array's tail when ncap exceeds its capacity.
__device__ void apply_grow_row(uint2 *arc, int32_t *beg, int32_t *end, int32_t *cap, long long *tail, int r,
                               long long ncap) {
    if (ncap <= cap[r]) return;
    const int32_t b = beg[r], used = end[r] - b;
    const long long base = atomicAdd(reinterpret_cast<unsigned long long *>(tail), (unsigned long long)ncap);
    for (int32_t j = 0; j < used; j++) arc[base + j] = arc[b + j];
    beg[r] = (int32_t)base;
    end[r] = (int32_t)(base + used);
    cap[r] = (int32_t)ncap;
}

__global__ void __launch_bounds__(APPLY_THREADS) k_apply(ApplyArgs A) {
    extern __shared__ unsigned long long apply_smem[];
    __shared__ unsigned long long need[2];
    __shared__ int nrec;
    int P = 32;
    while (P < A.nops) P <<= 1;
    unsigned long long *ka = apply_smem;        // (u << 32 | i), every valid op
    unsigned long long *kb = ka + P;            // (v << 32 | i), valid inserts
    int *hit = reinterpret_cast<int *>(kb + P);  // forward slot op i hit (-1: none)
    uint32_t *w0 = reinterpret_cast<uint32_t *>(hit + P);  // that slot's weight before op i
    const unsigned long long NONE = ~0ull;
    for (int z = 0; z < 3; z++)
        for (int i = threadIdx.x; i < A.zero_n[z]; i += blockDim.x) A.zero[z][i] = 0u;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        ka[i] = kb[i] = NONE;
        if (i < A.nops) {
            const int4 o = A.ops[i];
            hit[i] = -1;
            if (apply_valid(o, A.n)) {
                ka[i] = ((unsigned long long)(uint32_t)o.y << 32) | (uint32_t)i;
                if (o.x == 1) kb[i] = ((unsigned long long)(uint32_t)o.z << 32) | (uint32_t)i;
            }
        }
    }
    if (threadIdx.x == 0) {
        need[0] = need[1] = 0;
        nrec = 0;
    }
    __syncthreads();
    apply_sort2(ka, kb, P);
    // room: every row that outgrows its capacity moves to the tail
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        for (int side = 0; side < 2; side++) {
            const unsigned long long *k = side ? kb : ka;
            if (k[p] == NONE || (p > 0 && (k[p - 1] >> 32) == (k[p] >> 32))) continue;  // not a leader
            const int r = (int)(k[p] >> 32);
            int32_t add = 0;
            for (int q = p; q < P && k[q] != NONE && (k[q] >> 32) == (unsigned long long)r; q++)
                add += A.ops[(uint32_t)k[q]].x == 1;
            const int32_t *beg = side ? A.roff : A.off, *end = side ? A.roend : A.oend,
                          *cap = side ? A.rcap : A.cap;
            const long long c = grown_cap(end[r] - beg[r], cap[r], add);
            if (c > cap[r]) atomicAdd(&need[side], (unsigned long long)c);
        }
    }
    __syncthreads();
    const bool room = A.tails[0] + (long long)need[0] <= min(A.arc_lim, (long long)INT32_MAX) &&
                      A.tails[1] + (long long)need[1] <= min(A.rarc_lim, (long long)INT32_MAX);
    if (!room) {
        if (threadIdx.x == 0) {
            A.res[0] = 0;
            A.res[1] = APPLY_NO_ROOM;
        }
        return;
    }
    // deletes and weight changes, per tail row in batch order; then each
    // arc hit is classified once, from its weight before the batch and its
    // final state (deleted or heavier: subtree check; lighter: relax)
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        if (ka[p] == NONE || (p > 0 && (ka[p - 1] >> 32) == (ka[p] >> 32))) continue;
        const int a = (int)(ka[p] >> 32);
        int q1 = p;
        while (q1 < P && ka[q1] != NONE && (int)(ka[q1] >> 32) == a) q1++;
        for (int q = p; q < q1; q++) {
            const int i = (int)(uint32_t)ka[q];
            const int4 o = A.ops[i];
            if (o.x == 1) continue;
            const int b = o.z;
            const int jf = apply_find(A.arc, A.off[a], A.oend[a], (uint32_t)b, 0u, false);
            if (jf < 0) continue;  // no such arc: nothing to do
            const uint32_t wold = A.arc[jf].y;
            hit[i] = jf;
            w0[i] = wold;
            const int jr = apply_find(A.rarc, A.roff[b], A.roend[b], (uint32_t)a, wold, true);
            if (o.x == 0) {
                A.arc[jf].x = 0xFFFFFFFFu;
                if (jr >= 0) A.rarc[jr].x = 0xFFFFFFFFu;
            } else {
                A.arc[jf].y = (uint32_t)o.w;
                if (jr >= 0) A.rarc[jr].y = (uint32_t)o.w;
            }
        }
        for (int q = p; q < q1; q++) {
            const int i = (int)(uint32_t)ka[q];
            if (hit[i] < 0) continue;
            bool first = true;
            for (int q0 = p; q0 < q && first; q0++) first = hit[(uint32_t)ka[q0]] != hit[i];
            if (!first) continue;
            const uint2 fin = A.arc[hit[i]];
            int4 rec;
            if ((int32_t)fin.x < 0 || fin.y > w0[i]) rec = make_int4(UPD_TREE, a, A.ops[i].z, 0);
            else if (fin.y < w0[i]) rec = make_int4(UPD_LIGHTER, a, A.ops[i].z, (int)fin.y);
            else continue;
            A.ups[atomicAdd(&nrec, 1)] = rec;
        }
    }
    __syncthreads();
    // inserts: forward rows (leaders of ka), reverse rows (leaders of kb)
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        for (int side = 0; side < 2; side++) {
            const unsigned long long *k = side ? kb : ka;
            if (k[p] == NONE || (p > 0 && (k[p - 1] >> 32) == (k[p] >> 32))) continue;
            const int r = (int)(k[p] >> 32);
            int q1 = p;
            int32_t add = 0;
            for (; q1 < P && k[q1] != NONE && (int)(k[q1] >> 32) == r; q1++) add += A.ops[(uint32_t)k[q1]].x == 1;
            if (!add) continue;
            uint2 *arc = side ? A.rarc : A.arc;
            int32_t *beg = side ? A.roff : A.off, *end = side ? A.roend : A.oend, *cap = side ? A.rcap : A.cap;
            apply_grow_row(arc, beg, end, cap, A.tails + side, r, grown_cap(end[r] - beg[r], cap[r], add));
            int32_t e = end[r];
            for (int q = p; q < q1; q++) {
                const int4 o = A.ops[(uint32_t)k[q]];
                if (o.x != 1) continue;
                arc[e++] = make_uint2((uint32_t)(side ? o.y : o.z), (uint32_t)o.w);
                if (!side) A.ups[atomicAdd(&nrec, 1)] = make_int4(UPD_INS, o.y, o.z, o.w);
            }
            end[r] = e;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        A.res[0] = nrec;
        A.res[1] = 0;
    }
}

struct DynArgs {
    const int4 *upd;  // {kind, u, v, w}
    int nupd;
    const int *nupd_dev;   // non-null: the record count is on the device (k_apply)
    const int *apply_res;  // non-null: k_apply's result; a failed apply skips the launch
    int32_t *inv;     // invalidated nodes (n)
    int32_t *out;     // cost, path len, status, phases, invalidated, reseeded, relaxed, hops lowered
    int32_t *path;
    int32_t path_cap;
    int heur;         // 0: h = 0, 1: hops
    int initial;      // 1: first search from the source (no repair steps)
};

// Shared counter block for the repair steps (inside SearchCtl's pad space is
// not enough, so the dynamic kernel keeps its own).
struct DynCtl {
    int cnt[4];
    int inv_n;
    int far_add;
    int hops_lowered;
    int relaxed;
    int reseeded;
    int pad[7];
    int local_nf, local_odd;  // a walk's hand-back from CTA 0 (dyn_walk)
};

__device__ __forceinline__ SlotBufs slot_of_dyn(const SlotArrays &sa) {
    SlotBufs b;
    b.state = sa.state;
    b.touched = sa.touched;
    b.hops = sa.hops;
    b.q0 = sa.q;
    b.q1 = sa.q + sa.cap_q;
    b.f0 = sa.f;
    b.f1 = sa.f + sa.cap_f;
    b.ctl = sa.ctl;
    b.cap_q = sa.cap_q;
    b.cap_f = sa.cap_f;
    return b;
}

template <class Grp>
__device__ void dyn_level_end(const Grp &grp, DynCtl *dc, int it, int &nf) {
    const int PH = (it + 1) & 3, RS = (it + 3) & 3;
    grp.sync();
    if (grp.rank() == 0) dc->cnt[RS] = 0;
    nf = *(volatile int *)&dc->cnt[PH];
}

__device__ __forceinline__ GridGroup dyn_group(GridGroup *, const SlotBufs &B) {
    return GridGroup{{&B.ctl->bar_count, &B.ctl->bar_gen}, &B.ctl->status};
}
__device__ __forceinline__ CtaGroup dyn_group(CtaGroup *, const SlotBufs &B) { return CtaGroup{&B.ctl->status}; }

// Small frontiers in the repair walks (hop lowering, invalidation): a level
// of at most DYN_LOCAL_MAX nodes gives a few dozen threads work and still
// costs a grid barrier, so CTA 0 takes the walk's next levels alone (block
// barriers, a shared counter) while the grid waits once, and hands the walk
// back when a level outgrows DYN_LOCAL_BAIL.  step(x, out, counter) expands
// frontier node x, pushing into out at atomicAdd(counter).  On entry the
// frontier is in fb (nf nodes); returns true when the walk is over, else
// leaves the remaining frontier in fb with its size in nf for the grid.
#ifndef DYN_LOCAL_MAX
#define DYN_LOCAL_MAX 256
#endif
#ifndef DYN_LOCAL_BAIL
#define DYN_LOCAL_BAIL 2048
#endif
template <class Grp, class Step>
__device__ bool dyn_walk_local(const Grp &grp, int &nf, int32_t *&fa, int32_t *&fb, DynCtl *dc, int *lcnt,
                               Step &step) {
    if constexpr (!std::is_same<Grp, GridGroup>::value) {
        return false;  // one CTA: the grid loop already uses block barriers
    } else {
        if (nf > DYN_LOCAL_MAX) return false;
        if (blockIdx.x == 0) {
            int lnf = nf, odd = 0;
            int32_t *la = fa, *lb = fb;
            for (;;) {
                int32_t *t = la;
                la = lb;
                lb = t;
                odd ^= 1;
                if (threadIdx.x == 0) *lcnt = 0;
                __syncthreads();
                for (int i = threadIdx.x; i < lnf; i += blockDim.x) step(__ldcg(la + i), lb, lcnt);
                __syncthreads();
                lnf = *(volatile int *)lcnt;
                __syncthreads();  // every thread has read the count before the next reset
                if (lnf == 0 || lnf > DYN_LOCAL_BAIL) break;
            }
            if (threadIdx.x == 0) {
                dc->local_nf = lnf;
                dc->local_odd = odd;
            }
        }
        grp.sync();  // CTA 0's pushes and hand-back are visible to every CTA
        nf = *(volatile int *)&dc->local_nf;
        if (*(volatile int *)&dc->local_odd) {
            int32_t *t = fa;  // CTA 0 swapped its buffers an odd number of times
            fa = fb;
            fb = t;
        }
        return nf == 0;
    }
}

// Grp = GridGroup: every CTA of a cooperative launch (the initial search);
// Grp = CtaGroup: one CTA (update batches: the repair and the resumed
// search touch little of the graph, and block barriers are far cheaper than
// grid barriers between the repair steps and the search phases).
template <class Grp>
__global__ void __launch_bounds__(512, 2)
    k_dyn(DevGraph G, SlotArrays sa, uint32_t *hops, SearchParams P, DynArgs A, DynCtl *dc) {
    // a batch the device could not apply leaves graph and search untouched
    // (every CTA returns here, before any barrier; the host takes over)
    if (A.apply_res && *(volatile const int *)(A.apply_res + 1) != 0) return;
    const int nupd = A.nupd_dev ? *(volatile const int *)A.nupd_dev : A.nupd;
    __shared__ WarpRows wrows[16];
    __shared__ int lsh[1];  // level counter of a walk on one CTA
    SlotBufs B = slot_of_dyn(sa);
    const Grp grp = dyn_group(static_cast<Grp *>(nullptr), B);
    const int rank = grp.rank(), size = grp.size();
    const uint32_t scale = G.wmin;
    int32_t *fa = reinterpret_cast<int32_t *>(B.q0);
    int32_t *fb = reinterpret_cast<int32_t *>(B.q1);
    uint4 *far_buf = (*(volatile int *)&B.ctl->far_sel) ? B.f1 : B.f0;  // f re-derived (keep mode)
    const int64_t far_base = *(volatile int *)&B.ctl->far_n;

    if (!A.initial) {
        int it = 0, nf = 0;
        // ---- A. heuristic repair: lower hops over inserted arcs ----------
        if (A.heur == 1) {
            for (int i = rank; i < nupd; i += size) {
                const int4 up = A.upd[i];
                if (up.x != UPD_INS) continue;
                const uint32_t hv = __ldcg(hops + up.z);
                if (hv == HOPS_INF) continue;
                const uint32_t old = atomicMin(hops + up.y, hv + 1);
                if (hv + 1 < old) {
                    const int s = atomicAdd(&dc->cnt[(it + 1) & 3], 1);
                    fb[s] = up.y;  // each lowering pushes once; bounded by 2 cap_q
                    atomicAdd(&dc->hops_lowered, 1);
                }
            }
            dyn_level_end(grp, dc, it, nf);
            it++;
            // lowers the hops of u's in-neighbours from u's; pushes each
            // lowered node once per lowering (bounded by 2 cap_q)
            auto lower_from = [&](int u, int32_t *out, int *counter) {
                const uint32_t hu = __ldcg(hops + u);
                const int b = row_begin(G.roff, G.roend, u), e = row_end(G.roff, G.roend, u);
                for (int j0 = b; j0 < e; j0 += DYN_ROW_UNROLL) {
                    int p[DYN_ROW_UNROLL];
                    uint32_t hp[DYN_ROW_UNROLL];
#pragma unroll
                    for (int k = 0; k < DYN_ROW_UNROLL; k++) p[k] = j0 + k < e ? (int)__ldcg(G.rarc + j0 + k).x : -1;
#pragma unroll
                    for (int k = 0; k < DYN_ROW_UNROLL; k++) hp[k] = p[k] >= 0 ? __ldcg(hops + p[k]) : 0u;
#pragma unroll
                    for (int k = 0; k < DYN_ROW_UNROLL; k++) {
                        if (p[k] < 0 || hu + 1 >= hp[k]) continue;
                        const uint32_t old = atomicMin(hops + p[k], hu + 1);
                        if (hu + 1 < old) {
                            const int s = atomicAdd(counter, 1);
                            if (s < 2 * B.cap_q) out[s] = p[k];
                            else atomicOr(&B.ctl->status, ST_OVERFLOW);
                            atomicAdd(&dc->hops_lowered, 1);
                        }
                    }
                }
            };
            while (nf > 0) {
                if (dyn_walk_local<Grp>(grp, nf, fa, fb, dc, lsh, lower_from)) break;
                // a push past the buffer raised an overflow: its count is not a frontier
                if (*(volatile int *)&B.ctl->status & (ST_OVERFLOW | ST_TIMEOUT)) break;
                int32_t *t = fa;
                fa = fb;
                fb = t;
                const int PH = (it + 1) & 3;
                for (int i = rank; i < nf; i += size) lower_from(__ldcg(fa + i), fb, &dc->cnt[PH]);
                dyn_level_end(grp, dc, it, nf);
                it++;
                if (*(volatile int *)&B.ctl->status & (ST_OVERFLOW | ST_TIMEOUT)) break;
            }
        }
        // ---- B. invalidate subtrees hanging off removed / heavier tree arcs
        {
            const int PH = (it + 1) & 3;
            for (int i = rank; i < nupd; i += size) {
                const int4 up = A.upd[i];
                if (up.x != UPD_TREE) continue;
                const uint64_t sv = __ldcg(B.state + up.z);
                if (st_g(sv) < INF_G && st_parent(sv) == up.y &&
                    atomicCAS(B.state + up.z, sv, ~0ull) == sv) {
                    fb[atomicAdd(&dc->cnt[PH], 1)] = up.z;
                    A.inv[atomicAdd(&dc->inv_n, 1)] = up.z;
                }
            }
            dyn_level_end(grp, dc, it, nf);
            it++;
            // invalidates x's children in the tree (nodes whose parent is x);
            // a parallel arc's second CAS fails: each node is invalidated once
            auto invalidate_from = [&](int x, int32_t *out, int *counter) {
                const int b = row_begin(G.off, G.oend, x), e = row_end(G.off, G.oend, x);
                for (int j0 = b; j0 < e; j0 += DYN_ROW_UNROLL) {
                    int y[DYN_ROW_UNROLL];
                    uint64_t sy[DYN_ROW_UNROLL];
#pragma unroll
                    for (int k = 0; k < DYN_ROW_UNROLL; k++) y[k] = j0 + k < e ? (int)__ldcg(G.arc + j0 + k).x : -1;
#pragma unroll
                    for (int k = 0; k < DYN_ROW_UNROLL; k++) sy[k] = y[k] >= 0 ? __ldcg(B.state + y[k]) : ~0ull;
#pragma unroll
                    for (int k = 0; k < DYN_ROW_UNROLL; k++) {
                        if (y[k] >= 0 && st_g(sy[k]) < INF_G && st_parent(sy[k]) == x &&
                            atomicCAS(B.state + y[k], sy[k], ~0ull) == sy[k]) {
                            out[atomicAdd(counter, 1)] = y[k];
                            A.inv[atomicAdd(&dc->inv_n, 1)] = y[k];
                        }
                    }
                }
            };
            while (nf > 0) {
                if (dyn_walk_local<Grp>(grp, nf, fa, fb, dc, lsh, invalidate_from)) break;
                if (*(volatile int *)&B.ctl->status & (ST_OVERFLOW | ST_TIMEOUT)) break;
                int32_t *t = fa;
                fa = fb;
                fb = t;
                const int PH2 = (it + 1) & 3;
                for (int i = rank; i < nf; i += size) invalidate_from(__ldcg(fa + i), fb, &dc->cnt[PH2]);
                dyn_level_end(grp, dc, it, nf);
                it++;
            }
        }
        // ---- C. re-seed invalidated nodes from valid in-neighbours --------
        const int ninv = *(volatile int *)&dc->inv_n;
        uint2 *best = B.q1;  // one {g, parent} per invalidated node
        for (int i = rank; i < ninv; i += size) {
            const int x = A.inv[i];
            uint32_t bg = INF_G;
            int bp = -1;
            const int b = row_begin(G.roff, G.roend, x), e = row_end(G.roff, G.roend, x);
            for (int j0 = b; j0 < e; j0 += DYN_ROW_UNROLL) {
                uint2 a[DYN_ROW_UNROLL];
                uint32_t gp[DYN_ROW_UNROLL];
#pragma unroll
                for (int k = 0; k < DYN_ROW_UNROLL; k++)
                    a[k] = j0 + k < e ? __ldcg(G.rarc + j0 + k) : make_uint2(0xFFFFFFFFu, 0u);
#pragma unroll
                for (int k = 0; k < DYN_ROW_UNROLL; k++)
                    gp[k] = (int)a[k].x >= 0 ? st_g(__ldcg(B.state + (int)a[k].x)) : INF_G;
#pragma unroll
                for (int k = 0; k < DYN_ROW_UNROLL; k++) {
                    if (gp[k] >= INF_G) continue;
                    const uint64_t c = (uint64_t)gp[k] + a[k].y;
                    if (c < bg) {
                        bg = (uint32_t)c;
                        bp = (int)a[k].x;
                    }
                }
            }
            best[i] = make_uint2(bg, (uint32_t)bp);
        }
        grp.sync();
        for (int i = rank; i < ninv; i += size) {
            const uint2 bv = best[i];
            if (bv.x >= INF_G) continue;
            const int x = A.inv[i];
            B.state[x] = st_make(bv.x, (int32_t)bv.y);
            const int s = atomicAdd(&dc->far_add, 1);
            if (far_base + s < B.cap_f) far_buf[far_base + s] = make_uint4((uint32_t)x, bv.x, 0u, 0u);
            else atomicOr(&B.ctl->status, ST_OVERFLOW);
            atomicAdd(&dc->reseeded, 1);
        }
        grp.sync();
        // ---- D. relax heads of inserted / lighter arcs --------------------
        for (int i = rank; i < nupd; i += size) {
            const int4 up = A.upd[i];
            if (up.x != UPD_INS && up.x != UPD_LIGHTER) continue;
            const uint32_t gu = st_g(__ldcg(B.state + up.y));
            if (gu >= INF_G) continue;
            const uint64_t ng64 = (uint64_t)gu + (uint32_t)up.w;
            if (ng64 >= INF_G) continue;
            const uint32_t ng = (uint32_t)ng64;
            uint64_t cur = __ldcg(B.state + up.z);
            while (ng < st_g(cur)) {
                const uint64_t got = atomicCAS(B.state + up.z, cur, st_make(ng, up.y));
                if (got == cur) {
                    const int s = atomicAdd(&dc->far_add, 1);
                    if (far_base + s < B.cap_f) far_buf[far_base + s] = make_uint4((uint32_t)up.z, ng, 0u, 0u);
                    else atomicOr(&B.ctl->status, ST_OVERFLOW);
                    atomicAdd(&dc->relaxed, 1);
                    break;
                }
                cur = got;
            }
        }
        grp.sync();
        if (rank == 0) B.ctl->far_n = (int)min((int64_t)B.cap_f, far_base + *(volatile int *)&dc->far_add);
        grp.sync();
    }
    // ---- E. (resume) the A* search ---------------------------------------
    SearchResult r;
    if (A.heur == 1) r = run_search(grp, G, B, HeurHops{hops, scale, HOPS_INF, 0u}, P, wrows);
    else r = run_search(grp, G, B, HeurZero{}, P, wrows);
    if (rank == 0) {
        const int st = B.ctl->status;
        A.out[0] = (st & (ST_OVERFLOW | ST_TIMEOUT)) ? -1 : (r.cost >= INF_G ? DDP_INF : (int32_t)r.cost);
        A.out[1] = (st & (ST_OVERFLOW | ST_TIMEOUT)) ? 0 : write_path(B, P.s, P.t, A.path, A.path_cap, G.n, &B.ctl->status);
        A.out[2] = B.ctl->status;
        A.out[3] = r.iters;
        A.out[4] = *(volatile int *)&dc->inv_n;
        A.out[5] = *(volatile int *)&dc->reseeded;
        A.out[6] = *(volatile int *)&dc->relaxed;
        A.out[7] = *(volatile int *)&dc->hops_lowered;
        A.out[8] = (int32_t)min((unsigned long long)INT32_MAX, (unsigned long long)B.ctl->expanded);
        A.out[9] = (int32_t)min((unsigned long long)INT32_MAX, (unsigned long long)B.ctl->scanned);
    }
}

}  // namespace
}  // namespace ddp

using namespace ddp;

struct ddp_dyn {
    ddp_graph *g = nullptr;
    int32_t s = 0, t = 0;
    int hkind = DDP_H_ZERO;
    ddp_opts o{};
    SlotArrays sa;
    uint32_t *d_hops = nullptr;
    int32_t *d_inv = nullptr;
    int32_t *d_out = nullptr;
    int32_t *d_path = nullptr;
    DynCtl *d_dc = nullptr;
    int4 *d_upd = nullptr;
    int32_t upd_cap = 0;
    uint2 *d_cold = nullptr;  // cold tier of the retained far pile
    int64_t cold_cap = 0;
    int32_t *h_out = nullptr;  // pinned copy of d_out (16 words)
    double t_wait_us = 0;      // DDP_TRACE: host wait of the last launch
    int32_t cost = DDP_INF;
    int32_t path_len = 0;
    int64_t stats[10] = {0};
    int grid = 0;      // CTAs of the initial search
    int upd_grid = 0;  // CTAs of an update batch (1: the one-CTA kernel)
};

namespace ddp {

int dyn_upload(ddp_graph *g, bool sync) {
    DynMirror *m = g->dyn;
    const int32_t n = g->n;
    m->dev_meta = false;  // row capacities and tails may have changed here
    if (m->full) {
        if ((int64_t)m->arc.size() > m->arc_cap) {
            graph_free_dev(g, g->d_arc);
            g->d_arc = nullptr;
            DDP_CUDA(cudaMalloc(&g->d_arc, sizeof(uint2) * m->arc.size()));
            m->arc_cap = (int64_t)m->arc.size();
        }
        if ((int64_t)m->rarc.size() > m->rarc_cap) {
            graph_free_dev(g, g->d_rarc);
            g->d_rarc = nullptr;
            DDP_CUDA(cudaMalloc(&g->d_rarc, sizeof(uint2) * m->rarc.size()));
            m->rarc_cap = (int64_t)m->rarc.size();
        }
        DDP_CUDA(cudaMemcpy(g->d_arc, m->arc.data(), sizeof(uint2) * m->arc.size(), cudaMemcpyHostToDevice));
        DDP_CUDA(cudaMemcpy(g->d_rarc, m->rarc.data(), sizeof(uint2) * m->rarc.size(), cudaMemcpyHostToDevice));
        DDP_CUDA(cudaMemcpy(g->d_off, m->beg.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
        DDP_CUDA(cudaMemcpy(g->d_oend, m->end.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
        DDP_CUDA(cudaMemcpy(g->d_roff, m->rbeg.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
        DDP_CUDA(cudaMemcpy(g->d_roend, m->rend.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
        m->full = false;
        g->layout_gen++;
        m->dirty_arc.clear();
        m->dirty_rarc.clear();
        m->dirty_row.clear();
        m->dirty_rrow.clear();
        return DDP_OK;
    }
    // the touched arc slots and row bounds, sorted and without repeats
    auto uniq = [](auto &x) {
        std::sort(x.begin(), x.end());
        x.erase(std::unique(x.begin(), x.end()), x.end());
    };
    uniq(m->dirty_arc);
    uniq(m->dirty_rarc);
    uniq(m->dirty_row);
    uniq(m->dirty_rrow);
    int64_t ka = (int64_t)m->dirty_arc.size(), kra = (int64_t)m->dirty_rarc.size();
    int64_t kr = (int64_t)m->dirty_row.size(), krr = (int64_t)m->dirty_rrow.size();
    int rc = DDP_OK;
    if (g->hook.fn) {
        // a serving kernel holds the GPU: each list goes to its service CTA
        // (lists it cannot take stay for the launch below)
        auto hook_arcs = [&](std::vector<int64_t> &dirty, std::vector<uint2> &src, uint2 *dst, int64_t &k) {
            if (!k || rc) return;
            std::vector<long long> sl(dirty.begin(), dirty.end());
            std::vector<uint2> val((size_t)k);
            for (int64_t i = 0; i < k; i++) val[(size_t)i] = src[(size_t)dirty[(size_t)i]];
            const int h = g->hook.fn(g->hook.ctx, 0, dst, nullptr, sl.data(), val.data(), k);
            if (h == SCATTER_LAUNCH) return;
            rc = h;
            k = 0;
        };
        auto hook_rows = [&](std::vector<int32_t> &drow, std::vector<int32_t> &bb, std::vector<int32_t> &ee,
                             int32_t *db, int32_t *de, int64_t &k) {
            if (!k || rc) return;
            std::vector<int4> r((size_t)k);
            for (int64_t i = 0; i < k; i++) {
                const int32_t x = drow[(size_t)i];
                r[(size_t)i] = make_int4(x, bb[(size_t)x], ee[(size_t)x], 0);
            }
            const int h = g->hook.fn(g->hook.ctx, 1, db, de, r.data(), nullptr, k);
            if (h == SCATTER_LAUNCH) return;
            rc = h;
            k = 0;
        };
        hook_arcs(m->dirty_arc, m->arc, g->d_arc, ka);
        hook_arcs(m->dirty_rarc, m->rarc, g->d_rarc, kra);
        hook_rows(m->dirty_row, m->beg, m->end, g->d_off, g->d_oend, kr);
        hook_rows(m->dirty_rrow, m->rbeg, m->rend, g->d_roff, g->d_roend, krr);
    }
    const int64_t total = ka + kra + kr + krr;
    if (!rc && total) {
        // one staging buffer, one copy, one kernel: rows (int4) first, then
        // arc slots (int64), then arc values (uint2)
        const size_t bytes = sizeof(int4) * (size_t)(kr + krr) + (sizeof(long long) + sizeof(uint2)) * (size_t)(ka + kra);
        if ((int64_t)bytes > m->stage_cap) {
            graph_free_dev(g, m->d_stage);
            m->d_stage = nullptr;
            cudaFreeHost(m->h_stage);
            m->h_stage = nullptr;
            m->stage_cap = 0;
            const size_t cap = std::max<size_t>(bytes * 2, 1 << 16);
            DDP_CUDA(cudaMalloc(&m->d_stage, cap));
            DDP_CUDA(cudaHostAlloc(&m->h_stage, cap, cudaHostAllocDefault));
            m->stage_cap = (int64_t)cap;
        }
        int4 *hr = reinterpret_cast<int4 *>(m->h_stage);
        for (int64_t i = 0; i < kr; i++) {
            const int32_t x = m->dirty_row[(size_t)i];
            hr[i] = make_int4(x, m->beg[(size_t)x], m->end[(size_t)x], 0);
        }
        for (int64_t i = 0; i < krr; i++) {
            const int32_t x = m->dirty_rrow[(size_t)i];
            hr[kr + i] = make_int4(x, m->rbeg[(size_t)x], m->rend[(size_t)x], 0);
        }
        long long *hs = reinterpret_cast<long long *>(hr + kr + krr);
        uint2 *hv = reinterpret_cast<uint2 *>(hs + ka + kra);
        for (int64_t i = 0; i < ka; i++) {
            hs[i] = m->dirty_arc[(size_t)i];
            hv[i] = m->arc[(size_t)m->dirty_arc[(size_t)i]];
        }
        for (int64_t i = 0; i < kra; i++) {
            hs[ka + i] = m->dirty_rarc[(size_t)i];
            hv[ka + i] = m->rarc[(size_t)m->dirty_rarc[(size_t)i]];
        }
        DDP_CUDA(cudaMemcpyAsync(m->d_stage, m->h_stage, bytes, cudaMemcpyHostToDevice, g->stream));
        ScatterAll j;
        j.arc = g->d_arc;
        j.rarc = g->d_rarc;
        j.off = g->d_off;
        j.oend = g->d_oend;
        j.roff = g->d_roff;
        j.roend = g->d_roend;
        j.rows = reinterpret_cast<const int4 *>(m->d_stage);
        j.slots = reinterpret_cast<const long long *>(j.rows + kr + krr);
        j.vals = reinterpret_cast<const uint2 *>(j.slots + ka + kra);
        j.ka = ka;
        j.kra = kra;
        j.kr = kr;
        j.krr = krr;
        k_scatter_all<<<(int)((total + 255) / 256), 256, 0, g->stream>>>(j);
        DDP_CUDA(cudaGetLastError());  // stream-ordered; synchronised below or by the caller
    }
    m->dirty_arc.clear();
    m->dirty_rarc.clear();
    m->dirty_row.clear();
    m->dirty_rrow.clear();
    // the device graph is current when this returns (other streams read it),
    // unless the caller synchronises the graph's stream itself
    if (!rc && sync) DDP_CUDA(cudaStreamSynchronize(g->stream));
    return rc;
}

// Reads the device arrays back into the host copy after batches applied on
// the device.
int dyn_mirror_sync(ddp_graph *g) {
    DynMirror *m = g->dyn;
    if (!m || !m->stale) return DDP_OK;
    const size_t n = (size_t)g->n;
    long long tails[2];
    DDP_CUDA(cudaStreamSynchronize(g->stream));
    DDP_CUDA(cudaMemcpy(m->beg.data(), g->d_off, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    DDP_CUDA(cudaMemcpy(m->end.data(), g->d_oend, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    DDP_CUDA(cudaMemcpy(m->cap.data(), m->d_cap, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    DDP_CUDA(cudaMemcpy(m->rbeg.data(), g->d_roff, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    DDP_CUDA(cudaMemcpy(m->rend.data(), g->d_roend, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    DDP_CUDA(cudaMemcpy(m->rcap.data(), m->d_rcap, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    DDP_CUDA(cudaMemcpy(tails, m->d_tails, sizeof(tails), cudaMemcpyDeviceToHost));
    m->tail = tails[0];
    m->rtail = tails[1];
    DDP_CUDA(cudaMemcpy(m->arc.data(), g->d_arc, sizeof(uint2) * (size_t)m->tail, cudaMemcpyDeviceToHost));
    DDP_CUDA(cudaMemcpy(m->rarc.data(), g->d_rarc, sizeof(uint2) * (size_t)m->rtail, cudaMemcpyDeviceToHost));
    m->stale = false;
    return DDP_OK;
}

// Applies a batch of d's graph on the device (k_apply on the graph's
// stream, no synchronisation): the repair records go to d->d_upd, their
// count to d->d_out[DYN_OUT_APPLY] and k_apply's status to the next word
// (non-zero: nothing was applied, the batch must take the host path).
// k_apply also clears the counters, barrier and status of the k_dyn launch
// that follows.  Returns 1 (nothing launched) when the batch is too large
// for one CTA or a serving kernel owns the graph's updates.
int dyn_apply_device(ddp_dyn *d, int32_t nupd, const int32_t *flag, const int32_t *u, const int32_t *v,
                     const uint32_t *w) {
    ddp_graph *g = d->g;
    DynMirror *m = g->dyn;
    if (nupd > APPLY_MAX || g->hook.fn) return 1;
    const int32_t n = g->n;
    if (!m->h_ops) {
        DDP_CUDA(cudaHostAlloc(&m->h_ops, sizeof(int4) * APPLY_MAX, cudaHostAllocDefault));
        DDP_CUDA(cudaMalloc(&m->d_ops, sizeof(int4) * APPLY_MAX));
        DDP_CUDA(cudaFuncSetAttribute(k_apply, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      24 * APPLY_MAX));
    }
    if (!m->dev_meta) {
        // the host copy is current here (only device batches make it stale,
        // and they keep the device capacities current)
        const long long tails[2] = {m->tail, m->rtail};
        DDP_CUDA(cudaMemcpyAsync(m->d_cap, m->cap.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, g->stream));
        DDP_CUDA(cudaMemcpyAsync(m->d_rcap, m->rcap.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, g->stream));
        DDP_CUDA(cudaMemcpyAsync(m->d_tails, tails, sizeof(tails), cudaMemcpyHostToDevice, g->stream));
        DDP_CUDA(cudaStreamSynchronize(g->stream));  // the sources are pageable
        m->dev_meta = true;
    }
    // the pinned staging buffer is free: every update path synchronises the
    // graph's stream before returning
    for (int32_t i = 0; i < nupd; i++) {
        m->h_ops[i] = make_int4(flag[i], u[i], v[i], (int)w[i]);
        // admissible either way: a weight that found no arc only makes
        // wmin smaller than it needs to be
        if ((flag[i] == 1 || flag[i] == 2) && u[i] >= 0 && u[i] < n && v[i] >= 0 && v[i] < n) {
            if (w[i] < g->wmin) g->wmin = w[i];
            if (w[i] > g->wmax) g->wmax = w[i];
        }
    }
    if (nupd) DDP_CUDA(cudaMemcpyAsync(m->d_ops, m->h_ops, sizeof(int4) * nupd, cudaMemcpyHostToDevice, g->stream));
    ApplyArgs A;
    A.ops = m->d_ops;
    A.nops = nupd;
    A.n = n;
    A.arc = g->d_arc;
    A.rarc = g->d_rarc;
    A.off = g->d_off;
    A.oend = g->d_oend;
    A.cap = m->d_cap;
    A.roff = g->d_roff;
    A.roend = g->d_roend;
    A.rcap = m->d_rcap;
    A.tails = m->d_tails;
    A.arc_lim = (long long)m->arc.size();
    A.rarc_lim = (long long)m->rarc.size();
    A.ups = d->d_upd;
    A.res = d->d_out + DYN_OUT_APPLY;
    A.zero[0] = reinterpret_cast<uint32_t *>(d->d_dc);
    A.zero_n[0] = (int)(sizeof(DynCtl) / sizeof(uint32_t));
    A.zero[1] = &d->sa.ctl->bar_count;  // bar_count, bar_gen
    A.zero_n[1] = 2;
    A.zero[2] = reinterpret_cast<uint32_t *>(&d->sa.ctl->status);
    A.zero_n[2] = 1;
    int P = 32;
    while (P < nupd) P <<= 1;
    const bool timed = trace_on();
    if (timed && !m->ev[0])
        for (cudaEvent_t &e : m->ev) DDP_CUDA(cudaEventCreate(&e));
    if (timed) DDP_CUDA(cudaEventRecord(m->ev[0], g->stream));
    k_apply<<<1, APPLY_THREADS, 24 * (size_t)P, g->stream>>>(A);
    DDP_CUDA(cudaGetLastError());
    if (timed) DDP_CUDA(cudaEventRecord(m->ev[1], g->stream));
    g->update_count++;  // landmark distances no longer hold
    m->stale = true;
    return DDP_OK;
}

// dres: k_apply's result (d_out + DYN_OUT_APPLY) when the batch was applied
// on the device (the record count is read there, and *apply_status receives
// its status; a failed apply leaves the search untouched), else null.
static int dyn_launch(ddp_dyn *d, int initial, int nupd, const int *dres = nullptr, int *apply_status = nullptr) {
    const bool one_cta = !initial && d->upd_grid == 1;
    ddp_graph *g = d->g;
    DevGraph G = graph_view(g);
    SearchParams P{d->s, d->t, d->o.delta > 0 ? (uint32_t)d->o.delta : std::max(1u, (g->wmin + g->wmax) / 4),
                   d->o.K, 1, initial ? 0 : 1, 1};
    // a resumed search leaves entries with g >= the last cost (f >= g)
    // unexamined until it needs them
    if (!initial && d->cost >= 0 && d->cost != DDP_INF) {
        P.cold = d->d_cold;
        P.cold_cap = d->cold_cap;
        P.cold_x = (uint32_t)d->cost;
    }
    DynArgs A;
    A.upd = d->d_upd;
    A.nupd = nupd;
    A.nupd_dev = dres;
    A.apply_res = dres;
    A.inv = d->d_inv;
    A.out = d->d_out;
    A.path = d->d_path;
    A.path_cap = g->n;
    A.heur = d->hkind == DDP_H_BFS_HOPS ? 1 : 0;
    A.initial = initial;
    // fresh barrier / counters (k_apply cleared them on the device path);
    // the far pile position survives in ctl
    if (!dres) {
        DDP_CUDA(cudaMemsetAsync(d->d_dc, 0, sizeof(DynCtl), g->stream));
        DDP_CUDA(cudaMemsetAsync(&d->sa.ctl->bar_count, 0, 2 * sizeof(unsigned int), g->stream));
        DDP_CUDA(cudaMemsetAsync(&d->sa.ctl->status, 0, sizeof(int), g->stream));
    }
    void *args[] = {&G, &d->sa, &d->d_hops, &P, &A, &d->d_dc};
    if (one_cta)
        DDP_CUDA(cudaLaunchKernel((const void *)k_dyn<CtaGroup>, dim3(1), dim3(512), args, 0, g->stream));
    else
        DDP_CUDA(cudaLaunchCooperativeKernel((const void *)k_dyn<GridGroup>, dim3(initial ? d->grid : d->upd_grid),
                                             dim3(512), args, 0, g->stream));
    if (dres && trace_on() && g->dyn->ev[2]) DDP_CUDA(cudaEventRecord(g->dyn->ev[2], g->stream));
    // out[0..9] from k_dyn; out[DYN_OUT_APPLY..+1] from k_apply (device path)
    int32_t *out = d->h_out;
    DDP_CUDA(cudaMemcpyAsync(out, d->d_out, sizeof(int32_t) * (dres ? DYN_OUT_APPLY + 2 : 10),
                             cudaMemcpyDeviceToHost, g->stream));
    const auto tw = std::chrono::steady_clock::now();
    DDP_CUDA(cudaStreamSynchronize(g->stream));
    d->t_wait_us = std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - tw).count();
    if (apply_status) *apply_status = out[DYN_OUT_APPLY + 1];
    if (dres && out[DYN_OUT_APPLY + 1]) return DDP_OK;  // nothing ran: the caller applies the batch on the host
    if (out[2] & ST_TIMEOUT) return fail(DDP_ERR_TIMEOUT, "dynamic search: barrier wait timed out");
    if (out[2] & ST_OVERFLOW) return fail(DDP_ERR_QUEUE_OVERFLOW, "dynamic search: queue overflow");
    d->cost = out[0];
    d->path_len = out[1];
    for (int i = 0; i < 10; i++) d->stats[i] = out[i];
    return DDP_OK;
}

}  // namespace ddp


namespace ddp {

// Switches g to the dynamic layout (rows with slack and explicit ends) and
// builds its host mirror, once.
int dyn_graph_prepare(ddp_graph *g) {
    if (g->dyn) return DDP_OK;
    const int32_t n = g->n;
    std::vector<int32_t> off((size_t)n + 1), roff((size_t)n + 1);
    std::vector<uint2> arc((size_t)std::max<int64_t>(g->e, 1)), rarc((size_t)std::max<int64_t>(g->e_rev, 1));
    DDP_CUDA(cudaMemcpy(off.data(), g->d_off, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost));
    DDP_CUDA(cudaMemcpy(roff.data(), g->d_roff, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost));
    if (g->e) DDP_CUDA(cudaMemcpy(arc.data(), g->d_arc, sizeof(uint2) * g->e, cudaMemcpyDeviceToHost));
    if (g->e_rev) DDP_CUDA(cudaMemcpy(rarc.data(), g->d_rarc, sizeof(uint2) * g->e_rev, cudaMemcpyDeviceToHost));
    DynMirror *m = new DynMirror();
    m->n = n;
    std::vector<int32_t> ob(off.begin(), off.end() - 1), oe(off.begin() + 1, off.end());
    std::vector<int32_t> rb(roff.begin(), roff.end() - 1), re(roff.begin() + 1, roff.end());
    mirror_layout(ob, oe, arc, m->beg, m->end, m->cap, m->arc, m->tail);
    mirror_layout(rb, re, rarc, m->rbeg, m->rend, m->rcap, m->rarc, m->rtail);
    g->dyn = m;
    g->e = (int64_t)m->arc.size();
    g->e_rev = (int64_t)m->rarc.size();
    workspace_release(g);  // the single-query workspace was sized for the old arrays
    if (!g->d_oend) DDP_CUDA(cudaMalloc(&g->d_oend, sizeof(int32_t) * n));
    if (!g->d_roend) DDP_CUDA(cudaMalloc(&g->d_roend, sizeof(int32_t) * n));
    DDP_CUDA(cudaMalloc(&m->d_cap, sizeof(int32_t) * std::max(n, 1)));
    DDP_CUDA(cudaMalloc(&m->d_rcap, sizeof(int32_t) * std::max(n, 1)));
    DDP_CUDA(cudaMalloc(&m->d_tails, sizeof(long long) * 2));
    return dyn_upload(g);
}

// Applies one update batch to the mirror with the reference's semantics and
// uploads the touched slots.  ups receives the search-relevant updates.
int dyn_graph_apply(ddp_graph *g, int32_t nupd, const int32_t *flag, const int32_t *u, const int32_t *v,
                    const uint32_t *w, std::vector<int4> &ups, bool sync) {
    const auto t0 = std::chrono::steady_clock::now();
    int rcp = dyn_graph_prepare(g);
    if (rcp) return rcp;
    rcp = dyn_mirror_sync(g);
    if (rcp) return rcp;
    g->update_count++;  // landmark distances no longer hold
    DynMirror *m = g->dyn;
    const int32_t n = g->n;
    ups.clear();
    ups.reserve((size_t)nupd);
    // forward arc slots hit by deletes and weight changes, each with its
    // weight before the batch ({slot, u, v, w0}); an arc hit more than once
    // (say lighter, then heavier than before) is classified once, from its
    // pre-batch and final state, so no repair record carries a weight the
    // arc no longer has
    std::vector<int4> hit;
    // deletes and weight changes resolve against the pre-batch graph
    // (removeDelEdges runs before mergeDiff, DA_dyn_cpu.cu:1473-1484)
    for (int32_t i = 0; i < nupd; i++) {
        if (flag[i] != 0 && flag[i] != 2) continue;
        const int32_t a = u[i], b = v[i];
        if (a < 0 || a >= n || b < 0 || b >= n) continue;
        int32_t jf = -1;
        for (int32_t j = m->beg[(size_t)a]; j < m->end[(size_t)a]; j++)
            if ((int32_t)m->arc[(size_t)j].x == b) {
                jf = j;
                break;
            }
        if (jf < 0) continue;  // no such arc: nothing to do
        int32_t jr = -1;
        for (int32_t j = m->rbeg[(size_t)b]; j < m->rend[(size_t)b]; j++)
            if ((int32_t)m->rarc[(size_t)j].x == a && m->rarc[(size_t)j].y == m->arc[(size_t)jf].y) {
                jr = j;
                break;
            }
        hit.push_back(make_int4(jf, a, b, (int)m->arc[(size_t)jf].y));
        if (flag[i] == 0) {
            m->arc[(size_t)jf].x = 0xFFFFFFFFu;
            if (jr >= 0) m->rarc[(size_t)jr].x = 0xFFFFFFFFu;
        } else {
            m->arc[(size_t)jf].y = w[i];
            if (jr >= 0) m->rarc[(size_t)jr].y = w[i];
            if (w[i] < g->wmin) g->wmin = w[i];
            if (w[i] > g->wmax) g->wmax = w[i];
        }
        m->dirty_arc.push_back(jf);
        if (jr >= 0) m->dirty_rarc.push_back(jr);
    }
    // repair records: a deleted or heavier arc may be a tree arc of its head
    // (subtree check); a lighter one relaxes its head with its final weight
    std::stable_sort(hit.begin(), hit.end(), [](const int4 &x, const int4 &y) { return x.x < y.x; });
    for (size_t k = 0; k < hit.size(); k++) {
        if (k > 0 && hit[k].x == hit[k - 1].x) continue;  // the first hit holds the pre-batch weight
        const uint2 fin = m->arc[(size_t)hit[k].x];
        const uint32_t w0 = (uint32_t)hit[k].w;
        if ((int32_t)fin.x < 0 || fin.y > w0) ups.push_back(make_int4(UPD_TREE, hit[k].y, hit[k].z, 0));
        else if (fin.y < w0) ups.push_back(make_int4(UPD_LIGHTER, hit[k].y, hit[k].z, (int)fin.y));
    }
    // inserts, appended to their rows in batch order (createDiffGraph).  When
    // a row cannot grow, everything is laid out again with fresh slack and a
    // reserve sized for the inserts still to come (larger on each retry).
    const auto t_del = std::chrono::steady_clock::now();
    int relayouts = 0;
    for (int32_t i = 0; i < nupd; i++) {
        if (flag[i] != 1) continue;
        const int32_t a = u[i], b = v[i];
        if (a < 0 || a >= n || b < 0 || b >= n) continue;
        // both directions or neither
        while (!mirror_can_append(m->beg, m->end, m->cap, m->arc, m->tail, a) ||
               !mirror_can_append(m->rbeg, m->rend, m->rcap, m->rarc, m->rtail, b)) {
            if (relayouts >= 8) return fail(DDP_ERR_OOM, "dynamic graph: no room for the insert batch");
            int64_t remaining = 0;
            for (int32_t j = i; j < nupd; j++)
                if (flag[j] == 1) remaining++;
            const int64_t extra = remaining << relayouts;
            relayouts++;
            std::vector<int32_t> b0 = m->beg, e0 = m->end, rb0 = m->rbeg, re0 = m->rend;
            std::vector<uint2> a0 = m->arc, ra0 = m->rarc;
            mirror_layout(b0, e0, a0, m->beg, m->end, m->cap, m->arc, m->tail, extra);
            mirror_layout(rb0, re0, ra0, m->rbeg, m->rend, m->rcap, m->rarc, m->rtail, extra);
            m->full = true;
            g->e = (int64_t)m->arc.size();
            g->e_rev = (int64_t)m->rarc.size();
        }
        mirror_append(m->beg, m->end, m->cap, m->arc, m->tail, a, make_uint2((uint32_t)b, w[i]), m->dirty_arc,
                      m->dirty_row);
        mirror_append(m->rbeg, m->rend, m->rcap, m->rarc, m->rtail, b, make_uint2((uint32_t)a, w[i]), m->dirty_rarc,
                      m->dirty_rrow);
        ups.push_back(make_int4(UPD_INS, a, b, (int)w[i]));
        if (w[i] < g->wmin) g->wmin = w[i];
        if (w[i] > g->wmax) g->wmax = w[i];
    }
    if (!trace_on()) return dyn_upload(g, sync);
    const auto t1 = std::chrono::steady_clock::now();
    const int rc = dyn_upload(g, sync);
    const auto t2 = std::chrono::steady_clock::now();
    trace("dyn_apply: mirror %.1f us (deletes and weight changes %.1f us, inserts %.1f us, %d re-layouts), "
          "upload %.1f us",
          std::chrono::duration<double, std::micro>(t1 - t0).count(),
          std::chrono::duration<double, std::micro>(t_del - t0).count(),
          std::chrono::duration<double, std::micro>(t1 - t_del).count(), relayouts,
          std::chrono::duration<double, std::micro>(t2 - t1).count());
    return rc;
}

}  // namespace ddp

extern "C" {

int ddp_dyn_create(ddp_graph *g, int32_t source, int32_t target, int32_t hkind, const ddp_opts *opts,
                   ddp_dyn **out) {
    if (!g || !out) return fail(DDP_ERR_INVALID, "null argument");
    *out = nullptr;
    if (source < 0 || source >= g->n || target < 0 || target >= g->n)
        return fail(DDP_ERR_INVALID, "source/target out of range");
    if (hkind != DDP_H_ZERO && hkind != DDP_H_BFS_HOPS)
        return fail(DDP_ERR_INVALID, "dynamic search heuristic must be ZERO or BFS_HOPS");
    std::lock_guard<std::mutex> lk(g->mu);
    if (g->dyn_active) return fail(DDP_ERR_INVALID, "graph already has a dynamic search");
    const int32_t n = g->n;
    ddp_dyn *d = new ddp_dyn();
    d->g = g;
    graph_ref(g);
    d->s = source;
    d->t = target;
    d->hkind = hkind;
    if (opts) d->o = *opts;
    auto bail = [&](int rc) {
        ddp_dyn_free(d);
        return rc;
    };
    int rc0 = dyn_graph_prepare(g);
    if (rc0) return bail(rc0);
    g->dyn_active = true;
    cudaError_t e1;
    int rc;
    // one search slot with generous queues (keep mode retains the open list)
    const int64_t capq = (int64_t)n + 4096, capf = 2 * (int64_t)n + 4096;
    rc = slots_alloc(d->sa, n, 1, capq, capf, false, g->stream);
    if (rc) return bail(rc);
    e1 = cudaMalloc(&d->d_inv, sizeof(int32_t) * n);
    if (e1 == cudaSuccess) e1 = cudaMalloc(&d->d_out, sizeof(int32_t) * 16);
    if (e1 == cudaSuccess) e1 = cudaHostAlloc(&d->h_out, sizeof(int32_t) * 16, cudaHostAllocDefault);
    if (e1 == cudaSuccess) e1 = cudaMalloc(&d->d_path, sizeof(int32_t) * n);
    if (e1 == cudaSuccess) e1 = cudaMalloc(&d->d_dc, sizeof(DynCtl));
    if (e1 == cudaSuccess) e1 = cudaMalloc(&d->d_hops, sizeof(uint32_t) * n);
    d->cold_cap = capf;
    if (e1 == cudaSuccess) e1 = cudaMalloc(&d->d_cold, sizeof(uint2) * (size_t)capf);
    if (e1 != cudaSuccess) return bail(cuda_fail(e1, "cudaMalloc(dynamic state)"));
    DDP_CUDA(cudaMemsetAsync(d->sa.ctl, 0, sizeof(SearchCtl), g->stream));
    int per_sm = 0, sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dyn<GridGroup>, 512, 0);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // half the SMs by default: a batch repairs little, and fewer CTAs make
    // the grid barriers between repair steps cheaper (measured best on 1M
    // nodes with 1000-update batches)
    const int coresident = std::max(1, per_sm) * std::max(1, sms);
    d->grid = std::min(coresident, std::max(1, sms / 2));
    if (d->o.grid > 0) d->grid = std::min(coresident, d->o.grid);
    // update batches: the same grid as the initial search unless opts.group
    // asks otherwise (1 = the one-CTA kernel).  On 1M nodes with 1000-update
    // batches one CTA took 7.1 ms per batch against 1.23 ms on 76 CTAs: the
    // resumed search needs the grid's parallelism more than it pays for the
    // grid barriers.
    d->upd_grid = d->o.group > 0 ? std::min(coresident, d->o.group) : d->grid;
    if (hkind == DDP_H_BFS_HOPS) {
        // exact reverse BFS from the target into the dynamic hop array
        ddp_heuristic *h = nullptr;
        g->mu.unlock();
        rc = ddp_heuristic_build(g, target, DDP_H_BFS_HOPS, nullptr, nullptr, &h);
        g->mu.lock();
        if (rc) return bail(rc);
        cudaError_t ce = cudaMemcpy(d->d_hops, heuristic_hops_ptr(h), sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice);
        ddp_heuristic_free(h);
        if (ce != cudaSuccess) return bail(cuda_fail(ce, "hops copy"));
    }
    rc = dyn_launch(d, 1, 0);
    if (rc) return bail(rc);
    *out = d;
    return DDP_OK;
}

int ddp_dyn_update(ddp_dyn *d, int32_t nupd, const int32_t *flag, const int32_t *u, const int32_t *v,
                   const uint32_t *w, int32_t *out_cost) {
    if (!d || nupd < 0 || (nupd > 0 && (!flag || !u || !v || !w)))
        return fail(DDP_ERR_INVALID, "bad update arguments");
    ddp_graph *g = d->g;
    std::lock_guard<std::mutex> lk(g->mu);
    std::vector<int4> ups;
    const auto t0 = std::chrono::steady_clock::now();
    if (nupd > d->upd_cap) {
        cudaFree(d->d_upd);
        d->d_upd = nullptr;
        DDP_CUDA(cudaMalloc(&d->d_upd, sizeof(int4) * std::max(nupd, 1)));
        d->upd_cap = nupd;
    }
    // on the device when the batch fits one CTA: k_apply, then k_dyn on the
    // same stream (one upload, one synchronisation)
    int rc = dyn_apply_device(d, nupd, flag, u, v, w);
    if (rc == DDP_OK) {
        int st = 0;
        rc = dyn_launch(d, 0, 0, d->d_out + DYN_OUT_APPLY, &st);
        if (rc) return rc;
        if (!st) {
            if (trace_on()) {
                // ev[2] was recorded after k_dyn, before dyn_launch synchronised
                float ka = 0.f, kd = 0.f;
                cudaEventElapsedTime(&ka, g->dyn->ev[0], g->dyn->ev[1]);
                cudaEventElapsedTime(&kd, g->dyn->ev[1], g->dyn->ev[2]);
                trace("dyn_update: %d updates applied on the device, %.1f us in the call (k_apply %.1f us, "
                      "k_dyn repair + search %.1f us; host waited %.1f us)",
                      nupd, std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count(),
                      1000.0 * ka, 1000.0 * kd, d->t_wait_us);
            }
            if (out_cost) *out_cost = d->cost;
            return DDP_OK;
        }
        // no room at the arrays' tails: the host lays them out again
    } else if (rc != 1) {
        return rc;
    }
    // no synchronisation after the graph scatters: k_dyn runs on the same
    // stream, and dyn_launch synchronises it before returning
    rc = dyn_graph_apply(g, nupd, flag, u, v, w, ups, false);
    if (rc) return rc;
    const auto t1 = std::chrono::steady_clock::now();
    const int32_t k = (int32_t)ups.size();
    if (k > d->upd_cap) {
        cudaFree(d->d_upd);
        d->d_upd = nullptr;
        DDP_CUDA(cudaMalloc(&d->d_upd, sizeof(int4) * std::max(k, 1)));
        d->upd_cap = k;
    }
    if (k) DDP_CUDA(cudaMemcpyAsync(d->d_upd, ups.data(), sizeof(int4) * k, cudaMemcpyHostToDevice, g->stream));
    rc = dyn_launch(d, 0, k);
    if (rc) return rc;
    if (trace_on()) {
        const auto t2 = std::chrono::steady_clock::now();
        trace("dyn_update: %d updates, host apply + scatters %.1f us, repair + search (synchronised) %.1f us",
              nupd, std::chrono::duration<double, std::micro>(t1 - t0).count(),
              std::chrono::duration<double, std::micro>(t2 - t1).count());
    }
    if (out_cost) *out_cost = d->cost;
    return DDP_OK;
}

int ddp_dyn_cost(const ddp_dyn *d, int32_t *cost) {
    if (!d || !cost) return fail(DDP_ERR_INVALID, "null argument");
    *cost = d->cost;
    return DDP_OK;
}

int ddp_dyn_path(ddp_dyn *d, int32_t *buf, int32_t cap, int32_t *len) {
    if (!d || !len) return fail(DDP_ERR_INVALID, "null argument");
    *len = d->path_len;
    if (buf && cap > 0 && d->path_len > 0)
        DDP_CUDA(cudaMemcpy(buf, d->d_path, sizeof(int32_t) * std::min(cap, d->path_len), cudaMemcpyDeviceToHost));
    return DDP_OK;
}

int ddp_dyn_stats(const ddp_dyn *d, int64_t *stats) {
    if (!d || !stats) return fail(DDP_ERR_INVALID, "null argument");
    for (int i = 0; i < 10; i++) stats[i] = d->stats[i];
    return DDP_OK;
}

int ddp_dyn_grid(const ddp_dyn *d, int32_t *search_ctas, int32_t *update_ctas) {
    if (!d || !search_ctas || !update_ctas) return fail(DDP_ERR_INVALID, "null argument");
    *search_ctas = d->grid;
    *update_ctas = d->upd_grid;
    return DDP_OK;
}

int ddp_dyn_free(ddp_dyn *d) {
    if (!d) return DDP_OK;
    slots_free(d->sa);
    cudaFree(d->d_hops);
    cudaFree(d->d_cold);
    cudaFreeHost(d->h_out);
    cudaFree(d->d_inv);
    cudaFree(d->d_out);
    cudaFree(d->d_path);
    cudaFree(d->d_dc);
    cudaFree(d->d_upd);
    // the graph keeps its dynamic layout and mirror (other searches and
    // ddp_graph_read_csr see the updated graph)
    if (d->g) {
        d->g->dyn_active = false;
        graph_unref(d->g);
    }
    delete d;
    return DDP_OK;
}

}  // extern "C"

namespace ddp {
void dyn_mirror_free(DynMirror *m) { delete m; }

// Compacted CSR of a dynamic graph (live arcs in row order), n+1 offsets.
int dyn_read_csr(ddp_graph *g, int32_t *offsets, int32_t *cols, uint32_t *weights) {
    const int rc = dyn_mirror_sync(g);
    if (rc) return rc;
    const DynMirror *m = g->dyn;
    int64_t k = 0;
    for (int32_t u = 0; u < g->n; u++) {
        if (offsets) offsets[u] = (int32_t)k;
        for (int32_t j = m->beg[(size_t)u]; j < m->end[(size_t)u]; j++) {
            const uint2 a = m->arc[(size_t)j];
            if ((int32_t)a.x < 0) continue;
            if (cols) cols[k] = (int32_t)a.x;
            if (weights) weights[k] = a.y;
            k++;
        }
    }
    if (offsets) offsets[g->n] = (int32_t)k;
    return DDP_OK;
}

int64_t dyn_live_arcs(ddp_graph *g) {
    if (dyn_mirror_sync(g)) return -1;
    const DynMirror *m = g->dyn;
    int64_t k = 0;
    for (int32_t u = 0; u < g->n; u++)
        for (int32_t j = m->beg[(size_t)u]; j < m->end[(size_t)u]; j++)
            if ((int32_t)m->arc[(size_t)j].x >= 0) k++;
    return k;
}
}  // namespace ddp

extern "C" {

// Successive shortest paths by last-arc deletion, the method of
// k-short/DA_dyn_cpu.cu:1297-1340: after each path, delete the path's last
// arc (the first live (u, v) of the graph) and let the dynamic search repair.
int ddp_kpaths(ddp_graph *g, int32_t source, int32_t target, int32_t hkind, int32_t k, int32_t restore,
               int32_t *costs, int32_t *path_buf, int64_t path_cap, int64_t *path_offsets, int32_t *found) {
    if (!g || !costs || !path_offsets || !found || k < 1 || path_cap < 0 || (path_cap > 0 && !path_buf))
        return fail(DDP_ERR_INVALID, "bad k-paths arguments");
    ddp_dyn *d = nullptr;
    int rc = ddp_dyn_create(g, source, target, hkind, nullptr, &d);
    if (rc) return rc;
    std::vector<int4> removed;  // {u, v, w}
    std::vector<int32_t> path;
    int64_t used = 0;
    int32_t nfound = 0;
    path_offsets[0] = 0;
    for (int32_t i = 0; i < k; i++) {
        const int32_t cost = d->cost;
        costs[i] = cost;
        int32_t len = 0;
        if (cost != DDP_INF) {
            rc = ddp_dyn_path(d, nullptr, 0, &len);
            if (rc) break;
            path.resize((size_t)len);
            rc = ddp_dyn_path(d, path.data(), len, &len);
            if (rc) break;
            nfound++;
        }
        for (int32_t j = 0; j < len && used + j < path_cap; j++) path_buf[used + j] = path[(size_t)j];
        used += len;
        path_offsets[i + 1] = used;
        for (int32_t r = i + 1; r < k; r++) {  // in case the loop stops here
            costs[r] = DDP_INF;
            path_offsets[r + 1] = used;
        }
        if (cost == DDP_INF || len < 2 || i == k - 1) break;
        const int32_t u = path[(size_t)len - 2], v = path[(size_t)len - 1];
        uint32_t w = 0;
        {
            std::lock_guard<std::mutex> lk(g->mu);
            rc = dyn_mirror_sync(g);
            if (rc) break;
            const DynMirror *m = g->dyn;
            for (int32_t j = m->beg[(size_t)u]; j < m->end[(size_t)u]; j++)
                if ((int32_t)m->arc[(size_t)j].x == v) {
                    w = m->arc[(size_t)j].y;
                    break;
                }
        }
        removed.push_back(make_int4(u, v, (int)w, 0));
        const int32_t fl = 0;
        const uint32_t w0 = 0;
        rc = ddp_dyn_update(d, 1, &fl, &u, &v, &w0, nullptr);
        if (rc) break;
    }
    if (!rc && restore && !removed.empty()) {
        std::vector<int32_t> fl(removed.size(), 1), uu, vv;
        std::vector<uint32_t> ww;
        for (const int4 &x : removed) {
            uu.push_back(x.x);
            vv.push_back(x.y);
            ww.push_back((uint32_t)x.z);
        }
        rc = ddp_dyn_update(d, (int32_t)removed.size(), fl.data(), uu.data(), vv.data(), ww.data(), nullptr);
    }
    ddp_dyn_free(d);
    *found = nfound;
    if (!rc && used > path_cap) return fail(DDP_ERR_INVALID, "path buffer too small (path_offsets[k] holds the size needed)");
    return rc;
}

}  // extern "C"
