// Slot arrays and kernel argument blocks of the search kernels.
#pragma once

#include "common.cuh"

namespace ddp {

struct SearchCtl;

// Memory of `nslots` independent search slots (one per concurrent query).
struct SlotArrays {
    int32_t n = 0;
    int nslots = 0;
    int words = 1;        // 64-bit state words per node: 1, or 4 (paired slots: a 32-byte record)
    int64_t sstride = 0;  // state words per slot
    int hbits = 0;        // hashed paired slots: log2 of the records per slot
    bool pair = false;    // bidirectional queue layout (one ring, 8-byte far entries)
    int64_t cap_q = 0, cap_f = 0;
    unsigned long long *state = nullptr;  // nslots x n x words
    int32_t *touched = nullptr;           // nslots x n (null for paired slots)
    uint32_t *hops = nullptr;             // nslots x n (per-target heuristic) or null
    uint2 *q = nullptr;                   // nslots x 2 x cap_q
    uint4 *f = nullptr;                   // nslots x 2 x cap_f {node, g, f, 0}
    SearchCtl *ctl = nullptr;             // nslots
    uint32_t *epoch = nullptr;            // nslots: per-query tag counter of the hop array
};

// Graph maintenance jobs of a serving launch, run by its service CTA (or by
// k_svc when no serving kernel runs).  Lists live in host memory mapped into
// the device.  Kinds (k elements):
//   SVC_SCATTER_ARCS  ((uint2 *)p0)[((long long *)p2)[i]] = ((uint2 *)p3)[i]
//   SVC_SCATTER_ROWS  r = ((int4 *)p2)[i]: ((int *)p0)[r.x] = r.y, ((int *)p1)[r.x] = r.z
//   SVC_GATHER_ARCS   j = ((long long *)p2)[i]: ((uint2 *)p0)[j] = ((uint2 *)p1)[j]
//   SVC_GATHER_INTS   j = ((int *)p2)[i]: ((int *)p0)[j] = ((int *)p1)[j]
//   SVC_COPY_WORDS    ((uint32_t *)p0)[i] = ((uint32_t *)p1)[i]
enum { SVC_SCATTER_ARCS = 0, SVC_SCATTER_ROWS, SVC_GATHER_ARCS, SVC_GATHER_INTS, SVC_COPY_WORDS };
struct SvcSub {
    int kind, pad;
    long long k;
    unsigned long long p0, p1, p2, p3;
};
constexpr int SVC_MAX_SUB = 8;
// The host fills nsub and sub[] and publishes seq; the service CTA marks
// taken = seq, runs the subs in order, and marks done = seq.
struct SvcJob {
    int seq, taken, done, nsub;
    SvcSub sub[SVC_MAX_SUB];
};

struct BatchArgs {
    const int32_t *S, *T;
    int32_t nq;
    int32_t *cost, *plen, *paths;
    int32_t path_cap;
    int32_t *qstatus;
    long long *stats, *tstart, *tend;
    int *work, *status;
    uint32_t delta;
    int32_t K;
    int64_t bfs_budget;  // capped heuristic BFS (0 = run to completion)
    int group;           // CTAs per query slot
    int sync_engine;     // 1: phase-synchronous engine even for one-CTA slots
    // serving mode (continuous batching): requests are published in host
    // memory mapped into the device; slots wait for them
    int serve;
    const volatile int *pub;    // published request count
    const volatile int *pause;  // non-zero: stop claiming, exit
    int idle_limit;             // polls (~1 us each) before a slot votes to exit
    int *idle_votes;            // slots that found no work for idle_limit polls
    int *closing;               // set once every slot voted: all slots exit
    int serve_slots;            // search slots in the launch
    volatile SvcJob *svc;       // non-null: CTA serve_slots is the service CTA
    volatile int *done;         // per request: 1 once cost/ver are written
    int32_t *ver;               // per request: graph version it ran on
    int version;
    // versioned graphs (serving): version v lives in vtab[v % nver]
    const DevGraph *vtab;         // host memory, rewritten while the kernel runs
    int nver;
    const volatile int *cur_ver;  // latest published version (host memory)
    int *inflight;                // per buffer: searches running on it (host memory)
};

// The bidirectional batch kinds, and their k_batch instances (5: no
// potential, 6: Euclidean, 7: Manhattan potentials).
inline bool is_bidir_kind(int k) {
    return k == DDP_H_BIDIR || k == DDP_H_BIDIR_EUCLID || k == DDP_H_BIDIR_MANHATTAN;
}
// 8: DDP_H_BIDIR with hashed records (DDP_OPT_HASH); 9: DDP_H_BIDIR with
// 16-byte pairs (graphs with coordinates)
constexpr bool bidir_hk(int hk) { return hk >= 5 && hk <= 9; }
constexpr bool pair16_hk(int hk) { return hk == 9; }
int kernel_hk(int hkind, bool has_xy, bool hash);
int hk_slot_kind(int hk);

// Slot kinds (bits): a per-target hop array; paired forward/reverse state;
// paired records in a hash table of 2^hbits records instead of one per node.
// SLOT_PAIR16: 16-byte pairs (one 64-bit word per direction), a touched
// log of 2n entries and the paired queue layout.
enum { SLOT_HOPS = 1, SLOT_PAIR = 2, SLOT_HASH = 4, SLOT_PAIR16 = 8 };
size_t slot_bytes(int32_t n, int64_t cap_q, int64_t cap_f, int kind, int hbits = 0);
// log2 of the hashed records per slot for an n-node graph
int hash_bits(int32_t n);
// Runs maintenance subs with ordinary launches on st (no serving kernel runs).
cudaError_t svc_run_direct(const SvcSub *subs, int nsub, cudaStream_t st);
int slots_alloc(SlotArrays &sa, int32_t n, int nslots, int64_t cap_q, int64_t cap_f, int kind,
                cudaStream_t st, int hbits = 0);
void slots_free(SlotArrays &sa);
uint32_t *heuristic_hops_ptr(const ddp_heuristic *h);
cudaError_t launch_slots(int hk, int grid, int block, bool coop, DevGraph G, SlotArrays sa, BatchArgs A,
                         cudaStream_t st);
int slots_per_sm(int hk, int block);
int device_sms();
uint32_t auto_delta(const ddp_graph *g);
uint32_t auto_delta_bidir(const ddp_graph *g);
int64_t bfs_budget(int32_t n);

}  // namespace ddp
