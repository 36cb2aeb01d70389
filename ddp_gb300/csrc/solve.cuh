// Slot arrays and kernel argument blocks of the search kernels.
#pragma once

#include "common.cuh"

namespace ddp {

struct SearchCtl;

// Memory of `nslots` independent search slots (one per concurrent query).
struct SlotArrays {
    int32_t n = 0;
    int nslots = 0;
    int64_t cap_q = 0, cap_f = 0;
    unsigned long long *state = nullptr;  // nslots x n
    int32_t *touched = nullptr;           // nslots x n
    uint32_t *hops = nullptr;             // nslots x n (per-target heuristic) or null
    uint2 *q = nullptr;                   // nslots x 2 x cap_q
    uint2 *f = nullptr;                   // nslots x 2 x cap_f
    SearchCtl *ctl = nullptr;             // nslots
    uint32_t *epoch = nullptr;            // nslots: per-query tag counter of the hop array
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
    int idle_limit;             // polls (~1 us each) before an idle slot exits
    volatile int *done;         // per request: 1 once cost/ver are written
    int32_t *ver;               // per request: graph version it ran on
    int version;
};

size_t slot_bytes(int32_t n, int64_t cap_q, int64_t cap_f, bool hops);
int slots_alloc(SlotArrays &sa, int32_t n, int nslots, int64_t cap_q, int64_t cap_f, bool hops,
                cudaStream_t st);
void slots_free(SlotArrays &sa);
uint32_t *heuristic_hops_ptr(const ddp_heuristic *h);
cudaError_t launch_slots(int hkind, int grid, int block, bool coop, DevGraph G, SlotArrays sa, BatchArgs A,
                         cudaStream_t st);
int slots_per_sm(int hkind, int block);
int device_sms();
uint32_t auto_delta(const ddp_graph *g);
int64_t bfs_budget(int32_t n);

}  // namespace ddp
