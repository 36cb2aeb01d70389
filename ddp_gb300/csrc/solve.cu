// Heuristic build, single-query GA* and the batched multi-query engine.
//
// Replaces GA_star/bfs_hx.cu (heuristic program), LIB/include/a_star.cu
// (GPU_A_Star host loop of 5 kernels + ~12 host<->device crossings per
// iteration) with one cooperative kernel per query (single form) or one
// persistent kernel per batch (batched form).
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "engine.cuh"
#include "engine_async.cuh"
#include "engine_bidir.cuh"

#include <type_traits>
#include "graph.cuh"
#include "solve.cuh"

namespace ddp {

constexpr int MAX_WARPS = 16;  // blocks of at most 512 threads

// ---- slot arrays -------------------------------------------------------------
// Paired (bidirectional) slots hold a 32-byte record per node (two
// epoch-tagged units), no touched log, one ring and 8-byte far entries;
// the others one 8-byte state word per node, a touched log, two queues and
// 16-byte far entries.
// Hashed records per slot: a quarter of the nodes, between 2^16 and 2^20
// (a C4 query touches about 35k nodes; the table stays under 15 % full).
int hash_bits(int32_t n) {
    int b = 16;
    while (b < 20 && ((int64_t)1 << b) < (int64_t)n / 4) b++;
    return b;
}

size_t slot_bytes(int32_t n, int64_t cap_q, int64_t cap_f, int kind, int hbits) {
    const bool p16 = (kind & SLOT_PAIR16) != 0;
    const bool pair = (kind & SLOT_PAIR) != 0 || p16;
    const size_t recs = (kind & SLOT_HASH) ? ((size_t)1 << hbits) : (size_t)n;
    size_t b = 0;
    if (p16) {
        b += sizeof(unsigned long long) * 2 * (size_t)((n + 1) & ~1);  // state (an even node count)
        b += sizeof(int32_t) * 2 * (size_t)n;                          // touched (both directions)
    } else {
        b += sizeof(unsigned long long) * recs * (pair ? 4 : 1);  // state
        if (!pair) b += sizeof(int32_t) * (size_t)n;              // touched
    }
    if (kind & SLOT_HOPS) b += sizeof(uint32_t) * (size_t)n;
    b += (pair ? 1 : 2) * sizeof(uint2) * (size_t)cap_q;
    b += 2 * (pair ? sizeof(uint2) : sizeof(uint4)) * (size_t)cap_f;
    b += sizeof(SearchCtl);
    return b;
}

int slots_alloc(SlotArrays &sa, int32_t n, int nslots, int64_t cap_q, int64_t cap_f, int kind,
                cudaStream_t st, int hbits) {
    sa = SlotArrays();
    const bool hops = (kind & SLOT_HOPS) != 0;
    const bool p16 = (kind & SLOT_PAIR16) != 0;
    const bool pair = (kind & SLOT_PAIR) != 0 || p16;
    sa.n = n;
    sa.pair = pair;
    sa.words = p16 ? 2 : pair ? 4 : 1;
    sa.hbits = (kind & SLOT_HASH) ? hbits : 0;
    // 16-byte pairs: an even node count per slot, so that every slot (and
    // every node's 32-byte sector) starts on a 32-byte boundary
    sa.sstride = p16 ? 2 * (int64_t)((n + 1) & ~1)
                     : (sa.hbits ? ((int64_t)1 << sa.hbits) : (int64_t)n) * sa.words;
    sa.nslots = nslots;
    sa.cap_q = cap_q;
    sa.cap_f = cap_f;
    const size_t S = (size_t)nslots;
    DDP_CUDA(cudaMalloc(&sa.state, sizeof(unsigned long long) * (size_t)sa.sstride * S));
    if (!pair || p16) DDP_CUDA(cudaMalloc(&sa.touched, sizeof(int32_t) * (size_t)n * (p16 ? 2 : 1) * S));
    if (hops) DDP_CUDA(cudaMalloc(&sa.hops, sizeof(uint32_t) * (size_t)n * S));
    const size_t qn = pair ? 1 : 2;                             // rings per slot
    const size_t fb = pair ? sizeof(uint2) : sizeof(uint4);     // bytes per far entry
    DDP_CUDA(cudaMalloc(&sa.q, sizeof(uint2) * (size_t)cap_q * qn * S));
    DDP_CUDA(cudaMalloc(&sa.f, fb * (size_t)cap_f * 2 * S));
    DDP_CUDA(cudaMalloc(&sa.ctl, sizeof(SearchCtl) * S));
    DDP_CUDA(cudaMalloc(&sa.epoch, sizeof(uint32_t) * S));
    DDP_CUDA(cudaMemsetAsync(sa.epoch, 0, sizeof(uint32_t) * S, st));
    // unreached: all-ones words, or (epoch-tagged records) epoch 0, which
    // no query uses
    DDP_CUDA(cudaMemsetAsync(sa.state, (pair && !p16) ? 0 : 0xFF,
                             sizeof(unsigned long long) * (size_t)sa.sstride * S, st));
    if (hops) DDP_CUDA(cudaMemsetAsync(sa.hops, 0, sizeof(uint32_t) * (size_t)n * S, st));
    // queue slots start as "empty" (the asynchronous engine's ring marker)
    DDP_CUDA(cudaMemsetAsync(sa.q, 0xFF, sizeof(uint2) * (size_t)cap_q * qn * S, st));
    DDP_CUDA(cudaMemsetAsync(sa.ctl, 0, sizeof(SearchCtl) * S, st));
    return DDP_OK;
}

void slots_free(SlotArrays &sa) {
    cudaFree(sa.state);
    cudaFree(sa.touched);
    cudaFree(sa.hops);
    cudaFree(sa.q);
    cudaFree(sa.f);
    cudaFree(sa.ctl);
    cudaFree(sa.epoch);
    sa = SlotArrays();
}

__device__ __forceinline__ SlotBufs slot_of(const SlotArrays &sa, int i) {
    SlotBufs b;
    const size_t n = (size_t)sa.n;
    b.state = sa.state + (size_t)sa.sstride * i;
    b.touched = sa.touched ? sa.touched + n * (sa.words == 2 ? 2 : 1) * i : nullptr;
    b.hops = sa.hops ? sa.hops + n * i : nullptr;
    if (sa.pair) {
        // paired slots: one ring; far piles of 8-byte entries (the uint4
        // pointers only carry the address)
        b.q0 = sa.q + (size_t)sa.cap_q * i;
        b.q1 = b.q0;
        uint2 *fb = reinterpret_cast<uint2 *>(sa.f) + (size_t)sa.cap_f * 2 * i;
        b.f0 = reinterpret_cast<uint4 *>(fb);
        b.f1 = reinterpret_cast<uint4 *>(fb + sa.cap_f);
    } else {
        b.q0 = sa.q + (size_t)sa.cap_q * 2 * i;
        b.q1 = b.q0 + sa.cap_q;
        b.f0 = sa.f + (size_t)sa.cap_f * 2 * i;
        b.f1 = b.f0 + sa.cap_f;
    }
    b.ctl = sa.ctl + i;
    b.cap_q = sa.cap_q;
    b.cap_f = sa.cap_f;
    b.swords = sa.sstride;
    b.hbits = sa.hbits;
    return b;
}

__device__ __forceinline__ long long global_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---- kernels -------------------------------------------------------------------
// Clears the state words a finished search touched (slot 0 .. nslots-1).
__global__ void k_reset_touched(SlotArrays sa) {
    SlotBufs B = slot_of(sa, blockIdx.y);
    const int cnt = B.ctl->touched;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
        B.state[B.touched[i]] = ~0ull;
}

// Single-query reverse BFS (heuristic build) over the whole grid.
__global__ void __launch_bounds__(512) k_bfs_single(DevGraph G, SlotArrays sa, uint32_t *hops,
                                                    int32_t t, long long budget) {
    __shared__ WarpRows wrows[MAX_WARPS];
    SlotBufs B = slot_of(sa, 0);
    B.hops = hops;
    GridGroup grp{{&B.ctl->bar_count, &B.ctl->bar_gen}, &B.ctl->status};
    // q0 is the ring of the asynchronous engine: keep it clean
    const uint32_t cap = run_bfs_hops(grp, G, B, t, wrows, 0u, (int64_t)budget, true);
    if (grp.rank() == 0) B.ctl->hcap = cap;
}

// Single-query GA* over the whole grid (cooperative launch).
template <class Heur>
__global__ void __launch_bounds__(512, 2)
    k_solve_single(DevGraph G, SlotArrays sa, Heur H, SearchParams P, int32_t *out, int32_t *path,
                   int32_t path_cap) {
    __shared__ WarpRows wrows[MAX_WARPS];
    SlotBufs B = slot_of(sa, 0);
    GridGroup grp{{&B.ctl->bar_count, &B.ctl->bar_gen}, &B.ctl->status};
    SearchResult r = run_search(grp, G, B, H, P, wrows);
    if (grp.rank() == 0) {
        out[0] = r.cost >= INF_G ? DDP_INF : (int32_t)r.cost;
        out[1] = write_path(B, P.s, P.t, path, path_cap, G.n, &B.ctl->status);
        out[2] = B.ctl->status;
        out[3] = r.iters;
    }
}

// ---- landmarks (ALT heuristic) ---------------------------------------------

// Exhaustive search from P.s (P.t < 0) over the whole grid; dist[v] = d(s, v)
// or LM_UNREACHED.
__global__ void __launch_bounds__(512, 2)
    k_sssp(DevGraph G, SlotArrays sa, SearchParams P, int32_t *dist, int32_t *out) {
    __shared__ WarpRows wrows[MAX_WARPS];
    SlotBufs B = slot_of(sa, 0);
    GridGroup grp{{&B.ctl->bar_count, &B.ctl->bar_gen}, &B.ctl->status};
    run_search(grp, G, B, HeurZero{}, P, wrows);  // ends on a group barrier
    for (int64_t v = grp.rank(); v < G.n; v += grp.size()) {
        const uint32_t gv = st_g(__ldcg(B.state + v));
        dist[v] = gv >= INF_G ? LM_UNREACHED : (int32_t)gv;
    }
    if (grp.rank() == 0) out[2] = B.ctl->status;
}

// tab row v, column c <- dist[v]
__global__ void k_put_column(int32_t *tab, int32_t width, int32_t c, const int32_t *dist, int32_t n) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n) tab[v * width + c] = dist[v];
}

// 16- or 8-bit table entries from exhaustive-search distances: floor(d / scale)
template <class E>
__global__ void k_pack_landmarks(const int32_t *tab32, E *tab, int64_t count, int32_t scale) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t d = tab32[i];
        tab[i] = d == LM_UNREACHED ? (E)~(E)0 : (E)(d / scale);
    }
}

// h(v) of the landmark heuristic for target t (INF_G -> -1)
__global__ void k_alt_values(DevGraph G, int32_t t, int32_t *out) {
    const int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= G.n) return;
    const uint32_t h = HeurALT{G.lm, G.lm_L, G.lm_scale, t, G.lm_bits}(v);
    out[v] = h >= INF_G ? -1 : (int32_t)h;
}

// Batched GA*: each slot is a group of CTAs (one CTA, or `group` CTAs of a
// cooperative launch) that claims queries from a shared counter, so groups
// finishing short searches take the next query (dynamic load balance over
// uneven depths).  Fewer, wider groups keep fewer per-query state arrays live
// at once, which lets them stay resident in L2.
// One search of the slot: the asynchronous single-CTA engine when the slot is
// one CTA (and the caller did not ask for the phase-synchronous one), else
// the phase-synchronous group engine.
template <class Grp, class Heur>
__device__ SearchResult slot_search(const Grp &grp, const DevGraph &G, const SlotBufs &B, const Heur &H,
                                    const SearchParams &P, WarpRows *wrows, CtaQ *sq, bool async) {
    // throughput (many slots): load + CAS on improving arcs only, unless
    // the heuristic is cheap enough that one atomic per arc wins
    if (async) return run_search_cta<Heur, heur_cheap<Heur>::value>(G, B, H, P, wrows, sq);
    return run_search(grp, G, B, H, P, wrows);
}

template <int HK, class Grp>
__device__ void batch_loop(const Grp &grp, const DevGraph &G0, const SlotBufs &B, const BatchArgs &A,
                           uint32_t *epoch, WarpRows *wrows, CtaQ *sq, BiQ *bq, bool async) {
    SearchCtl *ctl = B.ctl;
    long long t0 = 0;
    int vbuf = -1;  // versioned serving: graph buffer the current search holds
    for (;;) {
        if (grp.rank() == 0) {
            int q;
            if (A.serve) {
                // claim the next published request.  A slot that finds no
                // work for idle_limit polls votes to exit and keeps polling
                // (new work takes its vote back); when every slot has voted,
                // all of them leave together, so the launch never shrinks
                // to a few slots while requests keep coming.
                q = -1;
                bool voted = false;
                // a slot that voted waits for the others at most ~500 idle
                // periods (slots that never became resident cannot vote)
                for (int idle = 0, waited = 0;;) {
                    if (*A.pause || *(volatile int *)A.closing) break;
                    const int p = *A.pub;
                    const int c = *(volatile int *)A.work;
                    if (c < p) {
                        if (voted) {
                            atomicSub(A.idle_votes, 1);
                            voted = false;
                        }
                        if (atomicCAS(A.work, c, c + 1) == c) {
                            q = c;
                            break;
                        }
                        continue;
                    }
                    if (idle < A.idle_limit) {
                        idle++;
                    } else if (!voted) {
                        atomicAdd(A.idle_votes, 1);
                        voted = true;
                    } else if (*(volatile int *)A.idle_votes >= A.serve_slots) {
                        atomicExch(A.closing, 1);
                        break;
                    } else if (++waited > 500 * A.idle_limit) {
                        break;
                    }
                    __nanosleep(1000);
                }
                __threadfence_system();  // requests were written before pub
                if (q < 0) q = A.nq;     // exit marker
                if (q < A.nq && A.vtab) {
                    // pin the latest graph version: count this search on its
                    // buffer, then re-read the version.  Buffer v % K is only
                    // rewritten for version v + K, after version v + K - 1 was
                    // published and the buffer's count was seen at zero, so
                    // the pin holds while fewer than K - 1 versions appeared
                    // in between.  A pin that keeps failing fails the request
                    // (cost -1: the host re-runs it).
                    ctl->cur_ver = -1;
                    for (uint32_t spins = 0; spins < 4096; spins++) {
                        const int v = *A.cur_ver;
                        const int b = v % A.nver;
                        atomicAdd(A.inflight + b, 1);
                        __threadfence_system();
                        if (*A.cur_ver - v < A.nver - 1) {
                            ctl->cur_ver = v;
                            vbuf = b;
                            break;
                        }
                        atomicSub(A.inflight + b, 1);
                    }
                }
            } else {
                q = atomicAdd(A.work, 1);
            }
            ctl->cur_q = q;
            ctl->status = 0;
            ctl->bfs_reached = 0;
            ctl->bfs_scanned = 0;
            if (HK == 1) {
                // per-query tag: the slot's hop array needs no clearing
                uint32_t ep = (*epoch + 1) & 0xFFFFFFu;
                if (ep == 0) ep = 1;  // tag 0 is never used (arrays start zeroed)
                *epoch = ep;
                ctl->tag = ep << 8;
            }
            if (bidir_hk(HK) && !pair16_hk(HK)) {
                // per-query epoch of the slot's records (0 = never used);
                // tag 0 asks for the records to be cleared once the
                // 32-bit epoch wraps
                const uint32_t ep = *epoch + 1;
                *epoch = ep == 0 ? 1u : ep;
                ctl->tag = ep;
            }
            t0 = global_ns();
        }
        grp.sync();
        if (bidir_hk(HK) && !pair16_hk(HK) && *(volatile uint32_t *)&ctl->tag == 0) {
            for (size_t i = grp.rank(); i < (size_t)B.swords; i += grp.size()) B.state[i] = 0ull;
            grp.sync();
            if (grp.rank() == 0) ctl->tag = 1;
            grp.sync();
        }
        const int q = *(volatile int *)&ctl->cur_q;
        if (q >= A.nq) break;
        const int qver = A.vtab ? *(volatile int *)&ctl->cur_ver : A.version;
        DevGraph G = G0;
        if (A.vtab && qver >= 0) {
            // the table (host memory) is rewritten while the kernel runs
            static_assert(sizeof(DevGraph) % 8 == 0, "DevGraph is copied in 8-byte words");
            const volatile unsigned long long *src =
                reinterpret_cast<const volatile unsigned long long *>(A.vtab + qver % A.nver);
            unsigned long long *dst = reinterpret_cast<unsigned long long *>(&G);
            for (int i = 0; i < (int)(sizeof(DevGraph) / 8); i++) dst[i] = src[i];
        }
        // serving requests live in host memory written while the kernel
        // runs: read them uncached
        const int32_t s = A.serve ? *(const volatile int32_t *)(A.S + q) : __ldg(A.S + q);
        const int32_t t = A.serve ? *(const volatile int32_t *)(A.T + q) : __ldg(A.T + q);
        if (qver < 0 || s < 0 || s >= G.n || t < 0 || t >= G.n) {
            if (grp.rank() == 0) {
                A.cost[q] = qver < 0 ? -1 : DDP_INF;
                if (A.plen) A.plen[q] = -1;
                if (A.qstatus) A.qstatus[q] = -1;
                if (A.serve) {
                    A.ver[q] = qver;
                    __threadfence_system();
                    A.done[q] = 1;
                }
                if (vbuf >= 0) {
                    atomicSub(A.inflight + vbuf, 1);
                    vbuf = -1;
                }
            }
            grp.sync();
            continue;
        }
        SearchParams P{s, t, A.delta, A.K, 0, 0, 0};
        SearchResult r;
        if (HK == 1) {
            const uint32_t tag = *(volatile uint32_t *)&ctl->tag;
            const uint32_t cap = run_bfs_hops(grp, G, B, t, wrows, tag, A.bfs_budget, async);
            r = slot_search(grp, G, B, HeurHops{B.hops, G.wmin, cap, tag}, P, wrows, sq, async);
        } else if (HK == 2) {
            int2 tp = reinterpret_cast<const int2 *>(G.xy)[t];
            r = slot_search(grp, G, B, HeurManhattan{G.xy, tp.x, tp.y, G.wmin}, P, wrows, sq, async);
        } else if (HK == 3) {
            int2 tp = reinterpret_cast<const int2 *>(G.xy)[t];
            r = slot_search(grp, G, B, HeurEuclid{G.xy, tp.x, tp.y, G.rho_fp}, P, wrows, sq, async);
        } else if (HK == 4) {
            r = slot_search(grp, G, B, HeurALT{G.lm, G.lm_L, G.lm_scale, t, G.lm_bits}, P, wrows, sq, async);
        } else if (bidir_hk(HK)) {
            // bidirectional: one-CTA slots only (the host never launches
            // these kinds with wider slots)
            if constexpr (std::is_same<Grp, CtaGroup>::value) {
                const uint32_t ep = *(volatile uint32_t *)&ctl->tag;
                if constexpr (HK == 5) {
                    r = run_bidir_cta(G, B, P, ep, wrows, bq, PotNone{}, RecDense{{}, B.state});
                } else if constexpr (HK == 8) {
                    const RecHash R{{}, B.state, (1u << B.hbits) - 1u, 32 - B.hbits};
                    r = run_bidir_cta(G, B, P, ep, wrows, bq, PotNone{}, R);
                } else if constexpr (HK == 9) {
                    r = run_bidir_cta(G, B, P, ep, wrows, bq, PotNone{}, RecPair16{B.state});
                } else {
                    const int2 sp = reinterpret_cast<const int2 *>(G.xy)[s];
                    const int2 tp = reinterpret_cast<const int2 *>(G.xy)[t];
                    if constexpr (HK == 6)
                        r = run_bidir_cta(G, B, P, ep, wrows, bq, PotEuclid{G.xy, sp, tp, G.rho_fp / 65536.0},
                                          RecDense{{}, B.state});
                    else
                        r = run_bidir_cta(G, B, P, ep, wrows, bq, PotManhattan{G.xy, sp, tp, G.wmin},
                                          RecDense{{}, B.state});
                }
            }
        } else {
            r = slot_search(grp, G, B, HeurZero{}, P, wrows, sq, async);
        }
        if ((async || bidir_hk(HK)) && (*(volatile int *)&ctl->status & (ST_OVERFLOW | ST_TIMEOUT))) {
            // an aborted asynchronous search may leave ring slots written:
            // clear the ring so the slot's next search starts clean
            for (int64_t i = grp.rank(); i < B.cap_q; i += grp.size()) B.q0[i].x = RING_EMPTY;
            grp.sync();
        }
        if (grp.rank() == 0) {
            const int st = ctl->status;
            int32_t len = 0;
            if (!(st & (ST_OVERFLOW | ST_TIMEOUT)) && A.paths) {
                if (HK == 8)
                    len = write_path_bidir(G, RecHash{{}, B.state, (1u << B.hbits) - 1u, 32 - B.hbits}, ctl->tag, s,
                                           t, bq->mu, A.paths + (size_t)q * A.path_cap, A.path_cap, &ctl->status);
                else if (pair16_hk(HK))
                    len = write_path_bidir(G, RecPair16{B.state}, ctl->tag, s, t, bq->mu,
                                           A.paths + (size_t)q * A.path_cap, A.path_cap, &ctl->status);
                else if (bidir_hk(HK))
                    len = write_path_bidir(G, RecDense{{}, B.state}, ctl->tag, s, t, bq->mu,
                                           A.paths + (size_t)q * A.path_cap, A.path_cap, &ctl->status);
                else
                    len = write_path(B, s, t, A.paths + (size_t)q * A.path_cap, A.path_cap, G.n,
                                     &ctl->status);
            }
            // a bidirectional search that found no meeting arc failed
            const int stf = ctl->status;
            A.cost[q] = ((st | stf) & (ST_OVERFLOW | ST_TIMEOUT)) ? -1
                        : (r.cost >= INF_G)                ? DDP_INF
                                                           : (int32_t)r.cost;
            if (A.plen) A.plen[q] = len;
            if (A.qstatus) A.qstatus[q] = ctl->status;
            if (A.serve) {
                A.ver[q] = qver;
                __threadfence_system();
                A.done[q] = 1;
            }
            if (vbuf >= 0) {
                atomicSub(A.inflight + vbuf, 1);
                vbuf = -1;
            }
            if (A.stats) {
                long long *st6 = A.stats + DDP_STATS * (size_t)q;
                st6[0] = (long long)ctl->expanded;
                st6[1] = (long long)ctl->scanned;
                st6[2] = (long long)ctl->relaxed;
                st6[3] = (long long)r.iters;
                st6[4] = HK == 1 ? (long long)ctl->bfs_reached : 0;
                st6[5] = HK == 1 ? (long long)ctl->bfs_scanned : 0;
                st6[6] = (long long)ctl->far_scanned;
                st6[7] = (long long)ctl->touched;
            }
            atomicOr(A.status, ctl->status);
        }
        grp.sync();
        const int cnt = *(volatile int *)&ctl->touched;
        if (pair16_hk(HK)) {
            // every word of a finished slot returns to all-ones, so the whole
            // 32-byte sector holding a logged node (it and its neighbour
            // node) is written: a full-sector store needs no read of the
            // old sector
            ulonglong4_32a ones;
            ones.x = ones.y = ones.z = ones.w = ~0ull;
            for (int i = grp.rank(); i < cnt; i += grp.size())
                reinterpret_cast<ulonglong4_32a *>(B.state)[B.touched[i] >> 1] = ones;
        } else if (!bidir_hk(HK)) {  // epoch-tagged records need no reset: the next query has a new epoch
            for (int i = grp.rank(); i < cnt; i += grp.size()) B.state[B.touched[i]] = ~0ull;
        }
        grp.sync();
        if (grp.rank() == 0) {
            if (A.tstart) A.tstart[q] = t0;
            if (A.tend) A.tend[q] = global_ns();
        }
    }
}

// One maintenance sub, spread over threads tid, tid + nth, ...
__device__ void svc_sub(const SvcSub &j, long long tid, long long nth) {
    const long long k = j.k;
    switch (j.kind) {
    case SVC_SCATTER_ARCS: {
        uint2 *dst = reinterpret_cast<uint2 *>(j.p0);
        const volatile long long *slot = reinterpret_cast<const volatile long long *>(j.p2);
        const volatile uint2 *val = reinterpret_cast<const volatile uint2 *>(j.p3);
        for (long long i = tid; i < k; i += nth) {
            const uint2 v = make_uint2(val[i].x, val[i].y);
            dst[slot[i]] = v;
        }
        break;
    }
    case SVC_SCATTER_ROWS: {
        int32_t *db = reinterpret_cast<int32_t *>(j.p0);
        int32_t *de = reinterpret_cast<int32_t *>(j.p1);
        const volatile int *rows = reinterpret_cast<const volatile int *>(j.p2);
        for (long long i = tid; i < k; i += nth) {
            const int r = rows[4 * i];
            db[r] = rows[4 * i + 1];
            de[r] = rows[4 * i + 2];
        }
        break;
    }
    case SVC_GATHER_ARCS: {
        uint2 *dst = reinterpret_cast<uint2 *>(j.p0);
        const uint2 *src = reinterpret_cast<const uint2 *>(j.p1);
        const volatile long long *slot = reinterpret_cast<const volatile long long *>(j.p2);
        for (long long i = tid; i < k; i += nth) {
            const long long x = slot[i];
            dst[x] = __ldcg(src + x);
        }
        break;
    }
    case SVC_GATHER_INTS: {
        int32_t *dst = reinterpret_cast<int32_t *>(j.p0);
        const int32_t *src = reinterpret_cast<const int32_t *>(j.p1);
        const volatile int *idx = reinterpret_cast<const volatile int *>(j.p2);
        for (long long i = tid; i < k; i += nth) {
            const int x = idx[i];
            dst[x] = __ldcg(src + x);
        }
        break;
    }
    case SVC_COPY_WORDS: {
        uint32_t *dst = reinterpret_cast<uint32_t *>(j.p0);
        const uint32_t *src = reinterpret_cast<const uint32_t *>(j.p1);
        // 16-byte body when both ends allow it (device allocations do)
        long long head = 0;
        if (((j.p0 | j.p1) & 15) == 0) {
            // eight loads in flight per thread (one CTA must still stream)
            const long long k4 = k / 4;
            uint4 *d4 = reinterpret_cast<uint4 *>(dst);
            const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
            long long i = tid;
            for (; i + 7 * nth < k4; i += 8 * nth) {
                uint4 r[8];
#pragma unroll
                for (int u = 0; u < 8; u++) r[u] = __ldcg(s4 + i + u * nth);
#pragma unroll
                for (int u = 0; u < 8; u++) d4[i + u * nth] = r[u];
            }
            for (; i < k4; i += nth) d4[i] = __ldcg(s4 + i);
            head = 4 * k4;
        }
        for (long long i = head + tid; i < k; i += nth) dst[i] = __ldcg(src + i);
        break;
    }
    default:
        break;
    }
}

__global__ void k_svc(SvcSub j) {
    svc_sub(j, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}

// Service CTA of a serving launch: runs the graph maintenance jobs of update
// batches while the search slots hold every SM.  It leaves when the slots
// close (or on pause).
__device__ void service_loop(const BatchArgs &A) {
    __shared__ SvcSub sub[SVC_MAX_SUB];
    __shared__ int job[3];  // run?, nsub, seq
    for (;;) {
        if (threadIdx.x == 0) {
            job[0] = 0;
            for (;;) {
                const int seq = A.svc->seq;
                if (seq != A.svc->done) {
                    A.svc->taken = seq;
                    __threadfence_system();
                    const int ns = min(max(A.svc->nsub, 0), SVC_MAX_SUB);
                    for (int i = 0; i < ns; i++) {
                        const volatile SvcSub &x = A.svc->sub[i];
                        sub[i].kind = x.kind;
                        sub[i].k = x.k;
                        sub[i].p0 = x.p0;
                        sub[i].p1 = x.p1;
                        sub[i].p2 = x.p2;
                        sub[i].p3 = x.p3;
                    }
                    job[0] = 1;
                    job[1] = ns;
                    job[2] = seq;
                    break;
                }
                if (*(volatile int *)A.closing || *A.pause) break;
                __nanosleep(2000);
            }
        }
        __syncthreads();
        if (!job[0]) return;
        for (int i = 0; i < job[1]; i++) {
            svc_sub(sub[i], threadIdx.x, blockDim.x);
            __syncthreads();  // subs run in order
        }
        __threadfence_system();
        __syncthreads();
        if (threadIdx.x == 0) A.svc->done = job[2];
        __syncthreads();
    }
}

// CTAs per SM the bidirectional instance is compiled for (its register
// budget per thread: 2 -> 64, 3 -> 40, 4 -> 32; the engine spills 220,
// 472 and 772 bytes per thread at those budgets, and three or four CTAs'
// spills outgrow the L1 left beside their shared memory).  Measured on the
// 4M-node batch of 4,096 pairs with ring claims spread over the warps:
// 2 -> 379k queries/s (304 slots), 3 -> 363k (456), 4 -> 228k (608).
#ifndef DDP_BIDIR_MIN_BLOCKS
#define DDP_BIDIR_MIN_BLOCKS 2
#endif
template <int HK>
__global__ void __launch_bounds__(512, (bidir_hk(HK) ? DDP_BIDIR_MIN_BLOCKS : 2)) k_batch(DevGraph G, SlotArrays sa, BatchArgs A) {
    __shared__ WarpRows wrows[MAX_WARPS];
    __shared__ CtaQ sq;
    __shared__ BiQ bq;
    if (A.svc && (int)blockIdx.x == A.serve_slots) {
        service_loop(A);
        return;
    }
    if (A.group <= 1) {
        SlotBufs B = slot_of(sa, blockIdx.x);
        CtaGroup grp{&B.ctl->status};
        batch_loop<HK>(grp, G, B, A, sa.epoch + blockIdx.x, wrows, &sq, &bq, !A.sync_engine);
    } else {
        const int slot = blockIdx.x / A.group;
        SlotBufs B = slot_of(sa, slot);
        SubGridGroup grp{{&B.ctl->bar_count, &B.ctl->bar_gen}, &B.ctl->status, A.group};
        batch_loop<HK>(grp, G, B, A, sa.epoch + slot, wrows, &sq, &bq, false);
    }
}

// Single query on one CTA with the asynchronous engine (narrow searches).
template <class Heur>
__global__ void __launch_bounds__(512, 2)
    k_solve_cta(DevGraph G, SlotArrays sa, Heur H, SearchParams P, int32_t *out, int32_t *path, int32_t path_cap) {
    __shared__ WarpRows wrows[MAX_WARPS];
    __shared__ CtaQ sq;
    SlotBufs B = slot_of(sa, 0);
    SearchResult r = run_search_cta<Heur, true>(G, B, H, P, wrows, &sq);  // one query: latency first
    if (threadIdx.x == 0) {
        out[0] = r.cost >= INF_G ? DDP_INF : (int32_t)r.cost;
        out[1] = (B.ctl->status & (ST_OVERFLOW | ST_TIMEOUT)) ? 0 : write_path(B, P.s, P.t, path, path_cap, G.n, &B.ctl->status);
        out[2] = B.ctl->status;
        out[3] = r.iters;
    }
    if (B.ctl->status & (ST_OVERFLOW | ST_TIMEOUT)) {
        __syncthreads();
        for (int64_t i = threadIdx.x; i < B.cap_q; i += blockDim.x) B.q0[i].x = RING_EMPTY;
    }
}

// ---- launch helpers ---------------------------------------------------------
static int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

template <class K>
static int coop_grid(K kernel, int block, int want) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
    int maxg = per_sm * sm_count();
    if (maxg < 1) maxg = 1;
    if (want > 0 && want < maxg) return want;
    return maxg;
}

template <class K>
static cudaError_t coop_launch(K kernel, int grid, int block, void **args, cudaStream_t st) {
    return cudaLaunchCooperativeKernel((const void *)kernel, dim3(grid), dim3(block), args, 0, st);
}

static bool is_bfs_kind(int k) { return k == DDP_H_BFS_HOPS || k == DDP_H_BFS_CAPPED; }

// Heuristic kind of the single-query engine that re-runs a batch query
// (the bidirectional form has no single-query counterpart: plain Dijkstra
// order gives the same cost).
static int rerun_kind(int hkind) { return is_bidir_kind(hkind) ? DDP_H_ZERO : hkind; }

// The k_batch instance of a heuristic kind.  Bidirectional kinds also pick
// their record layout: hashed records on request (DDP_OPT_HASH, plain
// kind); for the plain kind on graphs with coordinates, whose numbering
// (Morton order of points) puts a search's neighbours in shared sectors,
// 16-byte pairs (8-9 % more serving capacity on the 8M-point graph); else
// 32-byte epoch-tagged records (the potential-steered kinds too: on the
// 2048^2 maze they were faster, 16.4 against 17.8 ms).
int kernel_hk(int hkind, bool has_xy, bool hash) {
    if (is_bfs_kind(hkind)) return 1;
    if (hkind == DDP_H_MANHATTAN) return 2;
    if (hkind == DDP_H_EUCLID) return 3;
    if (hkind == DDP_H_LANDMARK) return 4;
#ifdef DDP_BIDIR_RECORDS32
    has_xy = false;  // build option: 32-byte records on every graph
#endif
    if (hkind == DDP_H_BIDIR) return hash ? 8 : has_xy ? 9 : 5;
    if (hkind == DDP_H_BIDIR_EUCLID) return 6;
    if (hkind == DDP_H_BIDIR_MANHATTAN) return 7;
    return 0;
}

// Slot layout of a k_batch instance.
int hk_slot_kind(int hk) {
    switch (hk) {
    case 1: return SLOT_HOPS;
    case 5:
    case 6:
    case 7: return SLOT_PAIR;
    case 8: return SLOT_PAIR | SLOT_HASH;
    case 9: return SLOT_PAIR16;
    default: return 0;
    }
}

static const void *batch_kernel_hk(int hk) {
    switch (hk) {
    case 1: return (const void *)k_batch<1>;
    case 2: return (const void *)k_batch<2>;
    case 3: return (const void *)k_batch<3>;
    case 4: return (const void *)k_batch<4>;
    case 5: return (const void *)k_batch<5>;
    case 6: return (const void *)k_batch<6>;
    case 7: return (const void *)k_batch<7>;
    case 8: return (const void *)k_batch<8>;
    case 9: return (const void *)k_batch<9>;
    default: return (const void *)k_batch<0>;
    }
}

// Nodes a capped heuristic BFS reaches before it stops (at the end of the
// level that crosses this count).
int64_t bfs_budget(int32_t n) { return std::max<int64_t>(4096, (int64_t)n / 32); }

// Launches the persistent slot kernel for heuristic kind `hkind`.
cudaError_t svc_run_direct(const SvcSub *subs, int nsub, cudaStream_t st) {
    for (int i = 0; i < nsub; i++) {
        if (subs[i].k <= 0) continue;
        const long long blocks = std::min<long long>((subs[i].k + 255) / 256, 4L * device_sms());
        k_svc<<<(unsigned)blocks, 256, 0, st>>>(subs[i]);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaStreamSynchronize(st);
}

cudaError_t launch_slots(int hk, int grid, int block, bool coop, DevGraph G, SlotArrays sa, BatchArgs A,
                         cudaStream_t st) {
    void *args[] = {&G, &sa, &A};
    const void *fn = batch_kernel_hk(hk);
    if (coop) return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(block), args, 0, st);
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, 0, st);
}

int slots_per_sm(int hk, int block) {
    int per_sm = 0;
    const void *fn = batch_kernel_hk(hk);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, 0);
    return per_sm;
}

int device_sms() { return sm_count(); }

// The bidirectional search keys its buckets by g.  On random digraphs (huge
// frontiers) narrow buckets pay (C4 family, 4,096 pairs: width 5 -> 319k
// queries/s, 8 -> 338k, 12 -> 314k, 25 -> 199k); on graphs with
// coordinates (thin frontiers) wide ones do (8M-point geometric graph,
// serving: width 27k -> 1.58k, 82k -> 1.90k queries/s; 2048^2 maze with unit
// weights: width 1-2 best).
uint32_t auto_delta_bidir(const ddp_graph *g) {
    const uint32_t d = (g->wmin + g->wmax) / (g->d_xy ? 4 : 12);
    return d < 1 ? 1 : d;
}

uint32_t auto_delta(const ddp_graph *g) {
    // bucket width ~ a typical arc weight: wide enough for parallel buckets,
    // narrow enough to keep re-expansions rare
    uint32_t d = (g->wmin + g->wmax) / 4;
    return d < 1 ? 1 : d;
}

}  // namespace ddp

using namespace ddp;

// ---- single-query workspace ------------------------------------------------
struct Workspace {
    SlotArrays sa;
    int32_t *d_out = nullptr;   // cost, path len, status, iters
    int32_t *d_path = nullptr;  // n
    int64_t cap = 0;
};

namespace ddp {
void workspace_release(ddp_graph *g) {
    if (!g->ws) return;
    slots_free(g->ws->sa);
    cudaFree(g->ws->d_out);
    cudaFree(g->ws->d_path);
    delete g->ws;
    g->ws = nullptr;
}

static int workspace_ensure(ddp_graph *g, int64_t cap) {
    if (g->ws && g->ws->cap >= cap) return DDP_OK;
    workspace_release(g);
    Workspace *w = new Workspace();
    g->ws = w;
    int rc = slots_alloc(w->sa, g->n, 1, cap, cap, false, g->stream);
    if (rc) {
        workspace_release(g);
        return rc;
    }
    w->cap = cap;
    DDP_CUDA(cudaMalloc(&w->d_out, sizeof(int32_t) * 8));
    DDP_CUDA(cudaMalloc(&w->d_path, sizeof(int32_t) * (size_t)g->n));
    return DDP_OK;
}
}  // namespace ddp

struct ddp_heuristic {
    ddp_graph *g = nullptr;
    int kind = DDP_H_ZERO;
    int32_t target = -1;
    uint32_t *d_hops = nullptr;  // BFS kind
    int32_t *d_h = nullptr;      // USER kind
    int32_t tx = 0, ty = 0;      // MANHATTAN kind
    uint32_t cap = HOPS_INF;     // hop cap of a BFS kind (HOPS_INF = exact)
};

struct ddp_query {
    int32_t cost = DDP_INF;
    std::vector<int32_t> path;
    int64_t stats[DDP_STATS] = {0, 0, 0, 0, 0, 0, 0, 0};
};

namespace ddp {
uint32_t *heuristic_hops_ptr(const ddp_heuristic *h) { return h ? h->d_hops : nullptr; }
}  // namespace ddp

extern "C" {

int ddp_heuristic_build(ddp_graph *g, int32_t target, int32_t kind, const int32_t *user_h,
                        int32_t *out_h, ddp_heuristic **out) {
    if (!g || !out) return fail(DDP_ERR_INVALID, "null argument");
    *out = nullptr;
    if (target < 0 || target >= g->n) return fail(DDP_ERR_INVALID, "target out of range");
    std::lock_guard<std::mutex> lk(g->mu);
    ddp_heuristic *h = new ddp_heuristic();
    h->g = g;
    graph_ref(g);
    h->kind = kind;
    h->target = target;
    auto bail = [&](int rc) {
        ddp_heuristic_free(h);
        return rc;
    };
    switch (kind) {
    case DDP_H_ZERO:
        if (out_h) std::fill(out_h, out_h + g->n, 0);
        break;
    case DDP_H_BFS_HOPS:
    case DDP_H_BFS_CAPPED: {
        int rc = workspace_ensure(g, (int64_t)g->n + 1024);
        if (rc) return bail(rc);
        cudaError_t e = cudaMalloc(&h->d_hops, sizeof(uint32_t) * (size_t)g->n);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(hops)"));
        DevGraph G = graph_view(g);
        SlotArrays sa = g->ws->sa;
        DDP_CUDA(cudaMemsetAsync(sa.ctl, 0, sizeof(SearchCtl), g->stream));
        int grid = coop_grid(k_bfs_single, 512, 0);
        long long budget = kind == DDP_H_BFS_CAPPED ? (long long)bfs_budget(g->n) : 0;
        void *args[] = {&G, &sa, &h->d_hops, &target, &budget};
        e = coop_launch(k_bfs_single, grid, 512, args, g->stream);
        if (e != cudaSuccess) return bail(cuda_fail(e, "k_bfs_single launch"));
        SearchCtl ctl;
        DDP_CUDA(cudaMemcpyAsync(&ctl, sa.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, g->stream));
        DDP_CUDA(cudaStreamSynchronize(g->stream));
        if (ctl.status & (ST_OVERFLOW | ST_TIMEOUT))
            return bail(fail(ctl.status & ST_TIMEOUT ? DDP_ERR_TIMEOUT : DDP_ERR_QUEUE_OVERFLOW,
                             "heuristic BFS did not complete"));
        h->cap = ctl.hcap;
        if (out_h) {
            std::vector<uint32_t> hops((size_t)g->n);
            DDP_CUDA(cudaMemcpy(hops.data(), h->d_hops, sizeof(uint32_t) * (size_t)g->n,
                                cudaMemcpyDeviceToHost));
            for (int32_t i = 0; i < g->n; i++) {
                if (hops[(size_t)i] == HOPS_INF) hops[(size_t)i] = h->cap;
            }
            for (int32_t i = 0; i < g->n; i++)
                out_h[i] = hops[(size_t)i] == HOPS_INF ? -1
                                                        : (int32_t)std::min<uint64_t>(
                                                              (uint64_t)hops[(size_t)i] * g->wmin,
                                                              (uint64_t)INT32_MAX - 1);
        }
        break;
    }
    case DDP_H_MANHATTAN: {
        if (!g->d_xy) return bail(fail(DDP_ERR_INVALID, "graph has no coordinates (ddp_graph_set_coords)"));
        h->tx = g->h_xy[2 * (size_t)target];
        h->ty = g->h_xy[2 * (size_t)target + 1];
        if (out_h)
            for (int32_t i = 0; i < g->n; i++) {
                int64_t d = llabs((long long)g->h_xy[2 * (size_t)i] - h->tx) +
                            llabs((long long)g->h_xy[2 * (size_t)i + 1] - h->ty);
                out_h[i] = (int32_t)std::min<int64_t>(d * g->wmin, INT32_MAX - 1);
            }
        break;
    }
    case DDP_H_EUCLID: {
        if (!g->d_xy) return bail(fail(DDP_ERR_INVALID, "graph has no coordinates (ddp_graph_set_coords)"));
        h->tx = g->h_xy[2 * (size_t)target];
        h->ty = g->h_xy[2 * (size_t)target + 1];
        if (out_h)
            for (int32_t i = 0; i < g->n; i++) {
                const int64_t dx = (int64_t)g->h_xy[2 * (size_t)i] - h->tx;
                const int64_t dy = (int64_t)g->h_xy[2 * (size_t)i + 1] - h->ty;
                const uint64_t r = isqrt_floor((uint64_t)(dx * dx + dy * dy));
                out_h[i] = (int32_t)std::min<uint64_t>((r * g->rho_fp) >> 16, INT32_MAX - 1);
            }
        break;
    }
    case DDP_H_USER: {
        if (!user_h) return bail(fail(DDP_ERR_INVALID, "user_h is null"));
        cudaError_t e = cudaMalloc(&h->d_h, sizeof(int32_t) * (size_t)g->n);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(h)"));
        DDP_CUDA(cudaMemcpy(h->d_h, user_h, sizeof(int32_t) * (size_t)g->n,
                            cudaMemcpyHostToDevice));
        if (out_h) std::memcpy(out_h, user_h, sizeof(int32_t) * (size_t)g->n);
        break;
    }
    case DDP_H_LANDMARK: {
        const DevGraph G = graph_view(g);
        if (!G.lm) return bail(fail(DDP_ERR_INVALID, "no current landmark table (ddp_landmarks_build)"));
        if (out_h) {
            int32_t *d = nullptr;
            cudaError_t e = cudaMalloc(&d, sizeof(int32_t) * (size_t)g->n);
            if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(h)"));
            k_alt_values<<<(g->n + 255) / 256, 256, 0, g->stream>>>(G, target, d);
            e = cudaGetLastError();
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(out_h, d, sizeof(int32_t) * (size_t)g->n, cudaMemcpyDeviceToHost, g->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
            cudaFree(d);
            if (e != cudaSuccess) return bail(cuda_fail(e, "landmark heuristic values"));
        }
        break;
    }
    default:
        return bail(fail(DDP_ERR_INVALID, "unknown heuristic kind"));
    }
    *out = h;
    return DDP_OK;
}

}  // extern "C"

namespace ddp {
// d(src, v) for every v (reverse: d(v, src)) into the device array dist.
static int sssp_into(ddp_graph *g, int32_t src, bool reverse, int32_t *dist) {
    DevGraph G = graph_view(g);
    if (reverse) {
        std::swap(G.off, G.roff);
        std::swap(G.arc, G.rarc);
        std::swap(G.oend, G.roend);
        std::swap(G.doff, G.droff);
        std::swap(G.darc, G.drarc);
    }
    SearchParams P{src, -1, auto_delta(g), 0, 0, 0, 0};
    int64_t cap = (int64_t)g->n + 1024;
    for (int attempt = 0; attempt < 4; attempt++) {
        int rc = workspace_ensure(g, cap);
        if (rc) return rc;
        Workspace *w = g->ws;
        DDP_CUDA(cudaMemsetAsync(w->sa.ctl, 0, sizeof(SearchCtl), g->stream));
        const int grid = coop_grid(k_sssp, 512, 0);
        void *args[] = {&G, &w->sa, &P, &dist, &w->d_out};
        cudaError_t e = coop_launch(k_sssp, grid, 512, args, g->stream);
        if (e != cudaSuccess) return cuda_fail(e, "k_sssp launch");
        DDP_CUDA(cudaMemsetAsync(w->sa.q, 0xFF, sizeof(uint2) * (size_t)w->sa.cap_q * 2, g->stream));
        k_reset_touched<<<dim3(256, 1), 256, 0, g->stream>>>(w->sa);
        DDP_CUDA(cudaGetLastError());
        int32_t res[4];
        DDP_CUDA(cudaMemcpyAsync(res, w->d_out, sizeof(res), cudaMemcpyDeviceToHost, g->stream));
        DDP_CUDA(cudaStreamSynchronize(g->stream));
        if (res[2] & ST_TIMEOUT) return fail(DDP_ERR_TIMEOUT, "landmark search barrier timed out");
        if (res[2] & ST_OVERFLOW) {
            cap *= 2;
            continue;
        }
        return DDP_OK;
    }
    return fail(DDP_ERR_QUEUE_OVERFLOW, "landmark search queue overflow after retries");
}
}  // namespace ddp

extern "C" {

int ddp_landmarks_build(ddp_graph *g, int32_t count, uint64_t seed, int32_t *out_ids) {
    return ddp_landmarks_build_bits(g, count, 16, seed, out_ids);
}

int ddp_landmarks_build_bits(ddp_graph *g, int32_t count, int32_t bits, uint64_t seed, int32_t *out_ids) {
    if (!g) return fail(DDP_ERR_INVALID, "null graph");
    if (bits != 16 && bits != 8) return fail(DDP_ERR_INVALID, "landmark entries are 16 or 8 bits");
    if (bits == 16 && (count < 4 || count > 64 || count % 4))
        return fail(DDP_ERR_INVALID, "landmark count must be 4, 8, ..., 64 (16-bit entries)");
    if (bits == 8 && (count < 8 || count > 128 || count % 8))
        return fail(DDP_ERR_INVALID, "landmark count must be 8, 16, ..., 128 (8-bit entries)");
    std::lock_guard<std::mutex> lk(g->mu);
    const int32_t n = g->n;
    const int32_t width = 2 * count;
    int32_t *dist = nullptr, *tab = nullptr;
    cudaError_t e = cudaMalloc(&dist, sizeof(int32_t) * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc(&tab, sizeof(int32_t) * (size_t)n * width);
    if (e != cudaSuccess) {
        cudaFree(dist);
        return cuda_fail(e, "cudaMalloc(landmarks)");
    }
    auto done = [&](int rc) {
        cudaFree(dist);
        if (rc) cudaFree(tab);
        return rc;
    };
    // farthest-point selection: the next landmark maximises the smallest
    // round trip d(L, v) + d(v, L) over the landmarks so far (nodes that no
    // landmark relates to come first); the first one is the farthest from a
    // seeded random node
    std::vector<int64_t> score((size_t)n, INT64_MAX);
    std::vector<int32_t> fw((size_t)n), bw((size_t)n);
    int32_t maxd = 0;  // largest finite landmark distance (sets the table's scale)
    auto measure = [&](int32_t src, int col) -> int {
        int rc = sssp_into(g, src, false, dist);
        if (rc) return rc;
        if (col >= 0) k_put_column<<<(n + 255) / 256, 256, 0, g->stream>>>(tab, width, col, dist, n);
        DDP_CUDA(cudaMemcpyAsync(fw.data(), dist, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, g->stream));
        DDP_CUDA(cudaStreamSynchronize(g->stream));
        rc = sssp_into(g, src, true, dist);
        if (rc) return rc;
        if (col >= 0) k_put_column<<<(n + 255) / 256, 256, 0, g->stream>>>(tab, width, col + count, dist, n);
        DDP_CUDA(cudaMemcpyAsync(bw.data(), dist, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, g->stream));
        DDP_CUDA(cudaStreamSynchronize(g->stream));
        for (int32_t v = 0; v < n; v++) {
            const bool f = fw[(size_t)v] != LM_UNREACHED, b = bw[(size_t)v] != LM_UNREACHED;
            if (col >= 0) {
                if (f) maxd = std::max(maxd, fw[(size_t)v]);
                if (b) maxd = std::max(maxd, bw[(size_t)v]);
            }
            const int64_t x = (f && b) ? (int64_t)fw[(size_t)v] + bw[(size_t)v]
                              : f       ? fw[(size_t)v]
                              : b       ? bw[(size_t)v]
                                        : INT64_MAX;
            score[(size_t)v] = std::min(score[(size_t)v], x);
        }
        return DDP_OK;
    };
    uint64_t x = seed + 0x9E3779B97F4A7C15ull;  // splitmix64
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    int rc = measure((int32_t)(x % (uint64_t)n), -1);
    if (rc) return done(rc);
    std::vector<int32_t> ids;
    {
        // the first landmark: farthest (round trip) from the random node
        int32_t best = 0;
        int64_t bs = -1;
        for (int32_t v = 0; v < n; v++) {
            const bool f = fw[(size_t)v] != LM_UNREACHED, b = bw[(size_t)v] != LM_UNREACHED;
            const int64_t y = (f ? fw[(size_t)v] : 0) + (b ? bw[(size_t)v] : 0);
            if (y > bs) {
                bs = y;
                best = v;
            }
        }
        ids.push_back(best);
    }
    std::fill(score.begin(), score.end(), INT64_MAX);
    for (int i = 0; i < count; i++) {
        if (i > 0) {
            int32_t best = 0;
            for (int32_t v = 1; v < n; v++)
                if (score[(size_t)v] > score[(size_t)best]) best = v;
            ids.push_back(best);
        }
        rc = measure(ids.back(), i);
        if (rc) return done(rc);
    }
    // entries q = floor(d / scale) with every finite q below the all-ones
    // unreachable marker: the smallest scale with maxd / scale <= marker - 1
    const int32_t top = bits == 16 ? 65534 : 254;
    const int32_t scale = std::max(1, (int32_t)(((int64_t)maxd + top - 1) / top));
    void *packed = nullptr;
    e = cudaMalloc(&packed, (size_t)(bits / 8) * (size_t)n * width);
    if (e != cudaSuccess) return done(cuda_fail(e, "cudaMalloc(landmarks)"));
    if (bits == 16)
        k_pack_landmarks<<<4 * device_sms(), 256, 0, g->stream>>>(tab, (uint16_t *)packed, (int64_t)n * width, scale);
    else
        k_pack_landmarks<<<4 * device_sms(), 256, 0, g->stream>>>(tab, (uint8_t *)packed, (int64_t)n * width, scale);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) {
        cudaFree(packed);
        return done(cuda_fail(e, "landmark table packing"));
    }
    cudaFree(g->d_lm);
    g->d_lm = reinterpret_cast<uint2 *>(packed);
    g->lm_scale = scale;
    g->lm_bits = bits;
    g->lm_L = count;
    g->lm_stamp = g->update_count;
    g->lm_ids = ids;
    if (out_ids) std::memcpy(out_ids, ids.data(), sizeof(int32_t) * (size_t)count);
    cudaFree(tab);  // the 32-bit staging table
    return done(DDP_OK);
}

int ddp_heuristic_free(ddp_heuristic *h) {
    if (!h) return DDP_OK;
    cudaFree(h->d_hops);
    cudaFree(h->d_h);
    graph_unref(h->g);
    delete h;
    return DDP_OK;
}

int ddp_solve(ddp_graph *g, const ddp_heuristic *h, int32_t source, int32_t target,
              const ddp_opts *opts, ddp_query **out) {
    if (!g || !out) return fail(DDP_ERR_INVALID, "null argument");
    *out = nullptr;
    if (source < 0 || source >= g->n || target < 0 || target >= g->n)
        return fail(DDP_ERR_INVALID, "source/target out of range");
    if (h && h->g != g) return fail(DDP_ERR_INVALID, "heuristic belongs to another graph");
    if (h && h->kind != DDP_H_ZERO && h->target != target)
        return fail(DDP_ERR_INVALID, "heuristic was built for another target");
    if (h && h->kind == DDP_H_LANDMARK && !graph_view(g).lm)
        return fail(DDP_ERR_INVALID, "landmark table is stale (the graph was updated)");
    ddp_opts o = opts ? *opts : ddp_opts{};
    std::lock_guard<std::mutex> lk(g->mu);
    cudaStream_t st = o.stream ? (cudaStream_t)o.stream : g->stream;
    const int block = o.block > 0 ? std::min(o.block, 512) : 512;
    int64_t cap = o.queue_cap > 0 ? o.queue_cap : (int64_t)g->n + 1024;
    const uint32_t delta = o.delta > 0 ? (uint32_t)o.delta : auto_delta(g);
    DevGraph G = graph_view(g);
    SearchParams P{source, target, delta, o.K, 0, 0, 0};
    for (int attempt = 0; attempt < 4; attempt++) {
        int rc = workspace_ensure(g, cap);
        if (rc) return rc;
        Workspace *w = g->ws;
        DDP_CUDA(cudaMemsetAsync(w->sa.ctl, 0, sizeof(SearchCtl), st));
        cudaError_t e;
        const int kind = h ? h->kind : DDP_H_ZERO;
        const bool one_cta = (o.flags & DDP_OPT_ONE_CTA) != 0;
        if (one_cta) {
            void *hp = nullptr;
            HeurHops Hh{h ? h->d_hops : nullptr, g->wmin, h ? h->cap : HOPS_INF, 0u};
            HeurManhattan Hm{g->d_xy, h ? h->tx : 0, h ? h->ty : 0, g->wmin};
            HeurEuclid He{g->d_xy, h ? h->tx : 0, h ? h->ty : 0, g->rho_fp};
            HeurArray Ha{h ? h->d_h : nullptr};
            HeurALT Hl{G.lm, G.lm_L, G.lm_scale, target, G.lm_bits};
            HeurZero Hz{};
            const void *fn;
            if (kind == DDP_H_BFS_HOPS || kind == DDP_H_BFS_CAPPED) { fn = (const void *)k_solve_cta<HeurHops>; hp = &Hh; }
            else if (kind == DDP_H_MANHATTAN) { fn = (const void *)k_solve_cta<HeurManhattan>; hp = &Hm; }
            else if (kind == DDP_H_EUCLID) { fn = (const void *)k_solve_cta<HeurEuclid>; hp = &He; }
            else if (kind == DDP_H_USER) { fn = (const void *)k_solve_cta<HeurArray>; hp = &Ha; }
            else if (kind == DDP_H_LANDMARK) { fn = (const void *)k_solve_cta<HeurALT>; hp = &Hl; }
            else { fn = (const void *)k_solve_cta<HeurZero>; hp = &Hz; }
            void *args[] = {&G, &w->sa, hp, &P, &w->d_out, &w->d_path, &g->n};
            e = cudaLaunchKernel(fn, dim3(1), dim3(block), args, 0, st);
        } else if (kind == DDP_H_BFS_HOPS || kind == DDP_H_BFS_CAPPED) {
            HeurHops H{h->d_hops, g->wmin, h->cap, 0u};
            int grid = coop_grid(k_solve_single<HeurHops>, block, o.grid);
            void *args[] = {&G, &w->sa, &H, &P, &w->d_out, &w->d_path, &g->n};
            e = coop_launch(k_solve_single<HeurHops>, grid, block, args, st);
        } else if (kind == DDP_H_MANHATTAN) {
            HeurManhattan H{g->d_xy, h->tx, h->ty, g->wmin};
            int grid = coop_grid(k_solve_single<HeurManhattan>, block, o.grid);
            void *args[] = {&G, &w->sa, &H, &P, &w->d_out, &w->d_path, &g->n};
            e = coop_launch(k_solve_single<HeurManhattan>, grid, block, args, st);
        } else if (kind == DDP_H_EUCLID) {
            HeurEuclid H{g->d_xy, h->tx, h->ty, g->rho_fp};
            int grid = coop_grid(k_solve_single<HeurEuclid>, block, o.grid);
            void *args[] = {&G, &w->sa, &H, &P, &w->d_out, &w->d_path, &g->n};
            e = coop_launch(k_solve_single<HeurEuclid>, grid, block, args, st);
        } else if (kind == DDP_H_USER) {
            HeurArray H{h->d_h};
            int grid = coop_grid(k_solve_single<HeurArray>, block, o.grid);
            void *args[] = {&G, &w->sa, &H, &P, &w->d_out, &w->d_path, &g->n};
            e = coop_launch(k_solve_single<HeurArray>, grid, block, args, st);
        } else if (kind == DDP_H_LANDMARK) {
            HeurALT H{G.lm, G.lm_L, G.lm_scale, target, G.lm_bits};
            int grid = coop_grid(k_solve_single<HeurALT>, block, o.grid);
            void *args[] = {&G, &w->sa, &H, &P, &w->d_out, &w->d_path, &g->n};
            e = coop_launch(k_solve_single<HeurALT>, grid, block, args, st);
        } else {
            HeurZero H{};
            int grid = coop_grid(k_solve_single<HeurZero>, block, o.grid);
            void *args[] = {&G, &w->sa, &H, &P, &w->d_out, &w->d_path, &g->n};
            e = coop_launch(k_solve_single<HeurZero>, grid, block, args, st);
        }
        if (e != cudaSuccess) return cuda_fail(e, "k_solve_single launch");
        if (!one_cta)  // the phase-synchronous engine leaves entries in q0/q1
            DDP_CUDA(cudaMemsetAsync(w->sa.q, 0xFF, sizeof(uint2) * (size_t)w->sa.cap_q * 2, st));
        k_reset_touched<<<dim3(256, 1), 256, 0, st>>>(w->sa);
        DDP_CUDA(cudaGetLastError());
        int32_t res[4];
        SearchCtl ctl;
        DDP_CUDA(cudaMemcpyAsync(res, w->d_out, sizeof(res), cudaMemcpyDeviceToHost, st));
        DDP_CUDA(cudaMemcpyAsync(&ctl, w->sa.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, st));
        DDP_CUDA(cudaStreamSynchronize(st));
        if (res[2] & ST_TIMEOUT) return fail(DDP_ERR_TIMEOUT, "search barrier timed out");
        if (res[2] & ST_OVERFLOW) {
            if (o.queue_cap > 0) return fail(DDP_ERR_QUEUE_OVERFLOW, "search queue overflow");
            cap *= 2;  // automatic capacity: grow and retry
            continue;
        }
        ddp_query *q = new ddp_query();
        q->cost = res[0];
        q->stats[0] = (int64_t)ctl.expanded;
        q->stats[1] = (int64_t)ctl.scanned;
        q->stats[2] = (int64_t)ctl.relaxed;
        q->stats[3] = res[3];
        q->stats[4] = 0;
        q->stats[5] = 0;
        q->stats[6] = (int64_t)ctl.far_scanned;
        q->stats[7] = (int64_t)ctl.touched;
        if (res[1] > 0) {
            q->path.resize((size_t)res[1]);
            cudaError_t ce = cudaMemcpy(q->path.data(), w->d_path, sizeof(int32_t) * (size_t)res[1],
                                        cudaMemcpyDeviceToHost);
            if (ce != cudaSuccess) {
                delete q;
                return cuda_fail(ce, "path readback");
            }
        }
        *out = q;
        return DDP_OK;
    }
    return fail(DDP_ERR_QUEUE_OVERFLOW, "search queue overflow after retries");
}

int ddp_query_cost(const ddp_query *q, int32_t *cost) {
    if (!q || !cost) return fail(DDP_ERR_INVALID, "null argument");
    *cost = q->cost;
    return DDP_OK;
}

int ddp_path_read(const ddp_query *q, int32_t *buf, int32_t cap, int32_t *len) {
    if (!q || !len) return fail(DDP_ERR_INVALID, "null argument");
    *len = (int32_t)q->path.size();
    if (buf && cap > 0)
        std::memcpy(buf, q->path.data(), sizeof(int32_t) * std::min<size_t>((size_t)cap, q->path.size()));
    return DDP_OK;
}

int ddp_query_stats(const ddp_query *q, int64_t *stats) {
    if (!q || !stats) return fail(DDP_ERR_INVALID, "null argument");
    for (int i = 0; i < DDP_STATS; i++) stats[i] = q->stats[i];
    return DDP_OK;
}

int ddp_query_free(ddp_query *q) {
    delete q;
    return DDP_OK;
}

}  // extern "C"

// ---- batched engine ----------------------------------------------------------
struct ddp_batch {
    ddp_graph *g = nullptr;
    int hkind = DDP_H_ZERO;
    ddp_opts o{};
    cudaStream_t stream = nullptr;
    int block = 512;
    SlotArrays sa;
    // device buffers sized for the largest batch seen
    int32_t cap_q_n = 0;
    int32_t *d_S = nullptr, *d_T = nullptr, *d_cost = nullptr, *d_plen = nullptr, *d_paths = nullptr;
    int32_t *d_qstatus = nullptr;
    long long *d_stats = nullptr, *d_t0 = nullptr, *d_t1 = nullptr;
    int *d_work = nullptr, *d_status = nullptr;
    int32_t path_cap = 0;
    int32_t last_n = 0;
    int32_t launches = 0;
    int group = 1;  // CTAs per query slot
    bool no_graph = false;
    int hk = 0;  // k_batch instance (heuristic kind and record layout)
    // CUDA graph of the last device-pointer solve and the kernel arguments
    // it was captured with: a replay is valid only while a fresh launch
    // would pass exactly the same arguments (graph arrays, landmark table,
    // batch buffers, options)
    cudaGraphExec_t gexec = nullptr;
    bool gkey_valid = false;
    DevGraph gkey_G{};
    BatchArgs gkey_A{};
    // arrays of the last solve that path reads go back to: the batch's own
    // after ddp_batch_solve, the caller's after ddp_batch_solve_device
    const int32_t *last_S = nullptr, *last_T = nullptr, *last_plen = nullptr;
    // paths of queries re-run on the single-query engine
    std::map<int32_t, std::vector<int32_t>> overflow_paths;
};

namespace ddp {

static int batch_grow(ddp_batch *b, int32_t n) {
    if (n <= b->cap_q_n) return DDP_OK;
    b->last_n = 0;  // the last solve's paths go with the old buffers
    cudaFree(b->d_S);
    cudaFree(b->d_T);
    cudaFree(b->d_cost);
    cudaFree(b->d_plen);
    cudaFree(b->d_paths);
    cudaFree(b->d_qstatus);
    cudaFree(b->d_stats);
    cudaFree(b->d_t0);
    cudaFree(b->d_t1);
    const size_t N = (size_t)n;
    DDP_CUDA(cudaMalloc(&b->d_S, sizeof(int32_t) * N));
    DDP_CUDA(cudaMalloc(&b->d_T, sizeof(int32_t) * N));
    DDP_CUDA(cudaMalloc(&b->d_cost, sizeof(int32_t) * N));
    DDP_CUDA(cudaMalloc(&b->d_plen, sizeof(int32_t) * N));
    DDP_CUDA(cudaMalloc(&b->d_paths, sizeof(int32_t) * N * (size_t)b->path_cap));
    DDP_CUDA(cudaMalloc(&b->d_qstatus, sizeof(int32_t) * N));
    DDP_CUDA(cudaMalloc(&b->d_stats, sizeof(long long) * DDP_STATS * N));
    DDP_CUDA(cudaMalloc(&b->d_t0, sizeof(long long) * N));
    DDP_CUDA(cudaMalloc(&b->d_t1, sizeof(long long) * N));
    b->cap_q_n = n;
    return DDP_OK;
}

// Kernel arguments of one batch launch.  Returns false when the landmark
// table the heuristic needs is stale (the graph changed since it was built).
static bool batch_args(ddp_batch *b, int32_t n, const int32_t *dS, const int32_t *dT, int32_t *dcost,
                       int32_t *dplen, DevGraph *G, BatchArgs *A0) {
    BatchArgs &A = *A0;
    std::memset(&A, 0, sizeof(A));
    A.S = dS;
    A.T = dT;
    A.nq = n;
    A.cost = dcost;
    A.plen = dplen;
    A.paths = b->d_paths;
    A.path_cap = b->path_cap;
    A.qstatus = b->d_qstatus;
    A.stats = b->d_stats;
    A.tstart = b->d_t0;
    A.tend = b->d_t1;
    A.work = b->d_work;
    A.status = b->d_status;
    A.delta = b->o.delta > 0                ? (uint32_t)b->o.delta
              : is_bidir_kind(b->hkind) ? auto_delta_bidir(b->g)
                                        : auto_delta(b->g);
    A.bfs_budget = b->hkind == DDP_H_BFS_CAPPED ? bfs_budget(b->g->n) : 0;
    A.K = b->o.K;
    A.group = b->group;
    A.sync_engine = (b->o.flags & DDP_OPT_SYNC) != 0;
    *G = graph_view(b->g);
    return !(b->hkind == DDP_H_LANDMARK && !G->lm);
}

static cudaError_t batch_launch_args(ddp_batch *b, DevGraph G, BatchArgs A) {
    cudaError_t e = cudaMemsetAsync(b->d_work, 0, sizeof(int) * 2, b->stream);
    if (e != cudaSuccess) return e;
    // fresh control blocks (barrier counters included) for every launch
    e = cudaMemsetAsync(b->sa.ctl, 0, sizeof(SearchCtl) * (size_t)b->sa.nslots, b->stream);
    if (e != cudaSuccess) return e;
    const int grid = b->sa.nslots * b->group;
    SlotArrays sa = b->sa;
    void *args[] = {&G, &sa, &A};
    const void *fn = batch_kernel_hk(b->hk);
    if (b->group > 1)
        return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(b->block), args, 0, b->stream);
    return cudaLaunchKernel(fn, dim3(grid), dim3(b->block), args, 0, b->stream);
}

// Field-by-field equality of the by-value kernel arguments (padding bytes
// are not compared).
static bool same_view(const DevGraph &x, const DevGraph &y) {
    return x.n == y.n && x.e == y.e && x.off == y.off && x.arc == y.arc && x.roff == y.roff &&
           x.rarc == y.rarc && x.xy == y.xy && x.wmin == y.wmin && x.rho_fp == y.rho_fp && x.doff == y.doff &&
           x.darc == y.darc && x.droff == y.droff && x.drarc == y.drarc && x.oend == y.oend &&
           x.roend == y.roend && x.lm == y.lm && x.lm_L == y.lm_L && x.lm_scale == y.lm_scale &&
           x.lm_bits == y.lm_bits;
}

static bool same_args(const BatchArgs &x, const BatchArgs &y) {
    return x.S == y.S && x.T == y.T && x.nq == y.nq && x.cost == y.cost && x.plen == y.plen &&
           x.paths == y.paths && x.path_cap == y.path_cap && x.qstatus == y.qstatus && x.stats == y.stats &&
           x.tstart == y.tstart && x.tend == y.tend && x.work == y.work && x.status == y.status &&
           x.delta == y.delta && x.K == y.K && x.bfs_budget == y.bfs_budget && x.group == y.group &&
           x.sync_engine == y.sync_engine;
}

}  // namespace ddp

extern "C" {

int ddp_batch_create(ddp_graph *g, int32_t hkind, const ddp_opts *opts, ddp_batch **out) {
    if (!g || !out) return fail(DDP_ERR_INVALID, "null argument");
    *out = nullptr;
    if (hkind != DDP_H_ZERO && !is_bfs_kind(hkind) && hkind != DDP_H_MANHATTAN && hkind != DDP_H_EUCLID &&
        hkind != DDP_H_LANDMARK && !is_bidir_kind(hkind))
        return fail(DDP_ERR_INVALID,
                    "batch heuristic must be ZERO, BFS_HOPS, BFS_CAPPED, MANHATTAN, EUCLID, LANDMARK or BIDIR");
    if (hkind == DDP_H_LANDMARK && !graph_view(g).lm)
        return fail(DDP_ERR_INVALID, "no current landmark table (ddp_landmarks_build)");
    if ((hkind == DDP_H_MANHATTAN || hkind == DDP_H_EUCLID || hkind == DDP_H_BIDIR_EUCLID ||
         hkind == DDP_H_BIDIR_MANHATTAN) && !g->d_xy)
        return fail(DDP_ERR_INVALID, "graph has no coordinates (ddp_graph_set_coords)");
    ddp_batch *b = new ddp_batch();
    b->g = g;
    graph_ref(g);
    b->hkind = hkind;
    if (opts) b->o = *opts;
    b->block = b->o.block > 0 ? std::min(b->o.block, 512) : 512;
    b->path_cap = 1024;
    cudaError_t e = b->o.stream ? cudaSuccess : cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (b->o.stream) b->stream = (cudaStream_t)b->o.stream;
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(e, "cudaStreamCreate");
    }
    // slots: occupancy-limited, then memory-limited (half of free memory)
    int per_sm = 0;
    b->hk = kernel_hk(hkind, g->d_xy != nullptr, (b->o.flags & DDP_OPT_HASH) != 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel_hk(b->hk), b->block, 0);
    b->group = is_bidir_kind(hkind) ? 1 : std::max(1, b->o.group);  // bidirectional slots are one CTA
    const int coresident = std::max(1, per_sm) * sm_count();
    if (b->group > coresident) b->group = coresident;
    int nslots = coresident / b->group;
    if (b->o.grid > 0) nslots = std::min(b->o.grid, b->group > 1 ? nslots : b->o.grid);
    // the bidirectional ring holds one bucket and spills to the far pile
    // when full, so it needs far less than a node count
    const int64_t cap = b->o.queue_cap > 0      ? b->o.queue_cap
                        : is_bidir_kind(hkind) ? std::min<int64_t>((int64_t)g->n + 4096, 1 << 18)
                                                : (int64_t)g->n + 4096;
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    // the far pile holds every open node beyond the current bucket: twice the
    // node count leaves room for stale copies between compactions
    const int64_t cap_f = b->o.queue_cap > 0 ? b->o.queue_cap : 2 * (int64_t)g->n + 4096;
    const int skind = hk_slot_kind(b->hk);
    const int hb = (skind & SLOT_HASH) ? hash_bits(g->n) : 0;
    const size_t per = slot_bytes(g->n, cap, cap_f, skind, hb);
    const size_t budget = freeb / 2;
    if ((size_t)nslots * per > budget) nslots = (int)std::max<size_t>(1, budget / per);
    int rc = slots_alloc(b->sa, g->n, nslots, cap, cap_f, skind, b->stream, hb);
    if (rc == DDP_OK) {
        cudaError_t e1 = cudaMalloc(&b->d_work, sizeof(int) * 2);
        if (e1 != cudaSuccess) rc = cuda_fail(e1, "cudaMalloc(work)");
        else b->d_status = b->d_work + 1;
    }
    if (rc) {
        ddp_batch_free(b);
        return rc;
    }
    *out = b;
    return DDP_OK;
}

int ddp_batch_solve_device(ddp_batch *b, int32_t n, const int32_t *d_sources,
                           const int32_t *d_targets, int32_t *d_cost, int32_t *d_path_len) {
    if (!b || n < 0 || (n > 0 && (!d_sources || !d_targets || !d_cost)))
        return fail(DDP_ERR_INVALID, "bad batch arguments");
    std::lock_guard<std::mutex> lk(b->g->mu);
    int rc = batch_grow(b, n);
    if (rc) return rc;
    if (n == 0) return DDP_OK;
    // path lengths go to the batch's own array when the caller wants none,
    // so that ddp_batch_path can still size the paths
    int32_t *plen = d_path_len ? d_path_len : b->d_plen;
    DevGraph G;
    BatchArgs A;
    if (!batch_args(b, n, d_sources, d_targets, d_cost, plen, &G, &A))
        return fail(DDP_ERR_INVALID, "landmark table is stale (graph updated since ddp_landmarks_build)");
    b->overflow_paths.clear();
    b->last_n = 0;  // no paths to read until this launch is queued
    if (!b->no_graph) {
        const bool hit = b->gexec && b->gkey_valid && same_view(G, b->gkey_G) && same_args(A, b->gkey_A);
        if (!hit) {
            if (b->gexec) {
                cudaGraphExecDestroy(b->gexec);
                b->gexec = nullptr;
            }
            b->gkey_valid = false;
            cudaGraph_t graph = nullptr;
            DDP_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = batch_launch_args(b, G, A);
            cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
            if (e == cudaSuccess && e2 == cudaSuccess) e = cudaGraphInstantiate(&b->gexec, graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                // capture was refused (e.g. a cooperative launch): launch
                // directly from now on
                (void)cudaGetLastError();
                if (b->gexec) cudaGraphExecDestroy(b->gexec);
                b->gexec = nullptr;
                b->no_graph = true;
            } else {
                b->gkey_G = G;
                b->gkey_A = A;
                b->gkey_valid = true;
            }
        }
    }
    if (b->no_graph) {
        cudaError_t e = batch_launch_args(b, G, A);
        if (e != cudaSuccess) return cuda_fail(e, "k_batch launch");
    } else {
        DDP_CUDA(cudaGraphLaunch(b->gexec, b->stream));
    }
    b->last_S = d_sources;
    b->last_T = d_targets;
    b->last_plen = plen;
    b->last_n = n;
    b->launches = 1;
    return DDP_OK;
}

int ddp_batch_solve(ddp_batch *b, int32_t n, const int32_t *sources, const int32_t *targets,
                    int32_t *out_cost, int32_t *out_path_len) {
    if (!b || n < 0 || (n > 0 && (!sources || !targets || !out_cost)))
        return fail(DDP_ERR_INVALID, "bad batch arguments");
    {
        std::lock_guard<std::mutex> lk(b->g->mu);
        int rc = batch_grow(b, n);
        if (rc) return rc;
        if (n == 0) return DDP_OK;
        b->overflow_paths.clear();
        DDP_CUDA(cudaMemcpyAsync(b->d_S, sources, sizeof(int32_t) * (size_t)n,
                                 cudaMemcpyHostToDevice, b->stream));
        DDP_CUDA(cudaMemcpyAsync(b->d_T, targets, sizeof(int32_t) * (size_t)n,
                                 cudaMemcpyHostToDevice, b->stream));
        DevGraph G;
        BatchArgs A;
        if (!batch_args(b, n, b->d_S, b->d_T, b->d_cost, b->d_plen, &G, &A))
            return fail(DDP_ERR_INVALID, "landmark table is stale (graph updated since ddp_landmarks_build)");
        cudaError_t e = batch_launch_args(b, G, A);
        if (e != cudaSuccess) return cuda_fail(e, "k_batch launch");
        b->last_S = b->d_S;
        b->last_T = b->d_T;
        b->last_plen = b->d_plen;
        b->last_n = n;
        b->launches = 1;
        DDP_CUDA(cudaMemcpyAsync(out_cost, b->d_cost, sizeof(int32_t) * (size_t)n,
                                 cudaMemcpyDeviceToHost, b->stream));
        if (out_path_len)
            DDP_CUDA(cudaMemcpyAsync(out_path_len, b->d_plen, sizeof(int32_t) * (size_t)n,
                                     cudaMemcpyDeviceToHost, b->stream));
        DDP_CUDA(cudaStreamSynchronize(b->stream));
    }
    // queries that outgrew the slot queues are re-run on the single-query
    // engine, which grows its queues as needed
    bool any = false;
    for (int32_t i = 0; i < n; i++) any |= out_cost[i] == -1;
    if (any) {
        for (int32_t i = 0; i < n; i++) {
            if (out_cost[i] != -1) continue;
            if (sources[i] < 0 || sources[i] >= b->g->n || targets[i] < 0 || targets[i] >= b->g->n)
                return fail(DDP_ERR_INVALID, "query endpoint out of range");
            ddp_heuristic *h = nullptr;
            int rc = ddp_heuristic_build(b->g, targets[i], rerun_kind(b->hkind), nullptr, nullptr, &h);
            if (rc) return rc;
            ddp_query *q = nullptr;
            ddp_opts so = b->o;
            so.queue_cap = 0;  // the single-query engine grows its queues itself
            so.grid = 0;
            rc = ddp_solve(b->g, h, sources[i], targets[i], &so, &q);
            ddp_heuristic_free(h);
            if (rc) return rc;
            out_cost[i] = q->cost;
            if (out_path_len) out_path_len[i] = (int32_t)q->path.size();
            b->overflow_paths[i] = q->path;
            ddp_query_free(q);
        }
    }
    return DDP_OK;
}

int ddp_batch_sync(ddp_batch *b) {
    if (!b) return fail(DDP_ERR_INVALID, "null batch");
    DDP_CUDA(cudaStreamSynchronize(b->stream));
    return DDP_OK;
}

int ddp_batch_path(ddp_batch *b, int32_t i, int32_t *buf, int32_t cap, int32_t *len) {
    if (!b || !len || i < 0 || i >= b->last_n) return fail(DDP_ERR_INVALID, "bad path request");
    auto it = b->overflow_paths.find(i);
    if (it != b->overflow_paths.end()) {
        *len = (int32_t)it->second.size();
        if (buf && cap > 0)
            std::memcpy(buf, it->second.data(), sizeof(int32_t) * std::min<size_t>(cap, it->second.size()));
        return DDP_OK;
    }
    int32_t l = 0;
    DDP_CUDA(cudaStreamSynchronize(b->stream));
    DDP_CUDA(cudaMemcpy(&l, b->last_plen + i, sizeof(int32_t), cudaMemcpyDeviceToHost));
    *len = l;
    if (l > b->path_cap) {
        // the slot buffer kept only a prefix; recompute the path on the
        // single-query engine
        ddp_heuristic *h = nullptr;
        int32_t s, t;
        DDP_CUDA(cudaMemcpy(&s, b->last_S + i, sizeof(int32_t), cudaMemcpyDeviceToHost));
        DDP_CUDA(cudaMemcpy(&t, b->last_T + i, sizeof(int32_t), cudaMemcpyDeviceToHost));
        int rc = ddp_heuristic_build(b->g, t, rerun_kind(b->hkind), nullptr, nullptr, &h);
        if (rc) return rc;
        ddp_query *q = nullptr;
        ddp_opts so = b->o;
        so.queue_cap = 0;
        so.grid = 0;
        rc = ddp_solve(b->g, h, s, t, &so, &q);
        ddp_heuristic_free(h);
        if (rc) return rc;
        *len = (int32_t)q->path.size();
        if (buf && cap > 0)
            std::memcpy(buf, q->path.data(), sizeof(int32_t) * std::min<size_t>(cap, q->path.size()));
        ddp_query_free(q);
        return DDP_OK;
    }
    if (buf && cap > 0 && l > 0)
        DDP_CUDA(cudaMemcpy(buf, b->d_paths + (size_t)i * b->path_cap,
                            sizeof(int32_t) * std::min(cap, l), cudaMemcpyDeviceToHost));
    return DDP_OK;
}

int ddp_batch_stats(ddp_batch *b, int64_t *stats, int64_t *t_start_ns, int64_t *t_end_ns) {
    if (!b) return fail(DDP_ERR_INVALID, "null batch");
    const size_t n = (size_t)b->last_n;
    DDP_CUDA(cudaStreamSynchronize(b->stream));
    if (stats && n)
        DDP_CUDA(cudaMemcpy(stats, b->d_stats, sizeof(long long) * DDP_STATS * n, cudaMemcpyDeviceToHost));
    if (t_start_ns && n)
        DDP_CUDA(cudaMemcpy(t_start_ns, b->d_t0, sizeof(long long) * n, cudaMemcpyDeviceToHost));
    if (t_end_ns && n)
        DDP_CUDA(cudaMemcpy(t_end_ns, b->d_t1, sizeof(long long) * n, cudaMemcpyDeviceToHost));
    return DDP_OK;
}

int ddp_batch_info(const ddp_batch *b, int32_t *slots, int64_t *queue_cap, int32_t *block) {
    if (!b) return fail(DDP_ERR_INVALID, "null batch");
    if (slots) *slots = b->sa.nslots;
    if (queue_cap) *queue_cap = b->sa.cap_q;
    if (block) *block = b->block;
    return DDP_OK;
}

int ddp_batch_group(const ddp_batch *b, int32_t *group) {
    if (!b || !group) return fail(DDP_ERR_INVALID, "null argument");
    *group = b->group;
    return DDP_OK;
}

int ddp_batch_launches(const ddp_batch *b, int32_t *launches) {
    if (!b || !launches) return fail(DDP_ERR_INVALID, "null argument");
    *launches = b->launches;
    return DDP_OK;
}

int ddp_batch_free(ddp_batch *b) {
    if (!b) return DDP_OK;
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    slots_free(b->sa);
    cudaFree(b->d_S);
    cudaFree(b->d_T);
    cudaFree(b->d_cost);
    cudaFree(b->d_plen);
    cudaFree(b->d_paths);
    cudaFree(b->d_qstatus);
    cudaFree(b->d_stats);
    cudaFree(b->d_t0);
    cudaFree(b->d_t1);
    cudaFree(b->d_work);
    if (b->stream && !b->o.stream) cudaStreamDestroy(b->stream);
    graph_unref(b->g);
    delete b;
    return DDP_OK;
}

}  // extern "C"
