// Asynchronous single-CTA A*: the search of one query by one CTA without a
// barrier per expansion wave.
//
// The phase-synchronous engine (engine.cuh, run_search) advances the search
// frontier by one arc per barrier; a narrow search with a good heuristic
// (grid mazes, geometric graphs) then costs one barrier round per hop of the
// path.  Here the current bucket (entries with f < T) is a work pool that
// warps drain and refill concurrently:
//   * a warp first continues on its own children (up to 64 entries staged in
//     shared memory: depth-first chasing of the frontier with no queue round
//     trip), and spills to a ring in global memory that any warp may claim
//     from;
//   * a `pending` counter in shared memory counts entries pushed and not yet
//     retired; children are counted before their parent retires, so
//     pending == 0 means the bucket is empty and no warp is working on it;
//   * ring slots hold {node, g} with node = 0xFFFFFFFF meaning "not written
//     yet"; a claimer waits (bounded) for a reserved slot to be written and
//     clears it after reading, so the ring is clean for the next bucket.
// Between buckets the CTA synchronises once and splits the far pile at the
// next threshold exactly as run_search does.  Stale entries (g changed since
// the push) and entries with f >= f(t) are dropped; keep mode retains them in
// the far pile, as in run_search.
#pragma once

#include "engine.cuh"

namespace ddp {

constexpr uint32_t RING_EMPTY = 0xFFFFFFFFu;

struct CtaQ {
    int head, tail;      // ring positions of the current bucket
    int pending;         // entries pushed to the bucket and not yet retired
    int far_cnt;         // far pushes appended this bucket
    int alt_cnt;         // split: far entries kept
    unsigned int minf;   // split: min f kept
    int status;
    unsigned int tg;     // g(t) as this CTA installed it (the target's label, kept in shared memory)
};

// Reserves k ring slots (lane 0 only); returns the first position or -1 when
// the ring would overflow (the caller then sends the entries to far).
__device__ __forceinline__ int ring_reserve(CtaQ *sq, int k, int cap) {
    for (;;) {
        const int t = *(volatile int *)&sq->tail;
        if (t + k > cap) return -1;
        if (atomicCAS(&sq->tail, t, t + k) == t) return t;
    }
}

// LATENCY picks the relaxation form: one atomic per arc (single queries and
// cheap heuristics) or a load, then h and a CAS on improving arcs only
// (table heuristics in batches).
template <class Heur, bool LATENCY>
__device__ SearchResult run_search_cta(const DevGraph &G, const SlotBufs &B, const Heur &H, const SearchParams &P,
                                       WarpRows *wrows, CtaQ *sq) {
    constexpr bool cheap = heur_cheap<Heur>::value;
    constexpr bool latency = LATENCY;
    SearchCtl *ctl = B.ctl;
    const int lane = lane_id();
    const int warp = threadIdx.x >> 5;
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
        sq->minf = 0xFFFFFFFFu;
        sq->status = 0;
        if (!P.resume) {
            ctl->touched = 1;
            B.state[P.s] = st_make(0, -1);
            B.touched[0] = P.s;
            ring[0] = make_uint2((uint32_t)P.s, 0u);
            sq->tail = 1;
            sq->pending = 1;
        }
        sq->tg = P.t >= 0 ? (unsigned int)st_g(__ldcg(B.state + P.t)) : 0xFFFFFFFFu;
    }
    const int64_t far_resume = P.resume ? (int64_t)(*(volatile int *)&ctl->far_n) : 0;
    const bool far_in_f1 = P.resume && (*(volatile int *)&ctl->far_sel) != 0;
    __syncthreads();

    uint4 *fcur = far_in_f1 ? B.f1 : B.f0, *falt = far_in_f1 ? B.f0 : B.f1;
    int64_t nfar = far_resume;
    const uint32_t ht = P.t >= 0 ? H(P.t) : 0u;
    uint32_t T = sat_add(H(P.s), P.delta);
    uint32_t Tsplit = T;
    bool do_expand = !P.resume;
    if (P.resume) T = Tsplit = 0;
    unsigned long long n_exp = 0, n_scan = 0, n_rel = 0;
    int phases = 0;
    const int64_t max_phases = 4 * (int64_t)G.n + (1 << 22);

    for (;;) {
        if (do_expand) {
            // ---- drain the bucket asynchronously -----------------------
            int c_f = 0, c_t = 0, c_loc = 0;  // staged far pushes, touches, own children
            for (;;) {
                // f(t) from the shared-memory copy of g(t): only this CTA relaxes t
                const uint64_t ft64 = (uint64_t)(*(volatile unsigned int *)&sq->tg) + ht;
                const uint32_t ft = ft64 >= 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)ft64;
                // 1. take work: own children first, else claim from the ring
                int n = 0;
                uint2 en = make_uint2(RING_EMPTY, 0u);
                int2 pre = make_int2(-1, -1);  // row bounds fetched when the child was pushed
                if (c_loc > 0) {
                    n = min(32, c_loc);
                    if (lane < n) {
                        en = wr.sn[c_loc - n + lane];
                        if (cheap) pre = wr.snr[c_loc - n + lane];
                    }
                    c_loc -= n;
                    __syncwarp();
                } else {
                    int h0 = 0;
                    if (lane == 0) {
                        n = -1;
                        for (uint32_t spins = 0;; spins++) {
                            const int h = *(volatile int *)&sq->head, t = *(volatile int *)&sq->tail;
                            if (h < t) {
                                const int k = min(32, t - h);
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
                            __nanosleep(64);
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
                // 2. entry stage (as run_search)
                int u = -1, rb = 0, deg = 0;
                uint32_t gu = 0;
                bool requeue = false;
                if (lane < n && en.x != RING_EMPTY) {
                    u = (int)en.x;
                    gu = en.y;
                    const bool have = cheap && pre.x >= 0;
                    // a child this warp just installed and chases at once is
                    // expanded without re-reading its state (latency mode): if
                    // another warp improved it meanwhile, the expansion with
                    // the older g only relaxes worse labels, which the newer
                    // entry corrects
                    const uint64_t su = (have && latency) ? st_make(gu, 0) : __ldcg(B.state + u);
                    // every entry of the current bucket was pushed with
                    // f = g + h(u) < T (near pushes, split moves and the
                    // source alike; T only grows), so while f(t) >= T the pop
                    // test f < f(t) passes without reading h again; keep mode
                    // re-derives it
                    const uint32_t hu = (ft < T || (P.keep && ft != 0xFFFFFFFFu)) ? H(u) : 0u;
                    const int r0 = have ? pre.x : row_begin(G.off, G.oend, u);
                    const int r1 = have ? pre.y : row_end(G.off, G.oend, u);
                    if (st_g(su) == gu && u != P.t) {
                        if ((uint64_t)gu + hu < ft) {
                            rb = r0;
                            deg = r1 - r0;
                            n_exp++;
                        } else if (P.keep) {
                            requeue = true;
                        }
                    }
                }
                stage_push(requeue, make_uint4((uint32_t)u, gu, 0u, 0u), wr.sf, c_f, &sq->far_cnt,  // keep mode: f re-derived
                           fcur, nfar, B.cap_f, ctl, 0);
                int total;
                const int ex = warp_excl_scan(deg, &total);
                wr.excl[lane] = ex;
                wr.rb[lane] = rb;
                wr.bdeg[lane] = deg;
                wr.drb[lane] = 0;
                wr.g[lane] = gu;
                wr.u[lane] = u;
                __syncwarp();
                n_scan += (lane == 0) ? (unsigned long long)total : 0ull;
                // AA arcs per lane per step; each stage issues all of its
                // loads / atomics before consuming any result.  Two in
                // latency mode; one in throughput mode, whose heuristic row
                // loads already fill the warp's memory pipeline (landmark
                // batches: 17.1k -> 19.0k q/s)
#ifndef DDP_ASYNC_ARCS_LATENCY
#define DDP_ASYNC_ARCS_LATENCY 2
#endif
#ifndef DDP_ASYNC_ARCS_THROUGHPUT
#define DDP_ASYNC_ARCS_THROUGHPUT 1
#endif
                constexpr int AA = latency ? DDP_ASYNC_ARCS_LATENCY : DDP_ASYNC_ARCS_THROUGHPUT;
                for (int kb = 0; kb < total; kb += 32 * AA) {
                    int v[AA], o[AA];
                    uint32_t ng[AA], hv[AA];
                    uint64_t cur[AA];
                    bool live[AA], wpos[AA];
#pragma unroll
                    for (int r = 0; r < AA; r++) {
                        const int k = kb + 32 * r + lane;
                        live[r] = false;
                        wpos[r] = true;
                        v[r] = 0;
                        ng[r] = 0;
                        o[r] = 0;
                        if (k < total) {
                            o[r] = row_owner(wr, k);
                            const uint2 a = row_arc(G, wr, o[r], k, true);
                            v[r] = (int)a.x;
                            wpos[r] = a.y != 0;
                            const uint64_t ng64 = (uint64_t)wr.g[o[r]] + a.y;
                            live[r] = v[r] >= 0 && ng64 < INF_G;
                            ng[r] = (uint32_t)ng64;
                        }
                    }
                    int2 rows[AA];
                    bool fresh[AA];  // latency mode: the atomic found v unreached
                    if (!P.keep && latency) {
                        // one atomic per arc: over a positive-weight arc,
                        // atomicMin on (g << 32 | parent) installs a smaller g
                        // (or, at equal g, a smaller parent id: an equal-cost
                        // alternative; parent chains still strictly decrease
                        // in g, so no cycle).  A zero-weight arc must not
                        // replace a parent on a tie (that could close a parent
                        // cycle): it tries a CAS from "unreached", then a
                        // strict-improvement CAS loop.  Cheap heuristics and
                        // the child's row bounds load beside the atomic.
#pragma unroll
                        for (int r = 0; r < AA; r++) {
                            rows[r] = make_int2(-1, -1);
                            if (cheap) {
                                hv[r] = live[r] ? H(v[r]) : 0u;
                                if (live[r]) rows[r] = make_int2(row_begin(G.off, G.oend, v[r]), row_end(G.off, G.oend, v[r]));
                            }
                            const uint64_t nv = st_make(ng[r], wr.u[o[r]]);
                            cur[r] = !live[r] ? 0ull
                                     : wpos[r] ? atomicMin(B.state + v[r], nv)
                                               : atomicCAS(B.state + v[r], ~0ull, nv);
                        }
#pragma unroll
                        for (int r = 0; r < AA; r++) {
                            fresh[r] = live[r] && cur[r] == ~0ull;
                            bool inst = fresh[r] || (live[r] && wpos[r] && ng[r] < st_g(cur[r]));
                            if (live[r] && !wpos[r] && !inst && ng[r] < st_g(cur[r])) {
                                const uint64_t nv = st_make(ng[r], wr.u[o[r]]);
                                uint64_t c0 = cur[r];
                                for (;;) {
                                    const uint64_t got = atomicCAS(B.state + v[r], c0, nv);
                                    if (got == c0) {
                                        inst = true;
                                        break;
                                    }
                                    c0 = got;
                                    if (ng[r] >= st_g(c0)) break;
                                }
                            }
                            live[r] = inst;
                            if (!cheap) hv[r] = live[r] ? H(v[r]) : 0u;
                        }
                    } else {
#pragma unroll
                        for (int r = 0; r < AA; r++) cur[r] = live[r] ? __ldcg(B.state + v[r]) : 0ull;
#pragma unroll
                        for (int r = 0; r < AA; r++) {
                            live[r] = live[r] && ng[r] < st_g(cur[r]);
                            hv[r] = live[r] ? H(v[r]) : 0u;
                            rows[r] = make_int2(-1, -1);
                            fresh[r] = false;
                        }
                    }
#pragma unroll
                    for (int r = 0; r < AA; r++) {
                        bool to_near = false, to_far = false, first = false;
                        const uint64_t fv = (uint64_t)ng[r] + hv[r];
                        const uint32_t fpush = fv >= 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)fv;
                        if (!P.keep && latency) {
                            // the atomic already installed g: log a first touch even
                            // when f >= f(t) prunes the push
                            if (live[r]) {
                                first = !P.no_touch_log && fresh[r];
                                if (v[r] == P.t) atomicMin(&sq->tg, ng[r]);
                                if (fv < ft) {
                                    if (fv < T) to_near = true;
                                    else to_far = true;
                                }
                            }
                        } else if (live[r] && (P.keep ? hv[r] < INF_G : fv < ft)) {
                            const uint64_t nv = st_make(ng[r], wr.u[o[r]]);
                            uint64_t c0 = cur[r];
                            for (;;) {
                                const uint64_t got = atomicCAS(B.state + v[r], c0, nv);
                                if (got == c0) {
                                    first = !P.no_touch_log && st_g(c0) >= INF_G;
                                    if (v[r] == P.t) atomicMin(&sq->tg, ng[r]);
                                    if (fv < T) to_near = true;
                                    else to_far = true;
                                    break;
                                }
                                c0 = got;
                                if (ng[r] >= st_g(c0)) break;
                            }
                        }
                        if (to_near || to_far) n_rel++;
                        // near pushes: counted in `pending` first, then kept as
                        // this warp's own work, or spilled to the ring when full
                        const unsigned mn = __ballot_sync(FULL, to_near);
                        if (mn) {
                            const int kn = __popc(mn);
                            const int rank_in = __popc(mn & ((1u << lane) - 1u));
                            if (lane == 0) atomicAdd(&sq->pending, kn);
                            __syncwarp();
                            if (c_loc + kn <= 64) {
                                if (to_near) {
                                    wr.sn[c_loc + rank_in] = make_uint2((uint32_t)v[r], ng[r]);
                                    if (cheap) wr.snr[c_loc + rank_in] = rows[r];
                                }
                                c_loc += kn;
                            } else {
                                int p0 = 0;
                                if (lane == 0) p0 = ring_reserve(sq, kn, cap);
                                p0 = __shfl_sync(FULL, p0, 0);
                                if (p0 >= 0) {
                                    if (to_near) {
                                        volatile uint2 *slot = reinterpret_cast<volatile uint2 *>(ring + p0 + rank_in);
                                        // one 8-byte store: readers see the old
                                        // empty marker or the whole entry
                                        *reinterpret_cast<volatile unsigned long long *>(slot) =
                                            ((unsigned long long)ng[r] << 32) | (uint32_t)v[r];
                                    }
                                } else {
                                    // ring full: the entries go to far (the next
                                    // split brings them back) and leave the bucket
                                    if (lane == 0) atomicSub(&sq->pending, kn);
                                    to_far = to_far || to_near;
                                }
                            }
                            __syncwarp();
                        }
                        stage_push(to_far, make_uint4((uint32_t)v[r], ng[r], fpush, 0u), wr.sf, c_f, &sq->far_cnt,
                                   fcur, nfar, B.cap_f, ctl, 0);
                        stage_push(first, v[r], wr.st, c_t, &ctl->touched, B.touched, 0, (int64_t)G.n, ctl, 0);
                    }
                }
                __syncwarp();
                // 3. retire the chunk (its children are already counted)
                if (lane == 0 && n > 0) atomicSub(&sq->pending, n);
                if (*(volatile int *)&sq->status & ST_TIMEOUT) break;
            }
            stage_flush(wr.sf, c_f, &sq->far_cnt, fcur, nfar, B.cap_f, ctl, 0);
            stage_flush(wr.st, c_t, &ctl->touched, B.touched, 0, (int64_t)G.n, ctl, 0);
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
            Tsplit = sat_add(T, P.delta);
            __syncthreads();
        }
        // ---- split the far pile at Tsplit ---------------------------------
        {
            const uint64_t st_t = P.t >= 0 ? __ldcg(B.state + P.t) : ~0ull;
            const uint64_t ft64 = (uint64_t)st_g(st_t) + (P.t >= 0 ? H(P.t) : 0u);
            const uint32_t ft = ft64 >= 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)ft64;
            unsigned int local_min = 0xFFFFFFFFu;
            int c_n = 0, c_f = 0;
            if (threadIdx.x == 0) ctl->far_scanned += (unsigned long long)nfar;
            for (int64_t base = (int64_t)warp * 32; base < nfar; base += (int64_t)(blockDim.x >> 5) * 32) {
                const int64_t idx = base + lane;
                bool to_near = false, keep = false;
                uint4 en = make_uint4(0u, 0u, 0u, 0u);
                if (idx < nfar) {
                    // entries carry f from their push (no node state read:
                    // stale entries are dropped when popped); keep mode
                    // re-checks, since h may have changed since the push
                    en = __ldcg(fcur + idx);
                    bool live = true;
                    uint64_t f = en.z;
                    if (P.keep) {
                        live = st_g(__ldcg(B.state + en.x)) == en.y;
                        f = (uint64_t)en.y + H((int)en.x);
                        en.z = f >= 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)f;
                    }
                    if (live) {
                        if (f < ft && f < Tsplit) {
                            to_near = true;
                        } else if (f < ft || (P.keep && f < INF_G)) {
                            keep = true;
                            local_min = min(local_min, (uint32_t)f);
                        }
                    }
                }
                // split output goes to ring positions [0, m): the ring is
                // clean and nobody reads it until the split is over
                stage_push(to_near, make_uint2(en.x, en.y), wr.sn, c_n, &sq->tail, ring, 0, (int64_t)cap, ctl, 0);
                stage_push(keep, en, wr.sf, c_f, &sq->alt_cnt, falt, 0, B.cap_f, ctl, 0);
            }
            stage_flush(wr.sn, c_n, &sq->tail, ring, 0, (int64_t)cap, ctl, 0);
            stage_flush(wr.sf, c_f, &sq->alt_cnt, falt, 0, B.cap_f, ctl, 0);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) local_min = min(local_min, __shfl_xor_sync(FULL, local_min, o));
            if (lane == 0 && local_min != 0xFFFFFFFFu) atomicMin(&sq->minf, local_min);
            __syncthreads();
            const int m = min(*(volatile int *)&sq->tail, cap);
            const int kept = *(volatile int *)&sq->alt_cnt;
            const unsigned int mf = *(volatile unsigned int *)&sq->minf;
            const int st = *(volatile int *)&ctl->status;
            phases++;
            __syncthreads();
            if (threadIdx.x == 0) {
                sq->alt_cnt = 0;
                sq->minf = 0xFFFFFFFFu;
                sq->head = 0;
                sq->pending = m;
            }
            uint4 *t2 = fcur;
            fcur = falt;
            falt = t2;
            nfar = kept;
            if (st & (ST_OVERFLOW | ST_TIMEOUT)) break;
            if (phases > max_phases) {
                if (threadIdx.x == 0) atomicOr(&ctl->status, ST_TIMEOUT);
                break;
            }
            if (m > 0) {
                T = Tsplit;
                do_expand = true;
            } else if (nfar == 0 || mf >= ft) {
                break;  // no open node with f < f(t)
            } else {
                Tsplit = sat_add(mf, P.delta);
                do_expand = false;
            }
            __syncthreads();
        }
    }

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
    if (threadIdx.x == 0) {
        ctl->far_n = (int)nfar;
        ctl->far_sel = fcur == B.f1 ? 1 : 0;
        ctl->iters = phases;
    }
    __syncthreads();
    SearchResult r;
    const uint64_t st_t = P.t >= 0 ? __ldcg(B.state + P.t) : ~0ull;
    const uint64_t c = (uint64_t)st_g(st_t) + (P.t >= 0 ? H(P.t) : 0u);
    r.cost = (st_g(st_t) >= INF_G || c >= INF_G) ? 0xFFFFFFFFu : (uint32_t)c;
    r.iters = phases;
    return r;
}

}  // namespace ddp
