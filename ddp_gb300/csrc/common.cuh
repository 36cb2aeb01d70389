// Shared internals of libddp_gb300: status/error plumbing, the device view
// of a graph, and group barriers with bounded waits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "ddp_gb300.h"

namespace ddp {

// ---- error plumbing ------------------------------------------------------
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
// Event trace to stderr, on when the environment sets DDP_TRACE=1.
bool trace_on();
void trace(const char *fmt, ...) __attribute__((format(printf, 1, 2)));

#define DDP_CUDA(call)                                              \
    do {                                                            \
        cudaError_t _e = (call);                                    \
        if (_e != cudaSuccess) return ::ddp::cuda_fail(_e, #call);  \
    } while (0)

// ---- constants -------------------------------------------------------------
// g = INF_G marks an unreached node; the state word packs (g << 32) | parent.
constexpr uint32_t INF_G = 0x7FFFFFFFu;
constexpr uint64_t STATE_INIT = (uint64_t(INF_G) << 32) | 0xFFFFFFFFull;
// hop value of a node that cannot reach the target
constexpr uint32_t HOPS_INF = 0xFFFFFFFFu;

__host__ __device__ __forceinline__ uint32_t st_g(uint64_t s) { return uint32_t(s >> 32); }
__host__ __device__ __forceinline__ int32_t st_parent(uint64_t s) { return int32_t(uint32_t(s)); }
__host__ __device__ __forceinline__ uint64_t st_make(uint32_t g, int32_t p) {
    return (uint64_t(g) << 32) | uint64_t(uint32_t(p));
}

// Device-side status bits (sticky, OR-ed into a per-run word).
enum : int {
    ST_OVERFLOW = 1,  // a queue outgrew its capacity
    ST_TIMEOUT = 2,   // a bounded barrier wait gave up
    ST_PATH_TRUNC = 4 // a path did not fit its buffer
};

// Arcs are stored interleaved as {col, weight}: one 8-byte load per arc.
// col < 0 marks a deleted arc.
struct DevGraph {
    int32_t n;
    int64_t e;
    const int32_t *off;   // n+1
    const uint2 *arc;     // e   {head, w}
    const int32_t *roff;  // n+1 reverse CSR
    const uint2 *rarc;    // e   {tail, w}
    const int32_t *xy;    // 2n coordinates (may be null)
    uint32_t wmin;
    uint32_t rho_fp;      // Euclidean heuristic scale, 16.16 fixed point
    // Arcs inserted by dynamic updates live in a second CSR (doff/darc)
    // until they are folded into the main one; null when absent.
    const int32_t *doff;  // n+1
    const uint2 *darc;
    const int32_t *droff; // n+1
    const uint2 *drarc;
    // Dynamic graphs keep explicit row ends (rows grow in place and move to
    // the end of the arc array when full): row u = [off[u], oend[u]).
    // Null for static graphs, where row u ends at off[u+1].
    const int32_t *oend;
    const int32_t *roend;
    // Landmark distances (ALT heuristic), null when not built: row v holds
    // lm_L values q(L_i, v) then lm_L values q(v, L_i), lm_bits (16 or 8)
    // each, with q = floor(d / lm_scale) and the all-ones entry
    // (LM_UNREACHED16 / LM_UNREACHED8) when there is no path.  Each half row
    // is a whole number of 8-byte words: lm_L is a multiple of 4 (16-bit)
    // or of 8 (8-bit).
    const uint2 *lm;
    int32_t lm_L;
    int32_t lm_scale;
    int32_t lm_bits;
};
constexpr int32_t LM_UNREACHED = 0x7FFFFFFF;  // exhaustive-search distances
constexpr uint32_t LM_UNREACHED16 = 0xFFFFu;  // 16-bit table entries
constexpr uint32_t LM_UNREACHED8 = 0xFFu;     // 8-bit table entries

__device__ __forceinline__ int row_end(const int32_t *off, const int32_t *oend, int u) {
    return oend ? __ldcg(oend + u) : __ldg(off + u + 1);
}

__device__ __forceinline__ int row_begin(const int32_t *off, const int32_t *oend, int u) {
    return oend ? __ldcg(off + u) : __ldg(off + u);
}

// ---- bounded-wait barriers -------------------------------------------------
// Spin limit for every device-side wait: ~2^22 polls with backoff (seconds),
// after which the waiter records ST_TIMEOUT and proceeds; callers check the
// status word after each barrier and leave their loops.
constexpr uint32_t SPIN_LIMIT = 1u << 22;

struct GridBarrier {
    unsigned int *count;  // arrivals in the current generation
    unsigned int *gen;    // generation counter
};

// Barrier over `nblocks` CTAs of a cooperative launch (co-residency
// guaranteed by cudaLaunchCooperativeKernel).  Bounded: gives up after
// SPIN_LIMIT polls and sets ST_TIMEOUT in *status.
__device__ __forceinline__ void grid_sync(const GridBarrier &b, unsigned int nblocks, int *status) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int *vgen = b.gen;
        unsigned int g = *vgen;
        __threadfence();
        unsigned int arrived = atomicAdd(b.count, 1u);
        if (arrived == nblocks - 1) {
            *b.count = 0;
            __threadfence();
            atomicAdd(b.gen, 1u);
        } else {
            uint32_t spins = 0;
            unsigned int ns = 32;
            while (*vgen == g) {
                if (++spins > SPIN_LIMIT) {
                    atomicOr(status, ST_TIMEOUT);
                    break;
                }
                __nanosleep(ns);
                if (ns < 256) ns <<= 1;
            }
        }
        __threadfence();
    }
    __syncthreads();
}

}  // namespace ddp
