// Reverse-BFS hop counts without any device allocation.
//
// Some callers cannot let a library call cudaMalloc: a service that hands all
// device memory to its own pool at start-up, or one that must not fail on a
// late allocation once it is serving.  For them ddp_bfs_hops_noalloc takes
// every input and output as a device pointer the caller already owns and
// keeps its own scratch (the BFS frontier queues, the level counters and the
// grid barrier) in the fixed array below.
//
// Cost of that choice: every GPU that loads this library holds the array
// (NOALLOC_BYTES, about 8 MiB) until the process exits, graphs are limited to
// DDP_NOALLOC_MAX_NODES nodes, and all calls share the one array, so calls
// that overlap on the GPU (different streams or threads) race and must be
// serialised by the caller.
#include <cstddef>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "ddp_gb300.h"

namespace ddp {
namespace {

constexpr int NA_BLOCK = 256;
constexpr size_t NA_CTRL = 256;  // control words at the start of the array
constexpr size_t NOALLOC_BYTES =
    NA_CTRL + 2 * sizeof(int32_t) * (size_t)DDP_NOALLOC_MAX_NODES;

// file-scope scratch; host code must not use its name as an address
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

struct NaCtrl {
    unsigned int bar_count, bar_gen;
    int status;
    int pad;
    int cnt[4];  // frontier sizes, rotating per level
};

// one set-up per device: the device address of the scratch array
std::mutex g_na_mu;
void *g_na_ptr[64] = {nullptr};

__global__ void __launch_bounds__(NA_BLOCK)
    k_bfs_noalloc(int32_t n, const int32_t *__restrict__ roff, const int32_t *__restrict__ rsrc,
                  int32_t target, int32_t *__restrict__ hops, unsigned char *scratch) {
    NaCtrl *c = reinterpret_cast<NaCtrl *>(scratch);
    int32_t *fa = reinterpret_cast<int32_t *>(scratch + NA_CTRL);
    int32_t *fb = fa + DDP_NOALLOC_MAX_NODES;
    GridBarrier bar{&c->bar_count, &c->bar_gen};
    const int rank = blockIdx.x * blockDim.x + threadIdx.x;
    const int size = gridDim.x * blockDim.x;

    for (int i = rank; i < n; i += size) hops[i] = -1;
    grid_sync(bar, gridDim.x, &c->status);
    if (rank == 0) {
        hops[target] = 0;
        fa[0] = target;
    }
    grid_sync(bar, gridDim.x, &c->status);
    int nf = 1, lvl = 0, it = 0;
    while (nf > 0) {
        const int PH = (it + 1) & 3, RS = (it + 3) & 3;
        for (int i = rank; i < nf; i += size) {
            const int u = __ldcg(fa + i);
            const int b = __ldg(roff + u), e = __ldg(roff + u + 1);
            for (int j = b; j < e; j++) {
                const int p = __ldg(rsrc + j);
                if (p < 0 || p >= n) continue;
                if (__ldcg(hops + p) == -1 && atomicCAS(hops + p, -1, lvl + 1) == -1) {
                    const int slot = atomicAdd(&c->cnt[PH], 1);
                    if (slot < DDP_NOALLOC_MAX_NODES) fb[slot] = p;  // each node claimed once
                }
            }
        }
        grid_sync(bar, gridDim.x, &c->status);
        if (rank == 0) c->cnt[RS] = 0;
        nf = *(volatile int *)&c->cnt[PH];
        const int st = *(volatile int *)&c->status;
        int32_t *t = fa;
        fa = fb;
        fb = t;
        lvl++;
        it++;
        if (st & ST_TIMEOUT) break;
    }
}

}  // namespace
}  // namespace ddp

using namespace ddp;

extern "C" int ddp_bfs_hops_noalloc(int32_t n, const int32_t *d_rev_offsets,
                                    const int32_t *d_rev_sources, int32_t target,
                                    int32_t *d_hops, void *stream) {
    if (n < 1 || n > DDP_NOALLOC_MAX_NODES)
        return fail(DDP_ERR_INVALID, "ddp_bfs_hops_noalloc: n must be in [1, DDP_NOALLOC_MAX_NODES]");
    if (!d_rev_offsets || !d_rev_sources || !d_hops)
        return fail(DDP_ERR_INVALID, "ddp_bfs_hops_noalloc: null device pointer");
    if (target < 0 || target >= n) return fail(DDP_ERR_INVALID, "ddp_bfs_hops_noalloc: target out of range");
    int dev = 0;
    DDP_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(DDP_ERR_INVALID, "ddp_bfs_hops_noalloc: device index >= 64");
    void *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (!g_na_ptr[dev]) {
            // first call on this device (it is current): look up the array's
            // device address once
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
            g_na_ptr[dev] = p;
        }
        scratch = g_na_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    // the array keeps the previous call's contents: zero the control words
    DDP_CUDA(cudaMemsetAsync(scratch, 0, NA_CTRL, st));
    int per_sm = 0, sms = 0;
    DDP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bfs_noalloc, NA_BLOCK, 0));
    DDP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int grid = per_sm * sms;
    if (grid < 1) grid = 1;
    unsigned char *sp = static_cast<unsigned char *>(scratch);
    void *args[] = {&n, &d_rev_offsets, &d_rev_sources, &target, &d_hops, &sp};
    DDP_CUDA(cudaLaunchCooperativeKernel((const void *)k_bfs_noalloc, dim3(grid), dim3(NA_BLOCK), args, 0, st));
    int status = 0;
    DDP_CUDA(cudaMemcpyAsync(&status, static_cast<unsigned char *>(scratch) + offsetof(NaCtrl, status),
                             sizeof(int), cudaMemcpyDeviceToHost, st));
    DDP_CUDA(cudaStreamSynchronize(st));
    if (status & ST_TIMEOUT) return fail(DDP_ERR_TIMEOUT, "ddp_bfs_hops_noalloc: barrier wait timed out");
    return DDP_OK;
}
