/* GPU_Graph<T> (LIB/include/graph.cuh:12-89): the Graph copied to the
 * device.  Like the reference it aliases the host arrays and shadows
 * get_offsets / get_edges with device pointers, plus get_weight()
 * (singular) for the device weights; __gpu_free() releases them.  It also
 * holds the engine's device-resident graph (ddp_handle()), which
 * GPU_A_Star searches. */
#ifndef DDP_LIB_GRAPH_CUH
#define DDP_LIB_GRAPH_CUH

#include <cuda_runtime.h>

#include "ddp_lib_detail.h"
#include "graph.h"

template <class T>
class GPU_Graph : public Graph<T> {
   private:
    int *d_offsets = nullptr;
    int *d_edges = nullptr;
    T *d_weights = nullptr;
    ddp_graph *handle = nullptr;

    static void cuda_check(cudaError_t e) {
        if (e != cudaSuccess) {
            std::fprintf(stderr, "[ddp] CUDA error: %s\n", cudaGetErrorString(e));
            std::exit((int)e);
        }
    }

   public:
    GPU_Graph() {}
    GPU_Graph(Graph<T> *cpu) {
        this->N = cpu->N;
        this->E = cpu->E;
        this->offsets = cpu->offsets;
        this->edges = cpu->edges;
        this->weights = cpu->weights;
        __gpu_alloc();
    }

    void __gpu_alloc() {
        const size_t n = this->N, e = this->E;
        cuda_check(cudaMalloc(&d_offsets, sizeof(int) * (n ? n : 1)));
        cuda_check(cudaMalloc(&d_edges, sizeof(int) * (e ? e : 1)));
        cuda_check(cudaMalloc(&d_weights, sizeof(T) * (e ? e : 1)));
        cuda_check(cudaMemcpy(d_offsets, this->offsets, sizeof(int) * n, cudaMemcpyHostToDevice));
        if (e) {
            cuda_check(cudaMemcpy(d_edges, this->edges, sizeof(int) * e, cudaMemcpyHostToDevice));
            cuda_check(cudaMemcpy(d_weights, this->weights, sizeof(T) * e, cudaMemcpyHostToDevice));
        }
        handle = ddp_lib::upload((int)this->N, (int)this->E, this->offsets, this->edges, this->weights);
    }

    void __gpu_free() {
        cudaFree(d_offsets);
        cudaFree(d_edges);
        cudaFree(d_weights);
        d_offsets = d_edges = nullptr;
        d_weights = nullptr;
        if (handle) ddp_graph_free(handle);
        handle = nullptr;
    }

    int *get_offsets() { return d_offsets; }
    int *get_edges() { return d_edges; }
    T *get_weight() { return d_weights; }
    ddp_graph *ddp_handle() const { return handle; }
};

#endif
