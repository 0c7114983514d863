// The small kernels around a search launch (reset, seed, collect), compiled
// once for the batched and the served forms.
#include "search_kernels.cuh"

namespace gh {
namespace search {
namespace {

// blockIdx.y = instance, blockIdx.x = slice of its arrays.
__global__ void k_search_fill(Inst* insts, const int* ids, int B) {
    const Inst* in = insts + (ids ? ids[blockIdx.y] : static_cast<int>(blockIdx.y));
    fill_instance(in, B, static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x,
                  static_cast<size_t>(gridDim.x) * blockDim.x);
}

__global__ void k_search_seed(Inst* insts, const int* ids, int count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        seed_instance(insts + (ids ? ids[i] : i));
}

// One block per listed instance.
__global__ void k_search_collect(Inst* insts, const int* ids, int final, int batchSize) {
    collect_instance(insts + (ids ? ids[blockIdx.x] : static_cast<int>(blockIdx.x)), final, batchSize);
}

}  // namespace

cudaError_t search_fill(Inst* insts, const int* ids, int count, int batchSize, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    k_search_fill<<<dim3(8, static_cast<unsigned>(count)), 256, 0, s>>>(insts, ids, batchSize);
    gh::impl::count_launch();
    return cudaGetLastError();
}

cudaError_t search_seed(Inst* insts, const int* ids, int count, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    k_search_seed<<<(count + 127) / 128, 128, 0, s>>>(insts, ids, count);
    gh::impl::count_launch();
    return cudaGetLastError();
}

cudaError_t search_collect(Inst* insts, const int* ids, int count, int final, int batchSize, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    k_search_collect<<<static_cast<unsigned>(count), 256, 0, s>>>(insts, ids, final, batchSize);
    gh::impl::count_launch();
    return cudaGetLastError();
}

}  // namespace search
}  // namespace gh
