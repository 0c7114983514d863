// Single-source shortest paths with the batched priority queue, and the
// R-MAT generator of its synthetic graphs.
//
// The caller pattern of applications/sssp_longfei_new/sssp.cu:19-132 (take a
// batch of (dist << 32 | vertex) keys, drop stale ones, relax the edges of
// the rest with atomicMin, insert the improved keys), written against this
// repository's device API (gh::Heap<uint64_t, ...>::deleteMin -- deleteRoot
// + deleteUpdate in one call -- and insertion) instead of that application's
// own heap.  Keys
// come out close to key order but not strictly (many blocks work at once), so
// a vertex can be improved after it was expanded; it is then re-inserted and
// expanded again (label correcting), and the final distances equal
// Dijkstra's.
#include <cuda_runtime.h>

#include <climits>
#include <cstdio>
#include <cstring>

#include "gpuheap.h"
#include "heap_launch.cuh"
#include "sssp_relax.cuh"
#include "worklist.cuh"
#include "trace.cuh"

struct gh_heap;  // defined in capi.cu; reached through gh_heap_device_view

namespace {

using u64 = unsigned long long;

__device__ __forceinline__ u64 mix64(u64 z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// R-MAT edge e: `scale` quadrant choices with probabilities (a, b, c, 1-a-b-c),
// one counter-based draw per (edge, level); weight uniform in [1, wmax].
__global__ void k_rmat(int scale, long long m, double a, double b, double c, u64 seed, unsigned wmax, int* src,
                       int* dst, unsigned* w) {
    for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < m;
         e += static_cast<long long>(gridDim.x) * blockDim.x) {
        unsigned s = 0, d = 0;
        for (int l = 0; l < scale; ++l) {
            const u64 r = mix64(seed + (static_cast<u64>(e) * 64 + l + 1) * 0x9e3779b97f4a7c15ULL);
            const double u = static_cast<double>(r >> 11) * (1.0 / 9007199254740992.0);
            const unsigned bs = u >= a + b ? 1u : 0u;
            const unsigned bd = (u >= a && u < a + b) || u >= a + b + c ? 1u : 0u;
            s = (s << 1) | bs;
            d = (d << 1) | bd;
        }
        src[e] = static_cast<int>(s);
        dst[e] = static_cast<int>(d);
        w[e] = 1u + static_cast<unsigned>(mix64((seed ^ 0xa5a5a5a5a5a5a5a5ULL) + (static_cast<u64>(e) + 1) *
                                                 0x9e3779b97f4a7c15ULL) % wmax);
    }
}

__global__ void k_sssp_init(unsigned* dist, int n, int source, gh::HeapState* st) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        dist[v] = v == source ? 0u : 0xffffffffu;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->busy = 1;  // block 0 holds the seed until it is inserted
}

// Shared memory of one block, ahead of the heap's own region.
struct SsspSmem {
    static __host__ __device__ size_t bytes(int B) {
        return static_cast<size_t>(B) * 8        // batch taken from the heap
               + 2 * static_cast<size_t>(B) * 8  // keys waiting to be inserted
               + (static_cast<size_t>(B) + 1) * 8 // degree prefix
               + 32 * 8 + 32;                     // warp sums, control words
    }
};

template <typename H>
__global__ void __launch_bounds__(1024) k_sssp(H heap, const long long* __restrict__ rowptr,
                                               const int* __restrict__ col, const unsigned* __restrict__ wt,
                                               unsigned* dist, int source) {
    static_assert(sizeof(typename H::key_type) == 8, "SSSP keys are dist << 32 | vertex");
    extern __shared__ __align__(16) unsigned char smem[];
    const int B = heap.batchSize;
    const int tid = threadIdx.x;
    u64* batch = reinterpret_cast<u64*>(smem);
    u64* emit = batch + B;
    long long* pre = reinterpret_cast<long long*>(emit + 2 * B);
    long long* wsum = pre + B + 1;
    int* ctl = reinterpret_cast<int*>(wsum + 32);
    const int heapOff = static_cast<int>(SsspSmem::bytes(B) / 4);
    gh::HeapState* st = heap.state;

    if (tid == 0) { ctl[0] = 0; ctl[1] = 0; }
    __syncthreads();
    if (blockIdx.x == 0 && source >= 0) {
        if (tid == 0) emit[0] = static_cast<u64>(source);  // distance 0
        __syncthreads();
        gh::app::insert_keys(heap, emit, 1, heapOff);
        __syncthreads();
        gh::app::batch_done(st);
    }
    u64 pops = 0, edges = 0, inserted = 0;
    unsigned long long waitStart = 0;
    int lastBusy = -1;
    for (;;) {
        if (gh::app::wait_for_keys(heap, &ctl[2], nullptr, lastBusy, waitStart)) break;
        const int size = gh::app::take_batch(heap, batch, heapOff);
        if (size == 0) {  // another block took the last keys first
            gh::app::batch_done(st);
            if (heap.failed()) break;
            continue;
        }
        pops += size;
        gh::app::sssp_relax_batch(heap, batch, size, pre, wsum, emit, &ctl[1], rowptr, col, wt, dist, heapOff, edges,
                                  inserted);
        gh::app::batch_done(st);
        if (heap.failed()) break;
    }
    if (tid == 0) {
        atomicAdd(&st->appStats[0], pops);
        atomicAdd(&st->appStats[1], edges);
        atomicAdd(&st->appStats[2], inserted);
    }
}

template <int V, int IPT>
cudaError_t launch_sssp(const void* viewBytes, int blocks, int threads, size_t smem, const long long* rowptr,
                        const int* col, const unsigned* w, unsigned* dist, int source, cudaStream_t s) {
    using H = gh::Heap<uint64_t, V, true, IPT>;
    H h;
    std::memcpy(&h, viewBytes, sizeof(H) <= 64 ? sizeof(H) : 64);
    cudaError_t e = cudaFuncSetAttribute(k_sssp<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    k_sssp<H><<<blocks, threads, smem, s>>>(h, rowptr, col, w, dist, source);
    gh::impl::count_launch();
    return cudaGetLastError();
}

}  // namespace

extern "C" gh_status gh_rmat_edges(int scale, long long m, double a, double b, double c, unsigned long long seed,
                                   unsigned max_weight, int* src_dev, int* dst_dev, unsigned* w_dev, void* stream) {
    if (scale < 1 || scale > 30 || m < 0 || max_weight < 1 || !(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0))
        return GH_ERR_INVALID;
    if (m == 0) return GH_OK;
    if (!src_dev || !dst_dev || !w_dev) return GH_ERR_INVALID;
    k_rmat<<<1024, 256, 0, static_cast<cudaStream_t>(stream)>>>(scale, m, a, b, c, seed, max_weight, src_dev, dst_dev,
                                                                 w_dev);
    gh::impl::count_launch();
    return cudaGetLastError() == cudaSuccess ? GH_OK : GH_ERR_CUDA;
}

extern "C" gh_status gh_sssp(gh_heap* h, int n, const long long* rowptr_dev, const int* col_dev, const unsigned* w_dev,
                             int source, unsigned* dist_dev, void* stream, unsigned long long* stats_host) {
    gh::trace::Range range_("gh_sssp");
    if (!h || n < 1 || !rowptr_dev || !col_dev || !w_dev || !dist_dev || source < 0 || source >= n) return GH_ERR_INVALID;
    int kind = 0, variant = 0, pb = 0, bn = 0, B = 0, threads = 0, grid = 0;
    gh_status st = gh_heap_info(h, &kind, &variant, &pb, &bn, &B, &threads, &grid);
    if (st != GH_OK) return st;
    if (kind != GH_KEY_U64 || !pb || threads > B) return GH_ERR_INVALID;  // emit buffer holds B + threads keys
    unsigned char view[64];
    st = gh_heap_device_view(h, view, sizeof(view));
    if (st != GH_OK) return st;
    gh::HeapState* hs = nullptr;
    std::memcpy(&hs, view + 16, sizeof(hs));  // Heap<K,...>: heapItems, status, state, ...
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    st = gh_heap_reset(h, stream);
    if (st != GH_OK) return st;
    k_sssp_init<<<256, 256, 0, s>>>(dist_dev, n, source, hs);
    gh::impl::count_launch();
    const size_t smem = SsspSmem::bytes(B) + 16 + gh::Heap<uint64_t, 0, true>::smemBytes(B);
    const int ipt = 2 * B / threads;
    cudaError_t e = cudaErrorInvalidValue;
    if (variant == GH_TOPDOWN) {
        if (ipt == 2) e = launch_sssp<gh::kTopDown, 2>(view, grid, threads, smem, rowptr_dev, col_dev, w_dev, dist_dev, source, s);
        if (ipt == 4) e = launch_sssp<gh::kTopDown, 4>(view, grid, threads, smem, rowptr_dev, col_dev, w_dev, dist_dev, source, s);
        if (ipt == 8) e = launch_sssp<gh::kTopDown, 8>(view, grid, threads, smem, rowptr_dev, col_dev, w_dev, dist_dev, source, s);
    } else {
        if (ipt == 2) e = launch_sssp<gh::kBottomUp, 2>(view, grid, threads, smem, rowptr_dev, col_dev, w_dev, dist_dev, source, s);
        if (ipt == 4) e = launch_sssp<gh::kBottomUp, 4>(view, grid, threads, smem, rowptr_dev, col_dev, w_dev, dist_dev, source, s);
        if (ipt == 8) e = launch_sssp<gh::kBottomUp, 8>(view, grid, threads, smem, rowptr_dev, col_dev, w_dev, dist_dev, source, s);
    }
    if (e != cudaSuccess) {
        std::fprintf(stderr, "gpuheap: gh_sssp launch: %s\n", cudaGetErrorString(e));
        return GH_ERR_CUDA;
    }
    gh::HeapState out;
    if (cudaMemcpyAsync(&out, hs, sizeof(out), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GH_ERR_CUDA;
    if (stats_host) {
        stats_host[0] = out.appStats[0];
        stats_host[1] = out.appStats[1];
        stats_host[2] = out.appStats[2];
    }
    if (out.err == gh::kErrTimeout) return GH_ERR_TIMEOUT;
    if (out.err == gh::kErrCapacity) return GH_ERR_CAPACITY;
    if (out.err) return GH_ERR_STATE;
    if (out.batchCount != 0 || out.partialBufferSize != 0) return GH_ERR_STATE;
    return GH_OK;
}
