// The heap's block primitives as entry points of their own, so that tests
// can check them in isolation against a sort: the two-batch merge that every
// insert and sift step uses (merge path per thread, gh::detail::merge_split_t),
// the owner-mode delete's warp-window merge (ballot split, bitonic network,
// shared-memory transposes; owner_delete.cuh) and the bitonic sort of an
// insert batch (gh::detail::bitonic_sort).  The reference tests its
// counterparts, imergePath and ibitonicSort (heap/heaputil.cuh:23-47,
// 99-158), with local_test/merge_path over batch 32..2048 x block
// 32..min(batch, 1024).
#include <cuda_runtime.h>

#include <cstdint>

#include "gpuheap.h"
#include "owner_delete.cuh"

namespace {

template <typename K>
__global__ void __launch_bounds__(1024) k_merge_path(const K* a, const K* b, int n, K* lo, K* hi) {
    extern __shared__ __align__(16) unsigned char sm[];
    K* sa = reinterpret_cast<K*>(sm);
    K* sb = sa + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        sa[i] = a[i];
        sb[i] = b[i];
    }
    __syncthreads();
    gh::detail::merge_split_rt<K>(sa, sb, lo, hi, n, threadIdx.x, 2 * n / static_cast<int>(blockDim.x));
}

template <typename K>
__global__ void __launch_bounds__(1024) k_merge_windows(const K* a, const K* b, int n, K* lo, K* hi) {
    constexpr int IPT = gh::impl::owner_ipt(sizeof(K));
    constexpr int S = 32 * IPT;
    constexpr int kScr = IPT == 32 ? 32 * 33 : 0;
    extern __shared__ __align__(16) unsigned char sm[];
    K* sa = reinterpret_cast<K*>(sm);
    K* sb = sa + n;
    K* scr = sb + n + (threadIdx.x >> 5) * kScr;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        sa[i] = a[i];
        sb[i] = b[i];
    }
    __syncthreads();
    // each warp merges its windows; the outputs go to global memory, so no
    // barrier is needed between a window's reads and its stores
    for (int w = threadIdx.x >> 5; w < 2 * n / S; w += blockDim.x >> 5) {
        K m[IPT];
        gh::impl::ow::window<K, IPT>(sa, sb, n, w * S, m, scr);
        gh::impl::ow::window_store<K, IPT>(lo, hi, n, w * S, m, scr);
        __syncwarp();
    }
}

template <typename K>
__global__ void __launch_bounds__(1024) k_sort_batch(const K* in, int n, K* out) {
    extern __shared__ __align__(16) unsigned char sm[];
    K* s = reinterpret_cast<K*>(sm);
    for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = in[i];
    __syncthreads();
    gh::detail::bitonic_sort(s, n);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = s[i];
}

bool pow2(int x) { return x > 0 && (x & (x - 1)) == 0; }
int key_bytes(int kind) { return kind == GH_KEY_U64 ? 8 : 4; }

gh_status launched(cudaError_t e) {
    if (e == cudaSuccess) e = cudaGetLastError();
    gh::impl::count_launch();
    return e == cudaSuccess ? GH_OK : GH_ERR_CUDA;
}

template <typename K>
gh_status merge_t(int method, const void* a, const void* b, int n, void* lo, void* hi, int threads, cudaStream_t s) {
    const K* ka = static_cast<const K*>(a);
    const K* kb = static_cast<const K*>(b);
    K* klo = static_cast<K*>(lo);
    K* khi = static_cast<K*>(hi);
    if (method == 0) {
        const size_t smem = 2 * static_cast<size_t>(n) * sizeof(K);
        cudaError_t e = cudaFuncSetAttribute(k_merge_path<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return GH_ERR_CUDA;
        k_merge_path<K><<<1, threads, smem, s>>>(ka, kb, n, klo, khi);
        return launched(cudaSuccess);
    }
    const size_t scr = gh::impl::owner_scratch(sizeof(K));
    const size_t smem = 2 * static_cast<size_t>(n) * sizeof(K) + (threads / 32) * scr;
    cudaError_t e = cudaFuncSetAttribute(k_merge_windows<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return GH_ERR_CUDA;
    k_merge_windows<K><<<1, threads, smem, s>>>(ka, kb, n, klo, khi);
    return launched(cudaSuccess);
}

template <typename K>
gh_status sort_t(const void* in, int n, void* out, int threads, cudaStream_t s) {
    const size_t smem = static_cast<size_t>(n) * sizeof(K);
    cudaError_t e = cudaFuncSetAttribute(k_sort_batch<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return GH_ERR_CUDA;
    k_sort_batch<K><<<1, threads, smem, s>>>(static_cast<const K*>(in), n, static_cast<K*>(out));
    return launched(cudaSuccess);
}

}  // namespace

extern "C" gh_status gh_merge_batches(int key_kind, int method, const void* a_dev, const void* b_dev, int n,
                                      void* lo_dev, void* hi_dev, int threads, void* stream) {
    if (key_kind < GH_KEY_U32 || key_kind > GH_KEY_U64 || (method != 0 && method != 1)) return GH_ERR_INVALID;
    if (!pow2(n) || n < 16 || n > 8192 || !pow2(threads) || threads < 32 || threads > 1024) return GH_ERR_INVALID;
    if (!a_dev || !b_dev || !lo_dev || !hi_dev) return GH_ERR_INVALID;
    const int kb = key_bytes(key_kind);
    if (method == 0) {
        const int ipt = 2 * n / threads;
        if (ipt < 1 || ipt > 16) return GH_ERR_INVALID;  // keys per thread of the merge path: 1..16
    } else {
        const int S = 32 * gh::impl::owner_ipt(kb);
        if (2 * n < S) return GH_ERR_INVALID;  // at least one whole window
        if (2 * static_cast<size_t>(n) * kb + (threads / 32) * gh::impl::owner_scratch(kb) > 227 * 1024)
            return GH_ERR_INVALID;
    }
    if (2 * static_cast<size_t>(n) * kb > 227 * 1024) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (key_kind == GH_KEY_U32) return merge_t<uint32_t>(method, a_dev, b_dev, n, lo_dev, hi_dev, threads, s);
    if (key_kind == GH_KEY_I32) return merge_t<int32_t>(method, a_dev, b_dev, n, lo_dev, hi_dev, threads, s);
    return merge_t<uint64_t>(method, a_dev, b_dev, n, lo_dev, hi_dev, threads, s);
}

extern "C" gh_status gh_sort_batch(int key_kind, const void* in_dev, int n, void* out_dev, int threads, void* stream) {
    if (key_kind < GH_KEY_U32 || key_kind > GH_KEY_U64) return GH_ERR_INVALID;
    if (!pow2(n) || n < 2 || n > 8192 || !pow2(threads) || threads < 32 || threads > 1024) return GH_ERR_INVALID;
    if (!in_dev || !out_dev) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (key_kind == GH_KEY_U32) return sort_t<uint32_t>(in_dev, n, out_dev, threads, s);
    if (key_kind == GH_KEY_I32) return sort_t<int32_t>(in_dev, n, out_dev, threads, s);
    return sort_t<uint64_t>(in_dev, n, out_dev, threads, s);
}
