// Seeded synthetic keys for the plain heap-sort workload, generated on the
// device.  Key i of a stream is a function of (seed, i) only -- the
// splitmix64 finaliser (Steele, Lea, Flood, OOPSLA 2014) applied to
// seed + (i + 1) * golden-ratio increment -- so any slice can be made
// independently and the CPU oracle can restate it exactly.
//   uniform: u32 in [0, 2^32 - 2] (UINT32_MAX is the padding key)
//   zipf:    rank r in [1, 2^16] by inverse CDF of Zipf(1.2) (computed on
//            the host with std::pow), scattered over the key space by a 32-bit
//            bijection (xor-shift / odd-multiply rounds) with cycle-walking
//            away from 0xffffffff
//   u64 keys are (u32 key << 32) | input index; i32 keys are u32 - 2^31.
// Sorted and reverse inputs are uniform keys sorted by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "gpuheap.h"
#include "heap_kernels.cuh"

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint32_t scatter32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU;
    x ^= x >> 15; x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

__global__ void k_gen(int kind, int zipf, uint64_t seed, long long n, void* out, const double* cdf, int ncdf) {
    const uint32_t zsalt = static_cast<uint32_t>(mix64(seed ^ 0x5a17f00dULL));
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const uint64_t r = mix64(seed + (static_cast<uint64_t>(i) + 1) * 0x9e3779b97f4a7c15ULL);
        uint32_t k;
        if (zipf) {
            const double u = static_cast<double>(r >> 11) * (1.0 / 9007199254740992.0);
            int lo = 0, hi = ncdf;  // first index with cdf >= u
            while (lo < hi) {
                const int m = (lo + hi) >> 1;
                if (cdf[m] < u) lo = m + 1;
                else hi = m;
            }
            uint32_t rank = static_cast<uint32_t>(lo) + 1;
            if (rank > static_cast<uint32_t>(ncdf)) rank = ncdf;
            uint32_t x = scatter32(rank ^ zsalt);
            while (x == 0xffffffffU) x = scatter32(x);
            k = x;
        } else {
            k = static_cast<uint32_t>(((r >> 32) * 0xffffffffULL) >> 32);
        }
        if (kind == GH_KEY_U64) static_cast<uint64_t*>(out)[i] = (static_cast<uint64_t>(k) << 32) | (static_cast<uint64_t>(i) & 0xffffffffULL);
        else if (kind == GH_KEY_I32) static_cast<int32_t*>(out)[i] = static_cast<int32_t>(static_cast<int64_t>(k) - 2147483648LL);
        else static_cast<uint32_t*>(out)[i] = k;
    }
}

}  // namespace

extern "C" gh_status gh_gen_keys(int key_kind, int zipf, unsigned long long seed, long long n, void* out_dev,
                                 void* stream) {
    if (key_kind < GH_KEY_U32 || key_kind > GH_KEY_U64 || n < 0 || (n > 0 && !out_dev)) return GH_ERR_INVALID;
    if (n == 0) return GH_OK;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return GH_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    constexpr int kZipfValues = 1 << 16;
    double* cdf = nullptr;
    if (zipf) {
        // Zipf(1.2) over 2^16 ranks, accumulated in rank order on the host
        std::vector<double> h(kZipfValues);
        double acc = 0.0;
        for (int r = 1; r <= kZipfValues; ++r) { acc += std::pow(static_cast<double>(r), -1.2); h[r - 1] = acc; }
        for (double& c : h) c /= acc;
        if (cudaMalloc(&cdf, sizeof(double) * kZipfValues) != cudaSuccess) return GH_ERR_CUDA;
        if (cudaMemcpyAsync(cdf, h.data(), sizeof(double) * kZipfValues, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            cudaFree(cdf);
            return GH_ERR_CUDA;
        }
    }
    k_gen<<<sms * 8, 256, 0, s>>>(key_kind, zipf ? 1 : 0, seed, n, out_dev, cdf, kZipfValues);
    gh::impl::count_launch();
    cudaError_t e = cudaGetLastError();
    if (cdf) {
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        cudaFree(cdf);
    }
    return e == cudaSuccess ? GH_OK : GH_ERR_CUDA;
}
