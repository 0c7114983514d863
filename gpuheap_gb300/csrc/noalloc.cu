// gh_sort_noalloc: the plain heap-sort with its heap in a fixed device array
// of this library instead of memory from cudaMalloc.
//
// Who needs it: code that cannot allocate device memory at the moment it
// sorts -- a caller inside a framework whose caching allocator has already
// reserved the GPU's memory (cudaMalloc then fails or fragments the pool),
// and latency-critical callers that cannot pay cudaMalloc/cudaFree's implicit
// device synchronization between steps.  They pass only the input and output
// buffers; everything else lives in kNoAllocScratchBytes of static device
// memory that every GPU using this library holds until the process exits.
#include <cuda_runtime.h>

#include <climits>
#include <cstdio>
#include <cstring>

#include "gpuheap.h"
#include "heap_launch.cuh"
#include "trace.cuh"

namespace {

// 16 MiB: the heap's nodes, lock words and counters for one sort.
constexpr size_t kNoAllocScratchBytes = size_t{16} << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Device address of the array on the current device (the host-side symbol
// is only a stand-in and must never reach a kernel).  Looked up on every
// call, with the device current: a cached address would dangle after a
// device reset reloads the module, and the lookup costs little next to a sort.
gh_status scratch_for_current_device(void** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        std::fprintf(stderr, "gpuheap: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
        return GH_ERR_CUDA;
    }
    *out = p;
    return GH_OK;
}

template <typename K>
cudaError_t run_sort(const gh::impl::Desc& d, const void* in, long long n, void* out, int threads, int grid,
                     cudaStream_t s) {
    const size_t keys = static_cast<size_t>(d.batchNum + 1) * d.batchSize;
    K lim;
    std::memcpy(&lim, &d.initBits, sizeof(K));
    // every call starts from a clean heap: the array keeps the previous call's contents
    gh::impl::k_fill<K><<<grid * 4, 256, 0, s>>>(static_cast<K*>(d.items), keys, lim);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(d.status, 0, sizeof(int) * (static_cast<size_t>(d.batchNum) + 2), s);
    if (e != cudaSuccess) return e;
    gh::impl::k_init_state<<<1, 32, 0, s>>>(d.state, 0);
    gh::impl::k_set_output<<<1, 32, 0, s>>>(d.state, 0, static_cast<int>(n));
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const gh::impl::LaunchArgs a{&d, threads, grid, s, nullptr};
    e = gh::impl::launch_insert<K>(a, static_cast<const K*>(in), n, d.batchSize);
    if (e != cudaSuccess) return e;
    return gh::impl::launch_erase<K>(a, static_cast<K*>(out));
}

}  // namespace

extern "C" gh_status gh_sort_noalloc(int key_kind, int variant, int partial_buffer, int batch_size,
                                     const void* in_dev, long long n, void* out_dev, void* stream) {
    gh::trace::Range range_("gh_sort_noalloc");
    if (key_kind < GH_KEY_U32 || key_kind > GH_KEY_U64) return GH_ERR_INVALID;
    if (variant != GH_TOPDOWN && variant != GH_BOTTOMUP) return GH_ERR_INVALID;
    if (batch_size < 16 || batch_size > 4096 || (batch_size & (batch_size - 1))) return GH_ERR_INVALID;
    if (n < 0 || (n > 0 && (!in_dev || !out_dev))) return GH_ERR_INVALID;
    // without the partial buffer a short last batch is padded to a full node
    // and its keys come out only with that padding, past out_dev's n keys
    if (!partial_buffer && n % batch_size != 0) {
        std::fprintf(stderr, "gpuheap: gh_sort_noalloc: without the partial buffer n (%lld) must be a multiple of "
                             "batch_size (%d)\n", n, batch_size);
        return GH_ERR_INVALID;
    }
    if (n == 0) return GH_OK;
    const int kb = key_kind == GH_KEY_U64 ? 8 : 4;
    const long long nodes = (n + batch_size - 1) / batch_size;  // full nodes a sort of n keys can hold
    if (nodes > INT_MAX / 4) return GH_ERR_CAPACITY;
    const int batchNum = static_cast<int>(nodes < 1 ? 1 : nodes);
    const size_t itemBytes = align_up(static_cast<size_t>(batchNum + 1) * batch_size * kb, 256);
    const size_t statusBytes = align_up(sizeof(int) * (static_cast<size_t>(batchNum) + 2), 256);
    const size_t need = itemBytes + statusBytes + sizeof(gh::HeapState);
    if (need > kNoAllocScratchBytes) {
        std::fprintf(stderr,
                     "gpuheap: gh_sort_noalloc: %lld keys need %zu bytes of heap, above its fixed %zu bytes\n", n,
                     need, kNoAllocScratchBytes);
        return GH_ERR_CAPACITY;
    }
    void* base = nullptr;
    gh_status st = scratch_for_current_device(&base);
    if (st != GH_OK) return st;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return GH_ERR_CUDA;

    gh::impl::Desc d{};
    d.items = base;
    d.status = reinterpret_cast<int*>(static_cast<unsigned char*>(base) + itemBytes);
    d.state = reinterpret_cast<gh::HeapState*>(static_cast<unsigned char*>(base) + itemBytes + statusBytes);
    d.initBits = key_kind == GH_KEY_U32 ? 0xffffffffull : key_kind == GH_KEY_I32 ? 0x7fffffffull : ~0ull;
    d.batchNum = batchNum;
    d.batchSize = batch_size;
    d.timeoutNs = 20000000000LL;
    d.variant = variant;
    d.pb = partial_buffer ? 1 : 0;
    d.keyBytes = kb;
    // threads as gh_heap_create's default: 16-byte merge runs per thread
    int ipt = 16 / kb, threads = 2 * batch_size / ipt;
    while (threads > 1024 && ipt < 8) { threads >>= 1; ipt <<= 1; }
    while (threads < 32 && ipt > 1) { threads <<= 1; ipt >>= 1; }

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (key_kind == GH_KEY_U32) e = run_sort<uint32_t>(d, in_dev, n, out_dev, threads, sms, s);
    else if (key_kind == GH_KEY_I32) e = run_sort<int32_t>(d, in_dev, n, out_dev, threads, sms, s);
    else e = run_sort<uint64_t>(d, in_dev, n, out_dev, threads, sms, s);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "gpuheap: gh_sort_noalloc: %s\n", cudaGetErrorString(e));
        return GH_ERR_CUDA;
    }
    int tail[2] = {0, 0};  // deleteCount, err
    e = cudaMemcpyAsync(&tail[0], &d.state->deleteCount, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&tail[1], &d.state->err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return GH_ERR_CUDA;
    if (tail[1] == gh::kErrTimeout) return GH_ERR_TIMEOUT;
    if (tail[1] != 0) return GH_ERR_STATE;
    return tail[0] == n ? GH_OK : GH_ERR_STATE;
}
