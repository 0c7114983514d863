// C ABI of the GB300 batched priority queue (declared in include/gpuheap.h).
//
// The reference selects key type and variant at compile time
// (test/Makefile:10-20); here they are run-time fields of the handle and
// dispatch to template instantiations of gh::Heap<K, Variant, PartialBuffer>.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <new>

#include "gpuheap.h"
#include "heap_launch.cuh"
#include "trace.cuh"

using gh::impl::Desc;

std::atomic<long long> gh::impl::g_launches{0};

struct gh_heap {
    Desc d;
    int keyKind;
    int blockThreads;  // 0 = automatic
    int grid;          // 0 = one block per SM
    int device;
    int numSMs;
    gh::impl::CheckResult* check;  // device scratch for gh_heap_check
    int* opSize;                   // device word for gh_heap_delete_batch
    void* scratch;                 // one batch of keys for gh_heap_retrieve
    // gh_heap_sort_host: device staging buffers, a copy stream and its events
    void* stageIn = nullptr;
    void* stageOut = nullptr;
    size_t stageBytes = 0;
    cudaStream_t copyStream = nullptr;
    cudaEvent_t sortEv[2 * 8 + 2] = {};
};

namespace {

gh_status cuda_fail(cudaError_t e) {
    if (e == cudaSuccess) return GH_OK;
    std::fprintf(stderr, "gpuheap: CUDA error %s\n", cudaGetErrorString(e));
    return GH_ERR_CUDA;
}
#define GH_CUDA(call)                                          \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_);           \
    } while (0)

bool pow2(int x) { return x > 0 && (x & (x - 1)) == 0; }

int key_bytes(int kind) { return kind == GH_KEY_U64 ? 8 : 4; }

// Threads per block: merge runs of 16 bytes per thread (ipt = 2*B/T keys),
// moved into [32, 1024] threads and ipt in {1, 2, 4, 8}.
int auto_threads(int batchSize, int keyBytes) {
    int ipt = 16 / keyBytes;
    int t = 2 * batchSize / ipt;
    while (t > 1024 && ipt < 8) { t >>= 1; ipt <<= 1; }
    while (t < 32 && ipt > 1) { t <<= 1; ipt >>= 1; }
    return t;
}

int threads_of(const gh_heap* h) {
    return h->blockThreads ? h->blockThreads : auto_threads(h->d.batchSize, h->d.keyBytes);
}
int grid_of(const gh_heap* h) { return h->grid ? h->grid : h->numSMs; }

gh_status device_error(const gh_heap* h) {
    int err = 0;
    cudaError_t e = cudaMemcpy(&err, &h->d.state->err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e);
    switch (err) {
        case 0: return GH_OK;
        case gh::kErrCapacity: return GH_ERR_CAPACITY;
        case gh::kErrTimeout: return GH_ERR_TIMEOUT;
        default: return GH_ERR_STATE;
    }
}

gh::impl::LaunchArgs args_of(const gh_heap* h, cudaStream_t s) {
    return gh::impl::LaunchArgs{&h->d, threads_of(h), grid_of(h), s, h->opSize};
}

// Calls f(K{}) with the heap's key type.
template <typename F>
gh_status with_key(const gh_heap* h, F&& f) {
    cudaError_t e;
    switch (h->keyKind) {
        case GH_KEY_U32: e = f(uint32_t{}); break;
        case GH_KEY_I32: e = f(int32_t{}); break;
        default: e = f(uint64_t{}); break;
    }
    return cuda_fail(e);
}

gh_status fill_items(gh_heap* h, cudaStream_t s) {
    const size_t n = static_cast<size_t>(h->d.batchNum + 1) * h->d.batchSize;
    const int blocks = std::max(1, std::min<int>(h->numSMs * 8, static_cast<int>((n + 255) / 256)));
    switch (h->keyKind) {
        case GH_KEY_U32: {
            uint32_t v; std::memcpy(&v, &h->d.initBits, 4);
            gh::impl::k_fill<uint32_t><<<blocks, 256, 0, s>>>(static_cast<uint32_t*>(h->d.items), n, v);
    gh::impl::count_launch();
            break;
        }
        case GH_KEY_I32: {
            int32_t v; std::memcpy(&v, &h->d.initBits, 4);
            gh::impl::k_fill<int32_t><<<blocks, 256, 0, s>>>(static_cast<int32_t*>(h->d.items), n, v);
    gh::impl::count_launch();
            break;
        }
        default: {
            uint64_t v = h->d.initBits;
            gh::impl::k_fill<uint64_t><<<blocks, 256, 0, s>>>(static_cast<uint64_t*>(h->d.items), n, v);
    gh::impl::count_launch();
            break;
        }
    }
    GH_CUDA(cudaGetLastError());
    GH_CUDA(cudaMemsetAsync(h->d.status, 0, sizeof(int) * (static_cast<size_t>(h->d.batchNum) + 2), s));
    gh::impl::k_init_state<<<1, 32, 0, s>>>(h->d.state, 0);
    gh::impl::count_launch();
    GH_CUDA(cudaGetLastError());
    return GH_OK;
}

const char* kCheckText[] = {"ok",
                            "node lock word is not AVAIL",
                            "node keys are not sorted",
                            "node starts below the last key of its parent",
                            "partial buffer is not sorted",
                            "partial buffer lies below the root",
                            "partial buffer lock word is not AVAIL"};

}  // namespace

extern "C" {

const char* gh_status_string(gh_status s) {
    switch (s) {
        case GH_OK: return "ok";
        case GH_ERR_INVALID: return "invalid argument";
        case GH_ERR_CAPACITY: return "heap capacity exceeded";
        case GH_ERR_TIMEOUT: return "device wait timed out";
        case GH_ERR_CUDA: return "CUDA error";
        case GH_ERR_STATE: return "heap holds an earlier device error";
    }
    return "unknown status";
}

gh_status gh_heap_create(gh_heap** out, int key_kind, int variant, int partial_buffer, int batch_num, int batch_size,
                         const void* init_limits) {
    if (!out) return GH_ERR_INVALID;
    *out = nullptr;
    if (key_kind < GH_KEY_U32 || key_kind > GH_KEY_U64) return GH_ERR_INVALID;
    if (variant != GH_TOPDOWN && variant != GH_BOTTOMUP) return GH_ERR_INVALID;
    if (!pow2(batch_size) || batch_size < 16 || batch_size > 4096) return GH_ERR_INVALID;
    if (batch_num < 1 || batch_num > (INT_MAX / 2 - 2)) return GH_ERR_INVALID;
    const int kb = key_bytes(key_kind);
    if (gh_heap_smem_bytes(key_kind, batch_size) > 227ull * 1024) return GH_ERR_INVALID;

    gh_heap* h = new (std::nothrow) gh_heap();
    if (!h) return GH_ERR_INVALID;
    std::memset(h, 0, sizeof(*h));
    h->keyKind = key_kind;
    h->d.variant = variant;
    h->d.pb = partial_buffer ? 1 : 0;
    h->d.batchNum = batch_num;
    h->d.batchSize = batch_size;
    h->d.keyBytes = kb;
    h->d.ownerDepth = -1;
    h->d.timeoutNs = 2000000000LL;  // 2 s: bulk deletes queue for node 0 in order, bulk inserts reserve targets
    uint64_t bits = 0;
    if (init_limits) std::memcpy(&bits, init_limits, kb);
    else if (key_kind == GH_KEY_U32) bits = 0xffffffffull;
    else if (key_kind == GH_KEY_I32) bits = 0x7fffffffull;
    else bits = ~0ull;
    h->d.initBits = bits;

    auto fail = [&](gh_status st) { gh_heap_destroy(h); return st; };
    if (cudaGetDevice(&h->device) != cudaSuccess) return fail(GH_ERR_CUDA);
    if (cudaDeviceGetAttribute(&h->numSMs, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess) return fail(GH_ERR_CUDA);
    const size_t itemBytes = static_cast<size_t>(batch_num + 1) * batch_size * kb;
    if (cudaMalloc(&h->d.items, itemBytes) != cudaSuccess) { cudaGetLastError(); return fail(GH_ERR_CUDA); }
    if (cudaMalloc(&h->d.status, sizeof(int) * (static_cast<size_t>(batch_num) + 2)) != cudaSuccess) { cudaGetLastError(); return fail(GH_ERR_CUDA); }
    if (cudaMalloc(&h->d.state, sizeof(gh::HeapState)) != cudaSuccess) { cudaGetLastError(); return fail(GH_ERR_CUDA); }
    if (cudaMalloc(&h->check, sizeof(gh::impl::CheckResult)) != cudaSuccess) { cudaGetLastError(); return fail(GH_ERR_CUDA); }
    if (cudaMalloc(&h->opSize, sizeof(int)) != cudaSuccess) { cudaGetLastError(); return fail(GH_ERR_CUDA); }
    if (cudaMalloc(&h->scratch, static_cast<size_t>(batch_size) * kb) != cudaSuccess) { cudaGetLastError(); return fail(GH_ERR_CUDA); }
    if (gh::impl::owner_depth(batch_size, kb) > 0) {
        if (cudaMalloc(&h->d.mbox, gh::impl::mbox_bytes(batch_size, kb)) != cudaSuccess) { cudaGetLastError(); return fail(GH_ERR_CUDA); }
        if (cudaMemset(h->d.mbox, 0, sizeof(gh::impl::Mailbox)) != cudaSuccess) { cudaGetLastError(); return fail(GH_ERR_CUDA); }
    }
    gh_status st = fill_items(h, nullptr);
    if (st != GH_OK) return fail(st);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(GH_ERR_CUDA);
    *out = h;
    return GH_OK;
}

gh_status gh_heap_destroy(gh_heap* h) {
    if (!h) return GH_OK;
    if (h->d.items) cudaFree(h->d.items);
    if (h->d.status) cudaFree(h->d.status);
    if (h->d.state) cudaFree(h->d.state);
    if (h->check) cudaFree(h->check);
    if (h->opSize) cudaFree(h->opSize);
    if (h->scratch) cudaFree(h->scratch);
    if (h->d.mbox) cudaFree(h->d.mbox);
    if (h->stageIn) cudaFree(h->stageIn);
    if (h->stageOut) cudaFree(h->stageOut);
    for (cudaEvent_t e : h->sortEv)
        if (e) cudaEventDestroy(e);
    if (h->copyStream) cudaStreamDestroy(h->copyStream);
    delete h;
    return GH_OK;
}

gh_status gh_heap_reset(gh_heap* h, void* stream) {
    if (!h) return GH_ERR_INVALID;
    return fill_items(h, static_cast<cudaStream_t>(stream));
}

gh_status gh_heap_set_timeout(gh_heap* h, double seconds) {
    // at most 60 s: a bottom-up park (two waits) must end before 2^29 later
    // inserts could reuse its ticket
    if (!h || !(seconds > 0) || seconds > 60.0) return GH_ERR_INVALID;
    h->d.timeoutNs = static_cast<long long>(seconds * 1e9);
    return GH_OK;
}

gh_status gh_heap_set_block_threads(gh_heap* h, int threads) {
    if (!h) return GH_ERR_INVALID;
    if (threads != 0) {
        if (!pow2(threads) || threads < 32 || threads > 1024 || threads > 2 * h->d.batchSize) return GH_ERR_INVALID;
        const int ipt = 2 * h->d.batchSize / threads;
        if (ipt != 1 && ipt != 2 && ipt != 4 && ipt != 8) return GH_ERR_INVALID;
    }
    h->blockThreads = threads;
    return GH_OK;
}

gh_status gh_heap_set_owner_depth(gh_heap* h, int depth) {
    if (!h) return GH_ERR_INVALID;
    if (depth > 0) {
        const int wpm = 2 * h->d.batchSize / (32 * gh::impl::owner_ipt(h->d.keyBytes));
        if (!h->d.mbox || depth < 2 || depth > gh::impl::kOwnerMaxR || depth * wpm > gh::impl::kOwnerWarps ||
            gh::impl::owner_smem(h->d.batchSize, h->d.keyBytes, depth) > 227 * 1024)
            return GH_ERR_INVALID;
    } else if (depth < -1) {
        return GH_ERR_INVALID;
    }
    h->d.ownerDepth = depth;
    return GH_OK;
}

gh_status gh_heap_set_grid(gh_heap* h, int blocks) {
    if (!h || blocks < 0) return GH_ERR_INVALID;
    h->grid = blocks;
    return GH_OK;
}

gh_status gh_heap_insert(gh_heap* h, const void* keys_dev, long long n, int chunk, void* stream) {
    gh::trace::Range range_("gh_heap_insert");
    if (!h || n < 0 || (n > 0 && !keys_dev)) return GH_ERR_INVALID;
    if (chunk == 0) chunk = h->d.batchSize;
    if (chunk < 1 || chunk > h->d.batchSize) return GH_ERR_INVALID;
    if (n == 0) return GH_OK;
    const gh::impl::LaunchArgs a = args_of(h, static_cast<cudaStream_t>(stream));
    return with_key(h, [&](auto k) {
        using K = decltype(k);
        return gh::impl::launch_insert<K>(a, static_cast<const K*>(keys_dev), n, chunk);
    });
}

namespace {
// Bulk delete into out_dev in ascending order, stopping at max_keys, at an
// empty heap or (threshold != NULL) at a smallest key not below *threshold.
gh_status delete_bulk(gh_heap* h, void* out_dev, long long max_keys, const void* threshold, long long* n_out,
                      void* stream) {
    if (!h || max_keys < 0 || (max_keys > 0 && !out_dev)) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int lim = static_cast<int>(std::min<long long>(max_keys, INT_MAX));
    gh::impl::k_set_output<<<1, 32, 0, s>>>(h->d.state, 0, lim);
    gh::impl::count_launch();
    GH_CUDA(cudaGetLastError());
    if (max_keys > 0) {
        const gh::impl::LaunchArgs a = args_of(h, s);
        gh_status st = with_key(h, [&](auto k) {
            using K = decltype(k);
            K t{};
            if (threshold) std::memcpy(&t, threshold, sizeof(K));
            return gh::impl::launch_erase<K>(a, static_cast<K*>(out_dev), threshold ? &t : nullptr);
        });
        if (st != GH_OK) return st;
    }
    gh::impl::k_set_output<<<1, 32, 0, s>>>(h->d.state, -1, INT_MAX);
    gh::impl::count_launch();
    GH_CUDA(cudaGetLastError());
    if (n_out) {
        int dc = 0;
        GH_CUDA(cudaMemcpyAsync(&dc, &h->d.state->deleteCount, sizeof(int), cudaMemcpyDeviceToHost, s));
        GH_CUDA(cudaStreamSynchronize(s));
        *n_out = dc;
        return device_error(h);
    }
    return GH_OK;
}
}  // namespace

gh_status gh_heap_delete(gh_heap* h, void* out_dev, long long max_keys, long long* n_out, void* stream) {
    gh::trace::Range range_("gh_heap_delete");
    return delete_bulk(h, out_dev, max_keys, nullptr, n_out, stream);
}

gh_status gh_heap_delete_below(gh_heap* h, void* out_dev, long long max_keys, const void* threshold,
                               long long* n_out, void* stream) {
    gh::trace::Range range_("gh_heap_delete_below");
    if (!threshold) return GH_ERR_INVALID;
    return delete_bulk(h, out_dev, max_keys, threshold, n_out, stream);
}

gh_status gh_heap_gc(gh_heap* h, const void* threshold, long long* kept, void* stream) {
    gh::trace::Range range_("gh_heap_gc");
    if (!h) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the used nodes, after the stream's work (the reference's invalidFilter
    // reads batchCount the same way, artifacts/astar/gc.cuh:153-154)
    int cnt[2] = {0, 0};
    GH_CUDA(cudaMemcpyAsync(cnt, &h->d.state->batchCount, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
    GH_CUDA(cudaStreamSynchronize(s));
    static_assert(offsetof(gh::HeapState, partialBufferSize) == offsetof(gh::HeapState, batchCount) + sizeof(int),
                  "batchCount and partialBufferSize are adjacent");
    gh_status st = device_error(h);
    if (st != GH_OK) return st;
    const size_t held = static_cast<size_t>(cnt[0]) * h->d.batchSize + cnt[1];
    void* buf = nullptr;
    GH_CUDA(cudaMallocAsync(&buf, 16 + std::max<size_t>(held, 1) * h->d.keyBytes, s));
    auto* keptDev = static_cast<unsigned long long*>(buf);
    void* scratch = static_cast<char*>(buf) + 16;
    st = GH_OK;
    cudaError_t e = cudaMemsetAsync(keptDev, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        const int blocks = std::max(1, std::min(h->numSMs * 8, cnt[0] + 1));
        const gh::impl::LaunchArgs a = args_of(h, s);
        st = with_key(h, [&](auto k) -> cudaError_t {
            using K = decltype(k);
            K t, fill;
            std::memcpy(&fill, &h->d.initBits, sizeof(K));
            if (threshold) std::memcpy(&t, threshold, sizeof(K));
            else t = fill;
            gh::impl::k_gc_compact<K><<<blocks, 256, 0, s>>>(static_cast<K*>(h->d.items), h->d.status, h->d.state,
                                                             h->d.batchSize, t, fill, static_cast<K*>(scratch), keptDev);
            gh::impl::count_launch();
            gh::impl::k_gc_reset<<<1, 1, 0, s>>>(h->d.state);
            gh::impl::count_launch();
            cudaError_t e2 = cudaGetLastError();
            if (e2 != cudaSuccess) return e2;
            return gh::impl::launch_insert_counted<K>(a, static_cast<const K*>(scratch), keptDev, h->d.batchSize);
        });
    } else {
        st = cuda_fail(e);
    }
    unsigned long long k = 0;
    if (st == GH_OK && kept) {
        e = cudaMemcpyAsync(&k, keptDev, sizeof(k), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) st = cuda_fail(e);
    }
    cudaError_t ef = cudaFreeAsync(buf, s);
    if (st != GH_OK) return st;
    GH_CUDA(ef);
    if (kept) {
        GH_CUDA(cudaStreamSynchronize(s));
        *kept = static_cast<long long>(k);
        return device_error(h);
    }
    return GH_OK;
}

gh_status gh_heap_concurrent(gh_heap* h, const void* keys_dev, long long n, int chunk, void* out_dev,
                             long long max_keys, long long* n_out, void* stream) {
    gh::trace::Range range_("gh_heap_concurrent");
    if (!h || n < 0 || (n > 0 && !keys_dev) || max_keys < 0 || (max_keys > 0 && !out_dev)) return GH_ERR_INVALID;
    if (chunk == 0) chunk = h->d.batchSize;
    if (chunk < 1 || chunk > h->d.batchSize) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    gh::impl::LaunchArgs a = args_of(h, s);
    if (a.grid < 2) a.grid = 2;  // one inserting and one deleting block at least
    const long long deletes = n / h->d.batchSize;
    const int lim = static_cast<int>(std::min<long long>(max_keys, INT_MAX));
    gh::impl::k_set_output<<<1, 32, 0, s>>>(h->d.state, 0, lim);
    gh::impl::count_launch();
    GH_CUDA(cudaGetLastError());
    if (n > 0) {
        gh_status st = with_key(h, [&](auto k) {
            using K = decltype(k);
            return gh::impl::launch_concurrent<K>(a, static_cast<const K*>(keys_dev), n, chunk, static_cast<K*>(out_dev),
                                                  max_keys > 0 ? deletes : 0);
        });
        if (st != GH_OK) return st;
    }
    gh::impl::k_set_output<<<1, 32, 0, s>>>(h->d.state, -1, INT_MAX);
    gh::impl::count_launch();
    GH_CUDA(cudaGetLastError());
    int dc = 0;
    GH_CUDA(cudaMemcpyAsync(&dc, &h->d.state->deleteCount, sizeof(int), cudaMemcpyDeviceToHost, s));
    GH_CUDA(cudaStreamSynchronize(s));
    if (n_out) *n_out = dc;
    return device_error(h);
}

gh_status gh_heap_insert_batch(gh_heap* h, const void* keys_dev, int size, void* stream) {
    if (!h || size < 0 || size > h->d.batchSize || (size > 0 && !keys_dev)) return GH_ERR_INVALID;
    if (size == 0) return GH_OK;
    gh::impl::LaunchArgs a = args_of(h, static_cast<cudaStream_t>(stream));
    a.grid = 1;
    a.reserve = false;  // one insertion() call, node 0 and all, as the reference makes it
    return with_key(h, [&](auto k) {
        using K = decltype(k);
        return gh::impl::launch_insert<K>(a, static_cast<const K*>(keys_dev), size, size);
    });
}

gh_status gh_heap_delete_batch(gh_heap* h, void* out_dev, int* size, void* stream) {
    if (!h || !out_dev) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const gh::impl::LaunchArgs a = args_of(h, s);
    gh_status st = with_key(h, [&](auto k) {
        using K = decltype(k);
        return gh::impl::launch_erase_one<K>(a, static_cast<K*>(out_dev));
    });
    if (st != GH_OK) return st;
    int sz = 0;
    GH_CUDA(cudaMemcpyAsync(&sz, h->opSize, sizeof(int), cudaMemcpyDeviceToHost, s));
    GH_CUDA(cudaStreamSynchronize(s));
    if (size) *size = sz;
    return device_error(h);
}

gh_status gh_heap_retrieve(gh_heap* h, void* out_dev, int size, int* n_out, void* stream) {
    gh::trace::Range range_("gh_heap_retrieve");
    if (!h || size < 0 || (size > 0 && !out_dev)) return GH_ERR_INVALID;
    if (!h->d.pb) return GH_ERR_INVALID;  // the remainder goes back through the partial buffer
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const gh::impl::LaunchArgs a = args_of(h, s);
    gh_status st = with_key(h, [&](auto k) {
        using K = decltype(k);
        return gh::impl::launch_retrieve<K>(a, static_cast<K*>(out_dev), size, static_cast<K*>(h->scratch));
    });
    if (st != GH_OK) return st;
    int got = 0;
    GH_CUDA(cudaMemcpyAsync(&got, h->opSize, sizeof(int), cudaMemcpyDeviceToHost, s));
    GH_CUDA(cudaStreamSynchronize(s));
    if (n_out) *n_out = got;
    return device_error(h);
}

gh_status gh_heap_sort(gh_heap* h, const void* in_dev, long long n, void* out_dev, void* stream) {
    gh::trace::Range range_("gh_heap_sort");
    if (!h || n < 0 || (n > 0 && (!in_dev || !out_dev))) return GH_ERR_INVALID;
    if (n > static_cast<long long>(h->d.batchNum) * h->d.batchSize) return GH_ERR_CAPACITY;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    gh_status st = fill_items(h, s);
    if (st != GH_OK) return st;
    st = gh_heap_insert(h, in_dev, n, h->d.batchSize, stream);
    if (st != GH_OK) return st;
    long long got = 0;
    st = gh_heap_delete(h, out_dev, n, &got, stream);
    if (st != GH_OK) return st;
    return got == n ? GH_OK : GH_ERR_STATE;
}

gh_status gh_heap_sort_host(gh_heap* h, const void* keys_host, long long n, void* out_host, void* stream) {
    gh::trace::Range range_("gh_heap_sort_host");
    constexpr int kPieces = 8;
    if (!h || n < 0 || (n > 0 && (!keys_host || !out_host))) return GH_ERR_INVALID;
    if (n > static_cast<long long>(h->d.batchNum) * h->d.batchSize) return GH_ERR_CAPACITY;
    const int B = h->d.batchSize;
    if (!h->d.pb && n % B != 0) return GH_ERR_INVALID;  // a padded last batch would not fit the output
    if (n == 0) return GH_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t kb = static_cast<size_t>(h->d.keyBytes), bytes = static_cast<size_t>(n) * kb;
    if (h->stageBytes < bytes) {
        if (h->stageIn) cudaFree(h->stageIn);
        if (h->stageOut) cudaFree(h->stageOut);
        h->stageIn = h->stageOut = nullptr;
        h->stageBytes = 0;
        GH_CUDA(cudaMalloc(&h->stageIn, bytes));
        GH_CUDA(cudaMalloc(&h->stageOut, bytes));
        h->stageBytes = bytes;
    }
    if (!h->copyStream) {
        GH_CUDA(cudaStreamCreateWithFlags(&h->copyStream, cudaStreamNonBlocking));
        for (cudaEvent_t& e : h->sortEv) GH_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    cudaStream_t c = h->copyStream;
    unsigned char* in = static_cast<unsigned char*>(h->stageIn);
    unsigned char* out = static_cast<unsigned char*>(h->stageOut);
    const unsigned char* hin = static_cast<const unsigned char*>(keys_host);
    unsigned char* hout = static_cast<unsigned char*>(out_host);
    // pieces of whole batches: the bulk insert reserves full batches, and the
    // deletes of a piece end on a batch boundary
    const long long per = (n + kPieces - 1) / kPieces;
    const long long piece = std::max<long long>(B, (per + B - 1) / B * B);
    int e = 0;
    // the copies start once the caller's stream is done with the staging buffers
    GH_CUDA(cudaEventRecord(h->sortEv[e], s));
    GH_CUDA(cudaStreamWaitEvent(c, h->sortEv[e++], 0));
    gh_status st = fill_items(h, s);
    if (st != GH_OK) return st;
    // keys in: piece i crosses on the copy stream while piece i - 1 is inserted
    for (long long off = 0; off < n; off += piece) {
        const long long len = std::min(piece, n - off);
        GH_CUDA(cudaMemcpyAsync(in + off * kb, hin + off * kb, len * kb, cudaMemcpyHostToDevice, c));
        GH_CUDA(cudaEventRecord(h->sortEv[e], c));
        GH_CUDA(cudaStreamWaitEvent(s, h->sortEv[e++], 0));
        st = gh_heap_insert(h, in + off * kb, len, B, stream);
        if (st != GH_OK) return st;
    }
    // keys out: piece j is deleted on the caller's stream, then crosses on
    // the copy stream while piece j + 1 is deleted
    for (long long off = 0; off < n; off += piece) {
        const long long len = std::min(piece, n - off);
        st = delete_bulk(h, out + off * kb, len, nullptr, nullptr, stream);
        if (st != GH_OK) return st;
        GH_CUDA(cudaEventRecord(h->sortEv[e], s));
        GH_CUDA(cudaStreamWaitEvent(c, h->sortEv[e++], 0));
        GH_CUDA(cudaMemcpyAsync(hout + off * kb, out + off * kb, len * kb, cudaMemcpyDeviceToHost, c));
    }
    // the caller's stream ends after the last copy
    GH_CUDA(cudaEventRecord(h->sortEv[e], c));
    GH_CUDA(cudaStreamWaitEvent(s, h->sortEv[e], 0));
    return GH_OK;
}

gh_status gh_heap_check(gh_heap* h, int* ok, char* msg, int msg_len, void* stream) {
    if (!h || !ok) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    gh::impl::CheckResult init{INT_MAX, 0, 0, 0};
    GH_CUDA(cudaMemcpyAsync(h->check, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    const int blocks = std::max(1, std::min(h->numSMs * 4, (h->d.batchNum + 7) / 8));
    switch (h->keyKind) {
        case GH_KEY_U32:
            gh::impl::k_check<uint32_t><<<blocks, 256, 0, s>>>(static_cast<const uint32_t*>(h->d.items), h->d.status,
                                                               h->d.state, h->d.variant, h->d.batchSize, h->check);
    gh::impl::count_launch();
            break;
        case GH_KEY_I32:
            gh::impl::k_check<int32_t><<<blocks, 256, 0, s>>>(static_cast<const int32_t*>(h->d.items), h->d.status,
                                                              h->d.state, h->d.variant, h->d.batchSize, h->check);
    gh::impl::count_launch();
            break;
        default:
            gh::impl::k_check<uint64_t><<<blocks, 256, 0, s>>>(static_cast<const uint64_t*>(h->d.items), h->d.status,
                                                               h->d.state, h->d.variant, h->d.batchSize, h->check);
    gh::impl::count_launch();
            break;
    }
    GH_CUDA(cudaGetLastError());
    gh::impl::CheckResult r;
    GH_CUDA(cudaMemcpyAsync(&r, h->check, sizeof(r), cudaMemcpyDeviceToHost, s));
    GH_CUDA(cudaStreamSynchronize(s));
    *ok = r.badNode == INT_MAX;
    if (msg && msg_len > 0) {
        if (*ok) std::snprintf(msg, msg_len, "ok");
        else std::snprintf(msg, msg_len, "node %d: %s (%d)", r.badNode, kCheckText[r.code >= 0 && r.code <= 6 ? r.code : 0], r.detail);
    }
    return device_error(h);
}

gh_status gh_heap_sync(gh_heap* h, void* stream) {
    if (!h) return GH_ERR_INVALID;
    GH_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    return device_error(h);
}

gh_status gh_heap_item_count(gh_heap* h, long long* n) {
    if (!h || !n) return GH_ERR_INVALID;
    int c[2];
    GH_CUDA(cudaMemcpy(c, h->d.state, sizeof(c), cudaMemcpyDeviceToHost));
    *n = static_cast<long long>(c[0]) * h->d.batchSize + c[1];
    return GH_OK;
}

gh_status gh_heap_node_count(gh_heap* h, int* n) {
    if (!h || !n) return GH_ERR_INVALID;
    GH_CUDA(cudaMemcpy(n, &h->d.state->batchCount, sizeof(int), cudaMemcpyDeviceToHost));
    return GH_OK;
}

gh_status gh_heap_is_empty(gh_heap* h, int* empty) {
    if (!h || !empty) return GH_ERR_INVALID;
    long long n = 0;
    gh_status st = gh_heap_item_count(h, &n);
    *empty = n == 0;
    return st;
}

gh_status gh_heap_snapshot(gh_heap* h, void* items_host, int* status_host, int* counters_host) {
    if (!h) return GH_ERR_INVALID;
    GH_CUDA(cudaDeviceSynchronize());
    if (items_host)
        GH_CUDA(cudaMemcpy(items_host, h->d.items, static_cast<size_t>(h->d.batchNum + 1) * h->d.batchSize * h->d.keyBytes,
                           cudaMemcpyDeviceToHost));
    if (status_host)
        GH_CUDA(cudaMemcpy(status_host, h->d.status, sizeof(int) * (static_cast<size_t>(h->d.batchNum) + 1), cudaMemcpyDeviceToHost));
    if (counters_host) {
        gh::HeapState st;
        GH_CUDA(cudaMemcpy(&st, h->d.state, sizeof(st), cudaMemcpyDeviceToHost));
        counters_host[0] = st.batchCount;
        counters_host[1] = st.partialBufferSize;
        counters_host[2] = st.deleteCount;
        counters_host[3] = st.err;
        counters_host[4] = st.errOp;
        counters_host[5] = st.errNode;
        counters_host[6] = st.errState;
    }
    return GH_OK;
}

gh_status gh_heap_restore(gh_heap* h, const void* items_host, const int* counters_host) {
    if (!h || !items_host || !counters_host) return GH_ERR_INVALID;
    const int bc = counters_host[0], ps = counters_host[1], dc = counters_host[2];
    if (bc < 0 || bc > h->d.batchNum || ps < 0 || ps >= h->d.batchSize || (!h->d.pb && ps != 0) || dc < 0)
        return GH_ERR_INVALID;
    static_assert(offsetof(gh::HeapState, partialBufferSize) == offsetof(gh::HeapState, batchCount) + sizeof(int) &&
                      offsetof(gh::HeapState, deleteCount) == offsetof(gh::HeapState, batchCount) + 2 * sizeof(int),
                  "batchCount, partialBufferSize and deleteCount are adjacent");
    GH_CUDA(cudaDeviceSynchronize());
    GH_CUDA(cudaMemcpy(h->d.items, items_host, static_cast<size_t>(h->d.batchNum + 1) * h->d.batchSize * h->d.keyBytes,
                       cudaMemcpyHostToDevice));
    GH_CUDA(cudaMemset(h->d.status, 0, sizeof(int) * (static_cast<size_t>(h->d.batchNum) + 2)));
    gh::impl::k_init_state<<<1, 32>>>(h->d.state, 0);
    gh::impl::count_launch();
    GH_CUDA(cudaGetLastError());
    GH_CUDA(cudaDeviceSynchronize());
    const int counters[3] = {bc, ps, dc};
    GH_CUDA(cudaMemcpy(&h->d.state->batchCount, counters, sizeof(counters), cudaMemcpyHostToDevice));
    return GH_OK;
}

gh_status gh_heap_inject_lock(gh_heap* h, int node, int state) {
    if (!h || node < 0 || node > h->d.batchNum) return GH_ERR_INVALID;
    GH_CUDA(cudaDeviceSynchronize());
    GH_CUDA(cudaMemcpy(h->d.status + node, &state, sizeof(int), cudaMemcpyHostToDevice));
    return GH_OK;
}

long long gh_launch_count(void) { return gh::impl::g_launches.load(); }

gh_status gh_heap_owner_stats(gh_heap* h, unsigned long long* out, int n) {
    if (!h || n < 0 || (n > 0 && !out)) return GH_ERR_INVALID;
    const int m = std::min(n, static_cast<int>(gh::impl::kStCount));
    for (int i = 0; i < n; ++i) out[i] = 0;
    if (!h->d.mbox || m == 0) return GH_OK;
    GH_CUDA(cudaDeviceSynchronize());
    const auto* mb = static_cast<const gh::impl::Mailbox*>(h->d.mbox);
    GH_CUDA(cudaMemcpy(out, mb->stats, sizeof(unsigned long long) * m, cudaMemcpyDeviceToHost));
    return GH_OK;
}

size_t gh_heap_view_bytes(void) { return 64; }
static_assert(sizeof(gh::Heap<uint64_t, 0, true>) <= 64, "device view size");

gh_status gh_heap_device_view(gh_heap* h, void* view_out, size_t view_bytes) {
    if (!h || !view_out || view_bytes < gh_heap_view_bytes()) return GH_ERR_INVALID;
    std::memset(view_out, 0, view_bytes);
    size_t got = 0;
    return with_key(h, [&](auto k) {
        gh::impl::device_view<decltype(k)>(h->d, view_out, &got);
        return got <= view_bytes ? cudaSuccess : cudaErrorInvalidValue;
    });
}

size_t gh_heap_smem_bytes(int key_kind, int batch_size) {
    return 4 * static_cast<size_t>(batch_size) * key_bytes(key_kind) + sizeof(gh::OpCtl) + 16;
}

gh_status gh_heap_info(gh_heap* h, int* key_kind, int* variant, int* partial_buffer, int* batch_num, int* batch_size,
                       int* block_threads, int* grid) {
    if (!h) return GH_ERR_INVALID;
    if (key_kind) *key_kind = h->keyKind;
    if (variant) *variant = h->d.variant;
    if (partial_buffer) *partial_buffer = h->d.pb;
    if (batch_num) *batch_num = h->d.batchNum;
    if (batch_size) *batch_size = h->d.batchSize;
    if (block_threads) *block_threads = threads_of(h);
    if (grid) *grid = grid_of(h);
    return GH_OK;
}

}  // extern "C"
