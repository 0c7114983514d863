// Device FIFO buffer: the bulk kernels of the reference's buffer test driver
// (artifacts/buffer/bufferTest.cu:13-56) over gh::Fifo<K>, and the C ABI of
// include/gpuheap_fifo.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>

#include "gpuheap_fifo.cuh"
#include "gpuheap_fifo.h"
#include "heap_kernels.cuh"
#include "trace.cuh"

namespace gh {
namespace impl {

// Pushes keys[0, n) in pieces of `chunk`, piece i by block (first + i*stride);
// with `split` each piece goes in as two pushes, its first third and the rest
// (bufferTest.cu:19-24).
template <typename K>
__device__ void push_pieces(const Fifo<K>& f, const K* __restrict__ keys, long long n, int chunk, int split,
                            int first, int stride) {
    const long long pieces = (n + chunk - 1) / chunk;
    for (long long i = first; i < pieces; i += stride) {
        const long long off = i * chunk;
        const int size = static_cast<int>(min(static_cast<long long>(chunk), n - off));
        if (split) {
            const int a = size / 3;
            f.push(keys + off, a);
            f.push(keys + off + a, size - a);
        } else {
            f.push(keys + off, size);
        }
        if (__syncthreads_or(threadIdx.x == 0 && f.failed())) return;
    }
}

// Takes keys until position `limit` has been claimed; out[p - base] gets the
// key at push-order position p.  Without `wait` it stops at the first empty
// claim (bufferTest.cu:49-56); with it, it waits for pushes (bufferTest.cu:29-35).
template <typename K>
__device__ void pop_until(const Fifo<K>& f, K* __restrict__ out, unsigned long long base, unsigned long long limit,
                          int chunk, int wait) {
    for (;;) {
        const typename Fifo<K>::Claim c = f.claim(chunk, limit);
        if (c.n > 0) {
            f.copy_out(c, out + (c.start - base));
            f.release(c);
            continue;
        }
        if (!wait) return;
        const int stop = threadIdx.x == 0 ? (f.wait_published(limit) ? 1 : 0) : 0;
        if (__syncthreads_or(stop)) return;
    }
}

template <typename K>
__global__ void __launch_bounds__(1024) k_fifo_push(Fifo<K> f, const K* __restrict__ keys, long long n, int chunk) {
    push_pieces(f, keys, n, chunk, 0, blockIdx.x, gridDim.x);
}

template <typename K>
__global__ void __launch_bounds__(1024) k_fifo_pop(Fifo<K> f, K* __restrict__ out, long long maxKeys, int chunk) {
    const unsigned long long base = f.state->mark;
    pop_until(f, out, base, base + maxKeys, chunk, 0);
}

// concurrentKernel: blocks [0, grid/2) push, the rest take maxKeys keys.
template <typename K>
__global__ void __launch_bounds__(1024) k_fifo_concurrent(Fifo<K> f, const K* __restrict__ keys, long long n,
                                                         int chunk, K* __restrict__ out, long long maxKeys) {
    const int pushers = gridDim.x / 2;
    if (static_cast<int>(blockIdx.x) < pushers) {
        push_pieces(f, keys, n, chunk, 1, blockIdx.x, pushers);
    } else {
        const unsigned long long base = f.state->mark;
        pop_until(f, out, base, base + maxKeys, chunk, 1);
    }
}

// One straight piece of a whole-call copy, kept out of line so the two
// pieces of a wrapped range share its registers.
template <typename K>
__device__ __noinline__ void grid_copy(K* __restrict__ dst, const K* __restrict__ src, long long n) {
    const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const long long T = static_cast<long long>(gridDim.x) * blockDim.x;
    fifo_detail::copy_keys(dst, src, n, t, T);
}

// Whole-call push, step 1 (one thread): one reservation for all n keys,
// then a bounded wait for room.
template <typename K>
__global__ void k_fifo_bulk_reserve(Fifo<K> f, unsigned long long n) {
    FifoState* s = f.state;
    const unsigned long long start = atomicAdd(&s->end, n);
    s->bulkStart = start;
    s->bulkDone = 0;
    const unsigned long long t0 = fifo_detail::now();
    while (start + n - fifo_detail::ld_acquire64(&s->begin) > f.capacity) {
        if (f.failed() || fifo_detail::now() - t0 > static_cast<unsigned long long>(f.timeoutNs)) {
            f.fail(1);
            return;
        }
        __nanosleep(200);
    }
}

// The last block of a whole-call launch to finish (thread 0) returns true.
__device__ __forceinline__ bool last_block(FifoState* s) {
    __threadfence();
    const bool last = atomicAdd(&s->bulkDone, 1) == static_cast<int>(gridDim.x) - 1;
    if (last) __threadfence();
    return last;
}

// Thread 0: waits (bounded) until *pos reaches `from`, then stores `to` --
// the in-order commit of a range whose owner is the only writer at `from`.
template <typename K>
__device__ __forceinline__ void commit(const Fifo<K>& f, unsigned long long* pos, unsigned long long from,
                                       unsigned long long to, int site) {
    const unsigned long long t0 = fifo_detail::now();
    while (fifo_detail::ld_acquire64(pos) != from) {
        if (f.failed() || fifo_detail::now() - t0 > static_cast<unsigned long long>(f.timeoutNs)) {
            f.fail(site);
            return;
        }
        __nanosleep(32);
    }
    fifo_detail::st_release64(pos, to);
}

// Whole-call push, step 2: the grid copies keys[0, n) to the reserved
// positions; the last block publishes them.
template <typename K>
__global__ void __launch_bounds__(512, 2) k_fifo_bulk_push(Fifo<K> f, const K* __restrict__ keys, long long n) {
    const unsigned long long start = f.state->bulkStart;
    if (!f.failed()) {
        const unsigned long long at = start & (f.capacity - 1);
        const long long first = static_cast<long long>(min(static_cast<unsigned long long>(n), f.capacity - at));
        grid_copy(f.items + at, keys, first);
        if (first < n) grid_copy(f.items, keys + first, n - first);
    }
    __syncthreads();
    if (threadIdx.x == 0 && last_block(f.state) && !f.failed()) commit(f, &f.state->write, start, start + n, 2);
}

// Whole-call pop, step 1 (one thread): claims min(maxKeys, published) keys.
template <typename K>
__global__ void k_fifo_bulk_claim(Fifo<K> f, long long maxKeys) {
    FifoState* s = f.state;
    unsigned long long r = 0;
    long long n = 0;
    if (!f.failed()) {
        const unsigned long long t0 = fifo_detail::now();
        for (;;) {
            r = fifo_detail::ld_acquire64(&s->read);
            const unsigned long long avail = fifo_detail::ld_acquire64(&s->write) - r;
            n = avail < static_cast<unsigned long long>(maxKeys) ? static_cast<long long>(avail) : maxKeys;
            if (n == 0 || fifo_detail::cas_acq_rel64(&s->read, r, r + n) == r) break;
            if (fifo_detail::now() - t0 > static_cast<unsigned long long>(f.timeoutNs)) {
                f.fail(3);
                n = 0;
                break;
            }
        }
    }
    s->mark = r;
    s->claimN = n;
    s->bulkDone = 0;
}

// Whole-call pop, step 2: the grid copies the claimed keys to out[0, n); the
// last block frees their slots.
template <typename K>
__global__ void __launch_bounds__(512, 2) k_fifo_bulk_pop(Fifo<K> f, K* __restrict__ out) {
    const unsigned long long start = f.state->mark;
    const long long n = f.state->claimN;
    const unsigned long long at = start & (f.capacity - 1);
    const long long first = static_cast<long long>(min(static_cast<unsigned long long>(n), f.capacity - at));
    grid_copy(out, f.items + at, first);
    if (first < n) grid_copy(out + first, f.items, n - first);
    __syncthreads();
    if (threadIdx.x == 0 && last_block(f.state) && n > 0) commit(f, &f.state->begin, start, start + n, 4);
}

__global__ void k_fifo_mark(FifoState* s) { s->mark = s->read; }

__global__ void k_fifo_reserve(FifoState* s, unsigned long long n) { s->end += n; }

}  // namespace impl
}  // namespace gh

struct gh_fifo {
    void* items;
    gh::FifoState* state;
    unsigned long long capacity;
    long long timeoutNs;
    int keyKind;
    int keyBytes;
    int blocks;   // 0 = as many as stay resident
    int threads;  // 0 = 512
    int device;
    int numSMs;
    int errSeen;                   // a call already reported the device's error
    unsigned long long knownBegin;  // begin at the last read (a lower bound)
    unsigned long long endBound;    // end at the last read plus keys pushed since
};

namespace {

gh_status fifo_cuda(cudaError_t e) {
    if (e == cudaSuccess) return GH_OK;
    std::fprintf(stderr, "gpuheap fifo: CUDA error %s\n", cudaGetErrorString(e));
    return GH_ERR_CUDA;
}
#define GHF_CUDA(call)                                  \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return fifo_cuda(e_);    \
    } while (0)

template <typename K>
gh::Fifo<K> view_of(const gh_fifo* f) {
    gh::Fifo<K> v;
    v.items = static_cast<K*>(f->items);
    v.state = f->state;
    v.capacity = f->capacity;
    v.timeoutNs = f->timeoutNs;
    return v;
}

template <typename F>
gh_status with_key(const gh_fifo* f, F&& fn) {
    switch (f->keyKind) {
        case GH_KEY_U32: return fn(uint32_t{});
        case GH_KEY_I32: return fn(int32_t{});
        default: return fn(uint64_t{});
    }
}

int threads_of(const gh_fifo* f) { return f->threads ? f->threads : 512; }
// The whole-call copy kernels are compiled for at most 512 threads a block.
int bulk_threads(const gh_fifo* f) { return std::min(threads_of(f), 512); }

// Blocks of a bulk call.  The concurrent kernel's pushers and poppers wait
// on one another, so its grid never exceeds what stays resident at once.
template <typename Kern>
gh_status grid_of(const gh_fifo* f, Kern kern, int* grid, int threads = 0) {
    int perSM = 0;
    GHF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, threads ? threads : threads_of(f), 0));
    const int resident = std::max(1, perSM) * f->numSMs;
    *grid = f->blocks ? std::min(f->blocks, resident) : resident;
    return GH_OK;
}

// Reads the state after the stream's work; a recorded device error is
// GH_ERR_TIMEOUT the first time a call sees it and GH_ERR_STATE after that.
gh_status sync_state(gh_fifo* f, cudaStream_t s, gh::FifoState* st) {
    GHF_CUDA(cudaMemcpyAsync(st, f->state, sizeof(*st), cudaMemcpyDeviceToHost, s));
    GHF_CUDA(cudaStreamSynchronize(s));
    f->knownBegin = st->begin;
    f->endBound = st->end;
    if (st->err == 0) return GH_OK;
    const gh_status r = f->errSeen ? GH_ERR_STATE : GH_ERR_TIMEOUT;
    f->errSeen = 1;
    return r;
}

gh_status launch_mark(const gh_fifo* f, cudaStream_t s) {
    gh::impl::k_fifo_mark<<<1, 1, 0, s>>>(f->state);
    gh::impl::count_launch();
    GHF_CUDA(cudaGetLastError());
    return GH_OK;
}

}  // namespace

extern "C" {

gh_status gh_fifo_create(gh_fifo** out, int key_kind, long long capacity) {
    if (!out) return GH_ERR_INVALID;
    *out = nullptr;
    if (key_kind < GH_KEY_U32 || key_kind > GH_KEY_U64) return GH_ERR_INVALID;
    if (capacity < 1 || capacity > (1LL << 34)) return GH_ERR_INVALID;
    unsigned long long cap = 1;
    while (cap < static_cast<unsigned long long>(capacity)) cap <<= 1;
    gh_fifo* f = new (std::nothrow) gh_fifo();
    if (!f) return GH_ERR_INVALID;
    std::memset(f, 0, sizeof(*f));
    f->capacity = cap;
    f->timeoutNs = 2000000000LL;
    f->keyKind = key_kind;
    f->keyBytes = key_kind == GH_KEY_U64 ? 8 : 4;
    auto fail = [&](gh_status st) { gh_fifo_destroy(f); return st; };
    if (cudaGetDevice(&f->device) != cudaSuccess) return fail(GH_ERR_CUDA);
    if (cudaDeviceGetAttribute(&f->numSMs, cudaDevAttrMultiProcessorCount, f->device) != cudaSuccess)
        return fail(GH_ERR_CUDA);
    if (cudaMalloc(&f->items, cap * f->keyBytes) != cudaSuccess) { cudaGetLastError(); return fail(GH_ERR_CUDA); }
    if (cudaMalloc(&f->state, sizeof(gh::FifoState)) != cudaSuccess) { cudaGetLastError(); return fail(GH_ERR_CUDA); }
    if (cudaMemset(f->state, 0, sizeof(gh::FifoState)) != cudaSuccess) return fail(GH_ERR_CUDA);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(GH_ERR_CUDA);
    *out = f;
    return GH_OK;
}

gh_status gh_fifo_destroy(gh_fifo* f) {
    if (!f) return GH_ERR_INVALID;
    if (f->items) cudaFree(f->items);
    if (f->state) cudaFree(f->state);
    delete f;
    return GH_OK;
}

gh_status gh_fifo_reset(gh_fifo* f, void* stream) {
    if (!f) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    GHF_CUDA(cudaMemsetAsync(f->state, 0, sizeof(gh::FifoState), s));
    GHF_CUDA(cudaStreamSynchronize(s));
    f->errSeen = 0;
    f->knownBegin = 0;
    f->endBound = 0;
    return GH_OK;
}

gh_status gh_fifo_set_timeout(gh_fifo* f, double seconds) {
    if (!f || !(seconds > 0) || seconds > 60.0) return GH_ERR_INVALID;
    f->timeoutNs = static_cast<long long>(seconds * 1e9);
    return GH_OK;
}

gh_status gh_fifo_set_launch(gh_fifo* f, int blocks, int threads) {
    if (!f || blocks < 0 || threads < 0 || threads > 1024 || threads % 32 != 0) return GH_ERR_INVALID;
    f->blocks = blocks;
    f->threads = threads;
    return GH_OK;
}

gh_status gh_fifo_push(gh_fifo* f, const void* keys_dev, long long n, int chunk, void* stream) {
    gh::trace::Range range_("gh_fifo_push");
    if (!f || n < 0 || (n > 0 && !keys_dev) || chunk < 0) return GH_ERR_INVALID;
    if (static_cast<unsigned long long>(chunk) > f->capacity) return GH_ERR_INVALID;
    if (f->errSeen) return GH_ERR_STATE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned long long add = static_cast<unsigned long long>(n);
    // The host's bound on the keys held (end since pushed, begin as last
    // read) decides without a synchronisation while it fits; otherwise the
    // exact positions after the stream's work decide.
    if (f->endBound - f->knownBegin + add > f->capacity) {
        gh::FifoState st;
        gh_status r = sync_state(f, s, &st);
        if (r != GH_OK) return r;
        if (st.end - st.begin + add > f->capacity) {
            std::fprintf(stderr, "gpuheap fifo: %llu keys held + %lld pushed exceed the ring's %llu\n",
                         st.end - st.begin, n, f->capacity);
            return GH_ERR_CAPACITY;
        }
    }
    if (n == 0) return GH_OK;
    gh_status r = with_key(f, [&](auto k) -> gh_status {
        using K = decltype(k);
        int grid = 0;
        if (chunk == 0) {  // one reservation for the whole call
            gh_status g = grid_of(f, gh::impl::k_fifo_bulk_push<K>, &grid, bulk_threads(f));
            if (g != GH_OK) return g;
            const long long per = 16LL * bulk_threads(f);
            grid = static_cast<int>(std::min<long long>(grid, (n + per - 1) / per));
            gh::impl::k_fifo_bulk_reserve<K><<<1, 1, 0, s>>>(view_of<K>(f), static_cast<unsigned long long>(n));
            gh::impl::count_launch();
            gh::impl::k_fifo_bulk_push<K><<<grid, bulk_threads(f), 0, s>>>(view_of<K>(f), static_cast<const K*>(keys_dev),
                                                                         n);
            gh::impl::count_launch();
            GHF_CUDA(cudaGetLastError());
            return GH_OK;
        }
        gh_status g = grid_of(f, gh::impl::k_fifo_push<K>, &grid);
        if (g != GH_OK) return g;
        const long long pieces = (n + chunk - 1) / chunk;
        grid = static_cast<int>(std::min<long long>(grid, pieces));
        gh::impl::k_fifo_push<K><<<grid, threads_of(f), 0, s>>>(view_of<K>(f), static_cast<const K*>(keys_dev), n,
                                                                chunk);
        gh::impl::count_launch();
        GHF_CUDA(cudaGetLastError());
        return GH_OK;
    });
    if (r == GH_OK) f->endBound += add;
    return r;
}

gh_status gh_fifo_pop(gh_fifo* f, void* out_dev, long long max_keys, int chunk, long long* n_out, void* stream) {
    gh::trace::Range range_("gh_fifo_pop");
    if (!f || max_keys < 0 || (max_keys > 0 && !out_dev) || chunk < 0) return GH_ERR_INVALID;
    if (f->errSeen) return GH_ERR_STATE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    gh_status st = GH_OK;
    if (chunk == 0) {  // one claim for the whole call
        st = with_key(f, [&](auto k) -> gh_status {
            using K = decltype(k);
            int grid = 0;
            gh_status g = grid_of(f, gh::impl::k_fifo_bulk_pop<K>, &grid, bulk_threads(f));
            if (g != GH_OK) return g;
            const long long per = 16LL * bulk_threads(f);
            grid = static_cast<int>(std::max<long long>(1, std::min<long long>(grid, (max_keys + per - 1) / per)));
            gh::impl::k_fifo_bulk_claim<K><<<1, 1, 0, s>>>(view_of<K>(f), max_keys);
            gh::impl::count_launch();
            gh::impl::k_fifo_bulk_pop<K><<<grid, bulk_threads(f), 0, s>>>(view_of<K>(f), static_cast<K*>(out_dev));
            gh::impl::count_launch();
            GHF_CUDA(cudaGetLastError());
            return GH_OK;
        });
        if (st != GH_OK) return st;
        if (!n_out) return GH_OK;
        gh::FifoState fs;
        st = sync_state(f, s, &fs);
        *n_out = fs.claimN;
        return st;
    }
    st = launch_mark(f, s);
    if (st != GH_OK) return st;
    if (max_keys > 0) {
        st = with_key(f, [&](auto k) -> gh_status {
            using K = decltype(k);
            int grid = 0;
            gh_status g = grid_of(f, gh::impl::k_fifo_pop<K>, &grid);
            if (g != GH_OK) return g;
            grid = static_cast<int>(std::min<long long>(grid, (max_keys + chunk - 1) / chunk));
            gh::impl::k_fifo_pop<K><<<grid, threads_of(f), 0, s>>>(view_of<K>(f), static_cast<K*>(out_dev), max_keys,
                                                                   chunk);
            gh::impl::count_launch();
            GHF_CUDA(cudaGetLastError());
            return GH_OK;
        });
        if (st != GH_OK) return st;
    }
    if (!n_out) return GH_OK;
    gh::FifoState fs;
    st = sync_state(f, s, &fs);
    *n_out = static_cast<long long>(fs.read - fs.mark);
    return st;
}

gh_status gh_fifo_concurrent(gh_fifo* f, const void* keys_dev, long long n, int chunk, void* out_dev,
                             long long max_keys, long long* n_out, void* stream) {
    gh::trace::Range range_("gh_fifo_concurrent");
    if (!f || n < 0 || (n > 0 && !keys_dev) || max_keys < 0 || (max_keys > 0 && !out_dev) || chunk < 0)
        return GH_ERR_INVALID;
    if (chunk == 0) chunk = static_cast<int>(std::min<unsigned long long>(1024, f->capacity));
    if (static_cast<unsigned long long>(chunk) > f->capacity) return GH_ERR_INVALID;
    if (f->errSeen) return GH_ERR_STATE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    gh::FifoState fs;
    gh_status st = sync_state(f, s, &fs);
    if (st != GH_OK) return st;
    const unsigned long long held = fs.end - fs.begin;
    if (static_cast<unsigned long long>(max_keys) > held + n) return GH_ERR_INVALID;
    if (held + n - max_keys > f->capacity) {
        std::fprintf(stderr, "gpuheap fifo: %llu keys held + %lld pushed - %lld taken exceed the ring's %llu\n",
                     held, n, max_keys, f->capacity);
        return GH_ERR_CAPACITY;
    }
    st = launch_mark(f, s);
    if (st != GH_OK) return st;
    st = with_key(f, [&](auto k) -> gh_status {
        using K = decltype(k);
        int perSM = 0;
        GHF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, gh::impl::k_fifo_concurrent<K>, threads_of(f),
                                                               0));
        const int resident = perSM * f->numSMs;
        if (resident < 2) return GH_ERR_INVALID;  // pushers and poppers must be resident together
        int grid = f->blocks ? std::min(f->blocks, resident) : resident;
        grid = std::max(grid, 2);
        gh::impl::k_fifo_concurrent<K><<<grid, threads_of(f), 0, s>>>(
            view_of<K>(f), static_cast<const K*>(keys_dev), n, chunk, static_cast<K*>(out_dev), max_keys);
        gh::impl::count_launch();
        GHF_CUDA(cudaGetLastError());
        return GH_OK;
    });
    if (st != GH_OK) return st;
    st = sync_state(f, s, &fs);
    if (n_out) *n_out = static_cast<long long>(fs.read - fs.mark);
    return st;
}

gh_status gh_fifo_count(gh_fifo* f, long long* n) {
    if (!f || !n) return GH_ERR_INVALID;
    GHF_CUDA(cudaDeviceSynchronize());
    gh::FifoState fs;
    gh_status st = sync_state(f, nullptr, &fs);
    *n = static_cast<long long>(fs.end - fs.begin);
    return st;
}

gh_status gh_fifo_positions(gh_fifo* f, unsigned long long* begin, unsigned long long* read, unsigned long long* write,
                            unsigned long long* end) {
    if (!f) return GH_ERR_INVALID;
    GHF_CUDA(cudaDeviceSynchronize());
    gh::FifoState fs;
    gh_status st = sync_state(f, nullptr, &fs);
    if (begin) *begin = fs.begin;
    if (read) *read = fs.read;
    if (write) *write = fs.write;
    if (end) *end = fs.end;
    return st;
}

gh_status gh_fifo_snapshot(gh_fifo* f, void* items_host, unsigned long long* positions_host) {
    if (!f || !items_host) return GH_ERR_INVALID;
    GHF_CUDA(cudaDeviceSynchronize());
    GHF_CUDA(cudaMemcpy(items_host, f->items, f->capacity * f->keyBytes, cudaMemcpyDeviceToHost));
    if (positions_host)
        return gh_fifo_positions(f, positions_host, positions_host + 1, positions_host + 2, positions_host + 3);
    return GH_OK;
}

size_t gh_fifo_view_bytes(void) { return sizeof(gh::Fifo<uint64_t>); }

gh_status gh_fifo_device_view(gh_fifo* f, void* view_out, size_t view_bytes) {
    if (!f || !view_out || view_bytes < gh_fifo_view_bytes()) return GH_ERR_INVALID;
    return with_key(f, [&](auto k) -> gh_status {
        using K = decltype(k);
        const gh::Fifo<K> v = view_of<K>(f);
        std::memcpy(view_out, &v, sizeof(v));
        return GH_OK;
    });
}

gh_status gh_fifo_inject_reservation(gh_fifo* f, long long n) {
    if (!f || n < 1) return GH_ERR_INVALID;
    gh::impl::k_fifo_reserve<<<1, 1>>>(f->state, static_cast<unsigned long long>(n));
    gh::impl::count_launch();
    GHF_CUDA(cudaGetLastError());
    GHF_CUDA(cudaDeviceSynchronize());
    return GH_OK;
}

gh_status gh_fifo_info(gh_fifo* f, int* key_kind, long long* capacity, int* blocks, int* threads, int* err_site) {
    if (!f) return GH_ERR_INVALID;
    if (key_kind) *key_kind = f->keyKind;
    if (capacity) *capacity = static_cast<long long>(f->capacity);
    if (threads) *threads = threads_of(f);
    if (blocks) {
        int grid = 0;
        gh_status st = with_key(f, [&](auto k) { return grid_of(f, gh::impl::k_fifo_push<decltype(k)>, &grid); });
        if (st != GH_OK) return st;
        *blocks = grid;
    }
    if (err_site) {
        gh::FifoState fs;
        GHF_CUDA(cudaDeviceSynchronize());
        GHF_CUDA(cudaMemcpy(&fs, f->state, sizeof(fs), cudaMemcpyDeviceToHost));
        *err_site = fs.err ? fs.errSite : 0;
    }
    return GH_OK;
}

}  // extern "C"
