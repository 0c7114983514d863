// The retrieving heap behind the C ABI (gh_rheap_*, gpuheap.h) and SSSP
// through its auxiliary buffer (gh_sssp_retrieve).
//
// The reference's counterparts: applications/sssp_longfei_new/heap.cuh
// (Heap<T>: insert, retrieve), heap_with_aux.cuh (Heap_With_Aux<T, Aux>:
// retrieve with chk_func) and sssp.cu:19-132 (ssspKernel: retrieve a batch
// of keys with their edge offsets, relax at most CONFIG_CHUNK_SIZE edges of
// each, put keys with edges left back into the auxiliary buffer, insert the
// improved vertices).  The device structure is include/gpuheap_retrieve.cuh.
#include <cuda_runtime.h>

#include <climits>
#include <cstring>
#include <new>

#include "gpuheap.h"
#include "gpuheap_retrieve.cuh"
#include "heap_kernels.cuh"
#include "trace.cuh"
#include "worklist.cuh"

struct gh_rheap {
    int keyKind = GH_KEY_U64;
    int batchNum = 0, batchSize = 0, threads = 0;
    unsigned long long initBits = ~0ull;
    long long timeoutNs = 2000000000LL;
    unsigned char* mem = nullptr;  // state, items, partial buffer, locks, taken
    gh::HeapState* state = nullptr;
    void* items = nullptr;
    void* pbuf = nullptr;
    int* lock = nullptr;
    int* taken = nullptr;
    int* scratch = nullptr;  // [0] taken count, [1..] concurrent-run cursors
};

namespace {

using u64 = unsigned long long;

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
int key_bytes(int kind) { return kind == GH_KEY_U64 ? 8 : 4; }

template <typename K>
gh::RetHeap<K> view(const gh_rheap* h) {
    gh::RetHeap<K> v;
    v.items = static_cast<K*>(h->items);
    v.pbuf = static_cast<K*>(h->pbuf);
    v.lock = h->lock;
    v.taken = h->taken;
    v.state = h->state;
    v.batchNum = h->batchNum;
    v.batchSize = h->batchSize;
    v.initLimit = static_cast<K>(h->initBits);
    v.timeoutNs = h->timeoutNs;
    return v;
}

template <typename K>
__global__ void k_rheap_fill(K* items, size_t n, K init) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        items[i] = init;
}

// Dynamic shared memory above the default 48 KB needs the kernel's opt-in.
template <typename F>
cudaError_t allow_smem(F kern, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

template <typename K>
__global__ void __launch_bounds__(1024) k_rheap_insert(gh::RetHeap<K> h, const K* keys, int count) {
    h.insert(keys, count, 0);
}

template <typename K>
__global__ void __launch_bounds__(1024) k_rheap_retrieve(gh::RetHeap<K> h, K* out, int size, int* got) {
    const int n = h.retrieve(out, size, 0);
    if (threadIdx.x == 0) *got = n;
}

// Blocks [0, inserters) insert keys[0, n) in chunks of `chunk` (chunk c to
// block c mod inserters); the other blocks retrieve `size` keys at a time
// until every inserter is done and the heap is empty.  Each retrieved run is
// appended to out at a cursor (runs[2r] = its start, runs[2r + 1] = its
// length).  cursors: [0] inserters done, [1] out cursor, [2] runs.
template <typename K>
__global__ void __launch_bounds__(1024) k_rheap_concurrent(gh::RetHeap<K> h, const K* keys, long long n, int chunk, int inserters, int size,
                                   K* out, long long maxOut, int* runs, int maxRuns, int* cursors) {
    __shared__ int s_word[2];
    if (static_cast<int>(blockIdx.x) < inserters) {
        const long long chunks = (n + chunk - 1) / chunk;
        for (long long c = blockIdx.x; c < chunks; c += inserters) {
            const long long at = c * chunk;
            const int cnt = static_cast<int>(n - at < chunk ? n - at : chunk);
            h.insert(keys + at, cnt, 0);
            if (h.failed()) break;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(cursors, 1);
        }
        return;
    }
    unsigned long long idleSince = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            const int done = gh::detail::ld_acquire(cursors);
            const long long held = h.held();
            int verdict = 0;  // 0 retrieve, 1 stop, 2 wait
            if (gh::detail::ld_relaxed(&h.state->err) != 0) verdict = 1;
            else if (held == 0 && done == inserters) verdict = 1;
            else if (held == 0) {
                const unsigned long long now = gh::detail::globaltimer();
                if (idleSince == 0) idleSince = now;
                if (now - idleSince > static_cast<unsigned long long>(h.timeoutNs)) verdict = 1;
                else verdict = 2;  // wait for the inserters
            } else {
                idleSince = 0;
            }
            s_word[0] = verdict;
        }
        __syncthreads();
        const int verdict = s_word[0];
        __syncthreads();
        if (verdict == 1) break;
        if (verdict == 2) {
            if (threadIdx.x == 0) __nanosleep(256);
            continue;
        }
        extern __shared__ __align__(16) unsigned char smem[];
        K* run = reinterpret_cast<K*>(smem + gh::RetHeap<K>::smemBytes(h.batchSize));
        const int got = h.retrieve(run, size, 0);
        if (got > 0) {
            if (threadIdx.x == 0) {
                const long long at = atomicAdd(reinterpret_cast<unsigned long long*>(cursors + 2),
                                               static_cast<unsigned long long>(got));
                const int r = atomicAdd(cursors + 4, 1);
                s_word[1] = at + got <= maxOut && r < maxRuns ? static_cast<int>(at) : -1;
                if (r < maxRuns) {
                    runs[2 * r] = static_cast<int>(at);
                    runs[2 * r + 1] = got;
                }
            }
            __syncthreads();
            const int at = s_word[1];
            if (at >= 0)
                for (int k = threadIdx.x; k < got; k += blockDim.x) out[at + k] = run[k];
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------------ SSSP
// Edge offset check of the reference (sssp.cu:9-17, update_offset): a key
// whose vertex has more than `chunk` edges past its offset goes back into
// the auxiliary buffer with the offset moved on by `chunk`.
struct ChunkCheck {
    const long long* rowptr;
    int chunk;
    __device__ bool operator()(u64 key, int& offset) const {
        const int v = static_cast<int>(key & 0xffffffffu);
        const long long deg = rowptr[v + 1] - rowptr[v];
        if (deg - offset > chunk) {
            offset += chunk;
            return true;
        }
        return false;
    }
};

// Shared memory of a block ahead of the heap's region (a multiple of 16
// bytes: the heap's buffers take 16-byte vector stores).
struct SsspRetSmem {
    static __host__ __device__ size_t bytes(int B) {
        const size_t raw = static_cast<size_t>(B) * 8      // keys handed out
                           + static_cast<size_t>(B) * 4    // their edge offsets
                           + static_cast<size_t>(B) * 8    // current keys
                           + static_cast<size_t>(B + 1) * 8  // edge prefix
                           + static_cast<size_t>(B) * 4    // current keys' offsets
                           + 64                            // control words
                           + 32 * 8;                       // warp sums of the scan
        return (raw + 15) / 16 * 16;
    }
};

// In-place inclusive prefix sum of x[0, n) over the block (a chunk of
// consecutive entries per thread, warp shuffles, then the warp totals);
// wsum: 32 shared slots.  Ends with a barrier.
__device__ void block_inclusive_scan(long long* x, int n, long long* wsum) {
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int per = (n + T - 1) / T;
    long long local = 0;
    for (int j = 0; j < per; ++j) {
        const int i = tid * per + j;
        if (i < n) local += x[i];
    }
    long long incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        long long v = lane < (T >> 5) ? wsum[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        wsum[lane] = v;
    }
    __syncthreads();
    long long run = incl - local + (warp ? wsum[warp - 1] : 0);
    for (int j = 0; j < per; ++j) {
        const int i = tid * per + j;
        if (i < n) { run += x[i]; x[i] = run; }
    }
    __syncthreads();
}

// ssspKernel (sssp.cu:19-132) on the retrieving heap with the auxiliary
// buffer: each block takes up to B keys, keeps those still current, relaxes
// at most `chunk` edges of each from its offset, and inserts the improved
// vertices in batches from its slice of `emit` (B * chunk keys).  The
// reference ends when every block has found nothing once (term_sig); here
// the busy-counter protocol of worklist.cuh ends the search: a block counts
// itself busy before it takes keys and leaves when it finds nothing held
// while no block is busy.
__global__ void __launch_bounds__(1024) k_sssp_retrieve(gh::RetHeapAux<u64, int> h, const long long* __restrict__ rowptr,
                                                        const int* __restrict__ col, const unsigned* __restrict__ wt,
                                                        unsigned* dist, u64* emitAll, int chunk) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int B = h.heap.batchSize, T = blockDim.x, tid = threadIdx.x;
    u64* keys = reinterpret_cast<u64*>(smem);
    int* offs = reinterpret_cast<int*>(keys + B);
    u64* cur = reinterpret_cast<u64*>(offs + B);
    long long* pre = reinterpret_cast<long long*>(cur + B);
    int* curOff = reinterpret_cast<int*>(pre + B + 1);
    int* ctl = curOff + B;  // 16 words
    long long* wsum = reinterpret_cast<long long*>(ctl + 16);  // 32 warp sums
    const int heapOff = static_cast<int>(SsspRetSmem::bytes(B));
    u64* emit = emitAll + static_cast<size_t>(blockIdx.x) * B * chunk;
    gh::HeapState* st = h.heap.state;
    const ChunkCheck check{rowptr, chunk};
    unsigned long long pops = 0, edges = 0, inserted = 0, waitStart = 0;
    int lastBusy = -1;
    for (;;) {
        // wait_for_keys (worklist.cuh) on the retrieving heap and its buffer
        if (tid == 0) {
            int verdict = 0;
            for (;;) {
                if (h.held() > 0) break;
                const int b = atomicAdd(&st->busy, 0);
                __threadfence();
                if (b == 0 && h.held() == 0) { verdict = 1; break; }
                if (gh::detail::ld_relaxed(&st->err) != 0) { verdict = 1; break; }
                const unsigned long long now = gh::detail::globaltimer();
                if (b != lastBusy || waitStart == 0) { lastBusy = b; waitStart = now; }
                if (now - waitStart > static_cast<unsigned long long>(h.heap.timeoutNs)) {
                    if (atomicCAS(&st->err, 0, gh::kErrTimeout) == 0) st->errOp = gh::kSiteLockPartial;
                    verdict = 1;
                    break;
                }
                __nanosleep(200);
            }
            if (!verdict) {
                atomicAdd(&st->busy, 1);
                __threadfence();
            }
            ctl[0] = verdict;
        }
        __syncthreads();
        const bool over = ctl[0] != 0;
        __syncthreads();
        if (over) break;
        lastBusy = -1;
        const int size = h.retrieve(keys, offs, B, check, heapOff);
        pops += size;
        // current keys and their edge counts (at most `chunk` from the offset)
        if (tid == 0) ctl[1] = 0;
        __syncthreads();
        for (int i = tid; i < size; i += T) {
            const u64 key = keys[i];
            const unsigned d = static_cast<unsigned>(key >> 32);
            const int v = static_cast<int>(key & 0xffffffffu);
            if (d <= __ldcg(dist + v)) {
                const int j = atomicAdd(&ctl[1], 1);
                cur[j] = key;
                curOff[j] = offs[i];
            }
        }
        __syncthreads();
        const int nc = ctl[1];
        // edges of each current key, then their exclusive prefix in pre[0, nc]
        for (int j = tid; j < nc; j += T) {
            const int v = static_cast<int>(cur[j] & 0xffffffffu);
            long long e = rowptr[v + 1] - rowptr[v] - curOff[j];
            if (e > chunk) e = chunk;
            pre[j + 1] = e > 0 ? e : 0;
        }
        if (tid == 0) {
            pre[0] = 0;
            ctl[2] = 0;
        }
        __syncthreads();
        block_inclusive_scan(pre + 1, nc, wsum);
        const long long total = pre[nc];
        edges += total;
        for (long long ei = tid; ei < total; ei += T) {
            int lo = 0, hi = nc;  // largest lo with pre[lo] <= ei
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (pre[mid] <= ei) lo = mid;
                else hi = mid;
            }
            const u64 key = cur[lo];
            const unsigned d = static_cast<unsigned>(key >> 32);
            const int v = static_cast<int>(key & 0xffffffffu);
            const long long e = rowptr[v] + curOff[lo] + (ei - pre[lo]);
            const int u = col[e];
            const u64 nd64 = static_cast<u64>(d) + wt[e];
            const unsigned nd = nd64 >= 0xffffffffULL ? 0xfffffffeu : static_cast<unsigned>(nd64);
            if (nd < __ldcg(dist + u)) {
                const unsigned old = atomicMin(dist + u, nd);
                if (nd < old) emit[atomicAdd(&ctl[2], 1)] = (static_cast<u64>(nd) << 32) | static_cast<unsigned>(u);
            }
        }
        __syncthreads();
        const int ne = ctl[2];
        for (int at = 0; at < ne; at += B) {
            const int c = ne - at < B ? ne - at : B;
            h.insert(emit + at, c, heapOff);
            inserted += c;
        }
        gh::app::batch_done(st);
        if (h.heap.failed()) break;
    }
    if (tid == 0) {
        atomicAdd(&st->appStats[4], pops);
        atomicAdd(&st->appStats[5], edges);
        atomicAdd(&st->appStats[6], inserted);
    }
}

__global__ void k_sssp_retrieve_init(unsigned* dist, int n, int source) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        dist[v] = v == source ? 0u : 0xffffffffu;
}

__global__ void __launch_bounds__(1024) k_sssp_retrieve_seed(gh::RetHeapAux<u64, int> h, int source) {
    extern __shared__ __align__(16) unsigned char smem[];
    u64* seed = reinterpret_cast<u64*>(smem);
    if (threadIdx.x == 0) seed[0] = static_cast<u64>(source);  // distance 0
    __syncthreads();
    h.insert(seed, 1, 16);
}

int threads_for(int B) { return B < 1024 ? B : 1024; }

}  // namespace

extern "C" {

gh_status gh_rheap_create(gh_rheap** out, int key_kind, int batch_num, int batch_size, const void* init_limit) {
    if (!out) return GH_ERR_INVALID;
    *out = nullptr;
    if (key_kind != GH_KEY_U32 && key_kind != GH_KEY_U64) return GH_ERR_INVALID;
    if (batch_size < 16 || batch_size > 2048 || (batch_size & (batch_size - 1))) return GH_ERR_INVALID;
    if (batch_num < 2 || batch_num > (1 << 24)) return GH_ERR_INVALID;
    gh_rheap* h = new (std::nothrow) gh_rheap();
    if (!h) return GH_ERR_INVALID;
    h->keyKind = key_kind;
    h->batchNum = batch_num;
    h->batchSize = batch_size;
    h->threads = threads_for(batch_size);
    const int kb = key_bytes(key_kind);
    if (init_limit) {
        h->initBits = 0;
        std::memcpy(&h->initBits, init_limit, kb);
    } else {
        h->initBits = kb == 8 ? ~0ull : 0xffffffffull;
    }
    const size_t stateB = align_up(sizeof(gh::HeapState), 256);
    const size_t itemsB = align_up(static_cast<size_t>(batch_num) * batch_size * kb, 256);
    const size_t pbB = align_up(static_cast<size_t>(batch_size) * kb, 256);
    const size_t lockB = align_up(static_cast<size_t>(batch_num) * 4, 256);
    const size_t scratchB = 256;
    if (cudaMalloc(&h->mem, stateB + itemsB + pbB + 2 * lockB + scratchB) != cudaSuccess) {
        cudaGetLastError();
        delete h;
        return GH_ERR_CUDA;
    }
    unsigned char* p = h->mem;
    h->state = reinterpret_cast<gh::HeapState*>(p);
    h->items = p + stateB;
    h->pbuf = p + stateB + itemsB;
    h->lock = reinterpret_cast<int*>(p + stateB + itemsB + pbB);
    h->taken = reinterpret_cast<int*>(p + stateB + itemsB + pbB + lockB);
    h->scratch = reinterpret_cast<int*>(p + stateB + itemsB + pbB + 2 * lockB);
    *out = h;
    const gh_status st = gh_rheap_reset(h, nullptr);
    if (st != GH_OK) {
        gh_rheap_destroy(h);
        *out = nullptr;
        return st;
    }
    return cudaDeviceSynchronize() == cudaSuccess ? GH_OK : GH_ERR_CUDA;
}

gh_status gh_rheap_destroy(gh_rheap* h) {
    if (!h) return GH_ERR_INVALID;
    if (h->mem) cudaFree(h->mem);
    delete h;
    return GH_OK;
}

gh_status gh_rheap_reset(gh_rheap* h, void* stream) {
    if (!h) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(h->state, 0, sizeof(gh::HeapState), s) != cudaSuccess ||
        cudaMemsetAsync(h->lock, 0, static_cast<size_t>(h->batchNum) * 4, s) != cudaSuccess ||
        cudaMemsetAsync(h->taken, 0, static_cast<size_t>(h->batchNum) * 4, s) != cudaSuccess)
        return GH_ERR_CUDA;
    // nodes and partial buffer to init_limit
    if (h->keyKind == GH_KEY_U64) {
        k_rheap_fill<u64><<<256, 256, 0, s>>>(static_cast<u64*>(h->items), static_cast<size_t>(h->batchNum) * h->batchSize, h->initBits);
        k_rheap_fill<u64><<<1, 256, 0, s>>>(static_cast<u64*>(h->pbuf), h->batchSize, h->initBits);
    } else {
        k_rheap_fill<unsigned><<<256, 256, 0, s>>>(static_cast<unsigned*>(h->items), static_cast<size_t>(h->batchNum) * h->batchSize,
                                                   static_cast<unsigned>(h->initBits));
        k_rheap_fill<unsigned><<<1, 256, 0, s>>>(static_cast<unsigned*>(h->pbuf), h->batchSize, static_cast<unsigned>(h->initBits));
    }
    gh::impl::count_launch();
    gh::impl::count_launch();
    return cudaGetLastError() == cudaSuccess ? GH_OK : GH_ERR_CUDA;
}

gh_status gh_rheap_set_timeout(gh_rheap* h, double seconds) {
    if (!h || !(seconds > 0.0) || seconds > 60.0) return GH_ERR_INVALID;
    h->timeoutNs = static_cast<long long>(seconds * 1e9);
    return GH_OK;
}

gh_status gh_rheap_insert(gh_rheap* h, const void* keys_dev, int count, void* stream) {
    gh::trace::Range range_("gh_rheap_insert");
    if (!h || count < 0 || count > h->batchSize || (count > 0 && !keys_dev)) return GH_ERR_INVALID;
    if (count == 0) return GH_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int T = h->threads;
    if (h->keyKind == GH_KEY_U64) {
        const size_t smem = gh::RetHeap<u64>::smemBytes(h->batchSize);
        if (allow_smem(k_rheap_insert<u64>, smem) != cudaSuccess) return GH_ERR_CUDA;
        k_rheap_insert<u64><<<1, T, smem, s>>>(view<u64>(h), static_cast<const u64*>(keys_dev), count);
    } else {
        const size_t smem = gh::RetHeap<unsigned>::smemBytes(h->batchSize);
        if (allow_smem(k_rheap_insert<unsigned>, smem) != cudaSuccess) return GH_ERR_CUDA;
        k_rheap_insert<unsigned><<<1, T, smem, s>>>(view<unsigned>(h), static_cast<const unsigned*>(keys_dev), count);
    }
    gh::impl::count_launch();
    return cudaGetLastError() == cudaSuccess ? GH_OK : GH_ERR_CUDA;
}

gh_status gh_rheap_retrieve(gh_rheap* h, void* out_dev, int* size, void* stream) {
    gh::trace::Range range_("gh_rheap_retrieve");
    if (!h || !size || *size < 0 || (*size > 0 && !out_dev)) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int T = h->threads;
    if (h->keyKind == GH_KEY_U64) {
        const size_t smem = gh::RetHeap<u64>::smemBytes(h->batchSize);
        if (allow_smem(k_rheap_retrieve<u64>, smem) != cudaSuccess) return GH_ERR_CUDA;
        k_rheap_retrieve<u64><<<1, T, smem, s>>>(view<u64>(h), static_cast<u64*>(out_dev), *size, h->scratch);
    } else {
        const size_t smem = gh::RetHeap<unsigned>::smemBytes(h->batchSize);
        if (allow_smem(k_rheap_retrieve<unsigned>, smem) != cudaSuccess) return GH_ERR_CUDA;
        k_rheap_retrieve<unsigned><<<1, T, smem, s>>>(view<unsigned>(h), static_cast<unsigned*>(out_dev), *size, h->scratch);
    }
    gh::impl::count_launch();
    if (cudaGetLastError() != cudaSuccess) return GH_ERR_CUDA;
    if (cudaMemcpyAsync(size, h->scratch, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GH_ERR_CUDA;
    return GH_OK;
}

gh_status gh_rheap_concurrent(gh_rheap* h, const void* keys_dev, long long n, int chunk, int inserters, int retrievers,
                              int size, void* out_dev, long long max_out, int* runs_dev, int max_runs,
                              long long* n_out, int* n_runs, void* stream) {
    gh::trace::Range range_("gh_rheap_concurrent");
    if (!h || n < 0 || chunk < 1 || chunk > h->batchSize || inserters < 1 || retrievers < 1 || size < 1 ||
        size > h->batchSize || (n > 0 && !keys_dev) || !out_dev || !runs_dev || max_runs < 1 || max_out < 0 ||
        inserters + retrievers > 65535)
        return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int T = h->threads;
    if (cudaMemsetAsync(h->scratch, 0, 64, s) != cudaSuccess) return GH_ERR_CUDA;
    const int grid = inserters + retrievers;
    if (h->keyKind == GH_KEY_U64) {
        const size_t smem = gh::RetHeap<u64>::smemBytes(h->batchSize) + static_cast<size_t>(h->batchSize) * 8;
        if (allow_smem(k_rheap_concurrent<u64>, smem) != cudaSuccess) return GH_ERR_CUDA;
        k_rheap_concurrent<u64><<<grid, T, smem, s>>>(view<u64>(h), static_cast<const u64*>(keys_dev), n, chunk, inserters,
                                                      size, static_cast<u64*>(out_dev), max_out, runs_dev, max_runs,
                                                      h->scratch);
    } else {
        const size_t smem = gh::RetHeap<unsigned>::smemBytes(h->batchSize) + static_cast<size_t>(h->batchSize) * 4;
        if (allow_smem(k_rheap_concurrent<unsigned>, smem) != cudaSuccess) return GH_ERR_CUDA;
        k_rheap_concurrent<unsigned><<<grid, T, smem, s>>>(view<unsigned>(h), static_cast<const unsigned*>(keys_dev), n,
                                                           chunk, inserters, size, static_cast<unsigned*>(out_dev),
                                                           max_out, runs_dev, max_runs, h->scratch);
    }
    gh::impl::count_launch();
    if (cudaGetLastError() != cudaSuccess) return GH_ERR_CUDA;
    int cur[6] = {0, 0, 0, 0, 0, 0};
    if (cudaMemcpyAsync(cur, h->scratch, sizeof(cur), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GH_ERR_CUDA;
    long long outN = 0;
    std::memcpy(&outN, cur + 2, 8);
    if (n_out) *n_out = outN;
    if (n_runs) *n_runs = cur[4];
    return (outN > max_out || cur[4] > max_runs) ? GH_ERR_CAPACITY : GH_OK;
}

gh_status gh_rheap_state(gh_rheap* h, void* items_host, void* pb_host, long long* counters_host) {
    if (!h) return GH_ERR_INVALID;
    if (cudaDeviceSynchronize() != cudaSuccess) return GH_ERR_CUDA;
    const int kb = key_bytes(h->keyKind);
    if (items_host &&
        cudaMemcpy(items_host, h->items, static_cast<size_t>(h->batchNum) * h->batchSize * kb, cudaMemcpyDeviceToHost) != cudaSuccess)
        return GH_ERR_CUDA;
    if (pb_host && cudaMemcpy(pb_host, h->pbuf, static_cast<size_t>(h->batchSize) * kb, cudaMemcpyDeviceToHost) != cudaSuccess)
        return GH_ERR_CUDA;
    if (counters_host) {
        gh::HeapState st;
        if (cudaMemcpy(&st, h->state, sizeof(st), cudaMemcpyDeviceToHost) != cudaSuccess) return GH_ERR_CUDA;
        counters_host[0] = st.batchCount;
        counters_host[1] = st.partialBufferSize;
        counters_host[2] = st.err;
        counters_host[3] = static_cast<long long>(st.appStats[gh::kRetSteals]);
        counters_host[4] = static_cast<long long>(st.appStats[gh::kRetFull]);
        counters_host[5] = st.errOp;
    }
    return GH_OK;
}

gh_status gh_sssp_retrieve(int n, const long long* rowptr_dev, const int* col_dev, const unsigned* w_dev, int source,
                           unsigned* dist_dev, int batch_size, int chunk, int blocks, long long capacity_keys,
                           void* stream, unsigned long long* stats_host) {
    gh::trace::Range range_("gh_sssp_retrieve");
    if (n < 1 || !rowptr_dev || !col_dev || !w_dev || !dist_dev || source < 0 || source >= n) return GH_ERR_INVALID;
    if (batch_size < 32 || batch_size > 1024 || (batch_size & (batch_size - 1)) || chunk < 1 || chunk > 4096 ||
        blocks < 1 || blocks > 4096 || capacity_keys < 0)
        return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    long long m = 0;
    if (cudaMemcpy(&m, rowptr_dev + n, sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess) return GH_ERR_CUDA;
    const long long keys = capacity_keys ? capacity_keys : (4LL * n > m / 2 ? 4LL * n : m / 2) + 16LL * batch_size;
    int bn = 2;
    while (static_cast<long long>(bn) * batch_size < keys) bn <<= 1;
    const u64 init = ~0ull;
    gh_rheap* h = nullptr;
    gh_status st = gh_rheap_create(&h, GH_KEY_U64, bn, batch_size, &init);
    if (st != GH_OK) return st;
    const int T = threads_for(batch_size);
    const long long auxCap = static_cast<long long>(batch_size) * blocks;
    u64* emit = nullptr;
    unsigned char* aux = nullptr;
    auto done = [&](gh_status r) {
        if (emit) cudaFree(emit);
        if (aux) cudaFree(aux);
        gh_rheap_destroy(h);
        return r;
    };
    if (cudaMalloc(&emit, static_cast<size_t>(blocks) * batch_size * chunk * 8) != cudaSuccess ||
        cudaMalloc(&aux, static_cast<size_t>(auxCap) * 12 + 256) != cudaSuccess) {
        cudaGetLastError();
        return done(GH_ERR_CUDA);
    }
    gh::RetHeapAux<u64, int> v;
    v.heap = view<u64>(h);
    v.auxCtl = reinterpret_cast<int*>(aux);
    v.auxKeys = reinterpret_cast<u64*>(aux + 256);
    v.auxData = reinterpret_cast<int*>(aux + 256 + static_cast<size_t>(auxCap) * 8);
    v.auxCap = static_cast<int>(auxCap);
    v.initAux = 0;
    const size_t smem = SsspRetSmem::bytes(batch_size) + gh::RetHeapAux<u64, int>::smemBytes(batch_size, T);
    if (cudaMemsetAsync(aux, 0, 256, s) != cudaSuccess) return done(GH_ERR_CUDA);
    if (cudaFuncSetAttribute(k_sssp_retrieve, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
        return done(GH_ERR_CUDA);
    k_sssp_retrieve_init<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, s>>>(dist_dev, n, source);
    if (allow_smem(k_sssp_retrieve_seed, 16 + gh::RetHeap<u64>::smemBytes(batch_size)) != cudaSuccess)
        return done(GH_ERR_CUDA);
    k_sssp_retrieve_seed<<<1, T, 16 + gh::RetHeap<u64>::smemBytes(batch_size), s>>>(v, source);
    k_sssp_retrieve<<<blocks, T, smem, s>>>(v, rowptr_dev, col_dev, w_dev, dist_dev, emit, chunk);
    gh::impl::count_launch();
    gh::impl::count_launch();
    gh::impl::count_launch();
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return done(GH_ERR_CUDA);
    gh::HeapState hs;
    if (cudaMemcpy(&hs, h->state, sizeof(hs), cudaMemcpyDeviceToHost) != cudaSuccess) return done(GH_ERR_CUDA);
    if (stats_host) {
        stats_host[0] = hs.appStats[4];
        stats_host[1] = hs.appStats[5];
        stats_host[2] = hs.appStats[6];
        stats_host[3] = hs.appStats[gh::kRetSteals];
    }
    const gh_status r = hs.err == 0 ? GH_OK
                        : hs.err == gh::kErrCapacity ? GH_ERR_CAPACITY
                        : hs.err == gh::kErrTimeout  ? GH_ERR_TIMEOUT
                                                     : GH_ERR_STATE;
    return done(r);
}

}  // extern "C"
