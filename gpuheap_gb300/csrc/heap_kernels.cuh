// Kernels behind the C ABI: bulk insert/delete drivers (the reference's
// insertKernel/deleteKernel of test/heap_test.cu:13-77), single-operation
// launches, device-side checkInsertHeap and state initialisation.
#pragma once
#include <climits>
#include <cstdint>

#include <atomic>

#include "gpuheap_device.cuh"

namespace gh {
namespace impl {

// Kernels this library has launched (reported by gh_launch_count).
extern std::atomic<long long> g_launches;
inline void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// Everything the host keeps about one heap, independent of the key type.
struct Desc {
    void* items;
    int* status;
    HeapState* state;
    uint64_t initBits;  // init_limits, in the low bytes
    int batchNum;
    int batchSize;
    long long timeoutNs;
    int variant;
    int pb;
    int keyBytes;
    void* mbox;  // owner-mode bulk delete: mailbox + lend buffers (null: plain deleteKernel only)
    int ownerDepth;  // owner-mode resident depth: -1 automatic, 0 off, else 2..4
};

// insertKernel: chunks of `chunk` keys, grid-strided over blocks.
template <typename H, typename K>
__global__ void __launch_bounds__(1024) k_insert(H h, const K* __restrict__ keys, long long n, int chunk) {
    const long long nchunks = (n + chunk - 1) / chunk;
    for (long long i = blockIdx.x; i < nchunks; i += gridDim.x) {
        const long long off = i * chunk;
        const long long rem = n - off;
        const int size = rem < chunk ? static_cast<int>(rem) : chunk;
        h.insertion(keys + off, size, 0);
        if (h.failed()) return;
    }
}

// Bulk insert of `m` full batches, step 1 (one thread): with the partial
// buffer empty, no error recorded and room for all of them, reserve targets
// batchCount+1 .. batchCount+m (batchCount moves past them now, as m
// node-0 hand-offs would have moved it); otherwise reserve nothing and the
// insert kernel takes node 0 per batch as the reference does.
static __global__ void k_reserve(HeapState* st, int batchNum, long long m) {
    const int bc = st->batchCount;
    const bool ok = m > 0 && st->err == 0 && st->partialBufferSize == 0 && bc + m <= batchNum;
    st->resvBase = bc;
    st->resvCount = ok ? static_cast<int>(m) : 0;
    st->resvTurn = bc + 1;
    if (ok) st->batchCount = bc + static_cast<int>(m);
}

// Step 2: the reserved targets' lock words take the state an insert holds
// its target in (top-down TARGET, bottom-up INUSE), so that an insert that
// reaches one before its own insert has written it waits there.
static __global__ void k_mark_reserved(const HeapState* st, int* status, int held) {
    const int base = st->resvBase, cnt = st->resvCount;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) status[base + 1 + i] = held;
}

// Step 3: insertKernel over the full batches; batch i goes to reserved
// target resvBase + 1 + i (batches in increasing order per block, so a
// block never waits on a target that it inserts later itself).  Without a
// reservation, insertion() as in k_insert.
template <typename H, typename K>
__global__ void __launch_bounds__(1024) k_insert_reserved(H h, const K* __restrict__ keys, long long m) {
    const int base = h.state->resvBase, cnt = h.state->resvCount;
    for (long long i = blockIdx.x; i < m; i += gridDim.x) {
        const K* src = keys + i * h.batchSize;
        if (cnt) h.insertionReserved(src, base + 1 + static_cast<int>(i), 0);
        else h.insertion(src, h.batchSize, 0);
        if (h.failed()) return;
    }
}

// One delete: deleteRoot, then deleteUpdate when it returns true, exactly
// as the reference's kernels call them.  Returns the number of keys written.
template <typename H, typename K>
__device__ __forceinline__ int delete_one(const H& h, K* out, K threshold, bool check) {
    int size = 0;
    h.deleteMinImpl(out, size, threshold, check, 0);
    return size;
}

// The reference's call pair itself, for the single-operation kernel.
template <typename H, typename K>
__device__ __forceinline__ int delete_root_update(const H& h, K* out) {
    int size = 0;
    if (h.deleteRoot(out, size)) h.deleteUpdate(0);
    return size;
}
template <typename H, typename K>
__device__ __forceinline__ int delete_one(const H& h, K* out) {
    return delete_one(h, out, h.init_limits, false);
}

// deleteKernel: every block deletes until the heap is empty, or (check)
// its smallest key is not below `threshold` (deleteRoot's app_t_val), or
// the output limit / an error stops it.  The blocks queue for node 0 by
// ticket (deleteRoot's `fair`), so none starves.
template <typename H, typename K>
__global__ void __launch_bounds__(1024) k_delete(H h, K* out, K threshold, int check) {
    for (;;) {
        int size = 0;
        h.deleteMinImpl(out, size, threshold, check != 0, 0, true);
        if (size == 0) break;
    }
}

// concurrentKernel (test/heap_test.cu:13-38): the first half of the grid
// inserts keys[0, n) in chunks of `chunk`, the second half makes
// `deletes` deleteRoot/deleteUpdate attempts, both grid-strided over their
// half, all at the same time.  An attempt on an empty heap writes nothing.
template <typename H, typename K>
__global__ void __launch_bounds__(1024) k_concurrent(H h, const K* __restrict__ keys, long long n, int chunk,
                                                     K* out, long long deletes) {
    const int half = gridDim.x / 2;
    if (static_cast<int>(blockIdx.x) < half) {
        const long long nchunks = (n + chunk - 1) / chunk;
        for (long long i = blockIdx.x; i < nchunks; i += half) {
            const long long off = i * chunk;
            const long long rem = n - off;
            h.insertion(keys + off, rem < chunk ? static_cast<int>(rem) : chunk, 0);
            if (h.failed()) return;
        }
    } else {
        for (long long i = blockIdx.x - half; i < deletes; i += gridDim.x - half) {
            delete_one(h, out);
            if (h.failed()) return;
        }
    }
}

// One retrieve of up to `want` keys by one block; the count goes to *sizeOut.
template <typename H, typename K>
__global__ void __launch_bounds__(1024) k_retrieve(H h, K* out, int want, K* scratch, int* sizeOut) {
    if constexpr (H::kHasPartialBuffer) {
        int size = want;
        h.retrieve(out, size, scratch, 0);
        if (threadIdx.x == 0) *sizeOut = size;
    }
}

// One delete by one block; the size goes to *sizeOut.
template <typename H, typename K>
__global__ void __launch_bounds__(1024) k_delete_one(H h, K* out, int* sizeOut) {
    const int size = delete_root_update(h, out);
    if (threadIdx.x == 0) *sizeOut = size;
}

template <typename K>
__global__ void k_fill(K* p, size_t n, K v) {
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = v;
}

static __global__ void k_init_state(HeapState* st, int deleteCount) {
    if (threadIdx.x == 0) {
        st->batchCount = 0;
        st->partialBufferSize = 0;
        st->deleteCount = deleteCount;
        st->outLimit = INT_MAX;
        st->insTicket = 0;
        st->resvBase = 0;
        st->resvCount = 0;
        st->resvTurn = 0;
        st->delTicket = 0;
        st->delServing = 0;
        st->err = 0;
        st->errOp = 0;
        st->errNode = 0;
        st->errState = 0;
        st->busy = 0;
        for (int q = 0; q < 8; ++q) st->appStats[q] = 0;
    }
}

// Sets the HEAP_SORT cursor (unless deleteCount < 0) and the output limit.
static __global__ void k_set_output(HeapState* st, int deleteCount, int outLimit) {
    if (threadIdx.x == 0) {
        if (deleteCount >= 0) st->deleteCount = deleteCount;
        st->outLimit = outLimit;
        st->delTicket = 0;
        st->delServing = 0;
    }
}

// Result of the device-side heap check.
// Garbage collection (the reference's invalidFilter + garbageCollection +
// HeapInsert, artifacts/astar/gc.cuh:77-180, artifacts/knapsack/gc.cuh:
// 30-180), all on the device.  Step 1: every used node (0 = partial buffer
// with its partialBufferSize keys, 1..batchCount full) keeps its keys below
// `threshold` -- a prefix, as nodes are sorted -- appended to `scratch` at a
// range that one atomicAdd per node claims; the node is refilled with
// `fill` (init_limits) and its lock word cleared.  The reference claims one
// slot per key with an atomicAdd.
template <typename K>
__global__ void __launch_bounds__(256) k_gc_compact(K* items, int* status, const HeapState* st, int B, K threshold,
                                                    K fill, K* __restrict__ scratch, unsigned long long* kept) {
    const int bc = st->batchCount, ps = st->partialBufferSize;
    __shared__ int s_cnt;
    __shared__ unsigned long long s_off;
    for (int i = blockIdx.x; i <= bc; i += gridDim.x) {
        K* nd = items + static_cast<size_t>(i) * B;
        const int len = i == 0 ? ps : B;
        if (threadIdx.x == 0) s_cnt = 0;
        __syncthreads();
        int c = 0;
        for (int j = threadIdx.x; j < len; j += blockDim.x) c += nd[j] < threshold ? 1 : 0;
        if (c) atomicAdd(&s_cnt, c);
        __syncthreads();
        const int cnt = s_cnt;
        if (threadIdx.x == 0) s_off = cnt ? atomicAdd(kept, static_cast<unsigned long long>(cnt)) : 0;
        __syncthreads();
        const unsigned long long off = s_off;
        for (int j = threadIdx.x; j < cnt; j += blockDim.x) scratch[off + j] = nd[j];
        __syncthreads();
        for (int j = threadIdx.x; j < B; j += blockDim.x) nd[j] = fill;
        if (threadIdx.x == 0) status[i] = 0;
        __syncthreads();
    }
}

// Step 2: the heap is empty again (the output cursor is kept).
static __global__ void k_gc_reset(HeapState* st) {
    st->batchCount = 0;
    st->partialBufferSize = 0;
}

// Step 3: insertKernel over scratch[0, *n) -- the count is read on the
// device, so the collection needs no round trip to the host.
template <typename H, typename K>
__global__ void __launch_bounds__(1024) k_insert_counted(H h, const K* __restrict__ keys, const unsigned long long* n,
                                                          int chunk) {
    const long long total = static_cast<long long>(*n);
    const long long nchunks = (total + chunk - 1) / chunk;
    for (long long i = blockIdx.x; i < nchunks; i += gridDim.x) {
        const long long off = i * chunk;
        const long long rem = total - off;
        h.insertion(keys + off, rem < chunk ? static_cast<int>(rem) : chunk, 0);
        if (h.failed()) return;
    }
}

struct CheckResult {
    int badNode;  // smallest failing node (INT_MAX when none)
    int code;     // what failed at badNode (see k_check)
    int detail;
    int pad;
};

__device__ __forceinline__ int rev_idx(int i) {
    if (i <= 1) return i;
    const int l = __clz(i) + 1;
    return static_cast<int>((__brev(static_cast<unsigned>(i)) >> l) | (1u << (32 - l)));
}

// checkInsertHeap on the device (heap/tditdd/heap.cuh:123-176,
// heap/buitdd/heap.cuh:118-172): one warp per node.  Codes: 1 status not
// AVAIL, 2 node unsorted, 3 node starts below its parent's end, 4 partial
// buffer unsorted, 5 partial buffer below the root, 6 partial buffer lock.
template <typename K>
__global__ void k_check(const K* __restrict__ items, const int* __restrict__ status, const HeapState* st,
                        int variant, int B, CheckResult* res) {
    const int bc = st->batchCount, ps = st->partialBufferSize;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    auto report = [&](int node, int code, int detail) {
        const int old = atomicMin(&res->badNode, node);
        if (old > node) { res->code = code; res->detail = detail; }
    };
    if (warp == 0) {
        if (lane == 0 && status[0] != 0) report(0, 6, status[0]);
        if (bc != 0 && ps != 0) {
            if (lane == 0 && items[2 * B - 1] > items[0]) report(0, 5, 0);
            for (int j = 1 + lane; j < ps; j += 32)
                if (items[j] < items[j - 1]) { report(0, 4, j); break; }
        }
    }
    for (int i = 1 + warp; i <= bc; i += nwarps) {
        const K* nd = items + static_cast<size_t>(i) * B;
        if (lane == 0) {
            if (status[i] != 0) report(i, 1, status[i]);
            if (i > 1) {
                const int p = variant == kTopDown ? i / 2 : rev_idx(rev_idx(i) >> 1);
                if (nd[0] < items[static_cast<size_t>(p) * B + B - 1]) report(i, 3, p);
            }
        }
        bool bad = false;
        int where = 0;
        for (int j = 1 + lane; j < B; j += 32)
            if (nd[j] < nd[j - 1]) { bad = true; where = j; break; }
        const unsigned m = __ballot_sync(0xffffffffu, bad);
        if (m) {
            const int src = __ffs(m) - 1;
            where = __shfl_sync(0xffffffffu, where, src);
            if (lane == 0) report(i, 2, where);
        }
    }
}

}  // namespace impl
}  // namespace gh
