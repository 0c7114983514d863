// Batched searches on the queue: many independent grid A* and 0/1 knapsack
// branch-and-bound instances of uneven size, each with its own heap, run by
// one persistent launch (or, as the baseline, one launch per instance).
//
// Caller patterns follow the reference's applications, written against this
// repository's device API (gh::Heap<uint64_t, ...>):
//   * A*: artifacts/astar/pq_model.cuh:299-371 and astar_item.cuh:12-53 (take
//     a batch of f << 32 | node keys, skip stale ones, expand, insert the
//     improved successors), on 4-connected grids of u8 cell costs
//     (0 = obstacle, a move costs the cost of the cell entered) with the
//     Manhattan heuristic; an incumbent (best goal cost so far, atomicMin)
//     prunes every key whose f is not below it, so the search drains and
//     the incumbent is the optimal cost;
//   * knapsack: artifacts/knapsack/models_pq.cuh:52-137 and
//     knapsackKernel.cuh:4-91 (take a batch of nodes, branch on the item at
//     the node's level: take it / skip it, prune on the Dantzig bound against
//     the best profit so far, atomicMax), best-first on the bound with ties
//     broken deepest first: the key is (INT32_MAX - bound) << 32 |
//     (1024 - level) << 20 | pool slot, and the node's (level, profit,
//     weight) sits in the instance's node pool (the reference keeps a 16-byte
//     record in the heap; here the heap stays on 8-byte keys).  Taking an
//     item keeps the parent's bound, so many nodes tie; deepest first reaches
//     good incumbents early, as a sequential best-first search does.
//
// Blocks find work through a task list: an instance appears once per block
// it should get (large grids several times, knapsacks once), largest first;
// blocks of one instance share its heap and stop by the protocol of
// worklist.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <thread>
#include <vector>

#include "gpuheap.h"
#include "heap_launch.cuh"
#include "worklist.cuh"

namespace {

using u64 = unsigned long long;
constexpr int kMaxKnapItems = 1024;
constexpr int kMaxSearchThreads = 512;  // 128 registers per thread
constexpr int kSlotBits = 20;            // knapsack key: pool slot bits below the level

__device__ __forceinline__ u64 knap_key(long long bound, int level, int slot) {
    return (static_cast<u64>(static_cast<unsigned>(INT_MAX - static_cast<int>(bound))) << 32) |
           (static_cast<u64>(kMaxKnapItems - level) << kSlotBits) | static_cast<unsigned>(slot);
}

// One instance, as the kernels see it (device array).
struct alignas(16) Inst {
    int kind;      // GH_SEARCH_ASTAR / GH_SEARCH_KNAPSACK
    int blocks;    // blocks that join it
    int batchNum;  // heap nodes
    int stop;      // set when an instance-level failure ends the search
    u64* items;
    int* status;
    gh::HeapState* state;
    // A*
    int width, height;
    const unsigned char* cost;
    unsigned* g;
    // knapsack: ratio-ordered items and exclusive prefix sums
    int n, poolCap;
    long long cap;
    const int* w;
    const int* p;
    const long long* W;
    const long long* P;
    int4* pool;  // (level, profit, weight, 0)
    int* freeList;
    int freeTop, bump;  // pool allocator, owned by the instance's single block
    // result and statistics
    int incumbent;  // A*: best goal cost (as unsigned); knapsack: best profit
    int failed;     // gh_status of a failure, 0 if none
    unsigned long long pops, expanded, inserted;
    int greedy;  // knapsack: profit of the greedy fill (first incumbent)
};

__device__ __forceinline__ unsigned astar_h(int v, int width, int height) {
    const int x = v % width, y = v / width;
    return static_cast<unsigned>((width - 1 - x) + (height - 1 - y));
}

// Dantzig bound of (level, profit, weight) from shared copies of the prefix
// sums (restates knapsackKernel.cuh:4-33 with a binary search for the break
// item and the fractional part floored).
__device__ __forceinline__ long long knap_bound(const long long* W, const long long* P, const int* w, const int* p,
                                                int n, long long cap, int level, long long profit, long long weight) {
    const long long rem = cap - weight;
    if (rem < 0) return -1;
    int lo = level, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (W[mid] - W[level] <= rem) lo = mid;
        else hi = mid - 1;
    }
    long long bound = profit + (P[lo] - P[level]);
    if (lo < n) bound += (rem - (W[lo] - W[level])) * p[lo] / w[lo];
    return bound;
}

// Reset of every instance's arrays: heap nodes to init keys, lock words to
// AVAIL, A* distances to infinity.  blockIdx.y = instance, blockIdx.x = slice.
__global__ void k_search_fill(Inst* insts, int B) {
    Inst* in = insts + blockIdx.y;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    const size_t first = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t keys = static_cast<size_t>(in->batchNum + 1) * B;
    for (size_t q = first; q < keys; q += stride) in->items[q] = ~0ull;
    for (size_t q = first; q < static_cast<size_t>(in->batchNum) + 2; q += stride) in->status[q] = 0;
    if (in->kind == GH_SEARCH_ASTAR) {
        const size_t cells = static_cast<size_t>(in->width) * in->height;
        for (size_t q = first; q < cells; q += stride) in->g[q] = 0xffffffffu;
    }
}

// Counters, incumbent and the seed key in the partial buffer (after the fill).
__global__ void k_search_seed(Inst* insts, int count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        Inst* in = insts + i;
        gh::HeapState* st = in->state;
        st->batchCount = 0;
        st->deleteCount = 0;
        st->outLimit = INT_MAX;
        st->insTicket = 0;
        st->err = st->errOp = st->errNode = st->errState = 0;
        st->busy = 0;
        for (int q = 0; q < 8; ++q) st->appStats[q] = 0;
        in->stop = 0;
        in->failed = 0;
        in->pops = in->expanded = in->inserted = 0;
        if (in->kind == GH_SEARCH_ASTAR) {
            const int goal = in->width * in->height - 1;
            const bool open = in->cost[0] != 0 && in->cost[goal] != 0;
            in->incumbent = open && goal == 0 ? 0 : static_cast<int>(0xffffffffu);
            if (open && goal != 0) {
                in->g[0] = 0;
                in->items[0] = static_cast<u64>(astar_h(0, in->width, in->height)) << 32;
            }
            st->partialBufferSize = open && goal != 0 ? 1 : 0;
        } else {
            in->freeTop = 0;
            in->bump = 1;
            in->incumbent = in->greedy;
            in->pool[0] = make_int4(0, 0, 0, 0);
            // root bound from the global prefix sums (knap_bound with level 0)
            int lo = 0, hi = in->n;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (in->W[mid] <= in->cap) lo = mid;
                else hi = mid - 1;
            }
            long long b = in->P[lo];
            if (lo < in->n) b += (in->cap - in->W[lo]) * in->p[lo] / in->w[lo];
            const bool live = b > in->greedy;
            if (live) in->items[0] = knap_key(b, 0, 0);
            st->partialBufferSize = live ? 1 : 0;
        }
    }
}

// Shared memory of a search block, ahead of the heap's region.
struct SearchSmem {
    static __host__ __device__ size_t emitKeys(int B, int T) { return static_cast<size_t>(B) + 4 * static_cast<size_t>(T); }
    static __host__ __device__ size_t bytes(int B, int T) {
        const size_t keys = (static_cast<size_t>(B) + emitKeys(B, T)) * 8;
        const size_t knap = static_cast<size_t>(kMaxKnapItems + 1) * 16 + static_cast<size_t>(kMaxKnapItems) * 8 +
                            static_cast<size_t>(B) * 16;
        return (keys + knap + 64 + 15) / 16 * 16;
    }
};

template <typename H>
__device__ __forceinline__ void flush_full(const H& heap, u64* emit, int* cnt, int B, int heapOff, unsigned long long& inserted) {
    __syncthreads();
    const int c = *cnt;
    if (c >= B) {
        heap.insertion(reinterpret_cast<typename H::key_type*>(emit), B, heapOff);
        for (int i = threadIdx.x; i < c - B; i += blockDim.x) emit[i] = emit[B + i];
        __syncthreads();
        if (threadIdx.x == 0) *cnt = c - B;
        inserted += B;
    }
    __syncthreads();
}

template <typename H>
__device__ __forceinline__ void flush_rest(const H& heap, u64* emit, int* cnt, int heapOff, unsigned long long& inserted) {
    __syncthreads();
    const int c = *cnt;
    if (c > 0) heap.insertion(reinterpret_cast<typename H::key_type*>(emit), c, heapOff);
    inserted += c;
    __syncthreads();
    if (threadIdx.x == 0) *cnt = 0;
    __syncthreads();
}

template <typename H>
__device__ void run_astar(const H& heap, Inst* in, unsigned char* smem, int heapOff) {
    const int B = heap.batchSize, T = blockDim.x, tid = threadIdx.x;
    u64* batch = reinterpret_cast<u64*>(smem);
    u64* emit = batch + B;
    int* ctl = reinterpret_cast<int*>(emit + SearchSmem::emitKeys(B, T));
    const int width = in->width, height = in->height;
    const int goal = width * height - 1;
    unsigned* g = in->g;
    const unsigned char* cost = in->cost;
    unsigned* inc = reinterpret_cast<unsigned*>(&in->incumbent);
    unsigned long long pops = 0, expanded = 0, inserted = 0, waitStart = 0;
    int lastBusy = -1;
    if (tid == 0) ctl[1] = 0;
    __syncthreads();
    for (;;) {
        if (gh::app::wait_for_keys(heap, &ctl[2], &in->stop, lastBusy, waitStart)) break;
        int size = 0;
        if (heap.deleteRoot(reinterpret_cast<typename H::key_type*>(batch), size)) heap.deleteUpdate(heapOff);
        pops += size;
        for (int base = 0; base < size; base += T) {
            const int i = base + tid;
            if (i < size) {
                const u64 key = batch[i];
                const unsigned f = static_cast<unsigned>(key >> 32);
                const int v = static_cast<int>(key & 0xffffffffu);
                const unsigned best = __ldcg(inc);
                const unsigned hv = astar_h(v, width, height);
                const unsigned gv = f - hv;
                if (f < best && gv <= __ldcg(g + v)) {  // not pruned, not stale
                    ++expanded;
                    const int x = v % width, y = v / width;
                    const int nb[4] = {x > 0 ? v - 1 : -1, x + 1 < width ? v + 1 : -1, y > 0 ? v - width : -1,
                                       y + 1 < height ? v + width : -1};
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int u = nb[k];
                        if (u < 0) continue;
                        const unsigned c = cost[u];
                        if (c == 0) continue;
                        const unsigned ng = gv + c;
                        if (u == goal) {
                            if (ng < __ldcg(g + u)) atomicMin(g + u, ng);
                            atomicMin(inc, ng);
                            continue;
                        }
                        const unsigned nf = ng + astar_h(u, width, height);
                        if (nf >= __ldcg(inc) || ng >= __ldcg(g + u)) continue;
                        if (ng < atomicMin(g + u, ng)) emit[atomicAdd(&ctl[1], 1)] = (static_cast<u64>(nf) << 32) | static_cast<unsigned>(u);
                    }
                }
            }
            flush_full(heap, emit, &ctl[1], B, heapOff, inserted);
        }
        flush_rest(heap, emit, &ctl[1], heapOff, inserted);
        gh::app::batch_done(heap.state);
        if (heap.failed()) break;
    }
    if (tid == 0) {
        atomicAdd(&in->pops, pops);
        atomicAdd(&in->inserted, inserted);
    }
    atomicAdd(&in->expanded, expanded);
}

template <typename H>
__device__ void run_knapsack(const H& heap, Inst* in, unsigned char* smem, int heapOff) {
    const int B = heap.batchSize, T = blockDim.x, tid = threadIdx.x;
    u64* batch = reinterpret_cast<u64*>(smem);
    u64* emit = batch + B;
    long long* sW = reinterpret_cast<long long*>(emit + SearchSmem::emitKeys(B, T));
    long long* sP = sW + kMaxKnapItems + 1;
    int* sw = reinterpret_cast<int*>(sP + kMaxKnapItems + 1);
    int* sp = sw + kMaxKnapItems;
    int4* nodes = reinterpret_cast<int4*>(sp + kMaxKnapItems);
    int* ctl = reinterpret_cast<int*>(nodes + B);
    const int n = in->n;
    const long long cap = in->cap;
    for (int i = tid; i <= n; i += T) { sW[i] = in->W[i]; sP[i] = in->P[i]; }
    for (int i = tid; i < n; i += T) { sw[i] = in->w[i]; sp[i] = in->p[i]; }
    if (tid == 0) { ctl[1] = 0; ctl[3] = in->freeTop; ctl[4] = in->bump; ctl[5] = 0; }
    __syncthreads();
    int* best = &in->incumbent;
    int4* pool = in->pool;
    int* freeList = in->freeList;
    const int poolCap = in->poolCap;
    unsigned long long pops = 0, expanded = 0, inserted = 0, waitStart = 0;
    int lastBusy = -1;
    for (;;) {
        if (gh::app::wait_for_keys(heap, &ctl[2], &in->stop, lastBusy, waitStart)) break;
        int size = 0;
        if (heap.deleteRoot(reinterpret_cast<typename H::key_type*>(batch), size)) heap.deleteUpdate(heapOff);
        pops += size;
        // read the popped nodes, then return their slots
        constexpr unsigned kSlotMask = (1u << kSlotBits) - 1;
        for (int i = tid; i < size; i += T) nodes[i] = pool[static_cast<unsigned>(batch[i]) & kSlotMask];
        __syncthreads();
        for (int i = tid; i < size; i += T) freeList[ctl[3] + i] = static_cast<int>(static_cast<unsigned>(batch[i]) & kSlotMask);
        __syncthreads();
        if (tid == 0) ctl[3] += size;
        __syncthreads();
        for (int base = 0; base < size; base += T) {
            const int i = base + tid;
            if (i < size) {
                const int4 nd = nodes[i];
                const int level = nd.x;
                const long long profit = nd.y, weight = nd.z;
                const long long b = knap_bound(sW, sP, sw, sp, n, cap, level, profit, weight);
                if (b > __ldcg(best) && level < n) {
                    ++expanded;
                    long long cb[2] = {-1, -1};
                    int cp[2] = {0, 0}, cw[2] = {0, 0};
                    if (weight + sw[level] <= cap) {  // take the item
                        cp[0] = static_cast<int>(profit + sp[level]);
                        cw[0] = static_cast<int>(weight + sw[level]);
                        atomicMax(best, cp[0]);
                        cb[0] = knap_bound(sW, sP, sw, sp, n, cap, level + 1, cp[0], cw[0]);
                    }
                    cp[1] = static_cast<int>(profit);  // skip it
                    cw[1] = static_cast<int>(weight);
                    cb[1] = knap_bound(sW, sP, sw, sp, n, cap, level + 1, cp[1], cw[1]);
#pragma unroll
                    for (int k = 0; k < 2; ++k) {
                        if (cb[k] <= __ldcg(best)) continue;
                        int slot;
                        const int top = atomicSub(&ctl[3], 1) - 1;
                        if (top >= 0) slot = freeList[top];
                        else slot = atomicAdd(&ctl[4], 1);
                        if (slot >= poolCap) { ctl[5] = 1; continue; }
                        pool[slot] = make_int4(level + 1, cp[k], cw[k], 0);
                        emit[atomicAdd(&ctl[1], 1)] = knap_key(cb[k], level + 1, slot);
                    }
                }
            }
            __syncthreads();
            if (tid == 0 && ctl[3] < 0) ctl[3] = 0;
            flush_full(heap, emit, &ctl[1], B, heapOff, inserted);
        }
        flush_rest(heap, emit, &ctl[1], heapOff, inserted);
        if (ctl[5]) {  // node pool exhausted
            if (tid == 0) { in->failed = GH_ERR_CAPACITY; gh::detail::st_relaxed(&in->stop, 1); }
        }
        gh::app::batch_done(heap.state);
        if (heap.failed() || ctl[5]) break;
    }
    if (tid == 0) {
        in->freeTop = ctl[3];
        in->bump = ctl[4];
        atomicAdd(&in->pops, pops);
        atomicAdd(&in->inserted, inserted);
    }
    atomicAdd(&in->expanded, expanded);
}

template <typename H>
__global__ void __launch_bounds__(kMaxSearchThreads, 1) k_search(H proto, Inst* insts, const int* tasks, int ntasks, int* next) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_task;
    const int heapOff = static_cast<int>(SearchSmem::bytes(proto.batchSize, blockDim.x) / 4);
    for (;;) {
        if (threadIdx.x == 0) s_task = atomicAdd(next, 1);
        __syncthreads();
        const int t = s_task;
        __syncthreads();
        if (t >= ntasks) break;
        Inst* in = insts + tasks[t];
        H h = proto;
        h.heapItems = reinterpret_cast<typename H::key_type*>(in->items);
        h.status = in->status;
        h.state = in->state;
        h.batchNum = in->batchNum;
        if (in->kind == GH_SEARCH_ASTAR) run_astar(h, in, smem, heapOff);
        else run_knapsack(h, in, smem, heapOff);
        __syncthreads();
    }
}

// Records instance failures from the heap's own error word.
__global__ void k_search_collect(Inst* insts, int count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        Inst* in = insts + i;
        const int err = in->state->err;
        if (err && !in->failed) in->failed = err == gh::kErrCapacity ? GH_ERR_CAPACITY : err == gh::kErrTimeout ? GH_ERR_TIMEOUT : GH_ERR_STATE;
        if (!in->failed && (in->state->batchCount != 0 || in->state->partialBufferSize != 0) && !in->stop)
            in->failed = GH_ERR_STATE;
    }
}

template <int V, int IPT>
cudaError_t launch_search(const gh::Heap<uint64_t, V, true, IPT>& proto, Inst* insts, const int* tasks, int ntasks,
                          int* next, int grid, int threads, size_t smem, cudaStream_t s) {
    using H = gh::Heap<uint64_t, V, true, IPT>;
    cudaError_t e = cudaFuncSetAttribute(k_search<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    k_search<H><<<grid, threads, smem, s>>>(proto, insts, tasks, ntasks, next);
    gh::impl::count_launch();
    return cudaGetLastError();
}

}  // namespace

// ---------------------------------------------------------------------- host side
struct HostInst {
    int kind;
    int width = 0, height = 0;
    std::vector<unsigned char> cost;
    std::vector<int> w, p;  // ratio-ordered
    std::vector<long long> W, P;
    long long cap = 0;
    int greedy = 0;
    int blocks = 1;
    long long work = 0;  // size estimate for the task order
};

struct gh_batch {
    int batchSize = 256, variant = GH_BOTTOMUP, threads = 0;
    long long timeoutNs = 2000000000LL;
    long long astarCellsPerBlock = 1 << 18;
    int astarMaxBlocks = 8;
    int device = 0, numSMs = 0;
    std::vector<HostInst> host;
    // device
    unsigned char* arena = nullptr;
    size_t arenaBytes = 0;
    Inst* insts = nullptr;
    int* tasks = nullptr;  // batched order, then per-instance segments
    int* next = nullptr;   // [0] batched counter, [1 + i] per-instance counters
    int ntasks = 0;
    std::vector<int> segOff, segLen;
    std::vector<Inst> hinst;
    cudaGraphExec_t graph = nullptr;
    cudaStream_t graphStream = nullptr;
    long long graphLaunches = 0;
    int grid = 0;  // blocks of the persistent launch
    bool built = false;
};

namespace {

int threads_for(const gh_batch* b) {
    if (b->threads) return b->threads;
    return std::min(kMaxSearchThreads, b->batchSize);  // 2 keys per thread per merge (4 at batch 1024)
}

size_t smem_for(const gh_batch* b) {
    const int T = threads_for(b);
    return SearchSmem::bytes(b->batchSize, T) + 16 + gh::Heap<uint64_t, 0, true>::smemBytes(b->batchSize);
}

int resident_blocks(const gh_batch* b) {
    int per = 0;
    const int T = threads_for(b);
    const size_t smem = smem_for(b);
    const int ipt = 2 * b->batchSize / T;
    cudaError_t e = cudaErrorInvalidValue;
    auto occ = [&](auto kern) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, T, smem);
    };
    if (b->variant == GH_TOPDOWN) {
        if (ipt == 2) e = occ(k_search<gh::Heap<uint64_t, gh::kTopDown, true, 2>>);
        if (ipt == 4) e = occ(k_search<gh::Heap<uint64_t, gh::kTopDown, true, 4>>);
    } else {
        if (ipt == 2) e = occ(k_search<gh::Heap<uint64_t, gh::kBottomUp, true, 2>>);
        if (ipt == 4) e = occ(k_search<gh::Heap<uint64_t, gh::kBottomUp, true, 4>>);
    }
    if (e != cudaSuccess || per < 1) per = 1;
    return per * b->numSMs;
}

cudaError_t launch(const gh_batch* b, const int* tasks, int ntasks, int* next, int grid, cudaStream_t s) {
    const int T = threads_for(b);
    const int ipt = 2 * b->batchSize / T;
    const size_t smem = smem_for(b);
    auto proto = [&](auto h) {
        h.heapItems = nullptr;
        h.status = nullptr;
        h.state = nullptr;
        h.init_limits = ~0ull;
        h.batchNum = 0;
        h.batchSize = b->batchSize;
        h.sortOutput = 0;
        h.timeoutNs = b->timeoutNs;
        return h;
    };
    if (b->variant == GH_TOPDOWN) {
        if (ipt == 2) return launch_search<gh::kTopDown, 2>(proto(gh::Heap<uint64_t, gh::kTopDown, true, 2>{}), b->insts, tasks, ntasks, next, grid, T, smem, s);
        if (ipt == 4) return launch_search<gh::kTopDown, 4>(proto(gh::Heap<uint64_t, gh::kTopDown, true, 4>{}), b->insts, tasks, ntasks, next, grid, T, smem, s);
    } else {
        if (ipt == 2) return launch_search<gh::kBottomUp, 2>(proto(gh::Heap<uint64_t, gh::kBottomUp, true, 2>{}), b->insts, tasks, ntasks, next, grid, T, smem, s);
        if (ipt == 4) return launch_search<gh::kBottomUp, 4>(proto(gh::Heap<uint64_t, gh::kBottomUp, true, 4>{}), b->insts, tasks, ntasks, next, grid, T, smem, s);
    }
    return cudaErrorInvalidValue;
}

void free_device(gh_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    if (b->arena) cudaFree(b->arena);
    b->arena = nullptr;
    b->insts = nullptr;
    b->tasks = nullptr;
    b->next = nullptr;
    b->built = false;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Heap nodes for an instance: a power of two holding its open-list bound.
int heap_nodes(long long keys, int B) {
    long long nodes = (keys + B - 1) / B;
    int bn = 1;
    while (bn < nodes) bn <<= 1;
    return bn;
}

gh_status reset_and_run(gh_batch* b, int mode, cudaStream_t s);

}  // namespace

extern "C" {

gh_status gh_batch_create(gh_batch** out, int batch_size, int variant, int block_threads) {
    if (!out) return GH_ERR_INVALID;
    *out = nullptr;
    if (batch_size < 32 || batch_size > 1024 || (batch_size & (batch_size - 1))) return GH_ERR_INVALID;
    if (variant != GH_TOPDOWN && variant != GH_BOTTOMUP) return GH_ERR_INVALID;
    if (block_threads != 0 && block_threads != batch_size && block_threads != batch_size / 2) return GH_ERR_INVALID;
    if (block_threads > kMaxSearchThreads) return GH_ERR_INVALID;
    gh_batch* b = new (std::nothrow) gh_batch();
    if (!b) return GH_ERR_INVALID;
    b->batchSize = batch_size;
    b->variant = variant;
    b->threads = block_threads;
    if (cudaGetDevice(&b->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&b->numSMs, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess) {
        delete b;
        return GH_ERR_CUDA;
    }
    *out = b;
    return GH_OK;
}

gh_status gh_batch_destroy(gh_batch* b) {
    if (!b) return GH_ERR_INVALID;
    free_device(b);
    if (b->graphStream) cudaStreamDestroy(b->graphStream);
    delete b;
    return GH_OK;
}

gh_status gh_batch_set_astar_blocks(gh_batch* b, long long cells_per_block, int max_blocks) {
    if (!b || cells_per_block < 1 || max_blocks < 1 || max_blocks > 64) return GH_ERR_INVALID;
    b->astarCellsPerBlock = cells_per_block;
    b->astarMaxBlocks = max_blocks;
    if (b->built) free_device(b);
    return GH_OK;
}

gh_status gh_batch_set_timeout(gh_batch* b, double seconds) {
    if (!b || !(seconds > 0) || seconds > 60.0) return GH_ERR_INVALID;
    b->timeoutNs = static_cast<long long>(seconds * 1e9);
    if (b->built) free_device(b);
    return GH_OK;
}

gh_status gh_batch_add_astar(gh_batch* b, int width, int height, const unsigned char* cost_host, int* id) {
    if (!b || !cost_host || width < 1 || height < 1 || static_cast<long long>(width) * height > (1LL << 30))
        return GH_ERR_INVALID;
    HostInst h;
    h.kind = GH_SEARCH_ASTAR;
    h.width = width;
    h.height = height;
    h.cost.assign(cost_host, cost_host + static_cast<size_t>(width) * height);
    h.work = static_cast<long long>(width) * height;
    if (id) *id = static_cast<int>(b->host.size());
    b->host.push_back(std::move(h));
    if (b->built) free_device(b);
    return GH_OK;
}

gh_status gh_batch_add_knapsack(gh_batch* b, int n, const int* weight_host, const int* profit_host, long long capacity,
                                int* id) {
    if (!b || n < 1 || n > kMaxKnapItems || !weight_host || !profit_host || capacity < 0) return GH_ERR_INVALID;
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        if (weight_host[i] < 1 || profit_host[i] < 0) return GH_ERR_INVALID;
        total += profit_host[i];
    }
    if (total >= INT_MAX / 2 || capacity >= (1LL << 40)) return GH_ERR_INVALID;
    HostInst h;
    h.kind = GH_SEARCH_KNAPSACK;
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
        return static_cast<long long>(profit_host[x]) * weight_host[y] > static_cast<long long>(profit_host[y]) * weight_host[x];
    });
    h.w.resize(n);
    h.p.resize(n);
    h.W.assign(n + 1, 0);
    h.P.assign(n + 1, 0);
    long long wt = 0, pr = 0;
    for (int i = 0; i < n; ++i) {
        h.w[i] = weight_host[ord[i]];
        h.p[i] = profit_host[ord[i]];
        h.W[i + 1] = h.W[i] + h.w[i];
        h.P[i + 1] = h.P[i] + h.p[i];
        if (wt + h.w[i] <= capacity) { wt += h.w[i]; pr += h.p[i]; }
    }
    h.cap = capacity;
    h.greedy = static_cast<int>(pr);
    h.work = n;
    if (id) *id = static_cast<int>(b->host.size());
    b->host.push_back(std::move(h));
    if (b->built) free_device(b);
    return GH_OK;
}

// Lays out the arena, uploads every instance and builds the task lists.
gh_status gh_batch_build(gh_batch* b, void* stream) {
    if (!b || b->host.empty() || b->host.size() > 65535) return GH_ERR_INVALID;  // fill grid: one y-row per instance
    free_device(b);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int B = b->batchSize;
    const int count = static_cast<int>(b->host.size());
    // sizes
    struct Lay { size_t items, status, state, cost, g, w, p, W, P, pool, freeList; int bn, poolCap; };
    std::vector<Lay> lay(count);
    size_t off = align_up(sizeof(Inst) * count, 256);
    size_t tasksOff = 0, nextOff = 0;
    std::vector<int> blocks(count, 1);
    for (int i = 0; i < count; ++i) {
        const HostInst& h = b->host[i];
        Lay& L = lay[i];
        long long keys;
        if (h.kind == GH_SEARCH_ASTAR) {
            const long long side = std::max(h.width, h.height);
            keys = std::max<long long>(64 * side, 16LL * B);
            const long long cells = static_cast<long long>(h.width) * h.height;
            blocks[i] = static_cast<int>(std::min<long long>(b->astarMaxBlocks, std::max<long long>(1, cells / b->astarCellsPerBlock)));
        } else {
            // batched branch-and-bound explores far more nodes than a
            // sequential one; pool slots must fit the key's 20 bits
            keys = std::min<long long>(1LL << 19, std::max<long long>({1LL << 16, 64LL * B, 256LL * static_cast<long long>(h.w.size())}));
        }
        L.bn = heap_nodes(keys, B);
        L.state = off; off = align_up(off + sizeof(gh::HeapState), 256);
        L.items = off; off = align_up(off + static_cast<size_t>(L.bn + 1) * B * 8, 256);
        L.status = off; off = align_up(off + static_cast<size_t>(L.bn + 2) * 4, 256);
        if (h.kind == GH_SEARCH_ASTAR) {
            const size_t cells = static_cast<size_t>(h.width) * h.height;
            L.cost = off; off = align_up(off + cells, 256);
            L.g = off; off = align_up(off + cells * 4, 256);
        } else {
            const int n = static_cast<int>(h.w.size());
            L.poolCap = std::min((L.bn + 1) * B + 4 * B, 1 << kSlotBits);
            L.w = off; off = align_up(off + n * 4, 256);
            L.p = off; off = align_up(off + n * 4, 256);
            L.W = off; off = align_up(off + (n + 1) * 8, 256);
            L.P = off; off = align_up(off + (n + 1) * 8, 256);
            L.pool = off; off = align_up(off + static_cast<size_t>(L.poolCap) * 16, 256);
            L.freeList = off; off = align_up(off + static_cast<size_t>(L.poolCap + B) * 4, 256);
        }
    }
    // task order: largest instances first, each instance's blocks together
    // (they start on one heap at about the same time)
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->host[x].work > b->host[y].work; });
    std::vector<int> batched;
    for (int i : order)
        for (int r = 0; r < blocks[i]; ++r) batched.push_back(i);
    b->ntasks = static_cast<int>(batched.size());
    b->segOff.assign(count, 0);
    b->segLen.assign(count, 0);
    std::vector<int> tasks(batched);
    for (int i = 0; i < count; ++i) {
        b->segOff[i] = static_cast<int>(tasks.size());
        b->segLen[i] = blocks[i];
        for (int r = 0; r < blocks[i]; ++r) tasks.push_back(i);
    }
    tasksOff = off; off = align_up(off + tasks.size() * 4, 256);
    nextOff = off; off = align_up(off + static_cast<size_t>(count + 1) * 4, 256);
    b->arenaBytes = off;
    if (cudaMalloc(&b->arena, off) != cudaSuccess) {
        cudaGetLastError();
        b->arena = nullptr;
        return GH_ERR_CUDA;
    }
    unsigned char* A = b->arena;
    b->insts = reinterpret_cast<Inst*>(A);
    b->tasks = reinterpret_cast<int*>(A + tasksOff);
    b->next = reinterpret_cast<int*>(A + nextOff);
    b->hinst.assign(count, Inst{});
    for (int i = 0; i < count; ++i) {
        const HostInst& h = b->host[i];
        const Lay& L = lay[i];
        Inst& d = b->hinst[i];
        std::memset(&d, 0, sizeof(d));
        d.kind = h.kind;
        d.blocks = blocks[i];
        d.batchNum = L.bn;
        d.items = reinterpret_cast<u64*>(A + L.items);
        d.status = reinterpret_cast<int*>(A + L.status);
        d.state = reinterpret_cast<gh::HeapState*>(A + L.state);
        if (h.kind == GH_SEARCH_ASTAR) {
            d.width = h.width;
            d.height = h.height;
            d.cost = A + L.cost;
            d.g = reinterpret_cast<unsigned*>(A + L.g);
            if (cudaMemcpyAsync(A + L.cost, h.cost.data(), h.cost.size(), cudaMemcpyHostToDevice, s) != cudaSuccess) return GH_ERR_CUDA;
        } else {
            const int n = static_cast<int>(h.w.size());
            d.n = n;
            d.cap = h.cap;
            d.poolCap = L.poolCap;
            d.w = reinterpret_cast<const int*>(A + L.w);
            d.p = reinterpret_cast<const int*>(A + L.p);
            d.W = reinterpret_cast<const long long*>(A + L.W);
            d.P = reinterpret_cast<const long long*>(A + L.P);
            d.pool = reinterpret_cast<int4*>(A + L.pool);
            d.freeList = reinterpret_cast<int*>(A + L.freeList);
            d.greedy = h.greedy;
            if (cudaMemcpyAsync(A + L.w, h.w.data(), n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                cudaMemcpyAsync(A + L.p, h.p.data(), n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                cudaMemcpyAsync(A + L.W, h.W.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                cudaMemcpyAsync(A + L.P, h.P.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
                return GH_ERR_CUDA;
        }
    }
    if (cudaMemcpyAsync(b->insts, b->hinst.data(), sizeof(Inst) * count, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b->tasks, tasks.data(), tasks.size() * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GH_ERR_CUDA;
    b->grid = std::min(resident_blocks(b), b->ntasks);
    b->built = true;
    return GH_OK;
}

// mode GH_BATCH_PERSISTENT: one persistent launch for every instance;
// GH_BATCH_GRAPH: the same, replayed from a captured CUDA graph;
// GH_BATCH_PLAIN: one launch per instance, back to back.
gh_status gh_batch_run(gh_batch* b, int mode, void* stream) {
    if (!b || !b->built) return GH_ERR_INVALID;
    if (mode != GH_BATCH_PERSISTENT && mode != GH_BATCH_GRAPH && mode != GH_BATCH_PLAIN) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (mode == GH_BATCH_GRAPH) {
        if (!b->graph) {
            if (!b->graphStream && cudaStreamCreateWithFlags(&b->graphStream, cudaStreamNonBlocking) != cudaSuccess)
                return GH_ERR_CUDA;
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(b->graphStream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return GH_ERR_CUDA;
            const long long before = gh::impl::g_launches.load();
            gh_status st = reset_and_run(b, GH_BATCH_PERSISTENT, b->graphStream);
            cudaError_t e = cudaStreamEndCapture(b->graphStream, &g);
            b->graphLaunches = gh::impl::g_launches.load() - before;
            gh::impl::g_launches.fetch_sub(b->graphLaunches);  // captured, not run
            if (st != GH_OK || e != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return st != GH_OK ? st : GH_ERR_CUDA;
            }
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { b->graph = nullptr; return GH_ERR_CUDA; }
        }
        if (cudaGraphLaunch(b->graph, s) != cudaSuccess) return GH_ERR_CUDA;
        gh::impl::g_launches.fetch_add(b->graphLaunches);  // fill, seed, search, collect
        return GH_OK;
    }
    return reset_and_run(b, mode, s);
}

gh_status gh_batch_results(gh_batch* b, long long* results, int* status, unsigned long long* stats, void* stream) {
    if (!b || !b->built) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int count = static_cast<int>(b->host.size());
    if (cudaMemcpyAsync(b->hinst.data(), b->insts, sizeof(Inst) * count, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GH_ERR_CUDA;
    gh_status worst = GH_OK;
    for (int i = 0; i < count; ++i) {
        const Inst& d = b->hinst[i];
        if (results) {
            if (d.kind == GH_SEARCH_ASTAR) results[i] = static_cast<long long>(static_cast<unsigned>(d.incumbent));
            else results[i] = d.incumbent;
        }
        if (status) status[i] = d.failed;
        if (stats) {
            stats[3 * i] = d.pops;
            stats[3 * i + 1] = d.expanded;
            stats[3 * i + 2] = d.inserted;
        }
        if (d.failed && worst == GH_OK) worst = static_cast<gh_status>(d.failed);
    }
    return worst;
}

gh_status gh_batch_info(gh_batch* b, int* count, int* tasks, int* grid, int* threads, long long* arena_bytes) {
    if (!b) return GH_ERR_INVALID;
    if (count) *count = static_cast<int>(b->host.size());
    if (tasks) *tasks = b->ntasks;
    if (grid) *grid = b->built ? b->grid : resident_blocks(b);
    if (threads) *threads = threads_for(b);
    if (arena_bytes) *arena_bytes = static_cast<long long>(b->arenaBytes);
    return GH_OK;
}

}  // extern "C"

namespace {

gh_status reset_and_run(gh_batch* b, int mode, cudaStream_t s) {
    const int count = static_cast<int>(b->host.size());
    if (cudaMemsetAsync(b->next, 0, static_cast<size_t>(count + 1) * 4, s) != cudaSuccess) return GH_ERR_CUDA;
    k_search_fill<<<dim3(8, count), 256, 0, s>>>(b->insts, b->batchSize);
    gh::impl::count_launch();
    k_search_seed<<<(count + 127) / 128, 128, 0, s>>>(b->insts, count);
    gh::impl::count_launch();
    if (cudaGetLastError() != cudaSuccess) return GH_ERR_CUDA;
    if (mode == GH_BATCH_PLAIN) {
        for (int i = 0; i < count; ++i) {
            if (launch(b, b->tasks + b->segOff[i], b->segLen[i], b->next + 1 + i, b->segLen[i], s) != cudaSuccess)
                return GH_ERR_CUDA;
        }
    } else {
        if (launch(b, b->tasks, b->ntasks, b->next, b->grid, s) != cudaSuccess) return GH_ERR_CUDA;
    }
    k_search_collect<<<std::max(1, std::min(count / 256 + 1, 1024)), 256, 0, s>>>(b->insts, count);
    gh::impl::count_launch();
    return cudaGetLastError() == cudaSuccess ? GH_OK : GH_ERR_CUDA;
}

}  // namespace

// ---------------------------------------------------------------------- workload generator
namespace {
inline u64 host_mix64(u64 z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
}  // namespace

extern "C" gh_status gh_gen_grid(int width, int height, unsigned long long seed, int obstacle_per_mille,
                                 unsigned char* out_host, int threads) {
    if (width < 1 || height < 1 || !out_host || obstacle_per_mille < 0 || obstacle_per_mille > 1000) return GH_ERR_INVALID;
    const long long cells = static_cast<long long>(width) * height;
    if (threads < 1) threads = 1;
    auto fill = [=](long long lo, long long hi) {
        for (long long i = lo; i < hi; ++i) {
            const u64 r = host_mix64(seed + (static_cast<u64>(i) + 1) * 0x9e3779b97f4a7c15ULL);
            const bool blocked = static_cast<int>((r >> 32) % 1000) < obstacle_per_mille;
            const unsigned char c = static_cast<unsigned char>(1 + (r & 0xffffffffu) % 9);
            out_host[i] = blocked && i != 0 && i != cells - 1 ? 0 : c;
        }
    };
    std::vector<std::thread> pool;
    const long long per = (cells + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const long long lo = t * per, hi = std::min(cells, lo + per);
        if (lo < hi) pool.emplace_back(fill, lo, hi);
    }
    for (auto& th : pool) th.join();
    return GH_OK;
}
