// Device side of the searches on the queue: many independent grid A* and 0/1 knapsack
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
// Knapsack instances can also run the reference's other two models on the
// same node pool: breadth-first through a FIFO ring (models_fifo.cuh:13-112,
// gh::Fifo) and the heap/FIFO switch (models.cuh:23-440): heap mode until
// `switchCounter` batches in a row insert children without raising the best
// profit, FIFO mode until that many batches in a row raise it; at a switch
// every live node moves across and nodes that can no longer beat the best
// are dropped (the reference's invalidFilter between modes).
//
// Blocks find work through a task list: an instance appears once per block
// it should get (large grids several times, knapsacks once), largest first;
// blocks of one instance share its heap and stop by the protocol of
// worklist.cuh.
#pragma once
#include <cuda_runtime.h>

#include <climits>

#include "gpuheap.h"
#include "gpuheap_fifo.cuh"
#include "heap_launch.cuh"
#include "sssp_relax.cuh"
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
    int kind;      // GH_SEARCH_ASTAR / GH_SEARCH_KNAPSACK / GH_SEARCH_SSSP
    int blocks;    // blocks that join it
    int batchNum;  // heap nodes
    int stop;      // set when an instance-level failure ends the search
    u64* items;
    int* status;
    gh::HeapState* state;
    // A*: grid, start and goal cell; SSSP: g holds the distances
    int width, height;
    const unsigned char* cost;
    unsigned* g;
    int start, goal;
    // SSSP: CSR graph with nv vertices, source vertex
    int nv, source;
    const long long* rowptr;
    const int* col;
    const unsigned* wt;
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
    int done;    // the search has finished (heap empty, no block inside)
    unsigned long long reached, distSum;  // SSSP: reachable vertices, sum of their distances
    // knapsack FIFO / switch models (ring == NULL: heap only)
    u64* ring;                  // ringCap keys, a power of two
    gh::FifoState* fifo;
    unsigned long long ringCap;
    int order;                  // GH_KNAP_HEAP / GH_KNAP_FIFO / GH_KNAP_SWITCH
    int switchCounter;          // batches in a row that trigger a switch
    int mode;                   // structure in use: 0 heap, 1 FIFO
    int switches;               // mode changes so far
};

// Prune thresholds (the app_t_val of deleteRoot, artifacts/astar/BGPQ_B/
// heap.cuh:260-289): keys at or above them cannot improve the incumbent, so
// the search leaves them in the heap and ends when only such keys are left.
// A*: key f<<32 | cell is expanded only while f < incumbent.
struct AstarThreshold {
    const unsigned* incumbent;
    template <typename H>
    __device__ __forceinline__ u64 operator()(const H&) const {
        return static_cast<u64>(__ldcg(incumbent)) << 32;
    }
};
// Knapsack: key (INT_MAX - bound)<<32 | ... is expanded only while bound > best.
struct KnapThreshold {
    const int* best;
    template <typename H>
    __device__ __forceinline__ u64 operator()(const H&) const {
        return static_cast<u64>(static_cast<unsigned>(INT_MAX - __ldcg(best))) << 32;
    }
};

__device__ __forceinline__ u64 prune_threshold(const Inst* in) {
    if (in->kind == GH_SEARCH_ASTAR) return static_cast<u64>(static_cast<unsigned>(in->incumbent)) << 32;
    if (in->kind == GH_SEARCH_KNAPSACK) return static_cast<u64>(static_cast<unsigned>(INT_MAX - in->incumbent)) << 32;
    return ~0ull;  // SSSP relaxes every key
}

// Manhattan distance to the goal cell (every move costs at least 1).
__device__ __forceinline__ unsigned astar_h(int v, int width, int goal) {
    const int x = v % width, y = v / width, gx = goal % width, gy = goal / width;
    return static_cast<unsigned>(abs(gx - x) + abs(gy - y));
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

// Reset of the listed instances' arrays (ids == NULL: the first gridDim.y):
// heap nodes to init keys, lock words to AVAIL, A* and SSSP distances to
// infinity.  blockIdx.y = instance, blockIdx.x = slice.
__global__ void k_search_fill(Inst* insts, const int* ids, int B) {
    Inst* in = insts + (ids ? ids[blockIdx.y] : static_cast<int>(blockIdx.y));
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    const size_t first = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t keys = static_cast<size_t>(in->batchNum + 1) * B;
    for (size_t q = first; q < keys; q += stride) in->items[q] = ~0ull;
    for (size_t q = first; q < static_cast<size_t>(in->batchNum) + 2; q += stride) in->status[q] = 0;
    if (in->kind == GH_SEARCH_ASTAR || in->kind == GH_SEARCH_SSSP) {
        const size_t cells = in->kind == GH_SEARCH_ASTAR ? static_cast<size_t>(in->width) * in->height
                                                         : static_cast<size_t>(in->nv);
        for (size_t q = first; q < cells; q += stride) in->g[q] = 0xffffffffu;
    }
    if (in->fifo) {
        unsigned long long* w = reinterpret_cast<unsigned long long*>(in->fifo);
        for (size_t q = first; q < sizeof(gh::FifoState) / 8; q += stride) w[q] = 0;
    }
}

// Counters, incumbent and the seed key in the partial buffer (after the
// fill), for the listed instances (ids == NULL: the first `count`).
__global__ void k_search_seed(Inst* insts, const int* ids, int count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        Inst* in = insts + (ids ? ids[i] : i);
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
        in->done = 0;
        in->pops = in->expanded = in->inserted = 0;
        in->reached = in->distSum = 0;
        if (in->kind == GH_SEARCH_ASTAR) {
            const int s = in->start, goal = in->goal;
            const bool open = in->cost[s] != 0 && in->cost[goal] != 0;
            in->incumbent = open && goal == s ? 0 : static_cast<int>(0xffffffffu);
            if (open && goal != s) {
                in->g[s] = 0;
                in->items[0] = (static_cast<u64>(astar_h(s, in->width, goal)) << 32) | static_cast<unsigned>(s);
            }
            st->partialBufferSize = open && goal != s ? 1 : 0;
        } else if (in->kind == GH_SEARCH_SSSP) {
            in->g[in->source] = 0;
            in->items[0] = static_cast<u64>(in->source);  // distance 0
            in->incumbent = 0;
            st->partialBufferSize = 1;
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
            in->mode = in->order == GH_KNAP_FIFO ? 1 : 0;
            in->switches = 0;
            if (in->mode == 1) {  // breadth-first: the root node goes into the ring
                if (live) in->ring[0] = knap_key(b, 0, 0);
                in->fifo->end = in->fifo->write = live ? 1 : 0;
                st->partialBufferSize = 0;
            } else {
                if (live) in->items[0] = knap_key(b, 0, 0);
                st->partialBufferSize = live ? 1 : 0;
            }
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

// Pushes the emitted keys into the ring.  One block owns the ring, so
// nothing frees slots while it pushes: a push that would not fit sets
// *overflow (the instance then fails with GH_ERR_CAPACITY) instead of
// waiting for room.
__device__ __forceinline__ void fifo_flush(const gh::Fifo<u64>& f, u64* emit, int* cnt, int* overflow,
                                           unsigned long long& inserted) {
    __syncthreads();
    const int c = *cnt;
    if (c > 0) {
        if (threadIdx.x == 0 && f.state->end - f.state->begin + static_cast<unsigned long long>(c) > f.capacity)
            *overflow = 1;
        __syncthreads();
        if (!*overflow) f.push(emit, c);
        inserted += c;
    }
    __syncthreads();
    if (threadIdx.x == 0) *cnt = 0;
    __syncthreads();
}

// Switch to the FIFO (models.cuh:358-372, heapDataToArray): every node's keys
// below the prune threshold -- a prefix, nodes are sorted -- go into the
// ring, and the heap is emptied.  The block owns the heap (one block per
// knapsack instance) and no key of it is in flight.
template <typename H>
__device__ void heap_to_fifo(const H& heap, const gh::Fifo<u64>& f, u64 threshold, int* ctl) {
    gh::HeapState* st = heap.state;
    const int bc = st->batchCount, ps = st->partialBufferSize;
    const int B = heap.batchSize;
    for (int i = 0; i <= bc; ++i) {
        u64* nd = reinterpret_cast<u64*>(heap.heapItems) + static_cast<size_t>(i) * B;
        const int len = i == 0 ? ps : B;
        if (threadIdx.x == 0) ctl[7] = 0;
        __syncthreads();
        int c = 0;
        for (int j = threadIdx.x; j < len; j += blockDim.x) c += nd[j] < threshold ? 1 : 0;
        if (c) atomicAdd(&ctl[7], c);
        __syncthreads();
        const int keep = ctl[7];
        if (keep > 0) f.push(nd, keep);  // fits: the ring is at least the node pool, one slot per live key
        for (int j = threadIdx.x; j < B; j += blockDim.x) nd[j] = ~0ull;
        if (threadIdx.x == 0) heap.status[i] = 0;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        st->batchCount = 0;
        st->partialBufferSize = 0;
    }
    __syncthreads();
}

// Switch back to the heap (models.cuh:262-280): the ring's keys are
// inserted in batches.
template <typename H>
__device__ void fifo_to_heap(const H& heap, const gh::Fifo<u64>& f, u64* batch, int heapOff) {
    const int B = heap.batchSize;
    for (;;) {
        const typename gh::Fifo<u64>::Claim c = f.claim(B);
        if (c.n == 0) break;
        f.copy_out(c, batch);
        f.release(c);
        __syncthreads();
        heap.insertion(reinterpret_cast<typename H::key_type*>(batch), c.n, heapOff);
        if (heap.failed()) break;
    }
}

template <typename H>
__device__ void run_astar(const H& heap, Inst* in, unsigned char* smem, int heapOff, int maxBatches) {
    const int B = heap.batchSize, T = blockDim.x, tid = threadIdx.x;
    u64* batch = reinterpret_cast<u64*>(smem);
    u64* emit = batch + B;
    int* ctl = reinterpret_cast<int*>(emit + SearchSmem::emitKeys(B, T));
    const int width = in->width, height = in->height;
    const int goal = in->goal;
    unsigned* g = in->g;
    const unsigned char* cost = in->cost;
    unsigned* inc = reinterpret_cast<unsigned*>(&in->incumbent);
    unsigned long long pops = 0, expanded = 0, inserted = 0, waitStart = 0;
    int lastBusy = -1, batches = 0;
    if (tid == 0) ctl[1] = 0;
    __syncthreads();
    const AstarThreshold prune{inc};
    for (;;) {
        if (maxBatches && batches++ == maxBatches) break;
        if (gh::app::wait_for_keys(heap, &ctl[2], &in->stop, lastBusy, waitStart, prune)) break;
        int size = 0;
        heap.deleteMin(reinterpret_cast<typename H::key_type*>(batch), size, prune(heap), heapOff);
        pops += size;
        for (int base = 0; base < size; base += T) {
            const int i = base + tid;
            if (i < size) {
                const u64 key = batch[i];
                const unsigned f = static_cast<unsigned>(key >> 32);
                const int v = static_cast<int>(key & 0xffffffffu);
                const unsigned best = __ldcg(inc);
                const unsigned hv = astar_h(v, width, goal);
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
                        const unsigned nf = ng + astar_h(u, width, goal);
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
__device__ void run_knapsack(const H& heap, Inst* in, unsigned char* smem, int heapOff, int maxBatches) {
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
    int lastBusy = -1, batches = 0;
    const KnapThreshold prune{best};
    const gh::Fifo<u64> fifo{in->ring, in->fifo, in->ringCap, heap.timeoutNs};
    int mode = in->mode;               // block-uniform: 0 heap, 1 FIFO
    int counter = 0, prevBest = 0;     // switch model, thread 0
    if (tid == 0) prevBest = __ldcg(best);
    for (;;) {
        if (maxBatches && batches++ == maxBatches) break;
        int size = 0;
        if (mode == 0) {
            if (gh::app::wait_for_keys(heap, &ctl[2], &in->stop, lastBusy, waitStart, prune)) break;
            heap.deleteMin(reinterpret_cast<typename H::key_type*>(batch), size, prune(heap), heapOff);
        } else {
            // breadth-first (models_fifo.cuh:46-52): the oldest batch of the ring;
            // the search is over when the ring is empty (one block owns it)
            if (__syncthreads_or(threadIdx.x == 0 && gh::detail::ld_relaxed(&in->stop) != 0)) break;
            const typename gh::Fifo<u64>::Claim c = fifo.claim(B);
            if (c.n == 0) break;
            fifo.copy_out(c, batch);
            fifo.release(c);
            size = c.n;
        }
        const unsigned long long insertedBefore = inserted;
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
            if (mode == 0) flush_full(heap, emit, &ctl[1], B, heapOff, inserted);
            else fifo_flush(fifo, emit, &ctl[1], &ctl[5], inserted);
        }
        if (mode == 0) flush_rest(heap, emit, &ctl[1], heapOff, inserted);
        else fifo_flush(fifo, emit, &ctl[1], &ctl[5], inserted);
        if (ctl[5]) {  // node pool or ring exhausted
            if (tid == 0) { in->failed = GH_ERR_CAPACITY; gh::detail::st_relaxed(&in->stop, 1); }
        }
        if (mode == 0) gh::app::batch_done(heap.state);
        if (heap.failed() || ctl[5] || __syncthreads_or(threadIdx.x == 0 && in->fifo != nullptr && fifo.failed())) break;
        if (in->order == GH_KNAP_SWITCH) {
            // models.cuh:102-117 (FIFO) and :210-227 (heap): count batches in
            // a row that inserted children with the best profit unchanged
            // (heap mode) or raised (FIFO mode)
            if (tid == 0) {
                const int nb = __ldcg(best);
                const bool ins = inserted > insertedBefore;
                counter = (ins && (mode == 0 ? nb == prevBest : nb > prevBest)) ? counter + 1 : 0;
                prevBest = nb;
                ctl[6] = counter >= in->switchCounter ? 1 : 0;
                if (ctl[6]) counter = 0;
            }
            __syncthreads();
            const int flip = ctl[6];
            __syncthreads();
            if (flip) {
                if (mode == 0) heap_to_fifo(heap, fifo, prune(heap), ctl);
                else fifo_to_heap(heap, fifo, batch, heapOff);
                mode ^= 1;
                if (tid == 0) { in->mode = mode; in->switches += 1; }
                if (heap.failed()) break;
            }
        }
    }
    if (tid == 0) {
        in->freeTop = ctl[3];
        in->bump = ctl[4];
        atomicAdd(&in->pops, pops);
        atomicAdd(&in->inserted, inserted);
    }
    atomicAdd(&in->expanded, expanded);
}

// SSSP from the instance's source: the label-correcting loop of the
// standalone SSSP kernel, one expansion step per taken batch.
template <typename H>
__device__ void run_sssp(const H& heap, Inst* in, unsigned char* smem, int heapOff, int maxBatches) {
    const int B = heap.batchSize, T = blockDim.x, tid = threadIdx.x;
    u64* batch = reinterpret_cast<u64*>(smem);
    u64* emit = batch + B;
    long long* pre = reinterpret_cast<long long*>(emit + SearchSmem::emitKeys(B, T));
    long long* wsum = pre + B + 1;
    int* ctl = reinterpret_cast<int*>(wsum + 32);
    unsigned long long pops = 0, edges = 0, inserted = 0, waitStart = 0;
    int lastBusy = -1, batches = 0;
    if (tid == 0) ctl[1] = 0;
    __syncthreads();
    for (;;) {
        if (maxBatches && batches++ == maxBatches) break;
        if (gh::app::wait_for_keys(heap, &ctl[2], &in->stop, lastBusy, waitStart)) break;
        int size = 0;
        heap.deleteMin(reinterpret_cast<typename H::key_type*>(batch), size, heapOff);
        pops += size;
        if (size > 0)
            gh::app::sssp_relax_batch(heap, batch, size, pre, wsum, emit, &ctl[1], in->rowptr, in->col, in->wt, in->g,
                                      heapOff, edges, inserted);
        gh::app::batch_done(heap.state);
        if (heap.failed()) break;
    }
    if (tid == 0) {
        atomicAdd(&in->pops, pops);
        atomicAdd(&in->expanded, edges);
        atomicAdd(&in->inserted, inserted);
    }
}

// Resident blocks per SM the build of the search kernel for blocks of up to
// 256 threads is compiled for (512-thread blocks: one).  On the batched
// workload (1024 grid A* + knapsack, batch 256) 3 measured 1011 ms per run,
// 2 (128 registers) 1056 ms, 4 1109 ms and 1 (255 registers, few spills)
// 1774 ms: resident blocks matter more than spills.
constexpr int kSmallSearchBlocksPerSM = 3;

// maxBatches > 0: each task takes at most that many batches, then the block
// moves on (the search resumes in a later launch from its heap).  MaxT is
// the largest block it runs with; the register budget follows from it and
// the blocks each SM should hold.
template <typename H, int MaxT>
__global__ void __launch_bounds__(MaxT, MaxT <= 256 ? kSmallSearchBlocksPerSM : 1)
    k_search(H proto, Inst* insts, const int* tasks, int ntasks, int* next, int maxBatches) {
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
        if (in->kind == GH_SEARCH_ASTAR) run_astar(h, in, smem, heapOff, maxBatches);
        else if (in->kind == GH_SEARCH_SSSP) run_sssp(h, in, smem, heapOff, maxBatches);
        else run_knapsack(h, in, smem, heapOff, maxBatches);
        __syncthreads();
    }
}

// After a launch, one block per listed instance (ids == NULL: instance
// blockIdx.x): records failures from the heap's error word, marks the
// search done when its heap holds no key below the prune threshold (no
// block is inside it once the launch has ended), and for a finished SSSP
// counts the reachable vertices and sums their distances (the query's
// digest).  final != 0: every search was run to the end, so a heap with a
// key below the threshold is an error.
__global__ void k_search_collect(Inst* insts, const int* ids, int final, int batchSize) {
    Inst* in = insts + (ids ? ids[blockIdx.x] : static_cast<int>(blockIdx.x));
    __shared__ int s_done;
    __shared__ unsigned long long s_red[2][32];
    if (threadIdx.x == 0) {
        const int err = in->state->err;
        if (err && !in->failed)
            in->failed = err == gh::kErrCapacity ? GH_ERR_CAPACITY : err == gh::kErrTimeout ? GH_ERR_TIMEOUT : GH_ERR_STATE;
        const int bc = in->state->batchCount;
        const bool empty = bc == 0 && in->state->partialBufferSize == 0;
        const bool ringEmpty = in->fifo == nullptr || in->fifo->end == in->fifo->begin;
        const bool finished = (empty || in->items[bc > 0 ? batchSize : 0] >= prune_threshold(in)) && ringEmpty;
        if (in->fifo && in->fifo->err && !in->failed) in->failed = GH_ERR_TIMEOUT;
        if (final && !in->failed && !finished && !in->stop) in->failed = GH_ERR_STATE;
        in->done = in->failed || in->stop || finished;
        s_done = in->done && !in->failed && in->kind == GH_SEARCH_SSSP;
    }
    __syncthreads();
    if (!s_done) return;
    unsigned long long cnt = 0, sum = 0;
    for (int v = threadIdx.x; v < in->nv; v += blockDim.x) {
        const unsigned dv = in->g[v];
        if (dv != 0xffffffffu) { ++cnt; sum += dv; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
        sum += __shfl_down_sync(0xffffffffu, sum, o);
    }
    if ((threadIdx.x & 31) == 0) { s_red[0][threadIdx.x >> 5] = cnt; s_red[1][threadIdx.x >> 5] = sum; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long c = 0, s2 = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) { c += s_red[0][w]; s2 += s_red[1][w]; }
        in->reached = c;
        in->distSum = s2;
    }
}

// The search kernel built for `threads` threads per block.
template <typename H>
inline auto search_kernel(int threads) {
    return threads <= 256 ? k_search<H, 256> : k_search<H, kMaxSearchThreads>;
}

template <typename H>
cudaError_t launch_search(const H& proto, Inst* insts, const int* tasks, int ntasks, int* next, int grid, int threads,
                          size_t smem, cudaStream_t s, int maxBatches) {
    const auto kern = search_kernel<H>(threads);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    kern<<<grid, threads, smem, s>>>(proto, insts, tasks, ntasks, next, maxBatches);
    gh::impl::count_launch();
    return cudaGetLastError();
}

// Host side: shape of a search launch, shared by the batched and served forms.
struct SearchConfig {
    int batchSize;
    int variant;
    int threads;  // 0 = min(batchSize, kMaxSearchThreads)
    long long timeoutNs;
    int numSMs;
};

inline int search_threads(const SearchConfig& c) {
    return c.threads ? c.threads : (c.batchSize < kMaxSearchThreads ? c.batchSize : kMaxSearchThreads);
}

inline size_t search_smem(const SearchConfig& c) {
    return SearchSmem::bytes(c.batchSize, search_threads(c)) + 16 + gh::Heap<uint64_t, 0, true>::smemBytes(c.batchSize);
}

// Calls f(Heap<uint64_t, variant, true, IPT>{}) for the configuration's layout and merge width.
template <typename F>
inline cudaError_t search_dispatch(const SearchConfig& c, F&& f) {
    const int ipt = 2 * c.batchSize / search_threads(c);
    if (c.variant == GH_TOPDOWN) {
        if (ipt == 2) return f(gh::Heap<uint64_t, gh::kTopDown, true, 2>{});
        if (ipt == 4) return f(gh::Heap<uint64_t, gh::kTopDown, true, 4>{});
    } else {
        if (ipt == 2) return f(gh::Heap<uint64_t, gh::kBottomUp, true, 2>{});
        if (ipt == 4) return f(gh::Heap<uint64_t, gh::kBottomUp, true, 4>{});
    }
    return cudaErrorInvalidValue;
}

// Blocks of one persistent launch: resident blocks per SM x SMs.
inline int search_resident_blocks(const SearchConfig& c) {
    int per = 0;
    const int T = search_threads(c);
    const size_t smem = search_smem(c);
    cudaError_t e = search_dispatch(c, [&](auto proto) {
        using H = decltype(proto);
        const auto kern = search_kernel<H>(T);
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, T, smem);
    });
    if (e != cudaSuccess || per < 1) per = 1;
    return per * c.numSMs;
}

inline cudaError_t search_launch(const SearchConfig& c, Inst* insts, const int* tasks, int ntasks, int* next, int grid,
                                 cudaStream_t s, int maxBatches) {
    const int T = search_threads(c);
    const size_t smem = search_smem(c);
    return search_dispatch(c, [&](auto h) {
        h.heapItems = nullptr;
        h.status = nullptr;
        h.state = nullptr;
        h.init_limits = ~0ull;
        h.batchNum = 0;
        h.batchSize = c.batchSize;
        h.sortOutput = 0;
        h.timeoutNs = c.timeoutNs;
        return launch_search(h, insts, tasks, ntasks, next, grid, T, smem, s, maxBatches);
    });
}

}  // namespace

