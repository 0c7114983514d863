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
#include "search_common.cuh"
#include "sssp_relax.cuh"
#include "worklist.cuh"

namespace gh {
namespace search {

__device__ __forceinline__ u64 knap_key(long long bound, int level, int slot) {
    return (static_cast<u64>(static_cast<unsigned>(INT_MAX - static_cast<int>(bound))) << 32) |
           (static_cast<u64>(kMaxKnapItems - level) << kSlotBits) | static_cast<unsigned>(slot);
}

// One instance, as the kernels see it (device array).

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
    if (in->kind == GH_SEARCH_ASTAR) return static_cast<u64>(static_cast<unsigned>(__ldcg(&in->incumbent))) << 32;
    if (in->kind == GH_SEARCH_KNAPSACK) return static_cast<u64>(static_cast<unsigned>(INT_MAX - __ldcg(&in->incumbent))) << 32;
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

// Reset of one instance's arrays: heap nodes to init keys, lock words to
// AVAIL, A* and SSSP distances to infinity, FIFO counters to zero.  Thread
// `first` of `stride` threads (the threads of several blocks, or of one).
__device__ inline void fill_instance(const Inst* in, int B, size_t first, size_t stride) {
    // nodes: (batchNum + 1) * B keys, an even count from a 256-byte aligned base
    const size_t pairs = static_cast<size_t>(in->batchNum + 1) * B / 2;
    ulonglong2* items = reinterpret_cast<ulonglong2*>(in->items);
    for (size_t q = first; q < pairs; q += stride) items[q] = make_ulonglong2(~0ull, ~0ull);
    for (size_t q = first; q < static_cast<size_t>(in->batchNum) + 2; q += stride) in->status[q] = 0;
    if (in->kind == GH_SEARCH_ASTAR || in->kind == GH_SEARCH_SSSP) {
        const size_t cells = in->kind == GH_SEARCH_ASTAR ? static_cast<size_t>(in->width) * in->height
                                                         : static_cast<size_t>(in->nv);
        uint4* g4 = reinterpret_cast<uint4*>(in->g);  // 256-byte aligned base
        for (size_t q = first; q < cells / 4; q += stride) g4[q] = make_uint4(~0u, ~0u, ~0u, ~0u);
        for (size_t q = cells / 4 * 4 + first; q < cells; q += stride) in->g[q] = 0xffffffffu;
    }
    if (in->fifo) {
        unsigned long long* w = reinterpret_cast<unsigned long long*>(in->fifo);
        for (size_t q = first; q < sizeof(gh::FifoState) / 8; q += stride) w[q] = 0;
    }
}

// Counters, incumbent and the seed key in the partial buffer of one
// instance, after its fill (one thread).
__device__ inline void seed_instance(Inst* in) {
    {
        gh::HeapState* st = in->state;
        // every counter, ticket and error word to zero: the block may have
        // held another instance's data before
        int* words = reinterpret_cast<int*>(st);
        for (int q = 0; q < static_cast<int>(sizeof(gh::HeapState) / 4); ++q) words[q] = 0;
        st->outLimit = INT_MAX;
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

// Inserts every full batch of the emitted keys and moves the rest (fewer
// than B) to the front, so that a round starts with fewer than B keys and
// its emits fit the B + 8 T slots.  The rest comes from behind at least one
// batch, so the parallel move never overlaps.
template <typename H>
__device__ __forceinline__ void flush_full(const H& heap, u64* emit, int* cnt, int B, int heapOff, unsigned long long& inserted) {
    __syncthreads();
    const int c = *cnt;
    if (c >= B) {
        int off = 0;
        for (; c - off >= B; off += B) gh::app::insert_keys(heap, emit + off, B, heapOff);
        for (int i = threadIdx.x; i < c - off; i += blockDim.x) emit[i] = emit[off + i];
        __syncthreads();
        if (threadIdx.x == 0) *cnt = c - off;
        inserted += off;
    }
    __syncthreads();
}

template <typename H>
__device__ __forceinline__ void flush_rest(const H& heap, u64* emit, int* cnt, int heapOff, unsigned long long& inserted) {
    __syncthreads();
    const int c = *cnt;
    if (c > 0) gh::app::insert_keys(heap, emit, c, heapOff);
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
        gh::app::insert_keys(heap, batch, c.n, heapOff);
        if (heap.failed()) break;
    }
}

template <typename H>
__device__ bool run_astar(const H& heap, Inst* in, unsigned char* smem, int heapOff, int maxBatches) {
    const int B = heap.batchSize, T = blockDim.x, tid = threadIdx.x;
    u64* batch = reinterpret_cast<u64*>(smem);
    u64* emit = batch + B;
    int* ctl = reinterpret_cast<int*>(emit + SearchSmem::emitKeys(B, T));
    const int width = in->width, height = in->height;
    const int goal = in->goal;
    const bool eight = in->moves == 8;
    unsigned* g = in->g;
    const unsigned char* cost = in->cost;
    unsigned* inc = reinterpret_cast<unsigned*>(&in->incumbent);
    unsigned long long pops = 0, expanded = 0, inserted = 0, waitStart = 0;
    int lastBusy = -1, batches = 0;
    if (tid == 0) ctl[1] = 0;
    __syncthreads();
    const AstarThreshold prune{inc};
    bool over = true;  // false: the batch budget ran out, the search goes on
    for (;;) {
        if (maxBatches && batches++ == maxBatches) { over = false; break; }
        if (gh::app::wait_for_keys(heap, &ctl[2], &in->stop, lastBusy, waitStart, prune)) break;
        int size = 0;
        size = gh::app::take_batch(heap, batch, prune(heap), heapOff);
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
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        // moves 4: left, right, up, down, each costing the cell
                        // entered; moves 8: the reference's model
                        // (artifacts/astar/pq_model.cuh:126-190): the eight
                        // neighbours in its order, open cells only, each
                        // direction with its fixed cost 3 2 2 2 1 3 1 2
                        if (k >= 4 && !eight) break;
                        const int dx = eight ? (k < 3 ? k - 1 : k < 5 ? (k == 3 ? -1 : 1) : k - 6)
                                             : (k == 0 ? -1 : k == 1 ? 1 : 0);
                        const int dy = eight ? (k < 3 ? -1 : k < 5 ? 0 : 1) : (k == 2 ? -1 : k == 3 ? 1 : 0);
                        const int nx = x + dx, ny = y + dy;
                        if (nx < 0 || ny < 0 || nx >= width || ny >= height) continue;
                        const int u = ny * width + nx;
                        const unsigned cu = cost[u];
                        if (cu == 0) continue;
                        const unsigned c = eight ? (0x21312223u >> (4 * k)) & 15u : cu;
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
    return over;
}

template <typename H>
__device__ bool run_knapsack(const H& heap, Inst* in, unsigned char* smem, int heapOff, int maxBatches) {
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
    bool over = true;  // false: the batch budget ran out, the search goes on
    for (;;) {
        if (maxBatches && batches++ == maxBatches) { over = false; break; }
        int size = 0;
        if (mode == 0) {
            if (gh::app::wait_for_keys(heap, &ctl[2], &in->stop, lastBusy, waitStart, prune)) break;
            size = gh::app::take_batch(heap, batch, prune(heap), heapOff);
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
    return over;
}

// SSSP from the instance's source: the label-correcting loop of the
// standalone SSSP kernel, one expansion step per taken batch.
template <typename H>
__device__ bool run_sssp(const H& heap, Inst* in, unsigned char* smem, int heapOff, int maxBatches) {
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
    bool over = true;  // false: the batch budget ran out, the search goes on
    for (;;) {
        if (maxBatches && batches++ == maxBatches) { over = false; break; }
        if (gh::app::wait_for_keys(heap, &ctl[2], &in->stop, lastBusy, waitStart)) break;
        int size = 0;
        size = gh::app::take_batch(heap, batch, heapOff);
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
    return over;
}

// One block per instance, after a launch or once the last block has left
// it: records failures from the heap's error word, marks the search done
// when its heap holds no key below the prune threshold, and for a finished
// SSSP counts the reachable vertices and sums their distances (the query's
// digest).  final != 0: the search was run to the end, so a heap with a key
// below the threshold is an error.  Every thread of the block calls it;
// loads go to L2, so a block that ran other instances before reads no
// stale lines.
__device__ inline void collect_instance(Inst* in, int final, int batchSize) {
    __shared__ int s_done;
    __shared__ unsigned long long s_red[2][32];
    if (threadIdx.x == 0) {
        gh::HeapState* st = in->state;
        const int err = __ldcg(&st->err);
        if (err && !in->failed)
            in->failed = err == gh::kErrCapacity ? GH_ERR_CAPACITY : err == gh::kErrTimeout ? GH_ERR_TIMEOUT : GH_ERR_STATE;
        const int bc = __ldcg(&st->batchCount);
        const bool empty = bc == 0 && __ldcg(&st->partialBufferSize) == 0;
        const bool ringEmpty = in->fifo == nullptr || __ldcg(&in->fifo->end) == __ldcg(&in->fifo->begin);
        const bool finished = (empty || __ldcg(&in->items[bc > 0 ? batchSize : 0]) >= prune_threshold(in)) && ringEmpty;
        if (in->fifo && __ldcg(&in->fifo->err) && !in->failed) in->failed = GH_ERR_TIMEOUT;
        const int stop = __ldcg(&in->stop);
        if (final && !in->failed && !finished && !stop) in->failed = GH_ERR_STATE;
        in->done = in->failed || stop || finished;
        s_done = in->done && !in->failed && in->kind == GH_SEARCH_SSSP;
    }
    __syncthreads();
    if (s_done) {
        unsigned long long cnt = 0, sum = 0;
        for (int v = threadIdx.x; v < in->nv; v += blockDim.x) {
            const unsigned dv = __ldcg(in->g + v);
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
    __syncthreads();
}

// ------------------------------------------------------ served, device loop
// Thread 0 of a block runs the control steps below; the state they share
// lives in ServeDev.  Three kinds of state:
//  * the admission state (pending requests, free slots, free arena ranges,
//    counters): only the holder of ServeDev::lock reads or writes it, with
//    volatile accesses (no stale L1 lines across blocks);
//  * the work-token queue: a bounded ring of cells, each with a sequence
//    word (cell i of lap k is free at seq i + k * cap, holds a token at
//    seq i + k * cap + 1); producers take a position with atomicAdd,
//    consumers with compare-and-swap, and the sequence words carry the
//    release/acquire order from the producer to the consumer;
//  * the rings in pinned host memory: records are filled first and their
//    sequence word is stored last with system-scope release; the reader
//    loads the sequence word with system-scope acquire.
// Every wait has a limit (waitNs for the lock and a queue cell, stallNs for
// a work token while no token moves); a wait that runs out records an error
// and makes every block leave.
namespace sv {

__device__ __forceinline__ u64 ld_acquire_sys(const u64* p) {
    u64 v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ u64 ld_relaxed_sys(const u64* p) {
    u64 v;
    asm volatile("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_sys(const int* p) {
    int v;
    asm volatile("ld.relaxed.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_sys(u64* p, u64 v) {
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_sys(u64* p, u64 v) {
    asm volatile("st.relaxed.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_sys(int* p, int v) {
    asm volatile("st.relaxed.sys.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ u64 ld_acquire_gpu(const u64* p) {
    u64 v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ u64 ld_relaxed_gpu(const u64* p) {
    u64 v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_gpu(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(u64* p, u64 v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Records a loop error and makes every block leave.
__device__ inline void fail(ServeDev* d, int code) {
    atomicCAS(&d->err, 0, code);
    st_relaxed_sys(&d->host->err, code);
    atomicExch(&d->exit, 1);
}

__device__ inline bool leaving(ServeDev* d) { return ld_relaxed_gpu(&d->exit) != 0; }

// Appends a token.  The ring has a cell for every token that can be out
// at once, so the cell is free or about to be (its last consumer is
// between its compare-and-swap and its release).
__device__ inline bool push(ServeDev* d, int v) {
    const u64 pos = atomicAdd(&d->enq, 1ull);
    ServeCell* c = d->cells + (pos & d->cellMask);
    const u64 t0 = gh::detail::globaltimer();
    while (ld_acquire_gpu(&c->seq) != pos) {
        if (gh::detail::globaltimer() - t0 > static_cast<u64>(d->waitNs)) {
            fail(d, kServeErrQueue);
            return false;
        }
        __nanosleep(64);
    }
    c->val = v;
    st_release_gpu(&c->seq, pos + 1);
    return true;
}

// Takes the oldest token, or returns -1 if none is ready.  An empty poll
// uses relaxed loads only; the acquire comes once a token is taken (an
// acquire load may drop the SM's L1 lines, which the blocks searching
// beside this one are using).
__device__ inline int pop(ServeDev* d) {
    for (int tries = 0; tries < 32; ++tries) {
        const u64 pos = ld_relaxed_gpu(&d->deq);
        ServeCell* c = d->cells + (pos & d->cellMask);
        const u64 s = ld_relaxed_gpu(&c->seq);
        if (s == pos + 1) {
            if (atomicCAS(&d->deq, pos, pos + 1) == pos) {
                ld_acquire_gpu(&c->seq);  // orders what the producer wrote before its release
                const int v = ld_relaxed_gpu(&c->val);
                st_release_gpu(&c->seq, pos + d->cellMask + 1);
                return v;
            }
        } else if (s < pos + 1) {
            return -1;  // empty, or its producer has not stored it yet
        }
    }
    return -1;
}

__device__ inline bool try_lock(ServeDev* d) {
    if (atomicCAS(&d->lock, 0, 1) != 0) return false;
    __threadfence();
    return true;
}

__device__ inline bool lock(ServeDev* d) {
    const u64 t0 = gh::detail::globaltimer();
    while (atomicCAS(&d->lock, 0, 1) != 0) {
        if (gh::detail::globaltimer() - t0 > static_cast<u64>(d->waitNs)) {
            fail(d, kServeErrLock);
            return false;
        }
        __nanosleep(128);
    }
    __threadfence();
    return true;
}

__device__ inline void unlock(ServeDev* d) {
    __threadfence();
    atomicExch(&d->lock, 0);
}

// Request records, word by word.
__device__ inline void copy_req(volatile ServeReq* dst, const volatile ServeReq* src) {
    volatile u64* o = reinterpret_cast<volatile u64*>(dst);
    const volatile u64* i = reinterpret_cast<const volatile u64*>(src);
    for (int k = 0; k < static_cast<int>(sizeof(ServeReq) / 8); ++k) o[k] = i[k];
}

__device__ inline void copy_req_from_host(volatile ServeReq* dst, const ServeReq* src) {
    volatile u64* o = reinterpret_cast<volatile u64*>(dst);
    const u64* i = reinterpret_cast<const u64*>(src);
    for (int k = 0; k < static_cast<int>(sizeof(ServeReq) / 8); ++k) o[k] = ld_relaxed_sys(i + k);
}

// First fit over the free ranges, kept sorted by offset (lock held).
__device__ inline bool arena_alloc(ServeDev* d, u64 bytes, u64* off) {
    volatile ServeRange* r = d->ranges;
    volatile ServeDev* v = d;
    const int n = v->nranges;
    for (int k = 0; k < n; ++k) {
        if (r[k].len < bytes) continue;
        *off = r[k].off;
        r[k].off = r[k].off + bytes;
        r[k].len = r[k].len - bytes;
        if (r[k].len == 0) {
            for (int j = k; j + 1 < n; ++j) { r[j].off = r[j + 1].off; r[j].len = r[j + 1].len; }
            v->nranges = n - 1;
        }
        return true;
    }
    return false;
}

// Returns a block, merging it with its neighbours (lock held).  There are
// at most one more free ranges than allocated blocks, so the array of
// maxSlots + 2 never overflows.
__device__ inline void arena_free(ServeDev* d, u64 off, u64 bytes) {
    volatile ServeRange* r = d->ranges;
    volatile ServeDev* v = d;
    const int n = v->nranges;
    int k = 0;
    while (k < n && r[k].off < off) ++k;
    const bool prev = k > 0 && r[k - 1].off + r[k - 1].len == off;
    const bool next = k < n && off + bytes == r[k].off;
    if (prev && next) {
        r[k - 1].len = r[k - 1].len + bytes + r[k].len;
        for (int j = k; j + 1 < n; ++j) { r[j].off = r[j + 1].off; r[j].len = r[j + 1].len; }
        v->nranges = n - 1;
    } else if (prev) {
        r[k - 1].len = r[k - 1].len + bytes;
    } else if (next) {
        r[k].off = off;
        r[k].len = r[k].len + bytes;
    } else if (n < d->maxRanges) {
        for (int j = n; j > k; --j) { r[j].off = r[j - 1].off; r[j].len = r[j - 1].len; }
        r[k].off = off;
        r[k].len = bytes;
        v->nranges = n + 1;
    }
}

// The host's view of the admission state (lock held).
__device__ inline void publish_status(ServeDev* d) {
    volatile ServeDev* v = d;
    ServeHost* h = d->host;
    st_relaxed_sys(reinterpret_cast<u64*>(&h->usedBytes), v->usedBytes);
    st_relaxed_sys(&h->slotsUsed, d->maxSlots - v->nfree);
    st_relaxed_sys(&h->pending, v->npend);
    st_relaxed_sys(&h->active, v->active);
    st_relaxed_sys(&h->admitted, v->admitted);
}

// Admission (lock held): the host's stop word, new requests out of the
// ring, then the pending requests in arrival order into free slots and
// memory (skipping those that do not fit yet), each admitted one as a setup
// token; last, the idle limit.
__device__ inline void admit(ServeDev* d) {
    volatile ServeDev* v = d;
    ServeHost* h = d->host;
    if (ld_relaxed_sys(&h->stop) != 0) {
        atomicExch(&d->exit, 1);
        return;
    }
    const u64 mask = static_cast<u64>(d->ringCap) - 1;
    u64 taken = v->reqTaken;
    int np = v->npend;
    bool changed = false;
    while (np < d->ringCap) {
        const ServeReq* r = d->ring + (taken & mask);
        if (ld_acquire_sys(&r->seq) != taken + 1) break;
        copy_req_from_host(d->pend + np, r);
        ++np;
        ++taken;
        changed = true;
    }
    if (changed) {
        v->reqTaken = taken;
        v->npend = np;
        st_release_sys(&h->reqTaken, taken);  // the records below `taken` may be written again
    }
    if (changed || v->freeEpoch != v->admitEpoch) {
        v->admitEpoch = v->freeEpoch;
        volatile int* freeSlots = d->freeSlots;
        int j = 0;
        for (int i = 0; i < np; ++i) {
            volatile ServeReq* q = d->pend + i;
            u64 off = 0;
            if (v->nfree > 0 && arena_alloc(d, q->bytes, &off)) {
                const int nf = v->nfree - 1;
                const int slot = freeSlots[nf];
                v->nfree = nf;
                q->off = off;
                copy_req(d->slotReq + slot, q);
                v->active = v->active + 1;
                v->usedBytes = v->usedBytes + q->bytes;
                v->admitted = v->admitted + 1;
                changed = true;
                if (!push(d, slot | kServeSetup)) return;
                continue;
            }
            if (j != i) copy_req(d->pend + j, q);
            ++j;
        }
        v->npend = j;
    }
    if (changed) publish_status(d);
    const u64 now = gh::detail::globaltimer();
    if (v->npend == 0 && v->active == 0) {
        if (v->idleSince == 0) v->idleSince = now;
        else if (now - v->idleSince > static_cast<u64>(d->idleNs)) atomicExch(&d->exit, 1);
    } else {
        v->idleSince = 0;
    }
    if (!changed) atomicExch(&d->admitAt, now + 1000);  // nothing new: let the others run for a microsecond
}

// Thread 0: the next token for this block, or -1 when the blocks leave.
__device__ inline int next_token(ServeDev* d) {
    u64 lastDeq = ~0ull, since = 0;
    unsigned backoff = 32;
    for (;;) {
        if (leaving(d)) return -1;
        const u64 now = gh::detail::globaltimer();
        if (now >= ld_relaxed_gpu(&d->admitAt) && try_lock(d)) {
            admit(d);
            unlock(d);
            if (leaving(d)) return -1;
        }
        const int t = pop(d);
        if (t >= 0) return t;
        const u64 dq = ld_relaxed_gpu(&d->deq);
        if (dq != lastDeq) {
            lastDeq = dq;
            since = now;
        } else if (now - since > static_cast<u64>(d->stallNs)) {
            fail(d, kServeErrWait);
            return -1;
        }
        __nanosleep(backoff);
        backoff = backoff < 2048 ? backoff * 2 : 2048;
    }
}

// Block-wide: the instance record of an admitted query from its request
// and its arena block, the reset of its arrays, its seed, then its search
// tokens.
__device__ inline void setup_query(ServeDev* d, int slot, int B) {
    Inst* in = d->insts + slot;
    __shared__ int s_blocks;
    if (threadIdx.x == 0) {
        const volatile ServeReq* q = d->slotReq + slot;
        const int kind = q->kind, bn = q->bn;
        const long long dist = kind == GH_SEARCH_SSSP ? static_cast<long long>(q->n)
                                                      : static_cast<long long>(q->width) * q->height;
        const QueryLayout L = query_layout(bn, B, dist);
        unsigned char* base = d->arena + q->off;
        u64* words = reinterpret_cast<u64*>(in);
        for (int k = 0; k < static_cast<int>(sizeof(Inst) / 8); ++k) words[k] = 0;
        in->kind = kind;
        in->blocks = q->blocks;
        in->batchNum = bn;
        in->state = reinterpret_cast<gh::HeapState*>(base);
        in->items = reinterpret_cast<u64*>(base + L.items);
        in->status = reinterpret_cast<int*>(base + L.status);
        in->g = reinterpret_cast<unsigned*>(base + L.g);
        if (kind == GH_SEARCH_SSSP) {
            in->nv = q->n;
            in->source = q->a;
            in->rowptr = q->rowptr;
            in->col = q->col;
            in->wt = q->w;
        } else {
            in->width = q->width;
            in->height = q->height;
            in->cost = q->cost;
            in->moves = q->moves;
            in->start = q->a;
            in->goal = q->b;
        }
        in->tokens = q->blocks;
        s_blocks = q->blocks;
    }
    __syncthreads();
    fill_instance(in, B, threadIdx.x, blockDim.x);
    __syncthreads();
    if (threadIdx.x == 0) {
        seed_instance(in);
        __threadfence();
        for (int k = 0; k < s_blocks; ++k)
            if (!push(d, slot)) break;
    }
    __syncthreads();
}

// Thread 0, after the last token of a query came back: the result, the
// slot and memory back to the free lists, then the completion record.
__device__ inline void complete(ServeDev* d, Inst* in, int slot) {
    volatile ServeDev* v = d;
    const volatile ServeReq* q = d->slotReq + slot;
    const long long qid = q->qid;
    const u64 off = q->off, bytes = q->bytes;
    const int failed = in->failed;
    const u64 r0 = in->kind == GH_SEARCH_SSSP ? in->reached : static_cast<u64>(static_cast<unsigned>(__ldcg(&in->incumbent)));
    const u64 r1 = in->kind == GH_SEARCH_SSSP ? in->distSum : 0;
    if (!lock(d)) return;
    arena_free(d, off, bytes);
    volatile int* freeSlots = d->freeSlots;
    freeSlots[v->nfree] = slot;
    v->nfree = v->nfree + 1;
    v->active = v->active - 1;
    v->usedBytes = v->usedBytes - bytes;
    v->freeEpoch = v->freeEpoch + 1;
    const u64 c = v->doneClaim;
    v->doneClaim = c + 1;
    publish_status(d);
    st_relaxed_sys(&d->host->completed, c + 1);
    unlock(d);
    atomicExch(&d->admitAt, 0ull);  // memory came free: admit at once
    ServeDone* r = d->done + (c & (static_cast<u64>(d->ringCap) - 1));
    st_relaxed_sys(reinterpret_cast<u64*>(&r->qid), static_cast<u64>(qid));
    st_relaxed_sys(&r->state, failed ? 3 : 2);
    st_relaxed_sys(&r->failed, failed);
    st_relaxed_sys(&r->r0, r0);
    st_relaxed_sys(&r->r1, r1);
    st_relaxed_sys(&r->tDone, gh::detail::globaltimer());
    st_release_sys(&r->seq, c + 1);
}

// Block-wide, after a stint on a query: its token goes back into the queue
// while the search goes on; once it is over, the block that returns the
// last token collects the result and completes the query.
__device__ inline void end_stint(ServeDev* d, Inst* in, int slot, bool over, int B) {
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        __threadfence();  // this block's writes to the query before its token moves on
        s_last = 0;
        if (!over) push(d, slot);
        else s_last = atomicSub(&in->tokens, 1) == 1;
        if (s_last) __threadfence();
    }
    __syncthreads();
    if (s_last) {
        collect_instance(in, 1, B);
        if (threadIdx.x == 0) complete(d, in, slot);
    }
    __syncthreads();
}

}  // namespace sv

// Resident blocks per SM the build of the search kernel for blocks of up to
// 256 threads is compiled for (512-thread blocks: one).  On the batched
// workload (1024 grid A* + knapsack, batch 256) 3 measured 1011 ms per run,
// 2 (128 registers) 1056 ms, 4 1109 ms and 1 (255 registers, few spills)
// 1774 ms: resident blocks matter more than spills.
constexpr int kSmallSearchBlocksPerSM = 3;

// The persistent search launch.  Without args.serve, blocks take instances
// from a task list (an instance appears once per block it should get);
// with it, they take work tokens from the device loop's queue (setup
// tokens, and one search token per block a query should get), until the
// loop's exit word is set.  args.maxBatches > 0: a block takes at most that
// many batches of a query, then moves on (the search resumes later from its
// heap).  MaxT is the largest block it runs with; the register budget
// follows from it and the blocks each SM should hold.
template <typename H, int MaxT>
__global__ void __launch_bounds__(MaxT, MaxT <= 256 ? kSmallSearchBlocksPerSM : 1) k_search(H proto, SearchArgs args) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_task;
    const int heapOff = static_cast<int>(SearchSmem::bytes(proto.batchSize, blockDim.x) / 4);
    for (;;) {
        if (threadIdx.x == 0) {
            if (args.serve) {
                s_task = sv::next_token(args.serve);
            } else {
                const int t = atomicAdd(args.next, 1);
                s_task = t < args.ntasks ? args.tasks[t] : -1;
            }
        }
        __syncthreads();
        const int task = s_task;
        __syncthreads();
        if (task < 0) break;
        if (task & kServeSetup) {
            sv::setup_query(args.serve, task & ~kServeSetup, proto.batchSize);
            continue;
        }
        Inst* in = args.insts + task;
        H h = proto;
        h.heapItems = reinterpret_cast<typename H::key_type*>(in->items);
        h.status = in->status;
        h.state = in->state;
        h.batchNum = in->batchNum;
        bool over;
        if (in->kind == GH_SEARCH_ASTAR) over = run_astar(h, in, smem, heapOff, args.maxBatches);
        else if (in->kind == GH_SEARCH_SSSP) over = run_sssp(h, in, smem, heapOff, args.maxBatches);
        else over = run_knapsack(h, in, smem, heapOff, args.maxBatches);
        __syncthreads();
        if (args.serve) sv::end_stint(args.serve, in, task, over, proto.batchSize);
    }
}

// Launch of the search kernel for one heap layout, the merge width following
// from the batch size and block threads.
template <int Variant>
inline cudaError_t launch_layout(const SearchConfig& c, const SearchArgs& a, int grid, cudaStream_t s) {
    const int T = search_threads(c);
    const size_t smem = search_smem(c);
    auto go = [&](auto h) -> cudaError_t {
        using H = decltype(h);
        h.heapItems = nullptr;
        h.status = nullptr;
        h.state = nullptr;
        h.init_limits = ~0ull;
        h.batchNum = 0;
        h.batchSize = c.batchSize;
        h.sortOutput = 0;
        h.timeoutNs = c.timeoutNs;
        const auto kern = T <= 256 ? k_search<H, 256> : k_search<H, kMaxSearchThreads>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        kern<<<grid, T, smem, s>>>(h, a);
        gh::impl::count_launch();
        return cudaGetLastError();
    };
    const int ipt = 2 * c.batchSize / T;
    if (ipt == 2) return go(gh::Heap<uint64_t, Variant, true, 2>{});
    if (ipt == 4) return go(gh::Heap<uint64_t, Variant, true, 4>{});
    return cudaErrorInvalidValue;
}

template <int Variant>
inline int blocks_per_sm_layout(const SearchConfig& c) {
    const int T = search_threads(c);
    const size_t smem = search_smem(c);
    auto occ = [&](auto h) -> int {
        using H = decltype(h);
        const auto kern = T <= 256 ? k_search<H, 256> : k_search<H, kMaxSearchThreads>;
        int per = 0;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, T, smem) != cudaSuccess) return 1;
        return per;
    };
    const int ipt = 2 * c.batchSize / T;
    if (ipt == 2) return occ(gh::Heap<uint64_t, Variant, true, 2>{});
    if (ipt == 4) return occ(gh::Heap<uint64_t, Variant, true, 4>{});
    return 1;
}

}  // namespace search
}  // namespace gh
