// Termination protocol for searches whose blocks share one heap (SSSP, grid
// A*, knapsack branch-and-bound).
//
// A block takes a batch (deleteRoot/deleteUpdate), expands it and inserts
// what it generates.  HeapState::busy counts the blocks between deciding to
// take a batch and finishing their inserts.  The search is over when the
// heap is empty while busy is 0: no block holds keys that could still be
// inserted.  A block that finds the heap empty only reads busy, so waiting
// blocks cannot keep each other alive; the block that takes a batch counts
// itself before it can empty the heap.  The reference's applications stop on
// a count of active blocks in the same way (applications/sssp_longfei_new/
// sssp.cu:19-132, artifacts/knapsack/models_pq.cuh:52-137 activeCount).
#pragma once
#include <type_traits>

#include "gpuheap_device.cuh"

namespace gh {
namespace app {

// Heap calls of the search loops, kept out of line.  Inlined into a search
// loop, insertion and deleteMin (with their merges) compete for registers
// with the loop's own state, and the compiler spills inside the merge
// loops; as calls, the heap code has the registers to itself and a call
// saves and restores a few of the caller's.
template <typename H>
__device__ __noinline__ void insert_keys(H heap, const unsigned long long* keys, int n, int heapOff) {
    heap.insertion(reinterpret_cast<const typename H::key_type*>(keys), n, heapOff);
}

// deleteRoot with a prune threshold (keys at or above it stay); returns the
// number of keys taken.
template <typename H>
__device__ __noinline__ int take_batch(H heap, unsigned long long* out, typename H::key_type threshold, int heapOff) {
    int size = 0;
    heap.deleteMin(reinterpret_cast<typename H::key_type*>(out), size, threshold, heapOff);
    return size;
}

template <typename H>
__device__ __noinline__ int take_batch(H heap, unsigned long long* out, int heapOff) {
    int size = 0;
    heap.deleteMin(reinterpret_cast<typename H::key_type*>(out), size, heapOff);
    return size;
}

// No prune threshold: every key is worth taking.
struct NoThreshold {
    template <typename H>
    __device__ __forceinline__ typename H::key_type operator()(const H& heap) const { return heap.init_limits; }
};

// Thread 0 waits until the heap holds keys below the prune threshold (then
// this block is counted busy and the call returns false: take a batch) or
// the search is over, `stop` (may be NULL) is set, or the heap has an error
// (returns true).  Every thread calls it; the result is block-uniform.
// `word` is a shared int.  `threshold(heap)` gives the current threshold
// (deleteRoot(items, size, app_t_val), artifacts/astar/BGPQ_B/heap.cuh:
// 260-289): keys at or above it are left in the heap, and the search is over
// once none below it is left and no block is busy.  A block that finds only
// such keys waits like one that finds the heap empty: it reads busy and
// never counts itself, so waiting blocks cannot keep each other alive.  The
// smallest key is read without locks; while blocks are busy it is a hint
// (a wrong one costs one empty deleteRoot or one early exit of this block,
// while busy blocks carry on), and the last block to finish reads it with
// no other block left inside the heap.  A wait with no change of busy for
// longer than the heap's time limit records a timeout and stops.
template <typename H, typename Threshold = NoThreshold>
__device__ __forceinline__ bool wait_for_keys(const H& heap, int* word, const int* stop, int& lastBusy,
                                              unsigned long long& waitStart, Threshold threshold = {}) {
    HeapState* st = heap.state;
    // with no threshold every key is worth taking, padding keys included
    auto below = [&](int bc) {
        if constexpr (std::is_same<Threshold, NoThreshold>::value) return true;
        else return heap.minKeyHint(bc) < threshold(heap);
    };
    if (threadIdx.x == 0) {
        int verdict = 0;
        for (;;) {
            if (stop && detail::ld_relaxed(stop) != 0) { verdict = 1; break; }
            const int bc = detail::ld_relaxed(&st->batchCount);
            const int ps = detail::ld_relaxed(&st->partialBufferSize);
            if ((bc || ps) && below(bc)) break;
            const int b = atomicAdd(&st->busy, 0);
            __threadfence();  // the counters below are read after busy
            if (b == 0) {
                const int bc2 = detail::ld_relaxed(&st->batchCount);
                const int ps2 = detail::ld_relaxed(&st->partialBufferSize);
                if ((bc2 == 0 && ps2 == 0) || !below(bc2)) { verdict = 1; break; }
            }
            if (detail::ld_relaxed(&st->err) != 0) { verdict = 1; break; }
            const unsigned long long now = detail::globaltimer();
            if (b != lastBusy || waitStart == 0) { lastBusy = b; waitStart = now; }
            if (now - waitStart > static_cast<unsigned long long>(heap.timeoutNs)) {
                heap.raise(kErrTimeout, kSiteLockPartial, 0, b);
                verdict = 1;
                break;
            }
            __nanosleep(200);
        }
        if (!verdict) {
            atomicAdd(&st->busy, 1);
            __threadfence();  // busy counts this block before it can empty the heap
        }
        *word = verdict;
    }
    __syncthreads();
    const bool r = *word != 0;
    __syncthreads();
    if (!r) lastBusy = -1;
    return r;
}

// The block has inserted everything it generated from its batch.
__device__ __forceinline__ void batch_done(HeapState* st) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicSub(&st->busy, 1);
    }
    __syncthreads();
}

}  // namespace app
}  // namespace gh
