// One SSSP expansion step on a taken batch of (dist << 32 | vertex) keys:
// the caller pattern of applications/sssp_longfei_new/sssp.cu:19-132 (skip
// stale keys, relax every edge of the rest with atomicMin, insert the
// improved keys).  Shared by the standalone SSSP kernel and the served
// queries.
//
// The block scans the degrees of the current keys, then relaxes the batch's
// edges in rounds of one edge per thread (a binary search over the scanned
// degrees finds each edge's vertex), appends improved keys to `emit` and
// inserts full batches as they form; the remainder is inserted at the end.
#pragma once
#include "gpuheap_device.cuh"
#include "worklist.cuh"

namespace gh {
namespace app {

// pre: size + 1 long longs; wsum: 32 long longs; emit: batchSize +
// blockDim.x keys; *cnt (shared) is 0 on entry and on return.
template <typename H>
__device__ __forceinline__ void sssp_relax_batch(const H& heap, const unsigned long long* batch, int size,
                                                 long long* pre, long long* wsum, unsigned long long* emit, int* cnt,
                                                 const long long* __restrict__ rowptr, const int* __restrict__ col,
                                                 const unsigned* __restrict__ wt, unsigned* dist, int heapOff,
                                                 unsigned long long& edges, unsigned long long& inserted) {
    using u64 = unsigned long long;
    const int B = heap.batchSize, T = blockDim.x, tid = threadIdx.x;
    // degrees of the keys that are still current (stale keys expand nothing)
    for (int i = tid; i < size; i += T) {
        const u64 key = batch[i];
        const unsigned d = static_cast<unsigned>(key >> 32);
        const int v = static_cast<int>(key & 0xffffffffu);
        pre[i + 1] = d <= __ldcg(dist + v) ? rowptr[v + 1] - rowptr[v] : 0;
    }
    __syncthreads();
    // exclusive scan of the degrees over the block (a chunk per thread)
    const int per = (size + T - 1) / T;
    long long local = 0;
    for (int j = 0; j < per; ++j) {
        const int i = tid * per + j;
        if (i < size) local += pre[i + 1];
    }
    long long incl = local;
    const int lane = tid & 31, warp = tid >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        long long x = lane < (T >> 5) ? wsum[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        wsum[lane] = x;
    }
    __syncthreads();
    long long run = incl - local + (warp ? wsum[warp - 1] : 0);
    for (int j = 0; j < per; ++j) {
        const int i = tid * per + j;
        if (i < size) { run += pre[i + 1]; pre[i + 1] = run; }
    }
    if (tid == 0) pre[0] = 0;
    __syncthreads();
    const long long total = pre[size];
    edges += total;
    // relax in rounds of one edge per thread; full batches go to the heap
    for (long long base = 0; base < total; base += T) {
        const long long ei = base + tid;
        if (ei < total) {
            int lo = 0, hi = size;  // largest lo with pre[lo] <= ei
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (pre[mid] <= ei) lo = mid;
                else hi = mid;
            }
            const u64 key = batch[lo];
            const unsigned d = static_cast<unsigned>(key >> 32);
            const int v = static_cast<int>(key & 0xffffffffu);
            const long long e = rowptr[v] + (ei - pre[lo]);
            const int u = col[e];
            const u64 nd64 = static_cast<u64>(d) + wt[e];
            const unsigned nd = nd64 >= 0xffffffffULL ? 0xfffffffeu : static_cast<unsigned>(nd64);
            if (nd < __ldcg(dist + u)) {
                const unsigned old = atomicMin(dist + u, nd);
                if (nd < old) emit[atomicAdd(cnt, 1)] = (static_cast<u64>(nd) << 32) | static_cast<unsigned>(u);
            }
        }
        __syncthreads();
        const int c = *cnt;
        if (c >= B) {
            insert_keys(heap, emit, B, heapOff);
            for (int i = tid; i < c - B; i += T) emit[i] = emit[B + i];
            __syncthreads();
            if (tid == 0) *cnt = c - B;
            inserted += B;
        }
        __syncthreads();
    }
    const int rest = *cnt;
    if (rest > 0) insert_keys(heap, emit, rest, heapOff);
    inserted += rest;
    __syncthreads();
    if (tid == 0) *cnt = 0;
    __syncthreads();
}

}  // namespace app
}  // namespace gh
