// gpuheap_fifo.cuh -- device FIFO buffer for block-collective batches.
//
// The reference's Buffer<K> (artifacts/buffer/buffer.cuh:6-218): a ring of
// `capacity` keys with four counters, begin <= read <= write <= end.  A push
// reserves [end, end + size) with atomicAdd, waits until the ring has room
// (its last slot is less than `capacity` past begin), writes its keys and
// publishes them by moving write from its start to its end -- pushes publish
// in the order they reserved (the reference commits with a CAS loop; here the
// owner waits for write to reach its start and stores, since no other block
// can move write from there).  A pop claims up to maxSize published keys by a
// CAS on read, copies them and frees their slots by moving begin, pops also
// in claim order.  Every thread of the block calls push / pop.
//
// Different by design: the capacity is a power of two (positions wrap with a
// mask), the pushers' counters (end, write) and the poppers' (read, begin)
// sit on separate 128-byte lines, slots are read through L2 (a slot is
// rewritten every lap), and every wait is bounded: past the time limit the
// block records FifoState::err and returns.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gh {

struct alignas(128) FifoState {
    unsigned long long end;    // next reservation
    unsigned long long write;  // published up to here
    unsigned long long pad0[14];
    unsigned long long read;   // claimed up to here
    unsigned long long begin;  // freed up to here
    unsigned long long pad1[14];
    int err;                   // 0, or 3 (a wait passed the time limit)
    int errSite;               // 1 room, 2 publish, 3 claim, 4 free, 5 empty
    unsigned long long mark;   // read position where the current bulk pop began
    unsigned long long bulkStart;  // first position of the current whole-call push
    long long claimN;          // keys of the current whole-call pop
    int bulkDone;              // blocks of the current whole-call launch that finished
    int pad3[23];
};
static_assert(sizeof(FifoState) == 384, "three 128-byte lines");

namespace fifo_detail {
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long cas_acq_rel64(unsigned long long* p, unsigned long long cmp,
                                                            unsigned long long val) {
    unsigned long long old;
    asm volatile("atom.acq_rel.gpu.global.cas.b64 %0, [%1], %2, %3;" : "=l"(old) : "l"(p), "l"(cmp), "l"(val) : "memory");
    return old;
}
__device__ __forceinline__ void st_release64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long now() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Loads of a copy's source: through L2 (__ldcg) from global memory -- ring
// slots are rewritten every lap and must not be served from a stale L1 line
// -- and plain loads from shared memory, which __ldcg cannot address.
template <bool kGlobal, typename T>
__device__ __forceinline__ T load_src(const T* p) {
    if constexpr (kGlobal) return __ldcg(p);
    else return *p;
}

// Copy of n keys by T threads, this one being thread t (a block or the whole
// grid).  When source and destination share their offset within 16 bytes
// the body moves as 16-byte vectors, four per thread in flight; otherwise
// four scalar keys per thread are loaded before they are stored.
template <bool kGlobal, typename K>
__device__ __forceinline__ void copy_keys_from(K* __restrict__ dst, const K* __restrict__ src, long long n, long long t,
                                               long long T) {
    constexpr int kVec = 16 / sizeof(K);
    const uintptr_t d = reinterpret_cast<uintptr_t>(dst), s = reinterpret_cast<uintptr_t>(src);
    if (((d ^ s) & 15) == 0 && n >= 4 * kVec) {
        const long long head = static_cast<long long>(((16 - (d & 15)) & 15) / sizeof(K));
        if (t < head) dst[t] = load_src<kGlobal>(src + t);
        const long long nv = (n - head) / kVec;
        uint4* dv = reinterpret_cast<uint4*>(dst + head);
        const uint4* sv = reinterpret_cast<const uint4*>(src + head);
        long long i = t;
#pragma unroll 1
        for (; i + 3 * T < nv; i += 4 * T) {
            const uint4 a = load_src<kGlobal>(sv + i), b = load_src<kGlobal>(sv + i + T),
                        c = load_src<kGlobal>(sv + i + 2 * T), e = load_src<kGlobal>(sv + i + 3 * T);
            dv[i] = a;
            dv[i + T] = b;
            dv[i + 2 * T] = c;
            dv[i + 3 * T] = e;
        }
#pragma unroll 1
        for (; i < nv; i += T) dv[i] = load_src<kGlobal>(sv + i);
#pragma unroll 1
        for (long long j = head + nv * kVec + t; j < n; j += T) dst[j] = load_src<kGlobal>(src + j);
        return;
    }
    long long i = t;
#pragma unroll 1
    for (; i + 3 * T < n; i += 4 * T) {
        const K a = load_src<kGlobal>(src + i), b = load_src<kGlobal>(src + i + T), c = load_src<kGlobal>(src + i + 2 * T),
                e = load_src<kGlobal>(src + i + 3 * T);
        dst[i] = a;
        dst[i + T] = b;
        dst[i + 2 * T] = c;
        dst[i + 3 * T] = e;
    }
#pragma unroll 1
    for (; i < n; i += T) dst[i] = load_src<kGlobal>(src + i);
}

// The source may be global or shared memory (a block's staging buffer).
template <typename K>
__device__ __forceinline__ void copy_keys(K* __restrict__ dst, const K* __restrict__ src, long long n, long long t,
                                          long long T) {
    if (__isShared(src)) copy_keys_from<false>(dst, src, n, t, T);
    else copy_keys_from<true>(dst, src, n, t, T);
}

}  // namespace fifo_detail

template <typename K>
struct Fifo {
    using key_type = K;
    K* items;
    FifoState* state;
    unsigned long long capacity;  // power of two
    long long timeoutNs;

    __device__ __forceinline__ K& slot(unsigned long long pos) const { return items[pos & (capacity - 1)]; }

    // Block-collective: src[0, n) into ring positions [pos, pos + n), as at
    // most two straight copies (the second after the ring wraps).
    __device__ __forceinline__ void to_ring(unsigned long long pos, const K* src, long long n) const {
        const unsigned long long at = pos & (capacity - 1);
        const long long first = static_cast<long long>(min(static_cast<unsigned long long>(n), capacity - at));
        fifo_detail::copy_keys(items + at, src, first, threadIdx.x, blockDim.x);
        if (first < n) fifo_detail::copy_keys(items, src + first, n - first, threadIdx.x, blockDim.x);
    }

    // Thread 0: records a timeout (sticky).
    __device__ __forceinline__ void fail(int site) const {
        if (atomicCAS(&state->err, 0, 3) == 0) state->errSite = site;
    }
    __device__ __forceinline__ bool failed() const { return *(volatile int*)&state->err != 0; }

    // insertToBuffer (buffer.cuh:127-170): appends src[0, size); size <= capacity.
    __device__ __forceinline__ void push(const K* src, int size) const {
        __shared__ unsigned long long s_start;
        __shared__ int s_ok;
        if (size <= 0) return;
        if (threadIdx.x == 0) {
            const unsigned long long start = atomicAdd(&state->end, static_cast<unsigned long long>(size));
            int ok = 1;
            const unsigned long long t0 = fifo_detail::now();
            // room for the whole chunk: its last slot is within one lap of begin
            while (start + size - fifo_detail::ld_acquire64(&state->begin) > capacity) {
                if (failed() || fifo_detail::now() - t0 > static_cast<unsigned long long>(timeoutNs)) {
                    fail(1);
                    ok = 0;
                    break;
                }
                __nanosleep(100);
            }
            s_start = start;
            s_ok = ok;
        }
        __syncthreads();
        const unsigned long long start = s_start;
        if (s_ok) to_ring(start, src, size);
        __syncthreads();
        if (threadIdx.x == 0 && s_ok) {
            // publish in reservation order (buffer.cuh:166-168).  Only the
            // owner of the range starting at `write` moves it, so once
            // `write` reaches `start` a release store commits.  A push that
            // timed out publishes nothing; the recorded error stops the rest.
            __threadfence();
            const unsigned long long t0 = fifo_detail::now();
            bool mine = true;
            while (fifo_detail::ld_acquire64(&state->write) != start) {
                if (failed() || fifo_detail::now() - t0 > static_cast<unsigned long long>(timeoutNs)) {
                    fail(2);
                    mine = false;
                    break;
                }
                __nanosleep(32);
            }
            if (mine) fifo_detail::st_release64(&state->write, start + size);
        }
        __syncthreads();
    }

    // A claim of `n` published keys starting at push-order position `start`.
    struct Claim {
        unsigned long long start;
        int n;
    };

    // First half of deleteFromBuffer (buffer.cuh:172-200), collective: claims
    // up to maxSize published keys, never past position `limit`.  n == 0 when
    // nothing is published below the limit (or a wait timed out).
    __device__ __forceinline__ Claim claim(int maxSize, unsigned long long limit = ~0ull) const {
        __shared__ unsigned long long s_start;
        __shared__ int s_n;
        if (threadIdx.x == 0) {
            int n = 0;
            unsigned long long r = 0;
            const unsigned long long t0 = fifo_detail::now();
            for (;;) {
                r = fifo_detail::ld_acquire64(&state->read);
                unsigned long long w = fifo_detail::ld_acquire64(&state->write);
                if (w > limit) w = limit;
                const unsigned long long avail = w > r ? w - r : 0;
                n = avail < static_cast<unsigned long long>(maxSize) ? static_cast<int>(avail) : maxSize;
                if (n == 0) break;
                if (fifo_detail::cas_acq_rel64(&state->read, r, r + n) == r) break;
                if (failed() || fifo_detail::now() - t0 > static_cast<unsigned long long>(timeoutNs)) {
                    fail(3);
                    n = 0;
                    break;
                }
            }
            s_start = r;
            s_n = n;
        }
        __syncthreads();
        Claim c{s_start, s_n};
        __syncthreads();
        return c;
    }

    // Copies a claimed range to dst[0, c.n) (collective).
    __device__ __forceinline__ void copy_out(const Claim& c, K* dst) const {
        const unsigned long long at = c.start & (capacity - 1);
        const long long first = static_cast<long long>(min(static_cast<unsigned long long>(c.n), capacity - at));
        fifo_detail::copy_keys(dst, items + at, first, threadIdx.x, blockDim.x);
        if (first < c.n) fifo_detail::copy_keys(dst + first, items, c.n - first, threadIdx.x, blockDim.x);
    }

    // Second half of deleteFromBuffer (buffer.cuh:206-213), collective: frees
    // the claimed slots, in claim order.
    __device__ __forceinline__ void release(const Claim& c) const {
        __syncthreads();
        if (threadIdx.x == 0 && c.n > 0) {
            __threadfence();
            const unsigned long long t0 = fifo_detail::now();
            bool mine = true;
            while (fifo_detail::ld_acquire64(&state->begin) != c.start) {
                if (failed() || fifo_detail::now() - t0 > static_cast<unsigned long long>(timeoutNs)) {
                    fail(4);
                    mine = false;
                    break;
                }
                __nanosleep(32);
            }
            if (mine) fifo_detail::st_release64(&state->begin, c.start + c.n);
        }
        __syncthreads();
    }

    // deleteFromBuffer (buffer.cuh:172-214): takes up to maxSize published
    // keys, in push order, into dst; size gets the count.  Returns false when
    // nothing was published.
    __device__ __forceinline__ bool pop(K* dst, int& size, int maxSize) const {
        const Claim c = claim(maxSize);
        size = c.n;
        if (c.n == 0) return false;
        copy_out(c, dst);
        release(c);
        return true;
    }

    // Thread 0: waits until a key below `limit` is published (returns false)
    // or everything below `limit` has been claimed (returns true).  Past the
    // time limit it records the timeout and returns true.
    __device__ __forceinline__ bool wait_published(unsigned long long limit) const {
        const unsigned long long t0 = fifo_detail::now();
        for (;;) {
            const unsigned long long r = fifo_detail::ld_acquire64(&state->read);
            if (r >= limit) return true;
            if (fifo_detail::ld_acquire64(&state->write) > r) return false;
            if (failed() || fifo_detail::now() - t0 > static_cast<unsigned long long>(timeoutNs)) {
                fail(5);
                return true;
            }
            __nanosleep(200);
        }
    }

    // Keys published and not yet claimed (a racy snapshot).
    __device__ __forceinline__ long long published() const {
        return static_cast<long long>(fifo_detail::ld_acquire64(&state->write) -
                                      fifo_detail::ld_acquire64(&state->read));
    }
};

}  // namespace gh
