// gpuheap_device.cuh -- device-side API of the GB300 batched priority queue.
//
// A drop-in for the reference's device member functions of Heap<K>
// (heap/{tditdd,tditdd_np,buitdd,buitdd_np}/heap.cuh): an application kernel
// receives a gh::Heap<K, Variant, PartialBuffer> by value (or pointer) and
// every thread of a block calls
//     heap.insertion(items, size, smemOffset)   (heap/tditdd/heap.cuh:536)
//     heap.deleteRoot(items, size)              (heap/tditdd/heap.cuh:267)
//     heap.deleteUpdate(smemOffset)             (heap/tditdd/heap.cuh:345)
// with the reference's meaning: operations are block-collective, a heap node
// is a sorted batch of batchSize keys, node 0 is the partial buffer, and
// `smemOffset` counts 4-byte words of dynamic shared memory reserved by the
// caller ahead of the heap's own region.  The variant, chosen by include path
// in the reference, is a template parameter here.
//
// What is different, by design, for sm_103a:
//   * nodes are moved global -> shared by TMA bulk copies (cp.async.bulk with
//     an mbarrier), merged in registers by a merge-path split of two sorted
//     batches and written straight from registers with 16-byte stores, so a
//     level step costs one bulk load, one merge and one store;
//   * the insert batch is sorted by a bitonic network whose short strides run
//     under __syncwarp instead of __syncthreads;
//   * locks use acquire/release atomics at GPU scope (the reference publishes
//     node data with plain stores), and node reads after a lock are ordered
//     by fence.proxy.async before the bulk copy;
//   * every wait is bounded by a time limit; on expiry the block records an
//     error in HeapState::err and returns, and every other block stops at its
//     next wait, so a broken heap never hangs the GPU;
//   * insertion checks capacity (the reference writes past batchNum).
//
// Requirements: batchSize is a power of two in [16, 8192]; blockDim.x is a
// power of two in [32, 1024] with batchSize / 8 <= blockDim.x <= 2 * batchSize; the heap
// needs smemBytes(batchSize) bytes of dynamic shared memory after
// 4 * smemOffset bytes (rounded up to 16).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gh {

enum Variant : int { kTopDown = 0, kBottomUp = 1 };

// Lock-word states.  Top-down heaps: heap/tditdd/heap.cuh:6-9 and the
// transition table at :242-258.  Bottom-up heaps: heap/buitdd/heap.cuh:6-9,
// table at :258-274.
struct TD { static constexpr int AVAIL = 0, INUSE = 1, TARGET = 2, MARKED = 3; };
struct BU { static constexpr int AVAIL = 0, INSHOLD = 1, DELMOD = 2, INUSE = 3; };

enum DeviceError : int { kErrNone = 0, kErrInvalid = 1, kErrCapacity = 2, kErrTimeout = 3 };

// Where a device error was raised (HeapState::errOp).
enum ErrSite : int {
    kSiteLockPartial = 1, kSiteLockRoot = 2, kSiteLockTarget = 3, kSiteLockPath = 4,
    kSiteLockLast = 5, kSiteLockChild = 6, kSiteHandOff = 7, kSiteBulkCopy = 8, kSiteCapacity = 9
};

// Heap counters and the sticky error record, one 128-byte line each.
struct alignas(128) HeapState {
    int batchCount;         // full nodes (reference: *batchCount)
    int partialBufferSize;  // keys held in node 0 (reference: *partialBufferSize)
    int deleteCount;        // HEAP_SORT output cursor (reference: *deleteCount)
    int outLimit;           // deleteRoot outputs nothing once the cursor would pass this
    int pad0[28];
    int err;                // first DeviceError raised, 0 if none
    int errOp;              // ErrSite
    int errNode;            // node whose wait failed
    int errState;           // lock word value last seen there
    int pad1[28];
};

// Per-operation control block at the end of the heap's shared-memory region.
struct OpCtl {
    unsigned long long bar;  // mbarrier for the bulk copies
    int abort;               // block-uniform "stop" flag
    int bc, ps, dc;          // counters read under the partial-buffer lock
    int w0, w1, w2, w3;      // broadcast words
    int pad[6];
};
static_assert(sizeof(OpCtl) == 64, "OpCtl layout");

namespace detail {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(int* p, int v) {
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int cas_acquire(int* p, int cmp, int val) {
    int old;
    asm volatile("atom.acquire.gpu.global.cas.b32 %0, [%1], %2, %3;" : "=r"(old) : "l"(p), "r"(cmp), "r"(val) : "memory");
    return old;
}
__device__ __forceinline__ int cas_acq_rel(int* p, int cmp, int val) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.cas.b32 %0, [%1], %2, %3;" : "=r"(old) : "l"(p), "r"(cmp), "r"(val) : "memory");
    return old;
}
__device__ __forceinline__ int max_acquire(int* p, int val) {
    int old;
    asm volatile("atom.acquire.gpu.global.max.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(val) : "memory");
    return old;
}
// Orders this thread's (and, through barriers and acquires, other threads')
// generic-proxy global accesses before later bulk-copy (async-proxy) ones.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(unsigned long long* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// One-dimensional TMA bulk copy global -> shared, completion on `bar`.
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Key bits as 32-bit words, without taking any register's address.
template <typename K>
__device__ __forceinline__ unsigned lo32(K k) {
    if constexpr (sizeof(K) == 8) return static_cast<unsigned>(static_cast<unsigned long long>(k));
    else return static_cast<unsigned>(k);
}
template <typename K>
__device__ __forceinline__ unsigned hi32(K k) {
    if constexpr (sizeof(K) == 8) return static_cast<unsigned>(static_cast<unsigned long long>(k) >> 32);
    else return 0u;
}

// Stores IPT consecutive keys from registers: 16-byte vectors when the
// destination is 16-byte aligned and the run a multiple of 16 bytes.
template <typename K, int IPT>
__device__ __forceinline__ void store_run(K* dst, const K (&r)[IPT]) {
    constexpr int bytes = IPT * static_cast<int>(sizeof(K));
    if constexpr (bytes % 16 == 0) {
        if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
            uint4* v = reinterpret_cast<uint4*>(dst);
            if constexpr (sizeof(K) == 4) {
#pragma unroll
                for (int q = 0; q < IPT / 4; ++q)
                    v[q] = make_uint4(lo32(r[4 * q]), lo32(r[4 * q + 1]), lo32(r[4 * q + 2]), lo32(r[4 * q + 3]));
            } else {
#pragma unroll
                for (int q = 0; q < IPT / 2; ++q)
                    v[q] = make_uint4(lo32(r[2 * q]), hi32(r[2 * q]), lo32(r[2 * q + 1]), hi32(r[2 * q + 1]));
            }
            return;
        }
    }
#pragma unroll
    for (int q = 0; q < IPT; ++q) dst[q] = r[q];
}

// Merge-path split of two sorted runs a[0,n) and b[0,n): the n smallest keys
// go to lo[0,n), the n largest to hi[0,n) (either may be null to discard).
// Thread t produces outputs [t*IPT, (t+1)*IPT): a binary search on its
// diagonal finds the split (a wins ties, as heap/heaputil.cuh:99-158 does),
// IPT sequential merge steps fill registers, a barrier lets lo/hi alias a/b,
// and the run is stored with vector stores.  Ends without a trailing barrier.
template <typename K, int IPT>
__device__ __forceinline__ void merge_split_t(const K* a, const K* b, K* lo, K* hi, int n) {
    const int d = static_cast<int>(threadIdx.x) * IPT;
    const bool active = d < 2 * n;
    K r[IPT];
    if (active) {
        int i0 = d > n ? d - n : 0, i1 = d < n ? d : n;
        while (i0 < i1) {
            const int m = (i0 + i1) >> 1;
            if (a[m] <= b[d - 1 - m]) i0 = m + 1;
            else i1 = m;
        }
        int i = i0, j = d - i0;
        K av = a[i < n ? i : n - 1], bv = b[j < n ? j : n - 1];
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const bool ta = (j >= n) || (i < n && av <= bv);
            r[k] = ta ? av : bv;
            if (ta) { ++i; av = a[i < n ? i : n - 1]; }
            else { ++j; bv = b[j < n ? j : n - 1]; }
        }
    }
    __syncthreads();
    if (active) {
        K* dst = d < n ? (lo ? lo + d : nullptr) : (hi ? hi + (d - n) : nullptr);
        if (dst) store_run<K, IPT>(dst, r);
    }
}

template <typename K, int FIXED_IPT = 0>
__device__ __forceinline__ void merge_split(const K* a, const K* b, K* lo, K* hi, int n) {
    if constexpr (FIXED_IPT > 0) {
        merge_split_t<K, FIXED_IPT>(a, b, lo, hi, n);
        return;
    }
    int ipt = (2 * n) / static_cast<int>(blockDim.x);
    if (ipt < 1) ipt = 1;
    switch (ipt) {
        case 1: merge_split_t<K, 1>(a, b, lo, hi, n); break;
        case 2: merge_split_t<K, 2>(a, b, lo, hi, n); break;
        case 4: merge_split_t<K, 4>(a, b, lo, hi, n); break;
        case 8: merge_split_t<K, 8>(a, b, lo, hi, n); break;
        default: merge_split_t<K, 16>(a, b, lo, hi, n); break;
    }
}

// In-place ascending bitonic sort of s[0,n) in shared memory, n a power of
// two.  Pair p of a stage with stride j touches (i, i + j) where
// i = (p / j) * 2j + p % j; for j <= 32 the pairs of one warp stay inside one
// aligned 64-key block, so those stages only need __syncwarp.
template <typename K>
__device__ __forceinline__ void bitonic_sort(K* s, int n) {
    const int half = n >> 1;
    const int T = static_cast<int>(blockDim.x);
    for (int k = 2; k <= n; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int p = static_cast<int>(threadIdx.x); p < half; p += T) {
                const int i = ((p / j) * 2 * j) + (p % j);
                const int x = i + j;
                const K u = s[i], v = s[x];
                const bool up = (i & k) == 0;
                if (up ? (u > v) : (u < v)) { s[i] = v; s[x] = u; }
            }
            const int next_j = j > 1 ? (j >> 1) : (k << 1) >> 1;
            if (j <= 32 && next_j <= 32 && !(j == 1 && k == n)) __syncwarp();
            else __syncthreads();
        }
    }
}

template <typename K>
__device__ __forceinline__ uint4 splat16(K v) {
    uint4 r;
    K* p = reinterpret_cast<K*>(&r);
#pragma unroll
    for (int q = 0; q < static_cast<int>(16 / sizeof(K)); ++q) p[q] = v;
    return r;
}

}  // namespace detail

template <typename K, int VARIANT, bool PB, int IPT = 0>
struct Heap {
    using key_type = K;
    K* heapItems;          // (batchNum + 1) nodes of batchSize keys, node 0 = partial buffer
    int* status;           // batchNum + 1 lock words
    HeapState* state;      // counters + error record
    K init_limits;         // padding key, strictly above every real key
    int batchNum;          // capacity in full nodes
    int batchSize;         // keys per node
    int sortOutput;        // 1: HEAP_SORT output at items + deleteCount
    long long timeoutNs;   // bound on every wait

    static __host__ __device__ size_t smemBytes(int bs) {
        return 3 * static_cast<size_t>(bs) * sizeof(K) + sizeof(OpCtl) + 16;
    }

    // ------------------------------------------------------------------ plumbing
    __device__ __forceinline__ K* region(int smemOffset) const {
        extern __shared__ __align__(16) unsigned char gh_dyn_smem[];
        size_t off = (static_cast<size_t>(smemOffset) * 4 + 15) & ~static_cast<size_t>(15);
        return reinterpret_cast<K*>(gh_dyn_smem + off);
    }
    __device__ __forceinline__ OpCtl* ctl(K* base) const { return reinterpret_cast<OpCtl*>(base + 3 * batchSize); }
    __device__ __forceinline__ K* node(int i) const { return heapItems + static_cast<size_t>(i) * batchSize; }
    __device__ __forceinline__ unsigned nodeBytes() const { return static_cast<unsigned>(batchSize * sizeof(K)); }

    // Records the first error (sticky).
    __device__ __forceinline__ void raise(int code, int site, int nodeIdx, int seen) const {
        if (atomicCAS(&state->err, 0, code) == 0) {
            state->errOp = site;
            state->errNode = nodeIdx;
            state->errState = seen;
            __threadfence();
        }
    }

    // Periodic check inside a wait: false once the time limit has passed
    // (the error is raised) or another block has already raised one.
    __device__ __forceinline__ bool keep_waiting(unsigned long long& t0, unsigned it, int site, int nodeIdx, int seen) const {
        if ((it & 15u) != 15u) return true;
        const unsigned long long now = detail::globaltimer();
        if (t0 == 0) t0 = now;
        if (now - t0 > static_cast<unsigned long long>(timeoutNs)) {
            raise(kErrTimeout, site, nodeIdx, seen);
            return false;
        }
        if ((it & 255u) == 255u && detail::ld_relaxed(&state->err) != 0) return false;
        return true;
    }

    // Spin until status[i] == from, then swap in `to` with acquire semantics.
    __device__ __forceinline__ bool lock(int i, int from, int to, int site) const {
        int* w = status + i;
        unsigned long long t0 = 0;
        for (unsigned it = 0;; ++it) {
            const int v = detail::ld_relaxed(w);
            if (v == from && detail::cas_acquire(w, from, to) == from) return true;
            if (!keep_waiting(t0, it, site, i, v)) return false;
        }
    }
    // Owner-side transition out of an exclusive state.
    __device__ __forceinline__ void unlock(int i, int to) const { detail::st_release(status + i, to); }

    // Block-wide setup: fresh mbarrier, abort if the heap already failed.
    struct Op {
        const Heap* h;
        OpCtl* c;
        unsigned phase;
        __device__ __forceinline__ Op(const Heap* hp, OpCtl* cp) : h(hp), c(cp), phase(0) {
            __syncthreads();
            if (threadIdx.x == 0) {
                c->abort = detail::ld_relaxed(&h->state->err) != 0;
                detail::mbar_init(&c->bar, 1);
            }
            __syncthreads();
        }
        __device__ __forceinline__ ~Op() {
            __syncthreads();
            if (threadIdx.x == 0) detail::mbar_inval(&c->bar);
        }
        // Thread 0 only: start one bulk transaction of `bytes`.
        __device__ __forceinline__ void expect(unsigned bytes) {
            detail::fence_proxy_async();
            detail::mbar_arrive_expect_tx(&c->bar, bytes);
        }
        // Block-wide: thread 0 waits for the transaction (bounded), the rest
        // wait at the barrier.  Returns false (block-uniform) on failure.
        __device__ __forceinline__ bool wait() {
            if (threadIdx.x == 0) {
                unsigned long long t0 = 0;
                bool ok = true;
                for (unsigned it = 0; !detail::mbar_try_wait(&c->bar, phase); ++it) {
                    if (!h->keep_waiting(t0, it, kSiteBulkCopy, -1, 0)) { ok = false; break; }
                }
                if (!ok) {
                    // The copies read valid global memory and must land before the
                    // shared memory is reused: give them a second bounded wait.
                    for (unsigned it = 0; it < (1u << 22) && !detail::mbar_try_wait(&c->bar, phase); ++it) {}
                    c->abort = 1;
                }
            }
            phase ^= 1u;
            __syncthreads();
            return !c->abort;
        }
    };

    // Block-wide copies between shared and global nodes (16-byte aligned).
    __device__ __forceinline__ void store_node(int i, const K* s) const {
        const int nv = batchSize * static_cast<int>(sizeof(K)) / 16;
        uint4* g = reinterpret_cast<uint4*>(node(i));
        const uint4* v = reinterpret_cast<const uint4*>(s);
        for (int q = threadIdx.x; q < nv; q += blockDim.x) g[q] = v[q];
    }
    __device__ __forceinline__ void fill_node(int i, int count) const {  // first `count` keys (multiple of 16 B) or scalar tail
        K* g = node(i);
        const int per = 16 / static_cast<int>(sizeof(K));
        const int nv = count / per;
        const uint4 pat = detail::splat16<K>(init_limits);
        for (int q = threadIdx.x; q < nv; q += blockDim.x) reinterpret_cast<uint4*>(g)[q] = pat;
        for (int q = nv * per + threadIdx.x; q < count; q += blockDim.x) g[q] = init_limits;
    }
    // Copies `count` keys of node i to dst (any alignment).
    __device__ __forceinline__ void copy_out(K* dst, int i, int count) const {
        const K* src = node(i);
        const int per = 16 / static_cast<int>(sizeof(K));
        if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
            const int nv = count / per;
            for (int q = threadIdx.x; q < nv; q += blockDim.x)
                reinterpret_cast<uint4*>(dst)[q] = __ldcg(reinterpret_cast<const uint4*>(src) + q);
            for (int q = nv * per + threadIdx.x; q < count; q += blockDim.x) dst[q] = __ldcg(src + q);
        } else {
            for (int q = threadIdx.x; q < count; q += blockDim.x) dst[q] = __ldcg(src + q);
        }
    }

    // Node layout helpers.  Bottom-up heaps store level-order nodes with the
    // bits below the leading one reversed (heap/buitdd/heap.cuh:233-236).
    __device__ __forceinline__ static int rev(int i) {
        if (i <= 1) return i;
        const int l = __clz(i) + 1;
        return static_cast<int>((__brev(static_cast<unsigned>(i)) >> l) | (1u << (32 - l)));
    }
    __device__ __forceinline__ static int parentOf(int i) { return VARIANT == kTopDown ? i >> 1 : rev(rev(i) >> 1); }
    __device__ __forceinline__ static int leftOf(int i) { return VARIANT == kTopDown ? i << 1 : rev(rev(i) << 1); }
    __device__ __forceinline__ static int rightOf(int l) { return VARIANT == kTopDown ? l + 1 : rev(rev(l) + 1); }
    // heap/tditdd/heap.cuh:263-265
    __device__ __forceinline__ static int nextOnPath(int cur, int target) {
        return target >> (__clz(cur) - __clz(target) - 1);
    }

    // ------------------------------------------------------------------ insertion
    // heap/tditdd/heap.cuh:536-753 (top-down) and heap/buitdd/heap.cuh:484-690
    // (bottom-up); without the partial buffer: the _np copies.
    __device__ __forceinline__ void insertion(const K* items, int size, int smemOffset) const {
        K* s0 = region(smemOffset);
        K* s1 = s0 + batchSize;
        K* s2 = s1 + batchSize;
        Op op(this, ctl(s0));
        OpCtl* c = op.c;
        if (c->abort) return;
        const int B = batchSize;
        const int tid = threadIdx.x;

        // stage and pad with init_limits, then sort (:557-562)
        for (int q = tid; q < B; q += blockDim.x) s0[q] = q < size ? items[q] : init_limits;
        __syncthreads();
        detail::bitonic_sort(s0, B);

        // lock the partial buffer; the counters are only changed under it
        if (tid == 0) {
            const bool ok = lock(0, 0, lockedState(), kSiteLockPartial);
            c->abort = !ok;
            if (ok) {
                c->bc = detail::ld_relaxed(&state->batchCount);
                c->ps = detail::ld_relaxed(&state->partialBufferSize);
            }
        }
        __syncthreads();
        if (c->abort) return;
        const int bc = c->bc, ps = c->ps;

        if constexpr (PB) {
            if (bc == 0 && size < B) {
                if (ps == 0) {  // case 1.1 (:575-584)
                    store_node(0, s0);
                    __syncthreads();
                    if (tid == 0) {
                        detail::st_relaxed(&state->partialBufferSize, size);
                        unlock(0, 0);
                    }
                    return;
                }
                if (tid == 0) { op.expect(nodeBytes()); detail::bulk_g2s(s1, node(0), nodeBytes(), &c->bar); }
                if (!op.wait()) return;
                if (size + ps < B) {  // case 1.2 (:586-598)
                    detail::merge_split<K, IPT>(s0, s1, node(0), static_cast<K*>(nullptr), B);
                    __syncthreads();
                    if (tid == 0) {
                        detail::st_relaxed(&state->partialBufferSize, ps + size);
                        unlock(0, 0);
                    }
                    return;
                }
                // case 1.3 (:600-620): the first full batch becomes the root
                if (tid == 0) {
                    bool ok = batchNum >= 1;
                    if (!ok) raise(kErrCapacity, kSiteCapacity, 1, 0);
                    ok = ok && lock(1, 0, lockedState(), kSiteLockRoot);
                    c->abort = !ok;
                    if (ok) detail::st_relaxed(&state->batchCount, 1);
                }
                __syncthreads();
                if (c->abort) return;
                detail::merge_split<K, IPT>(s0, s1, node(1), node(0), B);
                __syncthreads();
                if (tid == 0) {
                    detail::st_relaxed(&state->partialBufferSize, ps + size - B);
                    unlock(0, 0);
                    unlock(1, 0);
                }
                return;
            }
            if (tid == 0) { op.expect(nodeBytes()); detail::bulk_g2s(s1, node(0), nodeBytes(), &c->bar); }
            if (!op.wait()) return;
            if (size + ps < B) {  // case 2.1 (:625-648): no new full batch, merge through the root
                detail::merge_split<K, IPT>(s0, s1, s0, static_cast<K*>(nullptr), B);
                __syncthreads();
                if (tid == 0) {
                    const bool ok = lock(1, 0, lockedState(), kSiteLockRoot);
                    c->abort = !ok;
                    if (ok) { op.expect(nodeBytes()); detail::bulk_g2s(s1, node(1), nodeBytes(), &c->bar); }
                }
                __syncthreads();
                if (c->abort) return;
                if (!op.wait()) return;
                detail::merge_split<K, IPT>(s0, s1, node(1), node(0), B);
                __syncthreads();
                if (tid == 0) {
                    detail::st_relaxed(&state->partialBufferSize, ps + size);
                    unlock(0, 0);
                    unlock(1, 0);
                }
                return;
            }
            // case 2.2 (:650-662): the smaller B keys go on, the rest stay in node 0
            detail::merge_split<K, IPT>(s0, s1, s0, node(0), B);
            __syncthreads();
            if (tid == 0) detail::st_relaxed(&state->partialBufferSize, ps + size - B);
        }

        if constexpr (VARIANT == kTopDown) insert_topdown(op, s0, s1, bc);
        else insert_bottomup(op, s0, s1, s2, bc);
    }

    __device__ __forceinline__ static constexpr int lockedState() { return VARIANT == kTopDown ? TD::INUSE : BU::INUSE; }

    // Top-down path (heap/tditdd/heap.cuh:666-752).  Entered holding node 0;
    // the carried batch is in s0.
    __device__ __forceinline__ void insert_topdown(Op& op, K* s0, K* s1, int bc) const {
        OpCtl* c = op.c;
        const int tid = threadIdx.x;
        if (tid == 0) {
            const int target = bc + 1;
            bool ok = target <= batchNum;
            if (!ok) raise(kErrCapacity, kSiteCapacity, target, 0);
            if (ok) detail::st_relaxed(&state->batchCount, target);
            ok = ok && lock(target, TD::AVAIL, TD::TARGET, kSiteLockTarget);
            if (ok && target != 1) ok = lock(1, TD::AVAIL, TD::INUSE, kSiteLockRoot);
            c->abort = !ok;
            c->w0 = target;
        }
        __syncthreads();
        if (c->abort) return;
        const int target = c->w0;
        int cur = 1;
        while (cur != target) {
            if (tid == 0) {
                c->w1 = detail::ld_relaxed(status + target) == TD::MARKED;
                if (!c->w1) {
                    unlock(cur >> 1, TD::AVAIL);  // hand-over-hand: release the parent
                    op.expect(nodeBytes());
                    detail::bulk_g2s(s1, node(cur), nodeBytes(), &c->bar);
                }
            }
            __syncthreads();
            if (c->w1) break;  // a deleter has taken the target (:683-689)
            if (!op.wait()) return;
            detail::merge_split<K, IPT>(s0, s1, node(cur), s0, batchSize);
            cur = nextOnPath(cur, target);
            __syncthreads();
            if (tid == 0 && cur != target) c->abort = !lock(cur, TD::AVAIL, TD::INUSE, kSiteLockPath);
            __syncthreads();
            if (c->abort) return;
        }
        if (tid == 0) {
            const int old = detail::cas_acq_rel(status + target, TD::TARGET, TD::INUSE);
            c->w2 = old == TD::MARKED;
        }
        __syncthreads();
        if (c->w2) {
            // The deleter that marked the target holds the root and waits for
            // this batch there (:732-744).
            store_node(1, s0);
            __syncthreads();
            if (tid == 0) {
                unlock(cur >> 1, TD::AVAIL);
                if (target != cur) unlock(cur, TD::AVAIL);
                unlock(target, TD::TARGET);  // MARKED -> TARGET, release
            }
            return;
        }
        store_node(target, s0);
        __syncthreads();
        if (tid == 0) {
            unlock(cur >> 1, TD::AVAIL);
            unlock(cur, TD::AVAIL);
        }
    }

    // Bottom-up path (heap/buitdd/heap.cuh:616-689).  Entered holding node 0;
    // the carried batch is in s0.
    __device__ __forceinline__ void insert_bottomup(Op& op, K* s0, K* s1, K* s2, int bc) const {
        OpCtl* c = op.c;
        const int tid = threadIdx.x;
        if (tid == 0) {
            const int target = bc + 1;
            bool ok = target <= batchNum;
            if (!ok) raise(kErrCapacity, kSiteCapacity, target, 0);
            if (ok) detail::st_relaxed(&state->batchCount, target);
            ok = ok && lock(target, BU::AVAIL, BU::INUSE, kSiteLockTarget);
            if (ok) unlock(0, BU::AVAIL);
            c->abort = !ok;
            c->w0 = target;
        }
        __syncthreads();
        if (c->abort) return;
        int cur = c->w0;
        store_node(cur, s0);
        __syncthreads();
        if (tid == 0) unlock(cur, BU::INSHOLD);
        while (cur != 1) {
            const int p = parentOf(cur);
            if (tid == 0) {
                bool ok = lock(p, BU::AVAIL, BU::INUSE, kSiteLockPath);
                if (ok) {
                    // take our own node back from INSHOLD (or DELMOD if a
                    // deleter rewrote it meanwhile)
                    unsigned long long t0 = 0;
                    int prev;
                    for (unsigned it = 0; (prev = detail::max_acquire(status + cur, BU::INUSE)) == BU::INUSE; ++it) {
                        if (!keep_waiting(t0, it, kSiteLockPath, cur, prev)) { ok = false; break; }
                    }
                }
                c->abort = !ok;
                if (ok) {
                    op.expect(2 * nodeBytes());
                    detail::bulk_g2s(s1, node(p), nodeBytes(), &c->bar);
                    detail::bulk_g2s(s2, node(cur), nodeBytes(), &c->bar);
                }
            }
            __syncthreads();
            if (c->abort) return;
            if (!op.wait()) return;
            if (s1[0] >= s2[batchSize - 1]) {  // whole batch below the parent: swap (:647-661)
                store_node(p, s2);
                store_node(cur, s1);
            } else {
                detail::merge_split<K, IPT>(s2, s1, node(p), node(cur), batchSize);
            }
            __syncthreads();
            if (tid == 0) {
                unlock(p, BU::INSHOLD);
                unlock(cur, BU::AVAIL);
            }
            cur = p;
        }
        if (tid == 0) unlock(1, BU::AVAIL);  // INSHOLD -> INUSE -> AVAIL (:685-688)
    }

    // ------------------------------------------------------------------ deleteRoot
    // heap/tditdd/heap.cuh:267-341, heap/buitdd/heap.cuh:283-343.  Returns
    // true when deleteUpdate must follow (the root is taken and nodes 0 and 1
    // stay locked); `size` is the number of keys written.  Like the
    // reference it takes no shared-memory offset: its few broadcast words
    // live in a static __shared__ block, so the caller's dynamic shared
    // memory is untouched.
    __device__ __forceinline__ bool deleteRoot(K* items, int& size) const {
        __shared__ OpCtl dr;
        OpCtl* c = &dr;
        size = 0;
        const int tid = threadIdx.x;
        const int L = lockedState();
        __syncthreads();
        if (tid == 0) {
            c->abort = detail::ld_relaxed(&state->err) != 0;
            c->w0 = 0;  // 0: nothing, 1: partial buffer only, 2: root
            const bool ok = !c->abort && lock(0, 0, L, kSiteLockPartial);
            c->abort = !ok;
            if (ok) {
                const int bc = detail::ld_relaxed(&state->batchCount);
                const int ps = detail::ld_relaxed(&state->partialBufferSize);
                const int dc = detail::ld_relaxed(&state->deleteCount);
                const int lim = detail::ld_relaxed(&state->outLimit);
                c->bc = bc; c->ps = ps; c->dc = dc;
                const int want = bc > 0 ? batchSize : (PB ? ps : 0);
                if (want == 0 || (sortOutput && dc + want > lim)) {
                    unlock(0, 0);
                } else if (bc == 0) {
                    c->w0 = 1;
                } else {
                    const bool ok1 = lock(1, 0, L, kSiteLockRoot);
                    c->abort = !ok1;
                    if (ok1) {
                        c->w0 = 2;
                        if (sortOutput) detail::st_relaxed(&state->deleteCount, dc + batchSize);
                    }
                }
            }
        }
        __syncthreads();
        const int mode = c->w0;
        const bool stop = c->abort || mode == 0;
        const int dc = c->dc, ps = c->ps;
        __syncthreads();  // every thread has read dr before the next call rewrites it
        if (stop) return false;
        K* out = items + (sortOutput ? dc : 0);
        if (mode == 1) {  // only the partial buffer holds keys (:297-315)
            copy_out(out, 0, ps);
            __syncthreads();
            fill_node(0, ps);
            __syncthreads();
            if (tid == 0) {
                if (sortOutput) detail::st_relaxed(&state->deleteCount, dc + ps);
                detail::st_relaxed(&state->partialBufferSize, 0);
                unlock(0, 0);
            }
            size = ps;
            return false;
        }
        copy_out(out, 1, batchSize);  // (:328-329)
        __syncthreads();
        size = batchSize;
        return true;
    }

    // ------------------------------------------------------------------ deleteUpdate
    // Refills the root: heap/tditdd/heap.cuh:345-534, heap/buitdd/heap.cuh:348-482.
    __device__ __forceinline__ void deleteUpdate(int smemOffset) const {
        K* s0 = region(smemOffset);
        K* s1 = s0 + batchSize;
        K* s2 = s1 + batchSize;
        Op op(this, ctl(s0));
        OpCtl* c = op.c;
        if (c->abort) return;
        const int tid = threadIdx.x;
        const int B = batchSize;
        const int L = lockedState();

        // take the last node (:355-369)
        if (tid == 0) {
            const int last = detail::ld_relaxed(&state->batchCount);
            detail::st_relaxed(&state->batchCount, last - 1);
            c->w0 = last;
            c->w1 = 0;  // 0: last node taken, 1: in-flight insert handed its batch to the root
            if (last == 1) {
                unlock(1, 0);
                unlock(0, 0);
            } else if (VARIANT == kTopDown) {
                // (:371-402) either lock it, or mark an in-flight insert target
                unsigned long long t0 = 0;
                bool ok = true;
                for (unsigned it = 0;; ++it) {
                    if (detail::cas_acquire(status + last, TD::AVAIL, TD::INUSE) == TD::AVAIL) break;
                    if (detail::cas_acquire(status + last, TD::TARGET, TD::MARKED) == TD::TARGET) { c->w1 = 1; break; }
                    if (!keep_waiting(t0, it, kSiteLockLast, last, detail::ld_relaxed(status + last))) { ok = false; break; }
                }
                if (ok && c->w1) {
                    t0 = 0;
                    for (unsigned it = 0; detail::cas_acquire(status + last, TD::TARGET, TD::AVAIL) != TD::TARGET; ++it) {
                        if (!keep_waiting(t0, it, kSiteHandOff, last, detail::ld_relaxed(status + last))) { ok = false; break; }
                    }
                }
                c->abort = !ok;
            } else {
                // (:372-378) atomicMax takes the node from AVAIL, INSHOLD or DELMOD
                unsigned long long t0 = 0;
                int prev;
                bool ok = true;
                for (unsigned it = 0; (prev = detail::max_acquire(status + last, BU::INUSE)) == BU::INUSE; ++it) {
                    if (!keep_waiting(t0, it, kSiteLockLast, last, prev)) { ok = false; break; }
                }
                c->abort = !ok;
            }
            if (!c->abort && last != 1) {
                op.expect((PB ? 2u : 1u) * nodeBytes());
                detail::bulk_g2s(s0, node(c->w1 ? 1 : last), nodeBytes(), &c->bar);
                if (PB) detail::bulk_g2s(s1, node(0), nodeBytes(), &c->bar);
            }
        }
        __syncthreads();
        const int last = c->w0;
        if (last == 1 || c->abort) return;
        if (!op.wait()) return;
        if (!c->w1) {
            fill_node(last, B);  // reset the taken node (:396)
            __syncthreads();
            if (tid == 0) unlock(last, 0);
        }
        if constexpr (PB) {  // merge with the partial buffer (:404-416)
            detail::merge_split<K, IPT>(s0, s1, s0, node(0), B);
            __syncthreads();
        }
        if (tid == 0) unlock(0, 0);

        if constexpr (VARIANT == kTopDown) sift_topdown(op, s0, s1, s2);
        else sift_bottomup(op, s0, s1, s2);
    }

    // Top-down sift from the root (heap/tditdd/heap.cuh:418-532).  s0 holds
    // the batch being sifted; node `cur` is locked.
    __device__ __forceinline__ void sift_topdown(Op& op, K* s0, K* s1, K* s2) const {
        OpCtl* c = op.c;
        const int tid = threadIdx.x;
        const int B = batchSize;
        int cur = 1;
        for (;;) {
            const int l = cur << 1, r = l + 1;
            if (tid == 0) {
                // A child counts when its word can be locked from AVAIL; insert
                // targets (TARGET/MARKED) do not (:425-446).  Unlike the
                // reference, a TARGET left child does not hide an existing right
                // child: that right child's keys may be below the new content.
                bool ok = true;
                int have = 0;
                const int kids[2] = {l, r};
                for (int q = 0; q < 2 && ok; ++q) {
                    const int x = kids[q];
                    if (x > batchNum) continue;
                    unsigned long long t0 = 0;
                    for (unsigned it = 0;; ++it) {
                        const int v = detail::ld_relaxed(status + x);
                        if (v == TD::AVAIL) {
                            if (detail::cas_acquire(status + x, TD::AVAIL, TD::INUSE) == TD::AVAIL) { have |= 1 << q; break; }
                        } else if (v != TD::INUSE) {
                            break;  // an insert target: not a child yet
                        }
                        if (!keep_waiting(t0, it, kSiteLockChild, x, v)) { ok = false; break; }
                    }
                }
                c->abort = !ok;
                c->w0 = have;
                if (ok && have) {
                    op.expect((have == 3 ? 2u : 1u) * nodeBytes());
                    if (have & 1) detail::bulk_g2s(s1, node(l), nodeBytes(), &c->bar);
                    if (have & 2) detail::bulk_g2s(have == 3 ? s2 : s1, node(r), nodeBytes(), &c->bar);
                }
            }
            __syncthreads();
            if (c->abort) return;
            const int have = c->w0;
            if (have == 0) {  // no children (:452-460)
                store_node(cur, s0);
                __syncthreads();
                if (tid == 0) unlock(cur, TD::AVAIL);
                return;
            }
            if (!op.wait()) return;
            if (have != 3) {  // one child (:461-477)
                const int x = have == 1 ? l : r;
                detail::merge_split<K, IPT>(s0, s1, node(cur), node(x), B);
                __syncthreads();
                if (tid == 0) { unlock(cur, TD::AVAIL); unlock(x, TD::AVAIL); }
                return;
            }
            // two children (:479-531)
            const int larger = s1[B - 1] < s2[B - 1] ? r : l;
            const int smaller = larger == r ? l : r;
            detail::merge_split<K, IPT>(s1, s2, s1, node(larger), B);
            __syncthreads();
            if (tid == 0) unlock(larger, TD::AVAIL);
            if (s0[0] >= s1[B - 1]) {
                store_node(cur, s1);
            } else if (s0[B - 1] <= s1[0]) {
                store_node(cur, s0);
                store_node(smaller, s1);
                __syncthreads();
                if (tid == 0) { unlock(cur, TD::AVAIL); unlock(smaller, TD::AVAIL); }
                return;
            } else {
                detail::merge_split<K, IPT>(s0, s1, node(cur), s0, B);
            }
            __syncthreads();
            if (tid == 0) unlock(cur, TD::AVAIL);
            cur = smaller;
        }
    }

    // Bottom-up-layout sift from the root (heap/buitdd/heap.cuh:403-480).
    __device__ __forceinline__ void sift_bottomup(Op& op, K* s0, K* s1, K* s2) const {
        OpCtl* c = op.c;
        const int tid = threadIdx.x;
        const int B = batchSize;
        int cur = 1, curPrev = BU::AVAIL;
        for (;;) {
            const int l = leftOf(cur);
            const int r = l <= batchNum ? rightOf(l) : batchNum + 1;
            if (tid == 0) {
                // (:409-418) atomicMax takes a child from AVAIL, INSHOLD or
                // DELMOD; a child held INSHOLD by a bubbling insert is handed
                // back as DELMOD.
                bool ok = true;
                int prevs[2] = {BU::AVAIL, BU::AVAIL};
                const int kids[2] = {l, r};
                int have = 0;
                for (int q = 0; q < 2 && ok; ++q) {
                    const int x = kids[q];
                    if (x > batchNum) continue;
                    unsigned long long t0 = 0;
                    int prev;
                    for (unsigned it = 0; (prev = detail::max_acquire(status + x, BU::INUSE)) == BU::INUSE; ++it) {
                        if (!keep_waiting(t0, it, kSiteLockChild, x, prev)) { ok = false; break; }
                    }
                    if (ok) { have |= 1 << q; prevs[q] = prev == BU::INSHOLD ? BU::DELMOD : prev; }
                }
                c->abort = !ok;
                c->w0 = have;
                c->w1 = prevs[0];
                c->w2 = prevs[1];
                if (ok && have) {
                    op.expect((have == 3 ? 2u : 1u) * nodeBytes());
                    if (have & 1) detail::bulk_g2s(s1, node(l), nodeBytes(), &c->bar);
                    if (have & 2) detail::bulk_g2s(s2, node(r), nodeBytes(), &c->bar);
                }
            }
            __syncthreads();
            if (c->abort) return;
            const int have = c->w0, lPrev = c->w1, rPrev = c->w2;
            if (have == 0) {  // no child inside the allocation
                store_node(cur, s0);
                __syncthreads();
                if (tid == 0) unlock(cur, curPrev);
                return;
            }
            if (!op.wait()) return;
            if (have == 1) {  // only the left child lies inside the allocation
                detail::merge_split<K, IPT>(s0, s1, node(cur), node(l), B);
                __syncthreads();
                if (tid == 0) { unlock(cur, curPrev); unlock(l, lPrev); }
                return;
            }
            const int larger = s1[B - 1] < s2[B - 1] ? r : l;
            const int largerPrev = larger == r ? rPrev : lPrev;
            const int smaller = larger == r ? l : r;
            const int smallerPrev = larger == r ? lPrev : rPrev;
            detail::merge_split<K, IPT>(s1, s2, s1, node(larger), B);
            __syncthreads();
            if (tid == 0) unlock(larger, largerPrev);
            if (s0[0] >= s1[B - 1]) {
                store_node(cur, s1);
            } else if (s0[B - 1] < s1[0]) {
                store_node(cur, s0);
                store_node(smaller, s1);
                __syncthreads();
                if (tid == 0) { unlock(cur, curPrev); unlock(smaller, smallerPrev); }
                return;
            } else {
                detail::merge_split<K, IPT>(s0, s1, node(cur), s0, B);
            }
            __syncthreads();
            if (tid == 0) unlock(cur, curPrev);
            cur = smaller;
            curPrev = smallerPrev;
        }
    }

    // ------------------------------------------------------------------ counters
    // heap/tditdd/heap.cuh:210-215.  Call from ONE thread.
    __device__ __forceinline__ int getItemCount() const {
        if (!lock(0, 0, lockedState(), kSiteLockPartial)) return -1;
        const int n = detail::ld_relaxed(&state->partialBufferSize) + detail::ld_relaxed(&state->batchCount) * batchSize;
        unlock(0, 0);
        return n;
    }

    // Block-uniform: true once this heap has recorded an error.
    __device__ __forceinline__ bool failed() const {
        __shared__ int f;
        __syncthreads();
        if (threadIdx.x == 0) f = detail::ld_relaxed(&state->err) != 0;
        __syncthreads();
        const bool r = f != 0;
        __syncthreads();
        return r;
    }
};

// IPT = 2 * batchSize / blockDim.x fixed at compile time (0: chosen at run
// time, which costs registers).
template <typename K, int IPT = 0> using HeapTD = Heap<K, kTopDown, true, IPT>;
template <typename K, int IPT = 0> using HeapBU = Heap<K, kBottomUp, true, IPT>;
template <typename K, int IPT = 0> using HeapTDNoPartial = Heap<K, kTopDown, false, IPT>;
template <typename K, int IPT = 0> using HeapBUNoPartial = Heap<K, kBottomUp, false, IPT>;

}  // namespace gh
