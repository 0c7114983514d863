// gpuheap_device.cuh -- device-side API of the GB300 batched priority queue.
//
// A drop-in for the reference's device member functions of Heap<K>
// (heap/{tditdd,tditdd_np,buitdd,buitdd_np}/heap.cuh): an application kernel
// receives a gh::Heap<K, Variant, PartialBuffer> by value (or pointer) and
// every thread of a block calls
//     heap.insertion(items, size, smemOffset)   (heap/tditdd/heap.cuh:536)
//     heap.deleteRoot(items, size)              (heap/tditdd/heap.cuh:267)
//     heap.deleteRoot(items, size, threshold)   (artifacts/astar/BGPQ_B/heap.cuh:260)
//     heap.deleteUpdate(smemOffset)             (heap/tditdd/heap.cuh:345)
//     heap.retrieve(ret, size, scratch, smemOffset)
//                                               (applications/sssp_longfei_new/heap.cuh:79)
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
//     node data with plain stores); a bulk copy reads a node only after the
//     lock acquire that follows its writer's fence.acq_rel.gpu + release;
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
// A bottom-up insert parks its node with INSHOLD tagged by a ticket unique
// among concurrent inserts (kParkBase + ticket), so that on taking the node
// back it can tell whether anyone else held it meanwhile.  INUSE stays the
// largest value, so the deleters' atomicMax takes every other state.
struct BU {
    static constexpr int AVAIL = 0, INSHOLD = 1, DELMOD = 2, INUSE = 1 << 30;
    static constexpr int kParkBase = 4, kTicketMask = (1 << 29) - 1;
    __host__ __device__ static constexpr bool parked(int v) { return v == INSHOLD || (v >= kParkBase && v < INUSE); }
};

enum DeviceError : int { kErrNone = 0, kErrInvalid = 1, kErrCapacity = 2, kErrTimeout = 3 };

// Where a device error was raised (HeapState::errOp).
enum ErrSite : int {
    kSiteLockPartial = 1, kSiteLockRoot = 2, kSiteLockTarget = 3, kSiteLockPath = 4,
    kSiteLockLast = 5, kSiteLockChild = 6, kSiteHandOff = 7, kSiteBulkCopy = 8, kSiteCapacity = 9
};

// Heap counters, the sticky error record and application words, one
// 128-byte line each.
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
    int busy;               // applications: blocks between taking a batch and finishing its inserts
    int insTicket;          // bottom-up inserts: next park ticket (atomicAdd)
    int resvBase;           // bulk insert: targets resvBase+1 .. resvBase+resvCount are reserved
    int resvCount;          // 0: no reservation (the bulk insert takes node 0 per batch)
    int resvTurn;           // top-down reserved inserts take the root in target order: the next target
    int delTicket;          // bulk deletes: next ticket for node 0 (atomicAdd)
    int delServing;         // bulk deletes: the ticket whose holder may lock node 0 now
    int pad2[9];
    unsigned long long appStats[8];  // applications: counters (e.g. pops, expansions, relaxations)
};

// Per-operation control block at the end of the heap's shared-memory region:
// the mbarrier of the bulk copies and words that thread 0 (or the lock
// warps) broadcast to the block.
struct OpCtl {
    unsigned long long bar;  // mbarrier for the bulk copies
    int abort;               // block-uniform "stop" flag
    int bc, ps, dc;          // counters read under the partial-buffer lock
    int w[26];               // broadcast words
};
static_assert(sizeof(OpCtl) == 128, "OpCtl layout");

// A carried batch whose bulk load is still in flight on an mbarrier of its
// own (the owner-mode delete's workers start it before the sift's first
// level): `phase` is thread 0's parity of `bar`; once the batch is in,
// `cons` (global, if not null) is set to `consVal` with a release store.
struct CarriedInFlight {
    unsigned long long* bar;
    unsigned* phase;
    int* cons;
    int consVal;
};

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
__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
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
// Orders the block's earlier generic-proxy shared-memory accesses (after a
// barrier) before a later bulk copy (async proxy) writes the same buffers.
// Global node data needs no proxy fence here: every node a bulk copy reads
// was published by a fence.acq_rel.gpu + lock release, completing those
// writes at GPU scope (in L2, where the copy engine reads) before the lock
// word the reader acquired changed.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

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

// Bulk prefetch of `bytes` (multiple of 16, 16-byte aligned) into L2; a
// hint with no ordering or completion to track.
__device__ __forceinline__ void prefetch_l2(const void* src, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
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

// Shared-memory load through a 32-bit shared-window address.
template <typename K>
__device__ __forceinline__ K lds(unsigned addr) {
    if constexpr (sizeof(K) == 4) {
        unsigned v;
        asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(addr));
        return static_cast<K>(v);
    } else {
        unsigned long long v;
        asm volatile("ld.shared.b64 %0, [%1];" : "=l"(v) : "r"(addr));
        return static_cast<K>(v);
    }
}

// Merge-path split of two sorted runs a[0,n) and b[0,n) held in shared
// memory: the n smallest keys go to lo[0,n), the n largest to hi[0,n) (either
// may be null to discard; either may be shared or global).  Thread `tid` of
// the participating group produces outputs [tid*IPT, (tid+1)*IPT): a binary
// search on its diagonal finds the split (a wins ties, as
// heap/heaputil.cuh:99-158 does), IPT sequential steps fill registers, a
// barrier lets lo/hi alias a/b, and the run is stored with vector stores.
// Every thread of the block must call it (the barrier is block-wide); threads
// with tid*IPT >= 2n only take part in the barrier.  No trailing barrier.
template <typename K, int IPT>
__device__ __forceinline__ void merge_split_t(const K* a, const K* b, K* lo, K* hi, int n, int tid) {
    const int d = tid * IPT;
    const bool active = d < 2 * n;
    const unsigned sa = smem_u32(a), sb = smem_u32(b);
    constexpr unsigned S = sizeof(K);
    K r[IPT];
    if (active) {
        int i0 = d > n ? d - n : 0, i1 = d < n ? d : n;
        while (i0 < i1) {
            const int m = (i0 + i1) >> 1;
            const K x = lds<K>(sa + S * m), y = lds<K>(sb + S * (d - 1 - m));
            const bool p = x <= y;
            i0 = p ? m + 1 : i0;
            i1 = p ? i1 : m;
        }
        int i = i0, j = d - i0;
        K av = lds<K>(sa + S * (i < n ? i : n - 1)), bv = lds<K>(sb + S * (j < n ? j : n - 1));
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            const bool ta = (j >= n) || (i < n && av <= bv);
            r[k] = ta ? av : bv;
            if (ta) { ++i; av = lds<K>(sa + S * (i < n ? i : n - 1)); }
            else { ++j; bv = lds<K>(sb + S * (j < n ? j : n - 1)); }
        }
    }
    __syncthreads();
    if (active) {
        K* dst = d < n ? (lo ? lo + d : nullptr) : (hi ? hi + (d - n) : nullptr);
        if (dst) store_run<K, IPT>(dst, r);
    }
}

// Run-time IPT (= 2n*groups/blockDim) dispatch for callers without a fixed one.
template <typename K>
__device__ __forceinline__ void merge_split_rt(const K* a, const K* b, K* lo, K* hi, int n, int tid, int ipt) {
    switch (ipt) {
        case 1: merge_split_t<K, 1>(a, b, lo, hi, n, tid); break;
        case 2: merge_split_t<K, 2>(a, b, lo, hi, n, tid); break;
        case 4: merge_split_t<K, 4>(a, b, lo, hi, n, tid); break;
        case 8: merge_split_t<K, 8>(a, b, lo, hi, n, tid); break;
        default: merge_split_t<K, 16>(a, b, lo, hi, n, tid); break;
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

    // Four node buffers in shared memory: the carried batch (or insert
    // batch), the partial buffer (or loaded node) and the two children.
    static constexpr int kBufs = 4;
    static constexpr bool kHasPartialBuffer = PB;
    static constexpr int kVariant = VARIANT;
    static __host__ __device__ size_t smemBytes(int bs) {
        return kBufs * static_cast<size_t>(bs) * sizeof(K) + sizeof(OpCtl) + 16;
    }

    // Kid ownership after an acquire attempt.
    static constexpr int kAbsent = 0, kHeld = 1, kPending = 2;

    // ------------------------------------------------------------------ plumbing
    __device__ __forceinline__ K* region(int smemOffset) const {
        extern __shared__ __align__(16) unsigned char gh_dyn_smem[];
        size_t off = (static_cast<size_t>(smemOffset) * 4 + 15) & ~static_cast<size_t>(15);
        return reinterpret_cast<K*>(gh_dyn_smem + off);
    }
    __device__ __forceinline__ OpCtl* ctl(K* base) const { return reinterpret_cast<OpCtl*>(base + kBufs * batchSize); }
    __device__ __forceinline__ K* node(int i) const { return heapItems + static_cast<size_t>(i) * batchSize; }
    __device__ __forceinline__ unsigned nodeBytes() const { return static_cast<unsigned>(batchSize * sizeof(K)); }
    __device__ __forceinline__ static constexpr int lockedState() { return VARIANT == kTopDown ? TD::INUSE : BU::INUSE; }
    // Thread that runs the q-th of up to three concurrent lock waits: one per
    // warp when the block has three warps, else thread 0 for all.
    __device__ __forceinline__ int lockThread(int q) const { return blockDim.x >= 96 ? 32 * q : 0; }

    // Merge of two sorted batches; G = 2 splits the block into two groups
    // that merge two independent pairs at once.
    template <int G>
    __device__ __forceinline__ void mergeG(const K* a, const K* b, K* lo, K* hi, int tid) const {
        if constexpr (IPT > 0) detail::merge_split_t<K, IPT * G>(a, b, lo, hi, batchSize, tid);
        else detail::merge_split_rt<K>(a, b, lo, hi, batchSize, tid, (2 * batchSize * G) / static_cast<int>(blockDim.x));
    }
    __device__ __forceinline__ void merge(const K* a, const K* b, K* lo, K* hi) const {
        mergeG<1>(a, b, lo, hi, static_cast<int>(threadIdx.x));
    }

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
    __device__ __forceinline__ bool keep_waiting(unsigned long long& t0, unsigned it, int site, int nodeIdx,
                                                 int seen) const {
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

    // Swap status[i] from `from` to `to` (acquire); CAS first, then poll
    // until the word looks free and retry.
    __device__ __forceinline__ bool lock(int i, int from, int to, int site) const {
        int* w = status + i;
        unsigned long long t0 = 0;
        unsigned it = 0;
        for (;;) {
            int v = detail::cas_acquire(w, from, to);
            if (v == from) return true;
            do {
                if (!keep_waiting(t0, it++, site, i, v)) return false;
                v = detail::ld_relaxed(w);
            } while (v != from);
        }
    }
    // Owner-side transition out of an exclusive state (release).
    __device__ __forceinline__ void unlock(int i, int to) const { detail::st_release(status + i, to); }
    // After fence(): plain transitions, ordered by that fence.
    __device__ __forceinline__ static void fence() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
    __device__ __forceinline__ void setState(int i, int to) const { detail::st_relaxed(status + i, to); }

    // One attempt at a child: held (prev = state to restore), pending (held by
    // someone else) or absent (outside the allocation, or an insert target).
    __device__ __forceinline__ int tryChild(int x, int& prev) const {
        prev = 0;
        if (x > batchNum) return kAbsent;
        if constexpr (VARIANT == kTopDown) {
            const int v = detail::cas_acquire(status + x, TD::AVAIL, TD::INUSE);
            if (v == TD::AVAIL) return kHeld;
            return v == TD::INUSE ? kPending : kAbsent;
        } else {
            // heap/buitdd/heap.cuh:409-418: atomicMax takes AVAIL, INSHOLD or
            // DELMOD; a node a bubbling insert holds (INSHOLD) goes back as DELMOD.
            const int v = detail::max_acquire(status + x, BU::INUSE);
            if (v == BU::INUSE) return kPending;
            prev = BU::parked(v) ? BU::DELMOD : v;
            return kHeld;
        }
    }
    // Blocking version: held or absent, or -1 on timeout.
    __device__ __forceinline__ int takeChild(int x, int& prev) const {
        unsigned long long t0 = 0;
        for (unsigned it = 0;; ++it) {
            const int r = tryChild(x, prev);
            if (r != kPending) return r;
            if (!keep_waiting(t0, it, kSiteLockChild, x, lockedState())) return -1;
            if constexpr (VARIANT == kTopDown) {
                // poll before the next CAS
                while (detail::ld_relaxed(status + x) == TD::INUSE) {
                    if (!keep_waiting(t0, ++it, kSiteLockChild, x, TD::INUSE)) return -1;
                }
            }
        }
    }

    // Block-wide bulk-copy bookkeeping on one mbarrier; only thread 0 issues
    // and waits, the others meet it at a barrier.
    struct Op {
        const Heap* h;
        OpCtl* c;
        unsigned phase;
        bool inflight;
        __device__ __forceinline__ Op(const Heap* hp, OpCtl* cp) : h(hp), c(cp), phase(0), inflight(false) {
            __syncthreads();
            if (threadIdx.x == 0) {
                c->abort = 0;
                detail::mbar_init(&c->bar, 1);
            }
            __syncthreads();
        }
        __device__ __forceinline__ ~Op() {
            if (threadIdx.x == 0 && inflight) drain();
            __syncthreads();
            if (threadIdx.x == 0) detail::mbar_inval(&c->bar);
        }
        // Thread 0: start one transaction of `bytes` (copies follow).
        __device__ __forceinline__ void issue(unsigned bytes) {
            detail::fence_proxy_async_smem();
            detail::mbar_arrive_expect_tx(&c->bar, bytes);
            inflight = true;
        }
        // Thread 0: wait for the transaction in flight (bounded).
        __device__ __forceinline__ bool wait0() {
            if (!inflight) return true;
            unsigned long long t0 = 0;
            for (unsigned it = 0; !detail::mbar_try_wait(&c->bar, phase); ++it) {
                if (!h->keep_waiting(t0, it, kSiteBulkCopy, -1, 0)) {
                    drain();
                    return false;
                }
            }
            phase ^= 1u;
            inflight = false;
            return true;
        }
        // The copies read valid global memory and land in this block's shared
        // memory: give them a second bounded wait before it is reused.
        __device__ __forceinline__ void drain() {
            for (unsigned it = 0; it < (1u << 22) && !detail::mbar_try_wait(&c->bar, phase); ++it) {}
            phase ^= 1u;
            inflight = false;
        }
        // Block-wide wait; false (block-uniform) on failure.
        __device__ __forceinline__ bool wait() {
            if (threadIdx.x == 0 && !wait0()) c->abort = 1;
            __syncthreads();
            return !c->abort;
        }
    };

    __device__ __forceinline__ void load(K* dst, int i, unsigned long long* bar) const {
        detail::bulk_g2s(dst, node(i), nodeBytes(), bar);
    }

    // Block-wide copies between shared and global nodes (16-byte aligned).
    __device__ __forceinline__ void store_node(int i, const K* s) const {
        const int nv = batchSize * static_cast<int>(sizeof(K)) / 16;
        uint4* g = reinterpret_cast<uint4*>(node(i));
        const uint4* v = reinterpret_cast<const uint4*>(s);
        for (int q = threadIdx.x; q < nv; q += blockDim.x) g[q] = v[q];
    }
    __device__ __forceinline__ void fill_node(int i, int count) const {
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

    // Node layout.  Bottom-up heaps store level-order nodes with the bits
    // below the leading one reversed (heap/buitdd/heap.cuh:233-236).
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
    __device__ __forceinline__ int rightOrNone(int l) const { return l <= batchNum ? rightOf(l) : batchNum + 1; }

    // ------------------------------------------------------------------ insertion
    // heap/tditdd/heap.cuh:536-753 (top-down) and heap/buitdd/heap.cuh:484-690
    // (bottom-up); without the partial buffer: the _np copies.
    __device__ __forceinline__ void insertion(const K* items, int size, int smemOffset) const {
        K* s0 = region(smemOffset);
        K* s1 = s0 + batchSize;
        K* s2 = s1 + batchSize;
        Op op(this, ctl(s0));
        OpCtl* c = op.c;
        const int B = batchSize;
        const int tid = threadIdx.x;
        // bottom-up park ticket: drawn now, its latency hidden by the sort
        int parkTag = 0;
        if constexpr (VARIANT == kBottomUp) {
            if (tid == 0) parkTag = BU::kParkBase + (atomicAdd(&state->insTicket, 1) & BU::kTicketMask);
        }

        // stage and pad with init_limits, then sort (:557-562)
        for (int q = tid; q < B; q += blockDim.x) s0[q] = q < size ? items[q] : init_limits;
        __syncthreads();
        detail::bitonic_sort(s0, B);

        // lock the partial buffer (the counters are only changed under it) and
        // start loading it
        if (tid == 0) {
            const bool ok = lock(0, 0, lockedState(), kSiteLockPartial);
            c->abort = !ok;
            if (ok) {
                c->bc = detail::ld_relaxed(&state->batchCount);
                c->ps = detail::ld_relaxed(&state->partialBufferSize);
                // a full batch meeting an empty partial buffer merges with
                // padding only: that merge (case 2.2) changes nothing, skip it
                if (PB && !(c->ps == 0 && size == batchSize)) { op.issue(nodeBytes()); load(s1, 0, &c->bar); }
            }
        }
        __syncthreads();
        if (c->abort) return;
        const int bc = c->bc, ps = c->ps;

        if constexpr (PB) if (!(ps == 0 && size == B)) {
            if (!op.wait()) return;
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
                if (size + ps < B) {  // case 1.2 (:586-598)
                    merge(s0, s1, node(0), static_cast<K*>(nullptr));
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
                merge(s0, s1, node(1), node(0));
                __syncthreads();
                if (tid == 0) {
                    detail::st_relaxed(&state->partialBufferSize, ps + size - B);
                    fence();
                    setState(0, 0);
                    setState(1, 0);
                }
                return;
            }
            if (size + ps < B) {  // case 2.1 (:625-648): no new full batch, merge through the root
                merge(s0, s1, s0, static_cast<K*>(nullptr));
                __syncthreads();
                if (tid == 0) {
                    const bool ok = lock(1, 0, lockedState(), kSiteLockRoot);
                    c->abort = !ok;
                    if (ok) { op.issue(nodeBytes()); load(s1, 1, &c->bar); }
                }
                __syncthreads();
                if (c->abort) return;
                if (!op.wait()) return;
                merge(s0, s1, node(1), node(0));
                __syncthreads();
                if (tid == 0) {
                    detail::st_relaxed(&state->partialBufferSize, ps + size);
                    fence();
                    setState(0, 0);
                    setState(1, 0);
                }
                return;
            }
            // case 2.2 (:650-662): the smaller B keys go on, the rest stay in node 0
            merge(s0, s1, s0, node(0));
            __syncthreads();
            if (tid == 0) detail::st_relaxed(&state->partialBufferSize, ps + size - B);
        }

        if constexpr (VARIANT == kTopDown) insert_topdown(op, s0, s1, s2, bc);
        else insert_bottomup(op, s0, s1, s2, bc, parkTag);
    }

    // Insertion of one full batch into `target`, a node that a bulk driver
    // reserved before any of its inserts began: batchCount already counts
    // it and its lock word already holds the state the insert would have
    // claimed (TARGET top-down, INUSE bottom-up).  With the partial buffer
    // empty and the batch full, the reference's insertion changes node 0
    // not at all (case 2.2 with ps = 0 merges against padding) and holds it
    // only to draw the target, so this form takes no node-0 lock: the
    // bulk inserts pass the top of the heap without a serial hand-off.
    // Every other step is insertion()'s.  Callers: the bulk insert driver
    // only, with no deleter on the heap during its launch.
    __device__ __forceinline__ void insertionReserved(const K* items, int target, int smemOffset) const {
        K* s0 = region(smemOffset);
        K* s1 = s0 + batchSize;
        K* s2 = s1 + batchSize;
        Op op(this, ctl(s0));
        const int B = batchSize;
        const int tid = threadIdx.x;
        int parkTag = 0;
        if constexpr (VARIANT == kBottomUp) {
            if (tid == 0) parkTag = BU::kParkBase + (atomicAdd(&state->insTicket, 1) & BU::kTicketMask);
        }
        for (int q = tid; q < B; q += blockDim.x) s0[q] = items[q];
        __syncthreads();
        detail::bitonic_sort(s0, B);
        if constexpr (VARIANT == kTopDown) insert_topdown(op, s0, s1, s2, target - 1, true);
        else insert_bottomup(op, s0, s1, s2, target - 1, parkTag, true);
    }

    // Top-down path (heap/tditdd/heap.cuh:666-752).  Entered holding node 0;
    // the carried batch is in s0.  Each node on the root -> target path is
    // held while its merge runs; the next node is locked and its load started
    // before this one is released (locking it before the merge measured
    // slower: it lengthens the hold).
    // `reserved`: the target (bc + 1) was reserved by a bulk driver
    // (insertionReserved): no capacity check, counter update, target claim
    // or node-0 release here.
    __device__ __forceinline__ void insert_topdown(Op& op, K* s0, K* s1, K* s2, int bc, bool reserved = false) const {
        OpCtl* c = op.c;
        const int tid = threadIdx.x;
        if (tid == 0) {
            const int target = bc + 1;
            bool ok = true;
            if (!reserved) {
                ok = target <= batchNum;
                if (!ok) raise(kErrCapacity, kSiteCapacity, target, 0);
                if (ok) detail::st_relaxed(&state->batchCount, target);
                ok = ok && lock(target, TD::AVAIL, TD::TARGET, kSiteLockTarget);
            }
            if (ok && reserved) ok = waitTurn(target);
            if (ok && target != 1) {
                ok = lock(1, TD::AVAIL, TD::INUSE, kSiteLockRoot);
                if (ok) { op.issue(nodeBytes()); load(s1, 1, &c->bar); }
            }
            // reserved inserts enter the root in target order, as the
            // reference's do by claiming targets under the node-0 lock: a
            // later target's walk waits at an earlier one's (an ancestor's)
            // TARGET word, so the earlier insert must never queue behind it
            if (ok && reserved) detail::st_release(&state->resvTurn, target + 1);
            // the root is ours: release the partial buffer (the reference does
            // this at the top of the first path step, :692-694)
            if (ok && !reserved) unlock(0, TD::AVAIL);
            c->abort = !ok;
            c->w[0] = target;
        }
        __syncthreads();
        if (c->abort) return;
        const int target = c->w[0];
        int cur = 1;
        K* cn = s1;  // current node's keys
        K* nx = s2;  // next node's keys
        while (cur != target) {
            const int next = nextOnPath(cur, target);
            if (tid == 0) {
                // (:683-689) a deleter that took the target waits for this batch at the root
                c->w[1] = detail::ld_relaxed(status + target) == TD::MARKED;
                if (!c->w[1] && !op.wait0()) c->abort = 1;
            }
            __syncthreads();
            if (c->abort) return;
            if (c->w[1]) break;
            merge(s0, cn, node(cur), s0);
            __syncthreads();
            if (tid == 0) {
                bool ok = true;
                if (next != target) {
                    ok = lock(next, TD::AVAIL, TD::INUSE, kSiteLockPath);
                    if (ok) { op.issue(nodeBytes()); load(nx, next, &c->bar); }
                }
                fence();
                setState(cur, TD::AVAIL);
                c->abort = !ok;
            }
            __syncthreads();
            if (c->abort) return;
            cur = next;
            K* t = cn; cn = nx; nx = t;
        }
        if (tid == 0) {
            const int old = detail::cas_acq_rel(status + target, TD::TARGET, TD::INUSE);
            c->w[3] = old == TD::MARKED;
        }
        __syncthreads();
        if (c->w[3] || (cur != target)) {
            // (:732-744) the deleter that marked the target holds the root and
            // waits for this batch there
            store_node(1, s0);
            __syncthreads();
            if (tid == 0) {
                fence();
                if (cur != target) setState(cur, TD::AVAIL);
                setState(target, TD::TARGET);  // MARKED -> TARGET
            }
            return;
        }
        store_node(target, s0);
        __syncthreads();
        if (tid == 0) unlock(target, TD::AVAIL);
    }

    // Bottom-up path (heap/buitdd/heap.cuh:616-689).  Entered holding node 0;
    // the carried batch is in s0.  The reference parks its node as INSHOLD
    // before waiting for the parent; here one attempt at the parent comes
    // first and the park only happens when that attempt fails.
    //
    // A parked node is taken back with atomicMax; finding its own ticket
    // (parkTag, drawn by thread 0 when the insertion began) there proves
    // nobody held it meanwhile, so the cached batch is still the node's
    // content.  Tickets repeat after 2^29 inserts, which take over 170 s
    // (every insert holds node 0 for at least one ~330 ns L2 atomic); a park
    // lasts at most two waits of at most 60 s, so no park outlives its ticket.  Anything else (a deleter sifted through it, or took it as the
    // last node, reset it, and a new insert claimed it and parked there) makes
    // the node's memory authoritative, as the reference always reads it
    // (:643-673), and the batch is reloaded.
    //
    // Early stop: a level whose parent already ends at or below the batch
    // changes nothing, and while no one else has held this insert's nodes no
    // level above it would change either, so the walk stops there.  Once a
    // deleter has been through a parked node it walks on to the root like the
    // reference: that deleter merged the insert's small keys into the parent
    // it wrote, which can leave them below the grandparent, and only this walk
    // repairs that.  Stopping early in that case left parent/grandparent
    // inversions behind when inserts and deletes ran concurrently.
    __device__ __forceinline__ void insert_bottomup(Op& op, K* s0, K* s1, K* s2, int bc, int parkTag,
                                                    bool reserved = false) const {
        OpCtl* c = op.c;
        const int tid = threadIdx.x;
        const int B = batchSize;
        if (tid == 0) {
            const int target = bc + 1;
            bool ok = true;
            if (!reserved) {
                ok = target <= batchNum;
                if (!ok) raise(kErrCapacity, kSiteCapacity, target, 0);
                if (ok) detail::st_relaxed(&state->batchCount, target);
                ok = ok && lock(target, BU::AVAIL, BU::INUSE, kSiteLockTarget);
                if (ok) unlock(0, BU::AVAIL);
            }
            c->abort = !ok;
            c->w[0] = target;
        }
        __syncthreads();
        if (c->abort) return;
        int cur = c->w[0];
        store_node(cur, s0);
        __syncthreads();
        K* carried = s0;
        K* spare = s2;
        if (tid == 0) c->w[2] = 0;  // 1 once someone else has held one of this insert's nodes
        while (cur != 1) {
            const int p = parentOf(cur);
            if (tid == 0) {
                bool ok = true;
                int reload = 0;
                if (detail::cas_acquire(status + p, BU::AVAIL, BU::INUSE) != BU::AVAIL) {
                    // park our node so a deleter can pass through it, then wait
                    fence();
                    setState(cur, parkTag);
                    ok = lock(p, BU::AVAIL, BU::INUSE, kSiteLockPath);
                    if (ok) {
                        unsigned long long t0 = 0;
                        int prev;
                        for (unsigned it = 0; (prev = detail::max_acquire(status + cur, BU::INUSE)) == BU::INUSE; ++it) {
                            if (!keep_waiting(t0, it, kSiteLockPath, cur, prev)) { ok = false; break; }
                        }
                        reload = ok && prev != parkTag;
                        if (reload) c->w[2] = 1;
                    }
                }
                if (ok) {
                    op.issue((reload ? 2u : 1u) * nodeBytes());
                    load(s1, p, &c->bar);
                    if (reload) load(carried, cur, &c->bar);
                }
                c->abort = !ok;
            }
            __syncthreads();
            if (c->abort) return;
            if (!op.wait()) return;
            int done = 0;
            if (s1[0] >= carried[B - 1]) {  // whole batch below the parent: swap (:647-661)
                store_node(p, carried);
                store_node(cur, s1);
            } else if (s1[B - 1] <= carried[0] && c->w[2] == 0) {
                done = 1;  // already ordered, nodes never taken by others: nothing changes here or above
            } else {
                merge(carried, s1, spare, node(cur));
                __syncthreads();
                store_node(p, spare);
                K* t = carried; carried = spare; spare = t;
            }
            __syncthreads();
            if (tid == 0) {
                fence();
                setState(cur, BU::AVAIL);
                if (done) setState(p, BU::AVAIL);
            }
            if (done) return;
            cur = p;
        }
        if (tid == 0) unlock(1, BU::AVAIL);  // (:685-688)
    }

    // Thread 0 of a bulk-delete block: draws a ticket and waits (bounded)
    // until it is served, so that the blocks of a bulk delete take node 0 in
    // the order they asked for it.  Unlike racing on node 0's lock word, no
    // block can lose to the others for a whole phase.  Returns the ticket
    // (passed on with delServing once node 0 is held), or -2 on a failed wait.
    __device__ __forceinline__ int takeTurn() const {
        const int t = atomicAdd(&state->delTicket, 1);
        unsigned long long t0 = 0;
        for (unsigned it = 0; detail::ld_acquire(&state->delServing) != t; ++it)
            if (!keep_waiting(t0, it, kSiteLockPartial, 0, t)) return -2;
        return t;
    }

    // Thread 0: waits (bounded) until the reserved-insert turn reaches `target`.
    __device__ __forceinline__ bool waitTurn(int target) const {
        unsigned long long t0 = 0;
        for (unsigned it = 0; detail::ld_acquire(&state->resvTurn) != target; ++it)
            if (!keep_waiting(t0, it, kSiteLockRoot, 1, detail::ld_relaxed(&state->resvTurn))) return false;
        return true;
    }

    // ------------------------------------------------------------------ deleteRoot
    // heap/tditdd/heap.cuh:267-341, heap/buitdd/heap.cuh:283-343.  Returns
    // true when deleteUpdate must follow (the root is taken and nodes 0 and 1
    // stay locked); `size` is the number of keys written.  Like the
    // reference it takes no shared-memory offset: its few broadcast words
    // live in a static __shared__ block, so the caller's dynamic shared
    // memory is untouched.
    __device__ __forceinline__ bool deleteRoot(K* items, int& size) const {
        return deleteRootImpl(items, size, init_limits, false);
    }

    // deleteRoot(items, size, app_t_val) (artifacts/astar/BGPQ_B/heap.cuh:
    // 260-289): takes nothing (size 0) when the smallest key -- the root's
    // first, or the partial buffer's when no full node is left -- is not
    // below `threshold`: what is left can be pruned.  The key is read under
    // the locks that the delete takes anyway.
    __device__ __forceinline__ bool deleteRoot(K* items, int& size, K threshold) const {
        return deleteRootImpl(items, size, threshold, true);
    }

    // `check` false: no threshold at all (heap/tditdd/heap.cuh:267), so a heap
    // without the partial buffer also gives up its padding batches.
    // `fair`: the caller is one of many blocks of a bulk delete; it queues for
    // node 0 by ticket (takeTurn) instead of racing on the lock word.
    __device__ __forceinline__ bool deleteRootImpl(K* items, int& size, K threshold, bool check,
                                                   bool fair = false) const {
        __shared__ OpCtl dr;
        OpCtl* c = &dr;
        size = 0;
        const int tid = threadIdx.x;
        const int L = lockedState();
        __syncthreads();
        if (tid == 0) {
            c->w[0] = 0;  // 0: nothing, 1: partial buffer only, 2: root
            const int turn = fair ? takeTurn() : -1;
            const bool ok = turn != -2 && detail::ld_relaxed(&state->err) == 0 && lock(0, 0, L, kSiteLockPartial);
            if (turn >= 0) detail::st_release(&state->delServing, turn + 1);
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
                    if (!check || __ldcg(node(0)) < threshold) c->w[0] = 1;
                    else unlock(0, 0);
                } else {
                    // deleteUpdate will take node bc (a leaf, usually not in
                    // L2): start pulling it in while this block waits for the root
                    if (bc > 1) detail::prefetch_l2(node(bc), nodeBytes());
                    const bool ok1 = lock(1, 0, L, kSiteLockRoot);
                    c->abort = !ok1;
                    if (ok1 && check && !(__ldcg(node(1)) < threshold)) {
                        unlock(1, 0);
                        unlock(0, 0);
                    } else if (ok1) {
                        c->w[0] = 2;
                        if (sortOutput) detail::st_relaxed(&state->deleteCount, dc + batchSize);
                    }
                }
            }
        }
        __syncthreads();
        const int mode = c->w[0];
        const bool stop = c->abort || mode == 0;
        const int dc = c->dc, ps = c->ps;
        __syncthreads();  // every thread has read dr before the next call rewrites it
        if (stop) return false;
        K* out = items + (sortOutput ? dc : 0);
        if (mode == 1) {
            partial_out(out, ps, dc);
            size = ps;
            return false;
        }
        copy_out(out, 1, batchSize);  // (:328-329)
        __syncthreads();
        size = batchSize;
        return true;
    }

    // The smallest key as last published (the root's first, or the partial
    // buffer's when no full node is left), read without locks: a hint while
    // other blocks work on the heap, exact when none does.
    __device__ __forceinline__ K minKeyHint(int batchCount) const { return __ldcg(node(batchCount > 0 ? 1 : 0)); }

    // Only the partial buffer holds keys (:297-315): output and reset it,
    // release node 0.
    __device__ __forceinline__ void partial_out(K* out, int ps, int dc) const {
        copy_out(out, 0, ps);
        __syncthreads();
        fill_node(0, ps);
        __syncthreads();
        if (threadIdx.x == 0) {
            if (sortOutput) detail::st_relaxed(&state->deleteCount, dc + ps);
            detail::st_relaxed(&state->partialBufferSize, 0);
            unlock(0, 0);
        }
    }

    // ------------------------------------------------------------------ deleteUpdate
    // Refills the root: heap/tditdd/heap.cuh:345-534, heap/buitdd/heap.cuh:348-482.
    __device__ __forceinline__ void deleteUpdate(int smemOffset) const {
        K* base = region(smemOffset);
        Op op(this, ctl(base));
        OpCtl* c = op.c;
        if (threadIdx.x == 0) {
            const int last = detail::ld_relaxed(&state->batchCount);
            c->ps = detail::ld_relaxed(&state->partialBufferSize);
            detail::st_relaxed(&state->batchCount, last - 1);
            c->w[0] = last;
        }
        __syncthreads();
        const int last = c->w[0];
        if (last == 1) {  // (:357-369) the root was the only full node
            if (threadIdx.x == 0) { unlock(1, 0); unlock(0, 0); }
            return;
        }
        refill_and_sift(op, base, last);
    }

    // ------------------------------------------------------------------ deleteMin
    // deleteRoot(items, size, threshold) followed by deleteUpdate(smemOffset)
    // when it returns true, with the same result, for kernels that hold the
    // shared-memory region anyway.  Bottom-up: once the root is held, thread 0
    // takes the last node and one bulk transaction brings root, last node and
    // partial buffer into shared memory; the root goes to the output from
    // there.  The split calls read the root from global memory first and only
    // then take and load the last node, so this shortens the time the root
    // is held -- the period of back-to-back deletes -- by about one global
    // round trip.  Top-down keeps the split calls: its last node may be an
    // insert target whose batch is handed over at the root.
    __device__ __forceinline__ void deleteMin(K* items, int& size, K threshold, int smemOffset) const {
        deleteMinImpl(items, size, threshold, true, smemOffset);
    }
    __device__ __forceinline__ void deleteMin(K* items, int& size, int smemOffset) const {
        deleteMinImpl(items, size, init_limits, false, smemOffset);
    }
    __device__ __forceinline__ void deleteMinImpl(K* items, int& size, K threshold, bool check, int smemOffset,
                                                  bool fair = false) const {
        if constexpr (VARIANT == kTopDown) {
            if (deleteRootImpl(items, size, threshold, check, fair)) deleteUpdate(smemOffset);
        } else {
            deleteMinBottomUp(items, size, threshold, check, smemOffset, fair);
        }
    }

    __device__ __forceinline__ void deleteMinBottomUp(K* items, int& size, K threshold, bool check,
                                                      int smemOffset, bool fair = false) const {
        K* base = region(smemOffset);
        Op op(this, ctl(base));
        OpCtl* c = op.c;
        const int B = batchSize;
        const int tid = threadIdx.x;
        K* C = base;
        K* P = base + B;
        K* R = base + 2 * B;  // the root; the sift's first child buffer after it is written out
        size = 0;
        if (tid == 0) {
            c->w[0] = 0;  // 0: nothing, 1: partial buffer only, 2: root
            const int turn = fair ? takeTurn() : -1;
            const bool ok =
                turn != -2 && detail::ld_relaxed(&state->err) == 0 && lock(0, 0, BU::INUSE, kSiteLockPartial);
            if (turn >= 0) detail::st_release(&state->delServing, turn + 1);
            c->abort = !ok;
            if (ok) {
                const int bc = detail::ld_relaxed(&state->batchCount);
                const int ps = detail::ld_relaxed(&state->partialBufferSize);
                const int dc = detail::ld_relaxed(&state->deleteCount);
                const int lim = detail::ld_relaxed(&state->outLimit);
                c->bc = bc; c->ps = ps; c->dc = dc;
                const int want = bc > 0 ? B : (PB ? ps : 0);
                if (want == 0 || (sortOutput && dc + want > lim)) {
                    unlock(0, 0);
                } else if (bc == 0) {
                    if (!check || __ldcg(node(0)) < threshold) c->w[0] = 1;
                    else unlock(0, 0);
                } else {
                    if (bc > 1) detail::prefetch_l2(node(bc), nodeBytes());
                    const bool ok1 = lock(1, 0, BU::INUSE, kSiteLockRoot);
                    c->abort = !ok1;
                    if (ok1 && check && !(__ldcg(node(1)) < threshold)) {
                        unlock(1, 0);
                        unlock(0, 0);
                    } else if (ok1) {
                        c->w[0] = 2;
                        if (sortOutput) detail::st_relaxed(&state->deleteCount, dc + B);
                        detail::st_relaxed(&state->batchCount, bc - 1);
                        // take the last node (heap/buitdd/heap.cuh:372-378): atomicMax
                        // takes it from AVAIL, INSHOLD or DELMOD
                        bool okl = true;
                        if (bc > 1) {
                            unsigned long long t0 = 0;
                            int prev;
                            for (unsigned it = 0; (prev = detail::max_acquire(status + bc, BU::INUSE)) == BU::INUSE; ++it) {
                                if (!keep_waiting(t0, it, kSiteLockLast, bc, prev)) { okl = false; break; }
                            }
                        }
                        c->abort = !okl;
                        if (okl) {
                            const bool pb = PB && ps != 0 && bc > 1;
                            op.issue((1u + (bc > 1 ? 1u : 0u) + (pb ? 1u : 0u)) * nodeBytes());
                            load(R, 1, &c->bar);
                            if (bc > 1) load(C, bc, &c->bar);
                            if (pb) load(P, 0, &c->bar);
                        }
                    }
                }
            }
        }
        __syncthreads();
        const int mode = c->w[0];
        const bool stop = c->abort || mode == 0;
        const int bc = c->bc, ps = c->ps, dc = c->dc;
        __syncthreads();  // every thread has read the control words before they change
        if (stop) return;
        K* out = items + (sortOutput ? dc : 0);
        if (mode == 1) {
            partial_out(out, ps, dc);
            size = ps;
            return;
        }
        if (!op.wait()) return;
        smem_out(out, R, B);  // (:328-329)
        size = B;
        if (bc == 1) {  // the root was the only full node (:357-369)
            __syncthreads();
            if (tid == 0) { unlock(1, 0); unlock(0, 0); }
            return;
        }
        fill_node(bc, B);  // reset the taken node (:396)
        const bool pb = PB && ps != 0;
        if (pb) merge(C, P, C, node(0));
        __syncthreads();
        if (tid == 0) {
            fence();
            setState(bc, 0);
            setState(0, 0);
        }
        sift_loop(op, 1, 0, C, base + 2 * B, base + 3 * B);
    }

    // ------------------------------------------------------------------ retrieve
    // retrieve(ret, *size) (applications/sssp_longfei_new/heap.cuh:79-270):
    // the `size` smallest keys -- at most one batch, fewer when the heap holds
    // fewer -- into ret[0, size), ascending; `size` returns the count.  Built
    // from this heap's own operations: a delete takes the root (the B
    // smallest keys) into `scratch`, the first `size` go to ret and the rest
    // are inserted back, where they join the partial buffer, so no padding
    // enters the heap.  `scratch` holds batchSize keys (global or shared,
    // 16-byte aligned) outside the heap's shared-memory region; ret may not
    // overlap it.  Outputs at scratch[0] need a view with sortOutput = 0.
    // Heaps with the partial buffer only (the reference's retrieving heap
    // has one).
    __device__ __forceinline__ void retrieve(K* ret, int& size, K* scratch, int smemOffset) const {
        static_assert(PB, "retrieve needs the partial buffer");
        const int want = size < 0 ? 0 : size;
        int got = 0;
        if (want > 0) deleteMin(scratch, got, smemOffset);
        const int take = got < want ? got : want;
        for (int i = threadIdx.x; i < take; i += blockDim.x) ret[i] = scratch[i];
        __syncthreads();
        if (got > take) insertion(scratch + take, got - take, smemOffset);
        size = take;
    }

    // Block-wide copy of `count` keys from shared memory to dst.
    __device__ __forceinline__ void smem_out(K* dst, const K* s, int count) const {
        const int per = 16 / static_cast<int>(sizeof(K));
        if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
            const int nv = count / per;
            for (int q = threadIdx.x; q < nv; q += blockDim.x)
                reinterpret_cast<uint4*>(dst)[q] = reinterpret_cast<const uint4*>(s)[q];
            for (int q = nv * per + threadIdx.x; q < count; q += blockDim.x) dst[q] = s[q];
        } else {
            for (int q = threadIdx.x; q < count; q += blockDim.x) dst[q] = s[q];
        }
    }

    // The children of the node at one level, after they are locked and loaded.
    struct Level {
        int have, l, r, lPrev, rPrev, larger, smaller, lp, sp;
    };

    __device__ __forceinline__ void order(Level& lv, const K* Xc, const K* Yc) const {
        lv.larger = lv.smaller = lv.lp = lv.sp = 0;
        if (lv.have != 3) return;
        // the larger last key, the left child on a tie (tditdd_np :416), except
        // when both end in init_limits: then the larger first key, so that a
        // padded node's real keys never sink into a node past the heap
        const K xl = Xc[batchSize - 1], yl = Yc[batchSize - 1];
        lv.larger = (xl < yl || (xl == yl && !(xl < init_limits) && Xc[0] < Yc[0])) ? lv.r : lv.l;
        lv.smaller = lv.larger == lv.r ? lv.l : lv.r;
        lv.lp = lv.larger == lv.r ? lv.rPrev : lv.lPrev;
        lv.sp = lv.larger == lv.r ? lv.lPrev : lv.rPrev;
    }

    // TD: take the last node; if it is an in-flight insert target, mark it
    // and wait for the insert to hand its batch over at the root
    // (heap/tditdd/heap.cuh:371-393).  Thread 0; c->w[7] = 1 when handed over.
    __device__ __forceinline__ bool takeLastTopDown(int last, OpCtl* c) const {
        unsigned long long t0 = 0;
        c->w[7] = 0;
        for (unsigned it = 0;; ++it) {
            if (detail::cas_acquire(status + last, TD::AVAIL, TD::INUSE) == TD::AVAIL) return true;
            if (detail::cas_acquire(status + last, TD::TARGET, TD::MARKED) == TD::TARGET) break;
            if (!keep_waiting(t0, it, kSiteLockLast, last, detail::ld_relaxed(status + last))) return false;
        }
        c->w[7] = 1;
        t0 = 0;
        for (unsigned it = 0; detail::cas_acquire(status + last, TD::TARGET, TD::AVAIL) != TD::TARGET; ++it) {
            if (!keep_waiting(t0, it, kSiteHandOff, last, detail::ld_relaxed(status + last))) return false;
        }
        return true;
    }

    // deleteUpdate body once the root is copied out and batchCount lowered:
    // take the last node (:355-402), merge it with the partial buffer
    // (:404-416), release node 0 and the last node, then sift down from the
    // root.  Locks are taken as late and dropped as early as the protocol
    // allows: with many blocks in the pipeline, lock hold time is what
    // bounds throughput (taking the root's children before the partial-buffer
    // merge, or the next level's children one level ahead, measured slower).
    __device__ __forceinline__ void refill_and_sift(Op& op, K* base, int last) const {
        OpCtl* c = op.c;
        const int tid = threadIdx.x;
        const int B = batchSize;
        K* C = base;
        K* P = base + B;
        // an empty partial buffer is all padding: merging with it (:404-416)
        // changes nothing, so it is neither loaded nor merged
        const bool pb = PB && c->ps != 0;
        if (tid == 0) {
            bool ok = true;
            c->w[7] = 0;
            if constexpr (VARIANT == kTopDown) {
                ok = takeLastTopDown(last, c);
            } else {
                // (:372-378) atomicMax takes the node from AVAIL, INSHOLD or DELMOD
                unsigned long long t0 = 0;
                int prev;
                for (unsigned it = 0; (prev = detail::max_acquire(status + last, BU::INUSE)) == BU::INUSE; ++it) {
                    if (!keep_waiting(t0, it, kSiteLockLast, last, prev)) { ok = false; break; }
                }
            }
            if (ok) {
                op.issue((pb ? 2u : 1u) * nodeBytes());
                load(C, c->w[7] ? 1 : last, &c->bar);
                if (pb) load(P, 0, &c->bar);
            }
            c->abort = !ok;
        }
        __syncthreads();
        if (c->abort) return;
        const int lastTaken = !c->w[7];
        if (!op.wait()) return;
        if (lastTaken) fill_node(last, B);  // reset the taken node (:396)
        if (pb) merge(C, P, C, node(0));
        __syncthreads();
        if (tid == 0) {
            fence();
            if (lastTaken) setState(last, 0);
            setState(0, 0);
        }
        sift_loop(op, 1, 0, C, base + 2 * B, base + 3 * B);
    }

    // Block-wide: waits (bounded) for a carried batch loaded on its own
    // barrier, then releases its source; false (block-uniform) on failure,
    // after a second bounded wait, so that no copy lands after a return.
    __device__ __forceinline__ bool carried_in(CarriedInFlight* cf, OpCtl* c) const {
        if (!cf) return true;
        if (threadIdx.x == 0) {
            unsigned long long t0 = 0;
            bool ok = true;
            for (unsigned it = 0; !detail::mbar_try_wait(cf->bar, *cf->phase); ++it) {
                if (!keep_waiting(t0, it, kSiteBulkCopy, -1, 1)) {
                    for (unsigned i2 = 0; i2 < (1u << 22) && !detail::mbar_try_wait(cf->bar, *cf->phase); ++i2) {}
                    ok = false;
                    break;
                }
            }
            *cf->phase ^= 1u;
            if (ok && cf->cons) detail::st_release(cf->cons, cf->consVal);
            if (!ok) c->abort = 1;
        }
        __syncthreads();
        return !c->abort;
    }

    // Sift down from `cur` (held; curPrev = the state it returns to) with the
    // carried batch in C (heap/tditdd/heap.cuh:418-532, heap/buitdd/heap.cuh:
    // 403-480).  Per level: the two lock warps take the children at once,
    // one bulk transaction loads them, the children merge writes the larger
    // half straight to the larger child, the case analysis against C writes
    // the current node, and one fence releases both (a second fence to free
    // the larger child before the case analysis measured slower).
    //
    // `cf` (optional): the carried batch is still in flight on a barrier of
    // its own; the first level takes and loads the children meanwhile, then
    // waits for both (and releases cf->cons once the carried batch is in).
    __device__ __forceinline__ void sift_loop(Op& op, int cur, int curPrev, K* C, K* Xc, K* Yc,
                                              CarriedInFlight* cf = nullptr) const {
        OpCtl* c = op.c;
        const int tid = threadIdx.x;
        const int B = batchSize;
        for (;;) {
            Level lv;
            lv.l = leftOf(cur);
            lv.r = rightOrNone(lv.l);
            if (tid == lockThread(0)) { int p; c->w[3] = takeChild(lv.l, p); c->w[4] = p; }
            if (tid == lockThread(1)) { int p; c->w[5] = takeChild(lv.r, p); c->w[6] = p; }
            __syncthreads();
            if (c->w[3] < 0 || c->w[5] < 0) {
                carried_in(cf, c);
                return;
            }
            lv.have = (c->w[3] == kHeld ? 1 : 0) | (c->w[5] == kHeld ? 2 : 0);
            lv.lPrev = c->w[4];
            lv.rPrev = c->w[6];
            if (tid == 0 && lv.have) {
                op.issue(((lv.have & 1) + (lv.have >> 1)) * nodeBytes());
                if (lv.have & 1) load(Xc, lv.l, &c->bar);
                if (lv.have & 2) load(Yc, lv.r, &c->bar);
            }
            if (!op.wait()) {
                carried_in(cf, c);
                return;
            }
            if (cf) {
                if (!carried_in(cf, c)) return;
                cf = nullptr;
            }
            order(lv, Xc, Yc);
            int done = 1, single = 0;
            if (lv.have == 3 && !(C[0] < (Xc[B - 1] < Yc[B - 1] ? Xc[B - 1] : Yc[B - 1]))) {
                // The carried batch starts at or above one child's last key, so
                // at or above the B-th smallest key of the two children: the
                // current node becomes the smaller half of the children and
                // the carried batch goes on unchanged (the first case below),
                // so the merge writes both halves straight to their nodes.
                merge(Xc, Yc, node(cur), node(lv.larger));
                done = 0;
            } else {
                if (lv.have == 3) {
                    merge(Xc, Yc, Xc, node(lv.larger));
                    __syncthreads();
                }
                // case analysis against the carried batch
                if (lv.have == 0) {  // no children (:452-460)
                    store_node(cur, C);
                } else if (lv.have != 3) {  // one child (:461-477)
                    single = lv.have == 1 ? lv.l : lv.r;
                    merge(C, lv.have == 1 ? Xc : Yc, node(cur), node(single));
                } else if (C[0] >= Xc[B - 1]) {
                    store_node(cur, Xc);  // the carried batch goes on unchanged
                    done = 0;
                } else if (VARIANT == kTopDown || !PB ? (C[B - 1] <= Xc[0]) : (C[B - 1] < Xc[0])) {  // buitdd alone uses < (:451)
                    store_node(cur, C);
                    store_node(lv.smaller, Xc);
                } else {
                    merge(C, Xc, node(cur), C);
                    done = 0;
                }
            }
            __syncthreads();
            if (tid == 0) {
                fence();
                if (single) setState(single, single == lv.l ? lv.lPrev : lv.rPrev);
                if (lv.have == 3) setState(lv.larger, lv.lp);
                setState(cur, curPrev);
                if (done && lv.have == 3) setState(lv.smaller, lv.sp);
            }
            if (done) return;
            cur = lv.smaller;
            curPrev = lv.sp;
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
