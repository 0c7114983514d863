// gpuheap_retrieve.cuh -- the retrieving heap: partial retrieval in place.
//
// The reference's SSSP application (applications/sssp_longfei_new/heap.cuh)
// drives a heap of its own: 0-based nodes (children of i at 2i+1, 2i+2), its
// partial buffer in a separate array, top-down inserts, and
//
//   retrieve(ret, *size)  the `size` smallest keys (at most one batch,
//                         fewer when fewer are held), ascending; the root is
//                         refilled in place, from the partial buffer or,
//                         when that holds fewer than `size` keys, from the
//                         last node, whose other keys become the partial
//                         buffer; then the root sifts down (:79-270);
//   insert(items, count)  count <= batch keys (:272-382).
//
// A retrieve that needs the last node while an insert is still on its way
// down to it takes that insert's batch through the root: the per-node word
// `taken` moves 0 -> 1 (the insert marks its target, under the root's lock)
// -> 2 (the retrieve, holding the root and the target) -> 3 (the insert,
// having written its batch into the root instead of the target) -> 0 (the
// retrieve).  The hand-over is model-checked in oracle/lock_model.py
// (retrieve_steal_model) and the sequential behaviour is pinned bit for bit
// to the reference's own runs (oracle/retrieve_heap.py).
//
// RetHeapAux adds the reference's auxiliary (key, value) buffer
// (heap_with_aux.cuh:48-119): a retrieve takes buffered entries first, and
// a caller-given check puts an entry back into the buffer with a new value
// (the SSSP application walks a vertex's edges in chunks this way).
//
// Device code for one thread block per operation.  Lock words and `taken`
// are moved by thread 0 with acquire/release atomics; every wait has the
// time limit `timeoutNs` and records kErrTimeout in the state instead of
// hanging.  Node and partial-buffer data are read through L2 (ld.cg), so a
// block never sees stale L1 lines of a node another block wrote.  Keys are
// staged in three shared-memory buffers of one batch each; the merges and
// the sort are the BGPQ heap's (gpuheap_device.cuh: merge path with ties to
// the first run, bitonic sort), so results equal the reference's.
#pragma once
#include "gpuheap_device.cuh"

namespace gh {

// Counters in gh::HeapState: batchCount, partialBufferSize, the error
// record, busy (applications' termination), and these application counters.
enum RetStat : int { kRetSteals = 0, kRetFull = 1, kRetAuxFull = 2 };

template <typename K>
struct RetHeap {
    using key_type = K;
    K* items;          // batchNum * batchSize keys, node i at i * batchSize
    K* pbuf;           // batchSize keys: the partial buffer
    int* lock;         // batchNum lock words, 0 free, 1 held
    int* taken;        // batchNum words: 0, or 1..3 while an insert's target is handed over
    HeapState* state;  // batchCount, partialBufferSize, error record, busy, appStats
    int batchNum;
    int batchSize;     // a power of two in [16, 2048]; blocks of min(batchSize, 1024) threads
    K initLimit;       // above every real key
    long long timeoutNs;

    // Dynamic shared memory an operation needs at smemOffset (16-aligned).
    static __host__ __device__ size_t smemBytes(int B) { return 64 + 3 * static_cast<size_t>(B) * sizeof(K); }

    // Block-wide (every thread calls it): the heap recorded an error.
    __device__ bool failed() const {
        __shared__ int f;
        __syncthreads();
        if (threadIdx.x == 0) f = detail::ld_relaxed(&state->err) != 0;
        __syncthreads();
        const bool r = f != 0;
        __syncthreads();
        return r;
    }

    // --------------------------------------------------------------- pieces
  private:
    struct Smem {
        int* ctl;  // 16 words
        K* b1;
        K* b2;
        K* b3;
    };
    __device__ Smem smem_at(int smemOffset) const {
        extern __shared__ __align__(16) unsigned char gh_ret_smem[];
        unsigned char* base = gh_ret_smem + smemOffset;
        Smem s;
        s.ctl = reinterpret_cast<int*>(base);
        s.b1 = reinterpret_cast<K*>(base + 64);
        s.b2 = s.b1 + batchSize;
        s.b3 = s.b2 + batchSize;
        return s;
    }

    __device__ void raise(int code, int site, int node, int seen) const {
        if (atomicCAS(&state->err, 0, code) == 0) {
            state->errOp = site;
            state->errNode = node;
            state->errState = seen;
        }
    }

    // Block-wide: takes node i's lock (thread 0 spins with a time limit);
    // false, for every thread, when the wait ran out.
    __device__ bool lock_node(int i, int* ctl, int site) const {
        if (threadIdx.x == 0) {
            int ok = 1;
            const unsigned long long t0 = detail::globaltimer();
            while (detail::cas_acquire(lock + i, 0, 1) != 0) {
                if (detail::globaltimer() - t0 > static_cast<unsigned long long>(timeoutNs)) {
                    raise(kErrTimeout, site, i, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
            ctl[15] = ok;
        }
        __syncthreads();
        const bool ok = ctl[15] != 0;
        __syncthreads();
        return ok;
    }

    // Block-wide: every thread's writes, then node i's lock released.
    __device__ void unlock_node(int i) const {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            detail::st_release(lock + i, 0);
        }
    }

    __device__ void load(K* dst, const K* src, int n) const {
        for (int k = threadIdx.x; k < n; k += blockDim.x) dst[k] = __ldcg(src + k);
    }
    __device__ void store(K* dst, const K* src, int n) const {
        for (int k = threadIdx.x; k < n; k += blockDim.x) __stcg(dst + k, src[k]);
    }
    __device__ void fill(K* dst, int n) const {
        for (int k = threadIdx.x; k < n; k += blockDim.x) dst[k] = initLimit;
    }
    // a, b sorted in shared memory: the batchSize smallest to lo, the rest to
    // hi (shared or global, may alias a or b); ends with a barrier.  Blocks
    // of min(batchSize, 1024) threads: 2 keys a thread, 4 at batch 2048.
    __device__ void merge(const K* a, const K* b, K* lo, K* hi) const {
        if (2 * batchSize == 4 * static_cast<int>(blockDim.x))
            detail::merge_split_t<K, 4>(a, b, lo, hi, batchSize, threadIdx.x);
        else
            detail::merge_split_t<K, 2>(a, b, lo, hi, batchSize, threadIdx.x);
        __syncthreads();
    }
    __device__ K* node(int i) const { return items + static_cast<size_t>(i) * batchSize; }

    // The child of `cur` on the path to `target` (reference get_next_idx,
    // heap.cuh:50-54): target + 1 shifted right until it sits one level
    // below cur + 1.
    static __device__ int next_on_path(int cur, int target) {
        const int p = cur + 1, q = target + 1;
        return (q >> (__clz(p) - __clz(q) - 1)) - 1;
    }

  public:
    // ------------------------------------------------------------- insert
    // insert(items, count) (heap.cuh:272-382): 0 < count <= batchSize keys
    // (global or shared).  A full heap (batchCount >= batchNum - 1) takes
    // nothing and records kErrCapacity (the reference flags need_gc and
    // drops the keys).  Every thread of the block calls it.
    __device__ void insert(const K* keys, int count, int smemOffset) const {
        const Smem s = smem_at(smemOffset);
        const int B = batchSize;
        if (count <= 0) return;
        if (count > B) count = B;
        for (int k = threadIdx.x; k < count; k += blockDim.x) s.b1[k] = keys[k];
        if (!lock_node(0, s.ctl, kSiteLockRoot)) return;
        if (threadIdx.x == 0) {
            s.ctl[0] = detail::ld_relaxed(&state->batchCount);
            s.ctl[1] = detail::ld_relaxed(&state->partialBufferSize);
        }
        __syncthreads();
        const int bc = s.ctl[0], ps = s.ctl[1];
        __syncthreads();
        if (bc >= batchNum - 1) {
            if (threadIdx.x == 0) {
                raise(kErrCapacity, kSiteCapacity, bc, 0);
                atomicAdd(&state->appStats[kRetFull], 1ull);
            }
            unlock_node(0);
            return;
        }
        if (ps + count < B) {  // the partial buffer has room (:306-321)
            load(s.b1 + count, pbuf, ps);
            fill(s.b1 + count + ps, B - count - ps);
            __syncthreads();
            detail::bitonic_sort(s.b1, B);
            if (bc == 0) {
                store(pbuf, s.b1, B);
            } else {
                load(s.b2, node(0), B);
                __syncthreads();
                merge(s.b1, s.b2, node(0), pbuf);
            }
            if (threadIdx.x == 0) detail::st_relaxed(&state->partialBufferSize, ps + count);
            unlock_node(0);
            return;
        }
        // a full batch forms (:323-336)
        const int rem = B - count;
        const int rps = ps - rem;
        load(s.b1 + count, pbuf, rem);
        load(s.b2, pbuf + rem, rps);
        fill(s.b2 + rps, B - rps);
        __syncthreads();
        detail::bitonic_sort(s.b1, B);
        if (bc == 0) {  // straight into the root
            merge(s.b1, s.b2, node(0), pbuf);
            if (threadIdx.x == 0) {
                detail::st_relaxed(&state->partialBufferSize, rps);
                detail::st_relaxed(&state->batchCount, 1);
            }
            unlock_node(0);
            return;
        }
        // down the path from the root to the new last node (:338-380)
        store(pbuf, s.b2, B);
        const int target = bc;
        if (threadIdx.x == 0) {
            detail::st_relaxed(&state->partialBufferSize, rps);
            detail::st_relaxed(taken + target, 1);
            __threadfence();  // taken[target] before the count that makes target a node
            detail::st_release(&state->batchCount, bc + 1);
        }
        __syncthreads();
        int cur = 0;
        do {
            load(s.b2, node(cur), B);
            __syncthreads();
            merge(s.b1, s.b2, node(cur), s.b1);
            const int next = next_on_path(cur, target);
            if (!lock_node(next, s.ctl, next == target ? kSiteLockTarget : kSiteLockPath)) {
                unlock_node(cur);
                return;
            }
            unlock_node(cur);
            if (threadIdx.x == 0) s.ctl[2] = detail::ld_acquire(taken + target) == 2;
            __syncthreads();
            const bool abandon = s.ctl[2] != 0;
            __syncthreads();
            if (abandon) {
                // a retrieve holds the root and took the target: the batch
                // goes into the root, then 3 tells the retrieve it is there
                unlock_node(next);
                store(node(0), s.b1, B);
                __syncthreads();
                if (threadIdx.x == 0) {
                    __threadfence();
                    detail::st_release(taken + target, 3);
                }
                return;
            }
            cur = next;
        } while (cur != target);
        store(node(target), s.b1, B);
        __syncthreads();
        if (threadIdx.x == 0) detail::st_relaxed(taken + target, 0);
        unlock_node(target);
    }

    // ----------------------------------------------------------- retrieve
    // retrieve(ret, *size) (heap.cuh:79-270): writes the min(size, held,
    // batchSize) smallest keys to ret (global or shared), ascending, and
    // returns how many.  Every thread of the block calls it with the same
    // size.
    __device__ int retrieve(K* ret, int size, int smemOffset) const {
        const Smem s = smem_at(smemOffset);
        const int B = batchSize;
        int want = size < 0 ? 0 : (size > B ? B : size);
        if (!lock_node(0, s.ctl, kSiteLockRoot)) return 0;
        if (threadIdx.x == 0) {
            s.ctl[0] = detail::ld_relaxed(&state->batchCount);
            s.ctl[1] = detail::ld_relaxed(&state->partialBufferSize);
        }
        __syncthreads();
        const int bc = s.ctl[0], ps = s.ctl[1];
        __syncthreads();
        if (bc == 0) {  // from the partial buffer (:98-114)
            const int n = want < ps ? want : ps;
            for (int k = threadIdx.x; k < n; k += blockDim.x) ret[k] = __ldcg(pbuf + k);
            load(s.b1, pbuf + n, ps - n);
            __syncthreads();
            store(pbuf, s.b1, ps - n);
            if (threadIdx.x == 0) detail::st_relaxed(&state->partialBufferSize, ps - n);
            unlock_node(0);
            return n;
        }
        for (int k = threadIdx.x; k < want; k += blockDim.x) ret[k] = __ldcg(node(0) + k);
        const int rem = B - want;
        if (bc == 1) {  // only the root (:119-145)
            load(s.b1, node(0) + want, rem);
            if (ps >= want) {
                load(s.b1 + rem, pbuf, want);
                load(s.b2, pbuf + want, ps - want);
                __syncthreads();
                store(node(0), s.b1, B);
                store(pbuf, s.b2, ps - want);
                if (threadIdx.x == 0) detail::st_relaxed(&state->partialBufferSize, ps - want);
            } else {
                load(s.b1 + rem, pbuf, ps);
                __syncthreads();
                store(pbuf, s.b1, rem + ps);
                if (threadIdx.x == 0) {
                    detail::st_relaxed(&state->batchCount, 0);
                    detail::st_relaxed(&state->partialBufferSize, rem + ps);
                }
            }
            unlock_node(0);
            return want;
        }
        // refill the root from the partial buffer, then the last node (:147-199)
        load(s.b1, node(0) + want, rem);
        if (ps >= want) {
            load(s.b1 + rem, pbuf, want);
            load(s.b2, pbuf + want, ps - want);
            fill(s.b2 + (ps - want), B - (ps - want));
            __syncthreads();
            if (threadIdx.x == 0) detail::st_relaxed(&state->partialBufferSize, ps - want);
        } else {
            load(s.b1 + rem, pbuf, ps);
            const int gap = want - ps;
            const int last = bc - 1;
            if (!lock_node(last, s.ctl, kSiteLockLast)) {
                unlock_node(0);
                return 0;
            }
            if (threadIdx.x == 0) {
                // the count drops only with the last node locked: a block that
                // holds a node below the count finds it valid
                detail::st_relaxed(&state->batchCount, last);
                s.ctl[3] = detail::ld_acquire(taken + last);
            }
            __syncthreads();
            const int st = s.ctl[3];
            __syncthreads();
            const K* src = node(last);
            if (st == 0) {
                load(s.b1 + (B - gap), src, gap);
                load(s.b2, src + gap, B - gap);
                fill(s.b2 + (B - gap), gap);
                unlock_node(last);
            } else {
                // an insert is on its way down to `last` (taken 1): take its
                // batch through the root (model: retrieve_steal_model)
                if (threadIdx.x == 0) detail::st_release(taken + last, 2);
                unlock_node(last);
                if (threadIdx.x == 0) {
                    int ok = 1;
                    const unsigned long long t0 = detail::globaltimer();
                    while (detail::ld_acquire(taken + last) != 3) {
                        if (detail::globaltimer() - t0 > static_cast<unsigned long long>(timeoutNs)) {
                            raise(kErrTimeout, kSiteHandOff, last, detail::ld_relaxed(taken + last));
                            ok = 0;
                            break;
                        }
                        __nanosleep(64);
                    }
                    if (ok) {
                        detail::st_relaxed(taken + last, 0);
                        atomicAdd(&state->appStats[kRetSteals], 1ull);
                    }
                    s.ctl[4] = ok;
                }
                __syncthreads();
                const bool ok = s.ctl[4] != 0;
                __syncthreads();
                if (!ok) {
                    unlock_node(0);
                    return 0;
                }
                src = node(0);
                load(s.b1 + (B - gap), src, gap);
                load(s.b2, src + gap, B - gap);
                fill(s.b2 + (B - gap), gap);
            }
            __syncthreads();
            detail::bitonic_sort(s.b1, B);
            merge(s.b1, s.b2, s.b1, s.b2);
            if (threadIdx.x == 0) detail::st_relaxed(&state->partialBufferSize, B - gap);
        }
        store(pbuf, s.b2, B);
        // sift the new root down (:201-268); b1 holds it
        int cur = 0;
        for (;;) {
            const int l = 2 * cur + 1, r = l + 1;
            if (threadIdx.x == 0) s.ctl[5] = 0;
            if (l < batchNum) {
                if (!lock_node(l, s.ctl, kSiteLockChild)) return want;
                if (threadIdx.x == 0 && detail::ld_acquire(&state->batchCount) > l && detail::ld_relaxed(taken + l) == 0)
                    s.ctl[5] += 1;
            }
            if (r < batchNum) {
                if (!lock_node(r, s.ctl, kSiteLockChild)) return want;
                if (threadIdx.x == 0 && detail::ld_acquire(&state->batchCount) > r && detail::ld_relaxed(taken + r) == 0)
                    s.ctl[5] += 2;
            }
            __syncthreads();
            const int adj = s.ctl[5];
            __syncthreads();
            if (adj == 0) {  // a leaf here
                if (l < batchNum) unlock_node(l);
                if (r < batchNum) unlock_node(r);
                store(node(cur), s.b1, B);
                unlock_node(cur);
                break;
            }
            if (adj == 1 || adj == 2) {  // one child
                const int c = adj == 1 ? l : r, o = adj == 1 ? r : l;
                if (o < batchNum) unlock_node(o);
                load(s.b2, node(c), B);
                __syncthreads();
                merge(s.b1, s.b2, node(cur), s.b1);
                unlock_node(cur);
                cur = c;
                continue;
            }
            load(s.b2, node(l), B);
            load(s.b3, node(r), B);
            __syncthreads();
            if (s.b2[B - 1] <= s.b3[B - 1]) {  // the left child keeps the smaller keys
                merge(s.b2, s.b3, s.b2, s.b3);
                store(node(r), s.b3, B);
                unlock_node(r);
                merge(s.b1, s.b2, node(cur), s.b1);
                unlock_node(cur);
                cur = l;
            } else {
                merge(s.b2, s.b3, s.b3, s.b2);
                store(node(l), s.b2, B);
                unlock_node(l);
                merge(s.b1, s.b3, node(cur), s.b1);
                unlock_node(cur);
                cur = r;
            }
        }
        return want;
    }

    // The reference's signature: *size in, keys taken out.
    __device__ void retrieve(K* ret, int* size, int smemOffset) const {
        const int want = *size;
        __syncthreads();
        const int n = retrieve(ret, want, smemOffset);
        if (threadIdx.x == 0) *size = n;
        __syncthreads();
    }

    // Keys held (a hint while other blocks run).
    __device__ long long held() const {
        return static_cast<long long>(detail::ld_relaxed(&state->batchCount)) * batchSize +
               detail::ld_relaxed(&state->partialBufferSize);
    }
};

// The auxiliary buffer of heap_with_aux.cuh:48-119: (key, value) entries
// that a retrieve hands out before the heap's keys.
template <typename K, typename Aux>
struct RetHeapAux {
    static_assert(sizeof(Aux) == 4 || sizeof(Aux) == 8, "Aux is a 4- or 8-byte scalar");
    RetHeap<K> heap;
    K* auxKeys;     // auxCap entries
    Aux* auxData;
    int* auxCtl;    // [0] lock, [1] entries held
    int auxCap;
    Aux initAux;    // the value of an entry that comes from the heap

    static __host__ __device__ size_t smemBytes(int B, int threads) {
        return RetHeap<K>::smemBytes(B) + 16 + static_cast<size_t>(threads) * sizeof(Aux);
    }

    __device__ long long held() const { return heap.held() + detail::ld_relaxed(auxCtl + 1); }

    // retrieve(key_dst, aux_dst, count, chk_func, priv_data): up to
    // `count` (<= batchSize) entries; buffered ones first (the newest), then
    // the heap's smallest keys with initAux.  check(key, Aux& value) is
    // called for every entry handed out; when it returns true the entry
    // goes back into the buffer with the value it left (the caller keeps the
    // value it was handed).  Returns the number handed out.  Every thread
    // of the block calls it.
    template <typename Check>
    __device__ int retrieve(K* keyDst, Aux* auxDst, int count, Check check, int smemOffset) const {
        extern __shared__ __align__(16) unsigned char gh_ret_smem[];
        int* ctl = reinterpret_cast<int*>(gh_ret_smem + smemOffset + RetHeap<K>::smemBytes(heap.batchSize));
        Aux* tmp = reinterpret_cast<Aux*>(ctl + 4);
        const int B = heap.batchSize;
        if (count > B) count = B;
        if (count < 0) count = 0;
        if (!aux_lock(ctl)) return 0;
        if (threadIdx.x == 0) ctl[0] = detail::ld_relaxed(auxCtl + 1);
        __syncthreads();
        const int have = ctl[0];
        __syncthreads();
        int n;
        if (have > count) {  // the newest `count` buffered entries
            for (int k = threadIdx.x; k < count; k += blockDim.x) {
                keyDst[k] = __ldcg(auxKeys + have - count + k);
                auxDst[k] = load_aux(have - count + k);
            }
            if (threadIdx.x == 0) ctl[1] = have - count;
            n = count;
        } else {
            for (int k = threadIdx.x; k < have; k += blockDim.x) {
                keyDst[k] = __ldcg(auxKeys + k);
                auxDst[k] = load_aux(k);
            }
            if (threadIdx.x == 0) detail::st_relaxed(auxCtl + 1, 0);
            __syncthreads();
            n = have;
            if (count - have > 0) {
                aux_unlock();
                const int got = heap.retrieve(keyDst + have, count - have, smemOffset);
                for (int k = threadIdx.x; k < got; k += blockDim.x) auxDst[have + k] = initAux;
                n = have + got;
                if (!aux_lock(ctl)) return n;
                if (threadIdx.x == 0) ctl[1] = detail::ld_relaxed(auxCtl + 1);
            } else if (threadIdx.x == 0) {
                ctl[1] = 0;
            }
        }
        __syncthreads();
        // entries with work left go back into the buffer
        for (int base = 0; base < n; base += blockDim.x) {
            const int k = base + threadIdx.x;
            if (k < n) {
                tmp[threadIdx.x] = auxDst[k];
                if (check(keyDst[k], tmp[threadIdx.x])) {
                    const int at = atomicAdd(&ctl[1], 1);
                    if (at < auxCap) {
                        auxKeys[at] = keyDst[k];
                        auxData[at] = tmp[threadIdx.x];
                    } else {
                        atomicAdd(&heap.state->appStats[kRetAuxFull], 1ull);
                    }
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int size = ctl[1] < auxCap ? ctl[1] : auxCap;
            if (ctl[1] > auxCap) atomicCAS(&heap.state->err, 0, kErrCapacity);
            detail::st_relaxed(auxCtl + 1, size);
        }
        aux_unlock();
        return n;
    }

    __device__ void insert(const K* keys, int count, int smemOffset) const { heap.insert(keys, count, smemOffset); }

  private:
    // Entries other blocks wrote: read past L1 (Aux is a plain scalar).
    __device__ Aux load_aux(int k) const { return *reinterpret_cast<const volatile Aux*>(auxData + k); }

    __device__ bool aux_lock(int* ctl) const {
        if (threadIdx.x == 0) {
            int ok = 1;
            const unsigned long long t0 = detail::globaltimer();
            while (detail::cas_acquire(auxCtl, 0, 1) != 0) {
                if (detail::globaltimer() - t0 > static_cast<unsigned long long>(heap.timeoutNs)) {
                    if (atomicCAS(&heap.state->err, 0, kErrTimeout) == 0) heap.state->errOp = kSiteLockPartial;
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
            ctl[2] = ok;
        }
        __syncthreads();
        const bool ok = ctl[2] != 0;
        __syncthreads();
        return ok;
    }
    __device__ void aux_unlock() const {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            detail::st_release(auxCtl, 0);
        }
    }
};

}  // namespace gh
