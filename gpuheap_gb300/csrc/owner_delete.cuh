// Bulk delete with the top of the heap held in one block's shared memory.
//
// The reference's deleteKernel (test/heap_test.cu:60-77) has every block
// call deleteRoot/deleteUpdate (heap/tditdd/heap.cuh:267-534,
// heap/buitdd/heap.cuh:283-482) in a loop; consecutive deletes then follow
// each other down the heap two levels apart, and each level step pays an L2
// lock, a node load and a release fence (about 3 us on GB300), so the root
// is handed on every ~6 us.  Here the same deletes run in the same order
// with the same node updates, but:
//
//   * block 0, the owner, keeps node 0 (partial buffer) and levels 0..R of
//     the heap (nodes 1 .. 2^(R+1)-1) in shared memory for the whole launch
//     and holds their lock words; no other block touches those nodes;
//   * a delete's sift steps at levels 0..R-1 only read the children's last
//     keys to pick the path and only merge children into their parent, so
//     once the path is known they are independent: the owner plans the
//     path (one warp), then merges every level of it at once (one warp per
//     window of the merges);
//   * the sift continues below level R in a worker block (every other block
//     of the launch): the owner lends it the level-R node on the path
//     together with the carried batch through a mailbox in global memory,
//     and the worker runs deleteUpdate's sift loop from there with the
//     usual locks; when the worker is done with that node (its first level
//     leaves the node's lock word at kLentBack), the owner takes it back
//     and reloads it;
//   * three control warps of the owner overlap the global latency with the
//     merges: one takes the next delete's last node (lock, bulk load, reset
//     to init_limits, release), one copies lends into the mailbox, one
//     takes lent nodes back.
//
// The owner stops when the output limit is reached or the heap has too few
// nodes left for its resident levels; it then writes those levels back to
// their global nodes, restores the counters and releases the lock words,
// and the caller finishes with k_delete.  Every wait is bounded by the
// heap's time limit; on expiry the heap's sticky error is raised and every
// role stops at its next check.
#pragma once
#include <climits>
#include <cstdint>

#include "heap_kernels.cuh"

namespace gh {
namespace impl {

constexpr int kMboxEntries = 32;   // lends in flight between owner and workers
constexpr int kOwnerWarps = 29;    // compute warps of the owner block
constexpr int kOwnerMaxR = 4;      // deepest resident level
// Lock word a worker leaves on the lent level-R node when its first sift
// level is done: no other lock state (TD 0-3, BU 0, 1, 2, 1 << 30), so the
// owner's returner takes the node back on seeing it, without a CAS (no one
// else touches a lent node during a bulk delete).
constexpr int kLentBack = (1 << 30) + 1;

// Keys per lane of a merge window: 32 for 4-byte keys (a window of 1024
// keys, sorted with two shared-memory transposes), 16 for 8-byte keys (512,
// sorted with lane shuffles; 32 would not fit the registers).
__host__ __device__ constexpr int owner_ipt(int keyBytes) { return keyBytes == 8 ? 16 : 32; }

// Mailbox in global memory: lend q (q = 0, 1, ...) sits in entry q % 32 with
// its carried batch at data + entry * batchSize.
struct alignas(128) Mailbox {
    int claim;  // next lend number a worker takes
    int pad0[31];
    int done;   // the owner posts no lend numbered >= total
    int total;
    int pad1[30];
    int seq[kMboxEntries];   // entry e holds lend q once seq[e] == q + 1
    int cons[kMboxEntries];  // uses of entry e that a worker has read
    int node[kMboxEntries];  // the level-R node lent with it
    unsigned long long stats[16];  // counters of the launch, indexed by OwnerStat
};

// Indices of Mailbox::stats (SM cycles unless a count).
enum OwnerStat : int {
    kStDeletes = 0,     // deletes made by the owner
    kStWaitCarried,     // compute: waiting for the taker's last node
    kStWaitLent,        // compute: waiting for a lent level-R node to come back
    kStWaitRing,        // compute: waiting for room in the lend ring
    kStPlan,            // compute: path plans
    kStPass,            // compute: merge passes, general steps included
    kStGeneral,         // general sift steps (count)
    kStLoop,            // compute: the whole delete loop
    kStTakeLock,        // taker: last-node lock waits
    kStTakeLoad,        // taker: last-node bulk loads
    kStTakeIdle,        // taker: waiting for permission or a free buffer
    kStLends,           // lends posted (count)
    kStReloads,         // lent nodes taken back (count)
    kStPlanRead,        // compute: the plan's reads of the children (part of kStPlan)
    kStPassWork,        // compute: warp 0's own merge windows (part of kStPass)
    kStPassSync,        // compute: warp 0 waiting for the other windows (part of kStPass)
    kStCount = 16
};

// Shared-memory control words of the owner block (after its node slots).
struct alignas(16) OwnerCtl {
    unsigned long long st[16];                  // counters (OwnerStat), compute thread 0
    unsigned long long cbar[2];                 // bulk loads of the two carried-batch buffers
    unsigned long long rbar[1 << kOwnerMaxR];   // bulk reloads of lent level-R nodes
    unsigned long long sbar;                    // set-up loads
    int cReady[2];     // buffer b holds the last node of delete t once cReady[b] == t + 1
    int cFree[2];      // uses of buffer b finished (lent out or done with)
    int cEnd;          // delete number the taker found no last node for, else -1
    int takeAllowed;   // the taker may take last nodes for deletes < takeAllowed
    int lentState[1 << kOwnerMaxR];  // level-R node 2^R + i: 0 in its slot, 1 lent out, 2 lost (error)
    int reqNode[4], reqBuf[4];       // lend requests, ring of 4
    int lendReq;       // requests posted
    int lendDone;      // requests copied out
    int stop;          // compute warps are done; the control warps finish
    int bcFinal;       // batch count after the taker's last take
    int engaged;       // set-up outcome
    int bc0, ps, dc0, lim;
    // plan of one segment (compute thread 0 -> compute warps)
    int plStop, nm, gen, genL, genR, genLarger, genSmaller, lend;
    int mA[kOwnerMaxR], mB[kOwnerMaxR], mLo[kOwnerMaxR], mHi[kOwnerMaxR];
    int caseSel;
};

// Transpose scratch of one merge window (32 x 33 keys, one pad column).
inline size_t owner_scratch(int keyBytes) { return owner_ipt(keyBytes) == 32 ? 32 * 33 * keyBytes : 0; }
// Shared memory of the owner block: 2^(R+1) + 3 node slots, the merge
// windows' scratch, the control words.
inline size_t owner_smem(int batchSize, int keyBytes, int R) {
    const int windows = R * (2 * batchSize / (32 * owner_ipt(keyBytes)));
    return static_cast<size_t>((2 << R) + 3) * batchSize * keyBytes + windows * owner_scratch(keyBytes) +
           sizeof(OwnerCtl);
}
// Resident depth R for a batch size and key size (0: no owner mode): the
// deepest R <= 2 (batch >= 2048) or 3 whose shared memory fits in 216 KB
// and whose R merges fit the compute warps (one window per warp); depth 4
// only when asked for (gh_heap_set_owner_depth).
inline int owner_depth(int batchSize, int keyBytes) {
    if (batchSize < 512 || 2 * batchSize / 1024 > 8) return 0;
    // measured on GB300 (2^26 u32 keys): at batch 2048 depth 2 takes 4.5 us
    // per delete against 5.4 at depth 3 (the merges of a deeper pass cost
    // more than the lent nodes it saves waiting for); at 1024, 3 beats 4
    const int top = batchSize >= 2048 ? 2 : 3;
    for (int R = top; R >= 2; --R) {
        const int windows = R * (2 * batchSize / (32 * owner_ipt(keyBytes)));
        if (owner_smem(batchSize, keyBytes, R) <= 216 * 1024 && windows <= kOwnerWarps && windows >= R) return R;
    }
    return 0;
}
// Bytes of the mailbox and its lend buffers for a heap.
inline size_t mbox_bytes(int batchSize, int keyBytes) {
    return sizeof(Mailbox) + static_cast<size_t>(kMboxEntries) * batchSize * keyBytes;
}

namespace ow {

__device__ __forceinline__ void bar_compute() {
    asm volatile("bar.sync 1, %0;" ::"r"(kOwnerWarps * 32) : "memory");
}
// Polls read shared words relaxed and fence once they see what they wait
// for (fence_acq): an acquire on every poll would fence on every poll.
__device__ __forceinline__ int lds(const int* p) {
    int v;
    asm volatile("ld.relaxed.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(detail::smem_u32(p)) : "memory");
    return v;
}
__device__ __forceinline__ void fence_acq() { asm volatile("fence.acq_rel.cta;" ::: "memory"); }
__device__ __forceinline__ void sts_rel(int* p, int v) {
    asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"(detail::smem_u32(p)), "r"(v) : "memory");
}
__device__ __forceinline__ void stg_rel(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int level_of(int i) { return 31 - __clz(i); }

template <typename K>
__device__ __forceinline__ K key_max() {
    if constexpr (sizeof(K) == 8) return static_cast<K>(~0ull);
    else if constexpr (static_cast<K>(-1) < static_cast<K>(0)) return static_cast<K>(0x7fffffff);
    else return static_cast<K>(0xffffffffu);
}

// Start of the merge-path split at output diagonal D of sorted a[0,n) and
// b[0,n): the number of a's keys among the first D outputs (a wins ties).
// The warp probes 32 positions per round at an odd stride, so the probes of
// one round fall in 32 different banks; three rounds cover n = 2048.
template <typename K>
__device__ __forceinline__ int warp_split(const K* a, const K* b, int n, int D) {
    const int lane = threadIdx.x & 31;
    int L = D > n ? D - n : 0, H = D < n ? D : n;
    while (H > L) {
        const int step = ((H - L + 31) >> 5) | 1;
        const int p = L + (lane + 1) * step - 1;
        const bool t = p < H && a[p] <= b[D - 1 - p];
        const int c = __popc(__ballot_sync(0xffffffffu, t));
        const int nh = L + (c + 1) * step - 1;
        L = c == 0 ? L : L + c * step;
        H = nh < H ? nh : H;
    }
    return L;
}

// Merge-path splits at output diagonals D and E of sorted a[0,n) and
// b[0,n): the number of a's keys among the first D (E) outputs (a wins
// ties).  The warp probes 32 positions per round at an odd stride, so the
// probes of one round fall in 32 different banks.  The two searches run in
// the same rounds.
template <typename K>
__device__ __forceinline__ void warp_split2(const K* a, const K* b, int n, int D, int E, int& sD, int& sE) {
    const int lane = threadIdx.x & 31;
    int L1 = D > n ? D - n : 0, H1 = D < n ? D : n;
    int L2 = E > n ? E - n : 0, H2 = E < n ? E : n;
    while (H1 > L1 || H2 > L2) {
        const int s1 = ((H1 - L1 + 31) >> 5) | 1, s2 = ((H2 - L2 + 31) >> 5) | 1;
        const int p1 = L1 + (lane + 1) * s1 - 1, p2 = L2 + (lane + 1) * s2 - 1;
        const bool t1 = p1 < H1 && a[p1] <= b[D - 1 - p1];
        const bool t2 = p2 < H2 && a[p2] <= b[E - 1 - p2];
        const int c1 = __popc(__ballot_sync(0xffffffffu, t1));
        const int c2 = __popc(__ballot_sync(0xffffffffu, t2));
        const int n1 = L1 + (c1 + 1) * s1 - 1, n2 = L2 + (c2 + 1) * s2 - 1;
        L1 = c1 == 0 ? L1 : L1 + c1 * s1;
        H1 = n1 < H1 ? n1 : H1;
        L2 = c2 == 0 ? L2 : L2 + c2 * s2;
        H2 = n2 < H2 ? n2 : H2;
    }
    sD = L1;
    sE = L2;
}

// Bitonic merge of the registers: a bitonic sequence over m[0..IPT) of one
// lane comes out ascending.
template <typename K, int IPT>
__device__ __forceinline__ void sort_regs(K (&m)[IPT]) {
#pragma unroll
    for (int s = IPT / 2; s > 0; s >>= 1) {
#pragma unroll
        for (int r = 0; r < IPT; ++r)
            if ((r & s) == 0) {
                const K u = m[r], v = m[r + s];
                m[r] = u < v ? u : v;
                m[r + s] = u < v ? v : u;
            }
    }
}

// One merge window: outputs [D, D + S) of merge(a, b), S = 32*IPT, element
// k = r*32 + lane in m[r], gathered as a bitonic sequence and sorted by a
// bitonic network.  Two ways to gather it:
//   * 4-byte keys with the window inside lo or hi (n >= S): one split i0 at
//     D; the window's keys are the S smallest of the candidate runs
//     a[i0, i0+S) and b[j0, j0+S), and min(x_k, y_{S-1-k}) is that set as a
//     bitonic sequence (two reads a key);
//   * otherwise: the splits at D and D + S give the window's keys exactly,
//     a[i0, i1) and b[j0, j1); element k is a[i0 + k] for k < i1 - i0,
//     then b read backwards (one read a key, no padding key).
// Measured on GB300 (a window alone and in the owner's pass): the first is
// 3-6 % faster for 4-byte keys at batch 2048, where the second split costs
// more than the saved reads; the second is faster for 8-byte
// keys (half the reads and registers) and for a window across lo and hi
// (batch 512, whose splits are trivial).  Strides >= 32 compare keys inside
// a lane's registers; for strides < 32, IPT = 32 transposes the window
// through `scr` (32 x 33 keys of this warp: both access patterns hit 32
// different banks) so that they are inside the registers too, and back;
// IPT = 16 uses lane shuffles.  Reads shared memory only.
template <typename K, int IPT>
__device__ __forceinline__ void window(const K* a, const K* b, int n, int D, K (&m)[IPT], K* scr) {
    constexpr int S = 32 * IPT;
    const int lane = threadIdx.x & 31;
    if (IPT == 32 && n >= S) {
        const int i0 = warp_split(a, b, n, D), j0 = D - i0;
        const K top = key_max<K>();
#pragma unroll
        for (int r = 0; r < IPT; ++r) {
            const int k = r * 32 + lane;
            const int xi = i0 + k, yi = j0 + (S - 1 - k);
            const K x = xi < n ? a[xi] : top;
            const K y = yi < n ? b[yi] : top;
            m[r] = x < y ? x : y;
        }
    } else {
        int i0, i1;
        warp_split2(a, b, n, D, D + S, i0, i1);
        const int na = i1 - i0, j1 = D + S - i1;
        // element k < na: a[i0 + k]; k >= na: b[j1 - 1 - (k - na)], which is
        // in [j0, j1) since k < S; indexed from a (both lie in one shared array)
        const int ia = i0 + lane, ib = static_cast<int>(b - a) + (j1 - 1 + na - lane);
#pragma unroll
        for (int r = 0; r < IPT; ++r) m[r] = a[r * 32 + lane < na ? ia + r * 32 : ib - r * 32];
    }
    sort_regs<K, IPT>(m);
    if constexpr (IPT == 32) {
        // the sorted window stays in scr (element k at (k/32)*33 + k%32)
        // for window_store: nothing is held in registers across the barrier
#pragma unroll
        for (int r = 0; r < 32; ++r) scr[r * 33 + lane] = m[r];
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 32; ++q) m[q] = scr[lane * 33 + q];
        sort_regs<K, IPT>(m);
#pragma unroll
        for (int q = 0; q < 32; ++q) scr[lane * 33 + q] = m[q];
    } else {
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) {
            const bool upper = (lane & s) != 0;
#pragma unroll
            for (int r = 0; r < IPT; ++r) {
                const K o = __shfl_xor_sync(0xffffffffu, m[r], s);
                m[r] = upper ? (m[r] > o ? m[r] : o) : (m[r] < o ? m[r] : o);
            }
        }
    }
}
// Writes the window's outputs to lo[0, n) / hi[0, n) (from scr when IPT = 32).
// A window that lies in one of the two (every one when S divides n) takes
// one destination pointer; the one window across both (n = S/2) picks per key.
template <typename K, int IPT>
__device__ __forceinline__ void window_store(K* lo, K* hi, int n, int D, const K (&m)[IPT], const K* scr) {
    constexpr int S = 32 * IPT;
    const int lane = threadIdx.x & 31;
    if constexpr (IPT == 32) __syncwarp();
    if (D + S <= n || D >= n) {
        K* dst = (D < n ? lo + D : hi + (D - n)) + lane;
#pragma unroll
        for (int r = 0; r < IPT; ++r) dst[r * 32] = IPT == 32 ? scr[r * 33 + lane] : m[r];
    } else {
#pragma unroll
        for (int r = 0; r < IPT; ++r) {
            const int o = D + r * 32 + lane;
            const K v = IPT == 32 ? scr[r * 33 + lane] : m[r];
            if (o < n) lo[o] = v;
            else hi[o - n] = v;
        }
    }
}

// Posts lend request (node, buffer) to the lender warp; compute thread 0.
__device__ __forceinline__ void post_lend(OwnerCtl* oc, int node, int buf) {
    const int q = oc->lendReq;
    oc->reqNode[q & 3] = node;
    oc->reqBuf[q & 3] = buf;
    sts_rel(&oc->lendReq, q + 1);
}

}  // namespace ow

// ---------------------------------------------------------------- workers
// Blocks 1.. of the launch: take lends in order, load the carried batch and
// run deleteUpdate's sift from the lent node (heap/tditdd/heap.cuh:418-532,
// heap/buitdd/heap.cuh:403-480), whose first level leaves that node's lock
// word at kLentBack -- the owner's signal that it can take it back.
// The carried batch comes in on a barrier of its own while the sift's first
// level takes and loads the lent node's children (the two are independent):
// the lent node goes back to the owner one bulk load sooner.
template <typename H, typename K>
__device__ void owner_worker(const H& h, Mailbox* mb, const K* mdata) {
    K* base = h.region(0);
    const int B = h.batchSize;
    __shared__ int w_node, w_entry, w_q, w_exit;
    __shared__ unsigned long long w_cbar;  // the carried batch's bulk load
    __shared__ unsigned w_cphase;          // its parity (thread 0)
    if (threadIdx.x == 0) {
        detail::mbar_init(&w_cbar, 1);
        w_cphase = 0;
    }
    __syncthreads();
    for (;;) {
        typename H::Op op(&h, h.ctl(base));
        if (threadIdx.x == 0) {
            const int q = atomicAdd(&mb->claim, 1);
            const int e = q % kMboxEntries;
            int ex = 0;
            unsigned long long t0 = 0;
            for (unsigned it = 0;; ++it) {
                if (detail::ld_acquire(&mb->seq[e]) == q + 1) break;
                if (detail::ld_acquire(&mb->done) && q >= detail::ld_relaxed(&mb->total)) { ex = 1; break; }
                if (!h.keep_waiting(t0, it, kSiteHandOff, -1, q)) { ex = 1; break; }
                __nanosleep(64);
            }
            w_exit = ex;
            w_q = q;
            w_entry = e;
            if (!ex) {
                w_node = detail::ld_relaxed(&mb->node[e]);
                detail::fence_proxy_async_smem();
                detail::mbar_arrive_expect_tx(&w_cbar, h.nodeBytes());
                detail::bulk_g2s(base, mdata + static_cast<size_t>(e) * B, h.nodeBytes(), &w_cbar);
            }
        }
        __syncthreads();
        if (w_exit) break;
        CarriedInFlight cf{&w_cbar, &w_cphase, &mb->cons[w_entry], w_q / kMboxEntries + 1};
        h.sift_loop(op, w_node, kLentBack, base, base + 2 * B, base + 3 * B, &cf);
        if (h.failed()) break;
    }
    __syncthreads();
    if (threadIdx.x == 0) detail::mbar_inval(&w_cbar);
}

// ---------------------------------------------------------------- owner
template <typename H, typename K>
__device__ void owner_block(const H& h, K* out, Mailbox* mb, K* mdata, int R) {
    extern __shared__ __align__(16) unsigned char gh_dyn_smem[];
    constexpr int IPT = owner_ipt(sizeof(K));
    constexpr int S = 32 * IPT;
    const int B = h.batchSize;
    const int NR = (2 << R) - 1;       // resident nodes 1..NR; node i in slot i-1
    const int firstR = 1 << R;         // level-R nodes firstR .. NR
    const int sP = NR, sC = NR + 1, sT = NR + 3;
    const int wpm = 2 * B / S;         // windows per merge
    K* slots = reinterpret_cast<K*>(gh_dyn_smem);
    K* scratch = slots + static_cast<size_t>(NR + 4) * B;
    constexpr int kScr = IPT == 32 ? 32 * 33 : 0;  // keys of one window's scratch
    OwnerCtl* oc = reinterpret_cast<OwnerCtl*>(scratch + static_cast<size_t>(R * wpm) * kScr);
    auto slot = [&](int s) -> K* { return slots + static_cast<size_t>(s) * B; };
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    K* scr = scratch + static_cast<size_t>(warp < R * wpm ? warp : 0) * kScr;  // this warp's window scratch
    const unsigned nb = h.nodeBytes();
    constexpr int L = H::lockedState();

    // ---- set-up: every thread of the block
    if (tid == 0) {
        oc->cReady[0] = oc->cReady[1] = 0;
        oc->cFree[0] = oc->cFree[1] = 0;
        oc->cEnd = -1;
        oc->lendReq = oc->lendDone = 0;
        oc->stop = 0;
        oc->plStop = 0;
        for (int i = 0; i < (1 << kOwnerMaxR); ++i) oc->lentState[i] = 0;
        const int bc = detail::ld_relaxed(&h.state->batchCount);
        oc->bc0 = bc;
        oc->ps = detail::ld_relaxed(&h.state->partialBufferSize);
        oc->dc0 = detail::ld_relaxed(&h.state->deleteCount);
        oc->lim = detail::ld_relaxed(&h.state->outLimit);
        oc->bcFinal = bc;
        oc->engaged = detail::ld_relaxed(&h.state->err) == 0 && bc >= (2 << R) + 1 &&
                      static_cast<long long>(oc->dc0) + B <= oc->lim;
        oc->takeAllowed = 1;
        detail::mbar_init(&oc->cbar[0], 1);
        detail::mbar_init(&oc->cbar[1], 1);
        detail::mbar_init(&oc->sbar, 1);
        for (int i = 0; i < (1 << kOwnerMaxR); ++i) detail::mbar_init(&oc->rbar[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (oc->engaged && warp == 0) {
        // hold node 0 and every resident node: nobody else uses the heap during a bulk delete
        bool ok = true;
        for (int i = lane; i <= NR; i += 32) ok = ok && h.lock(i, 0, L, i == 0 ? kSiteLockPartial : kSiteLockRoot);
        ok = __all_sync(0xffffffffu, ok);
        if (lane == 0) {
            oc->engaged = ok;
            if (ok) {
                const bool pbLoad = H::kHasPartialBuffer && oc->ps != 0;
                detail::mbar_arrive_expect_tx(&oc->sbar, (NR + (pbLoad ? 1u : 0u)) * nb);
                for (int i = 1; i <= NR; ++i) h.load(slot(i - 1), i, &oc->sbar);
                if (pbLoad) h.load(slot(sP), 0, &oc->sbar);
                unsigned long long t0 = 0;
                for (unsigned it = 0; !detail::mbar_try_wait(&oc->sbar, 0); ++it)
                    if (!h.keep_waiting(t0, it, kSiteBulkCopy, -1, 0)) { oc->engaged = 0; break; }
            }
        }
    }
    __syncthreads();
    if (!oc->engaged) {
        // not deep enough (or a failed wait, which left the heap's error
        // raised): no lend will come; k_delete does the work
        if (tid == 0) {
            mb->total = 0;
            ow::stg_rel(&mb->done, 1);
        }
        return;
    }

    if (warp < kOwnerWarps) {
        // ================================================= compute warps
        const int ct = tid;
        long long dc = oc->dc0;
        const int lim = oc->lim;
        const int ps = oc->ps;
        unsigned long long* st = oc->st;  // in shared memory: thread 0 alone counts
        if (ct == 0)
            for (int i = 0; i < kStCount; ++i) st[i] = 0;
        const long long tLoop = clock64();
        for (int d = 0;; ++d) {
            const int b = d & 1;
            K* C = slot(sC + b);
            if (ct == 0) {
                int stop = 0;
                // the heap's error word lives in global memory: a round trip,
                // so only every 64th delete reads it (the bounded waits below
                // stop on an error anyway)
                if (((d & 63) == 63 && detail::ld_relaxed(&h.state->err) != 0) || dc + B > lim) {
                    stop = 1;
                } else {
                    const long long tw = clock64();
                    unsigned long long t0 = 0;
                    for (unsigned it = 0;; ++it) {
                        if (ow::lds(&oc->cReady[b]) == d + 1) break;
                        if (ow::lds(&oc->cEnd) == d) { stop = 1; break; }
                        if (!h.keep_waiting(t0, it, kSiteLockLast, -1, d)) { stop = 1; break; }
                    }
                    ow::fence_acq();
                    st[kStWaitCarried] += clock64() - tw;
                }
                // the next delete's last node may be taken during this one
                if (!stop && dc + 2 * B <= lim) ow::sts_rel(&oc->takeAllowed, d + 2);
                oc->plStop = stop;
            }
            ow::bar_compute();
            if (oc->plStop) break;

            // refill: the last node merged with the partial buffer (:404-416)
            if (H::kHasPartialBuffer && ps != 0) {
                K m[IPT];
                const bool act = warp < wpm;
                if (act) ow::window<K, IPT>(C, slot(sP), B, warp * S, m, scr);
                ow::bar_compute();
                if (act) ow::window_store<K, IPT>(C, slot(sP), B, warp * S, m, scr);
                ow::bar_compute();
            }
            // deleteRoot's output (:328-329): the root's keys, before the pass
            // rewrites node 1; warps 1.. copy, so that warp 0, which plans and
            // signals with release stores, has no global stores in flight
            if (warp > 0) {
                K* dst = out + dc;
                const K* src = slot(0);
                const int t = ct - 32, nt = (kOwnerWarps - 1) * 32;
                if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
                    const int nv = static_cast<int>(nb / 16);
                    for (int q = t; q < nv; q += nt)
                        reinterpret_cast<uint4*>(dst)[q] = reinterpret_cast<const uint4*>(src)[q];
                } else {
                    for (int q = t; q < B; q += nt) dst[q] = src[q];
                }
            }
            int cur = 1;
            int lendNode = 0;
            for (;;) {
                long long tPass = 0;
                if (warp == 0) {
                    const long long tPlan = clock64();
                    long long tWait = 0;
                    // plan: follow the smaller child while the carried batch
                    // starts at or above one child's last key (the fast case
                    // of the sift, where the node takes the children's lower
                    // half and the carried batch goes on unchanged).  Lane i
                    // first reads the children of resident node i+1 (which is
                    // larger, by the heap/tditdd_np/heap.cuh:416 tie rule, and
                    // their smaller last key); the walk then takes one
                    // shuffle per level.  Children lent out are read on the way.
                    auto children = [&](int l, int r, int& larger, int& smaller, K& mn) {
                        const K* X = slot(l - 1);
                        const K* Y = slot(r - 1);
                        const K xl = X[B - 1], yl = Y[B - 1];
                        larger = (xl < yl || (xl == yl && !(xl < h.init_limits) && X[0] < Y[0])) ? r : l;
                        smaller = larger == r ? l : r;
                        mn = xl < yl ? xl : yl;
                    };
                    int pLarger = 0, pSmaller = 0, pOk = 0;
                    K pMin = K();
                    if (lane < firstR - 1) {
                        const int v = lane + 1, l = H::leftOf(v), r = H::rightOf(l);
                        pOk = ow::level_of(l) < R ||
                              (ow::lds(&oc->lentState[l - firstR]) == 0 && ow::lds(&oc->lentState[r - firstR]) == 0);
                        if (pOk) {
                            if (ow::level_of(l) == R) ow::fence_acq();  // after the reloads' completion
                            children(l, r, pLarger, pSmaller, pMin);
                        }
                    }
                    const K c0 = C[0];
                    __syncwarp();
                    if (lane == 0) st[kStPlanRead] += clock64() - tPlan;
                    int nm = 0, gen = 0, node = cur, lev = ow::level_of(cur);
                    while (lev < R) {
                        const int i = node - 1;
                        int larger = __shfl_sync(0xffffffffu, pLarger, i);
                        int smaller = __shfl_sync(0xffffffffu, pSmaller, i);
                        K mn = __shfl_sync(0xffffffffu, pMin, i);
                        const int ok = __shfl_sync(0xffffffffu, pOk, i);
                        const int l = H::leftOf(node), r = H::rightOf(l);
                        if (!ok) {
                            // a lent child must be back in its slot first
                            const long long tw = clock64();
                            if (lane == 0) {
                                for (int k = 0; k < 2; ++k) {
                                    const int x = k ? r : l;
                                    unsigned long long t0 = 0;
                                    for (unsigned it = 0; ow::lds(&oc->lentState[x - firstR]) != 0; ++it)
                                        if (!h.keep_waiting(t0, it, kSiteLockChild, x, 1)) break;
                                }
                                ow::fence_acq();
                            }
                            __syncwarp();
                            tWait += clock64() - tw;
                            children(l, r, larger, smaller, mn);
                        }
                        if (c0 < mn) {
                            gen = node;
                            if (lane == 0) {
                                oc->genL = l;
                                oc->genR = r;
                                oc->genLarger = larger;
                                oc->genSmaller = smaller;
                            }
                            break;
                        }
                        if (lane == 0) {
                            oc->mA[nm] = l - 1;
                            oc->mB[nm] = r - 1;
                            oc->mLo[nm] = node - 1;
                            oc->mHi[nm] = larger - 1;
                        }
                        ++nm;
                        node = smaller;
                        ++lev;
                    }
                    if (lane == 0) {
                        oc->nm = nm;
                        oc->gen = gen;
                        oc->lend = (!gen && lev == R) ? node : 0;
                        if (oc->lend) {
                            // post the lend now: the worker's first step needs
                            // nothing from this pass
                            const long long tw = clock64();
                            unsigned long long t0 = 0;
                            for (unsigned it = 0; oc->lendReq - ow::lds(&oc->lendDone) >= 4; ++it)
                                if (!h.keep_waiting(t0, it, kSiteHandOff, -1, 0)) break;
                            st[kStWaitRing] += clock64() - tw;
                            ow::post_lend(oc, oc->lend, b);
                            ++st[kStLends];
                        }
                        tPass = clock64();
                        st[kStWaitLent] += tWait;
                        st[kStPlan] += tPass - tPlan - tWait;
                        st[kStGeneral] += gen != 0;
                    }
                }
                ow::bar_compute();
                const int nm = oc->nm, gen = oc->gen;
                if (oc->lend) lendNode = oc->lend;
                // the pass: every planned level's children merge at once
                {
                    K m[IPT];
                    const int q = warp / wpm;
                    const bool act = q < nm;
                    if (act) ow::window<K, IPT>(slot(oc->mA[q]), slot(oc->mB[q]), B, (warp - q * wpm) * S, m, scr);
                    const long long tw = ct == 0 ? clock64() : 0;
                    ow::bar_compute();
                    if (ct == 0) {
                        const long long tb = clock64();
                        st[kStPassWork] += tw - tPass;
                        st[kStPassSync] += tb - tw;
                    }
                    if (act) ow::window_store<K, IPT>(slot(oc->mLo[q]), slot(oc->mHi[q]), B, (warp - q * wpm) * S, m, scr);
                    ow::bar_compute();
                }
                if (!gen) {
                    if (ct == 0) st[kStPass] += clock64() - tPass;
                    break;
                }
                // the general sift step at node `gen` (heap/tditdd/heap.cuh:
                // 418-532): children merge, lower half to T, upper half to the
                // larger child, then the case analysis against the carried batch
                {
                    K m[IPT];
                    const bool act = warp < wpm;
                    if (act) ow::window<K, IPT>(slot(oc->genL - 1), slot(oc->genR - 1), B, warp * S, m, scr);
                    ow::bar_compute();
                    if (act) ow::window_store<K, IPT>(slot(sT), slot(oc->genLarger - 1), B, warp * S, m, scr);
                    ow::bar_compute();
                }
                if (ct == 0) {
                    const K* T = slot(sT);
                    int sel;
                    if (!(C[0] < T[B - 1])) sel = 0;  // node takes T, the carried batch goes on
                    else if (H::kVariant == kTopDown || !H::kHasPartialBuffer ? (C[B - 1] <= T[0]) : (C[B - 1] < T[0]))
                        sel = 1;  // node takes C, the smaller child takes T: done (buitdd alone uses <, :451)
                    else sel = 2;  // merge C with T: lower to the node, upper carried on
                    oc->caseSel = sel;
                }
                ow::bar_compute();
                const int sel = oc->caseSel;
                const int g = gen, sm = oc->genSmaller;
                if (sel == 0) {
                    for (int q = ct; q < B; q += kOwnerWarps * 32) slot(g - 1)[q] = slot(sT)[q];
                } else if (sel == 1) {
                    for (int q = ct; q < B; q += kOwnerWarps * 32) {
                        slot(g - 1)[q] = C[q];
                        slot(sm - 1)[q] = slot(sT)[q];
                    }
                } else {
                    K m[IPT];
                    const bool act = warp < wpm;
                    if (act) ow::window<K, IPT>(C, slot(sT), B, warp * S, m, scr);
                    ow::bar_compute();
                    if (act) ow::window_store<K, IPT>(slot(g - 1), C, B, warp * S, m, scr);
                }
                ow::bar_compute();
                if (ct == 0) st[kStPass] += clock64() - tPass;
                if (sel == 1) break;
                cur = sm;
                if (ow::level_of(cur) == R) {
                    // the sift goes on below the resident levels: lend cur
                    // with the (possibly changed) carried batch
                    if (ct == 0) {
                        const long long tw = clock64();
                        unsigned long long t0 = 0;
                        for (unsigned it = 0; oc->lendReq - ow::lds(&oc->lendDone) >= 4; ++it)
                            if (!h.keep_waiting(t0, it, kSiteHandOff, -1, 0)) break;
                        st[kStWaitRing] += clock64() - tw;
                        ow::post_lend(oc, cur, b);
                        ++st[kStLends];
                    }
                    lendNode = cur;
                    break;
                }
            }
            if (ct == 0) {
                // the lent node's slot was read by this delete's pass: only now
                // may the returner reload it
                if (lendNode) ow::sts_rel(&oc->lentState[lendNode - firstR], 1);
                else atomicAdd(&oc->cFree[b], 1);  // no lend: the buffer is free again
            }
            dc += B;
        }
        if (ct == 0) {
            h.state->deleteCount = static_cast<int>(dc);
            st[kStDeletes] = static_cast<unsigned long long>((dc - oc->dc0) / B);
            st[kStLoop] = clock64() - tLoop;
            for (int i = 0; i < 8; ++i) mb->stats[i] = st[i];
            mb->stats[kStLends] = st[kStLends];
            for (int i = kStPlanRead; i < kStCount; ++i) mb->stats[i] = st[i];
            ow::sts_rel(&oc->stop, 1);
        }
    } else if (warp == kOwnerWarps) {
        // ================================================= taker
        int bc = oc->bc0;
        unsigned long long tkLock = 0, tkLoad = 0, tkIdle = 0;
        for (int t = 0;; ++t) {
            const int b = t & 1;
            int go = 0;
            if (lane == 0) {
                const long long ti = clock64();
                unsigned long long t0 = 0;
                for (unsigned it = 0;; ++it) {
                    if (ow::lds(&oc->stop)) break;
                    if (ow::lds(&oc->takeAllowed) > t && ow::lds(&oc->cFree[b]) >= (t >> 1)) { go = 1; break; }
                    if (!h.keep_waiting(t0, it, kSiteLockLast, -1, t)) break;
                    __nanosleep(32);
                }
                ow::fence_acq();
                tkIdle += clock64() - ti;
                if (go && bc < (2 << R)) {  // the last node would be resident: the owner is done
                    ow::sts_rel(&oc->cEnd, t);
                    go = 0;
                }
                if (go) {
                    // deleteUpdate takes the last node (:355-402): lock it
                    const long long tl = clock64();
                    bool ok;
                    if constexpr (H::kVariant == kTopDown) {
                        ok = h.lock(bc, TD::AVAIL, TD::INUSE, kSiteLockLast);
                    } else {
                        ok = true;
                        unsigned long long t1 = 0;
                        for (unsigned it = 0; detail::max_acquire(h.status + bc, BU::INUSE) == BU::INUSE; ++it)
                            if (!h.keep_waiting(t1, it, kSiteLockLast, bc, BU::INUSE)) { ok = false; break; }
                    }
                    const long long tb = clock64();
                    tkLock += tb - tl;
                    if (ok) {
                        detail::fence_proxy_async_smem();
                        detail::mbar_arrive_expect_tx(&oc->cbar[b], nb);
                        h.load(slot(sC + b), bc, &oc->cbar[b]);
                        unsigned long long t1 = 0;
                        for (unsigned it = 0; !detail::mbar_try_wait(&oc->cbar[b], (t >> 1) & 1); ++it)
                            if (!h.keep_waiting(t1, it, kSiteBulkCopy, bc, 0)) { ok = false; break; }
                    }
                    tkLoad += clock64() - tb;
                    if (ok) ow::sts_rel(&oc->cReady[b], t + 1);
                    else ow::sts_rel(&oc->cEnd, t);
                    go = ok ? 2 : 0;
                }
            }
            go = __shfl_sync(0xffffffffu, go, 0);
            if (go != 2) break;
            // reset the taken node (:396) and release it
            {
                K* g = h.node(bc);
                const int nv = static_cast<int>(nb / 16);
                const uint4 pat = detail::splat16<K>(h.init_limits);
                for (int q = lane; q < nv; q += 32) reinterpret_cast<uint4*>(g)[q] = pat;
            }
            __syncwarp();
            if (lane == 0) {
                H::fence();
                h.setState(bc, 0);
            }
            --bc;
        }
        if (lane == 0) {
            oc->bcFinal = bc;
            mb->stats[kStTakeLock] = tkLock;
            mb->stats[kStTakeLoad] = tkLoad;
            mb->stats[kStTakeIdle] = tkIdle;
        }
    } else if (warp == kOwnerWarps + 1) {
        // ================================================= lender
        for (int q = 0;; ++q) {
            int go = 0;
            if (lane == 0) {
                unsigned long long t0 = 0;
                for (unsigned it = 0;; ++it) {
                    if (ow::lds(&oc->lendReq) > q) { go = 1; break; }
                    if (ow::lds(&oc->stop)) {
                        ow::fence_acq();
                        if (ow::lds(&oc->lendReq) <= q) break;
                    }
                    if (!h.keep_waiting(t0, it, kSiteHandOff, -1, q)) break;
                    __nanosleep(32);
                }
                ow::fence_acq();
                if (go) {
                    // the entry's previous lend must have been read by its worker
                    const int e = q % kMboxEntries;
                    unsigned long long t1 = 0;
                    for (unsigned it = 0; detail::ld_acquire(&mb->cons[e]) != q / kMboxEntries; ++it)
                        if (!h.keep_waiting(t1, it, kSiteHandOff, -1, q)) { go = 0; break; }
                }
            }
            go = __shfl_sync(0xffffffffu, go, 0);
            if (!go) {
                if (lane == 0) {
                    mb->total = q;
                    ow::stg_rel(&mb->done, 1);
                }
                break;
            }
            const int e = q % kMboxEntries;
            const int b = oc->reqBuf[q & 3];
            {
                const uint4* src = reinterpret_cast<const uint4*>(slot(sC + b));
                uint4* dst = reinterpret_cast<uint4*>(mdata + static_cast<size_t>(e) * B);
                const int nv = static_cast<int>(nb / 16);
                for (int v = lane; v < nv; v += 32) dst[v] = src[v];
            }
            __syncwarp();
            if (lane == 0) {
                mb->node[e] = oc->reqNode[q & 3];
                H::fence();
                ow::stg_rel(&mb->seq[e], q + 1);
                atomicAdd(&oc->cFree[b], 1);
                ow::sts_rel(&oc->lendDone, q + 1);
            }
        }
    } else {
        // ================================================= returner
        // lane i watches level-R node 2^R + i while it is lent
        const int nR = 1 << R;
        unsigned phase = 0, reloads = 0;
        unsigned long long t0 = 0;
        unsigned it = 0;
        for (;;) {
            // `stop` first: the compute warps mark their last lend before they
            // set it, so a scan that follows a seen `stop` finds every lend
            const int stop = __shfl_sync(0xffffffffu, lane == 0 ? ow::lds(&oc->stop) : 0, 0);
            ow::fence_acq();
            int st = 0;
            if (lane < nR) {
                st = ow::lds(&oc->lentState[lane]);
                if (st == 1) {
                    const int x = firstR + lane;
                    if (detail::ld_acquire(h.status + x) == kLentBack) {
                        h.setState(x, L);  // held by the owner again
                        detail::fence_proxy_async_smem();
                        detail::mbar_arrive_expect_tx(&oc->rbar[lane], nb);
                        h.load(slot(x - 1), x, &oc->rbar[lane]);
                        unsigned long long t1 = 0;
                        bool ok = true;
                        for (unsigned i2 = 0; !detail::mbar_try_wait(&oc->rbar[lane], phase); ++i2)
                            if (!h.keep_waiting(t1, i2, kSiteBulkCopy, x, 0)) { ok = false; break; }
                        phase ^= 1u;
                        ++reloads;
                        st = ok ? 0 : 2;
                        ow::sts_rel(&oc->lentState[lane], st);
                        t0 = 0;
                        it = 0;
                    } else if (!h.keep_waiting(t0, it++, kSiteLockChild, x, 0)) {
                        st = 2;
                        ow::sts_rel(&oc->lentState[lane], st);
                    }
                }
            }
            const bool pending = __any_sync(0xffffffffu, st == 1);
            if (stop && !pending) {
                for (int o = 16; o > 0; o >>= 1) reloads += __shfl_xor_sync(0xffffffffu, reloads, o);
                if (lane == 0) mb->stats[kStReloads] = reloads;
                break;
            }
            __nanosleep(pending ? 32 : 128);
        }
    }
    __syncthreads();

    // ---- write-back: resident nodes and the partial buffer to their global
    // nodes, counters, then every lock word released
    {
        const int nv = static_cast<int>(nb / 16);
        for (int i = 1; i <= NR; ++i) {
            const uint4* src = reinterpret_cast<const uint4*>(slot(i - 1));
            uint4* dst = reinterpret_cast<uint4*>(h.node(i));
            for (int v = tid; v < nv; v += blockDim.x) dst[v] = src[v];
        }
        if (H::kHasPartialBuffer && oc->ps != 0) {
            const uint4* src = reinterpret_cast<const uint4*>(slot(sP));
            uint4* dst = reinterpret_cast<uint4*>(h.node(0));
            for (int v = tid; v < nv; v += blockDim.x) dst[v] = src[v];
        }
    }
    __syncthreads();
    if (tid == 0) {
        h.state->batchCount = oc->bcFinal;
        H::fence();
        for (int i = 0; i <= NR; ++i) h.setState(i, 0);
        detail::mbar_inval(&oc->cbar[0]);
        detail::mbar_inval(&oc->cbar[1]);
        detail::mbar_inval(&oc->sbar);
        for (int i = 0; i < (1 << kOwnerMaxR); ++i) detail::mbar_inval(&oc->rbar[i]);
    }
}

// Block 0 owns the top of the heap, the rest are workers.  blockDim.x must
// be 1024 (29 compute warps and 3 control warps in the owner).
template <typename H, typename K>
__global__ void __launch_bounds__(1024) k_delete_owner(H h, K* out, Mailbox* mb, K* mdata, int R) {
    if (blockIdx.x == 0) owner_block<H, K>(h, out, mb, mdata, R);
    else owner_worker<H, K>(h, mb, mdata);
}

}  // namespace impl
}  // namespace gh
