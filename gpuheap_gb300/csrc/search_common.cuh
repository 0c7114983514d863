// Types and host entry points shared by the batched searches (search.cu), the
// served queries (serve.cu) and the translation units that compile the
// search kernels once (search_inst_td.cu, search_inst_bu.cu, search_util.cu).
//
// Only those three units instantiate device code; the host units see the
// instance record, the launch shape and plain function declarations.
#pragma once
#include <cuda_runtime.h>

#include <climits>
#include <cstddef>

#include "gpuheap.h"
#include "gpuheap_device.cuh"
#include "gpuheap_fifo.cuh"

namespace gh {
namespace search {

using u64 = unsigned long long;
constexpr int kMaxKnapItems = 1024;
constexpr int kMaxSearchThreads = 512;  // 128 registers per thread
constexpr int kSlotBits = 20;            // knapsack key: pool slot bits below the level

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
    int tokens;                 // served, device loop: work tokens of the query still out
    int moves;                  // A*: 0 or 4, cost grid (4 neighbours); 8, the reference's bitmap model
};

// Shared memory of a search block, ahead of the heap's region.  Emitted
// keys: a full batch is inserted after every round of one key a thread, so
// B + 8 T holds what a round adds (an A* key has up to eight neighbours).
struct SearchSmem {
    static __host__ __device__ size_t emitKeys(int B, int T) { return static_cast<size_t>(B) + 8 * static_cast<size_t>(T); }
    static __host__ __device__ size_t bytes(int B, int T) {
        const size_t keys = (static_cast<size_t>(B) + emitKeys(B, T)) * 8;
        const size_t knap = static_cast<size_t>(kMaxKnapItems + 1) * 16 + static_cast<size_t>(kMaxKnapItems) * 8 +
                            static_cast<size_t>(B) * 16;
        return (keys + knap + 64 + 15) / 16 * 16;
    }
};

// Shape of a search launch, shared by the batched and served forms.
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

// ------------------------------------------------ served queries, device loop
// The host posts requests into a ring in pinned host memory and reads
// completions from another; the resident search launch admits requests
// into free slots and arena memory, runs them and frees them, without a
// host round trip per step.

// Arena block of a served query: its heap's counters, nodes and lock words,
// then its distance array (`dist` entries), each 256-byte aligned.
struct QueryLayout {
    size_t items, status, g, bytes;  // offsets from the block's start (the counters sit at 0), total size
};
__host__ __device__ inline size_t align256(size_t x) { return (x + 255) / 256 * 256; }
__host__ __device__ inline QueryLayout query_layout(int bn, int B, long long dist) {
    QueryLayout L;
    L.items = align256(sizeof(gh::HeapState));
    L.status = L.items + align256(static_cast<size_t>(bn + 1) * B * 8);
    L.g = L.status + align256(static_cast<size_t>(bn + 2) * 4);
    L.bytes = L.g + align256(static_cast<size_t>(dist) * 4);
    return L;
}

// A request (host writes every field, then seq; the device reads seq first).
struct alignas(16) ServeReq {
    unsigned long long seq;  // r + 1 once record r of the ring is complete
    long long qid;           // the host's query id
    int kind, a, b, blocks;  // GH_SEARCH_SSSP / GH_SEARCH_ASTAR, endpoints, work tokens
    int bn, n, width, height;  // heap nodes; graph vertices or grid shape
    unsigned long long bytes;  // arena bytes of the query
    unsigned long long off;    // arena offset, set at admission
    const long long* rowptr;
    const int* col;
    const unsigned* w;
    const unsigned char* cost;
    int moves;  // A*: 4 (cost grid) or 8 (the reference's bitmap model)
    int pad[3];
};
static_assert(sizeof(ServeReq) == 112, "request record layout");

// A completion (the device writes every field, then seq).
struct alignas(16) ServeDone {
    unsigned long long seq;  // c + 1 once completion c is complete
    long long qid;
    int state, failed;       // 2 finished, 3 failed; the failure's gh_status
    unsigned long long r0, r1;
    unsigned long long tDone;  // device global timer (ns)
    unsigned long long pad[2];
};
static_assert(sizeof(ServeDone) == 64, "completion record layout");

// Words in pinned host memory: `stop` from the host; the rest from the
// device (relaxed system-scope stores by the admission lock's holder).
struct alignas(128) ServeHost {
    int stop;
    int pad0[31];
    unsigned long long reqTaken;  // requests the device has read out of the ring
    long long usedBytes;          // arena bytes of admitted queries
    int slotsUsed, pending, active, err;
    unsigned long long admitted, completed;
    int pad1[18];
};
static_assert(sizeof(ServeHost) == 256, "host words layout");

// A cell of the work-token queue (a bounded multi-producer multi-consumer
// ring with one sequence word per cell).
struct alignas(16) ServeCell {
    unsigned long long seq;
    int val;
    int pad;
};

struct ServeRange {
    unsigned long long off, len;
};

// A work token: a slot (take batches of its query) or a slot with this bit
// (set the query up: instance record, fill, seed, then its search tokens).
constexpr int kServeSetup = 1 << 30;

// Device errors of the loop (ServeHost::err).
enum ServeErr { kServeOk = 0, kServeErrQueue = 1, kServeErrLock = 2, kServeErrWait = 3 };

struct ServeDev {
    // admission state: read and written by the holder of `lock` only
    int lock, exit, err, npend;
    int nfree, nranges, active, freeEpoch;
    int admitEpoch, pad0;
    unsigned long long reqTaken, idleSince, usedBytes, doneClaim, admitted;
    unsigned long long pad1[8];
    // token queue positions, each on its own line
    alignas(128) unsigned long long enq;
    unsigned long long pad2[15];
    alignas(128) unsigned long long deq;
    unsigned long long pad3[15];
    alignas(128) unsigned long long admitAt;  // global timer before which no block tries to admit
    unsigned long long pad4[15];
    // set by the host before the first launch
    alignas(128) ServeReq* ring;  // pinned, ringCap records
    ServeDone* done;              // pinned, ringCap records
    ServeHost* host;              // pinned
    ServeReq* pend;               // ringCap: read, not admitted yet (arrival order)
    ServeReq* slotReq;            // maxSlots: the request each slot holds
    int* freeSlots;               // maxSlots
    ServeRange* ranges;           // maxRanges free arena ranges, by offset
    ServeCell* cells;             // cellMask + 1
    Inst* insts;                  // maxSlots
    unsigned char* arena;
    unsigned long long arenaBytes, cellMask;
    int ringCap, maxSlots, maxRanges, batchSize;
    long long idleNs;   // exit after this long with nothing admitted or pending
    long long waitNs;   // limit of a wait for a queue cell or the lock
    long long stallNs;  // limit of a wait for a work token while no token moves
};

// Arguments of a search launch: a static task list (batched form, host
// step of the served form) or, with serve != NULL, the device loop.
struct SearchArgs {
    Inst* insts;
    const int* tasks;
    int ntasks;
    int* next;
    int maxBatches;  // > 0: a block takes at most this many batches of a query, then moves on
    ServeDev* serve;
};

// Defined by search_inst_td.cu and search_inst_bu.cu (one layout each).
cudaError_t search_launch_topdown(const SearchConfig& c, const SearchArgs& a, int grid, cudaStream_t s);
cudaError_t search_launch_bottomup(const SearchConfig& c, const SearchArgs& a, int grid, cudaStream_t s);
int search_blocks_per_sm_topdown(const SearchConfig& c);
int search_blocks_per_sm_bottomup(const SearchConfig& c);

inline cudaError_t search_launch(const SearchConfig& c, const SearchArgs& a, int grid, cudaStream_t s) {
    return c.variant == GH_TOPDOWN ? search_launch_topdown(c, a, grid, s) : search_launch_bottomup(c, a, grid, s);
}

// Blocks of one persistent launch: resident blocks per SM x SMs.
inline int search_resident_blocks(const SearchConfig& c) {
    int per = c.variant == GH_TOPDOWN ? search_blocks_per_sm_topdown(c) : search_blocks_per_sm_bottomup(c);
    if (per < 1) per = 1;
    return per * c.numSMs;
}

// Defined by search_util.cu.  Reset of the listed instances' arrays (ids ==
// NULL: the first `count`); counters and seed keys; the after-launch
// collection (failures, done, SSSP digests).
cudaError_t search_fill(Inst* insts, const int* ids, int count, int batchSize, cudaStream_t s);
cudaError_t search_seed(Inst* insts, const int* ids, int count, cudaStream_t s);
cudaError_t search_collect(Inst* insts, const int* ids, int count, int final, int batchSize, cudaStream_t s);

}  // namespace search
}  // namespace gh
