// Batched searches on the queue: many independent grid A* and 0/1 knapsack
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
// Blocks find work through a task list: an instance appears once per block
// it should get (large grids several times, knapsacks once), largest first;
// blocks of one instance share its heap and stop by the protocol of
// worklist.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <thread>
#include <vector>

#include "gpuheap.h"
#include "heap_kernels.cuh"
#include "search_common.cuh"
#include "trace.cuh"

using namespace gh::search;

// ---------------------------------------------------------------------- host side
struct HostInst {
    int kind;
    int width = 0, height = 0;
    std::vector<unsigned char> cost;
    std::vector<int> w, p;  // ratio-ordered
    std::vector<long long> W, P;
    long long cap = 0;
    int greedy = 0;
    int blocks = 1;
    long long work = 0;  // size estimate for the task order
    int moves = 4;       // A*: 4 (cost grid) or 8 (the reference's bitmap model)
};

struct gh_batch {
    int batchSize = 256, variant = GH_BOTTOMUP, threads = 0;
    long long timeoutNs = 2000000000LL;
    long long astarCellsPerBlock = 1 << 18;
    int astarMaxBlocks = 8;
    int knapOrder = GH_KNAP_HEAP, switchCounter = 20;
    int device = 0, numSMs = 0;
    std::vector<HostInst> host;
    // device
    unsigned char* arena = nullptr;
    size_t arenaBytes = 0;
    Inst* insts = nullptr;
    int* tasks = nullptr;  // batched order, then per-instance segments
    int* next = nullptr;   // [0] batched counter, [1 + i] per-instance counters
    int ntasks = 0;
    std::vector<int> segOff, segLen;
    std::vector<Inst> hinst;
    cudaGraphExec_t graph = nullptr;
    cudaStream_t graphStream = nullptr;
    long long graphLaunches = 0;
    int grid = 0;  // blocks of the persistent launch
    bool built = false;
    std::vector<cudaEvent_t> plainEv;  // one-launch-per-instance runs: an event before each launch and one after
};

namespace {

SearchConfig config_of(const gh_batch* b) {
    return SearchConfig{b->batchSize, b->variant, b->threads, b->timeoutNs, b->numSMs};
}
int threads_for(const gh_batch* b) { return search_threads(config_of(b)); }
int resident_blocks(const gh_batch* b) { return search_resident_blocks(config_of(b)); }
cudaError_t launch(const gh_batch* b, const int* tasks, int ntasks, int* next, int grid, cudaStream_t s) {
    return search_launch(config_of(b), SearchArgs{b->insts, tasks, ntasks, next, 0, nullptr}, grid, s);
}

void free_device(gh_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    if (b->arena) cudaFree(b->arena);
    b->arena = nullptr;
    b->insts = nullptr;
    b->tasks = nullptr;
    b->next = nullptr;
    b->built = false;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Heap nodes for an instance: a power of two holding its open-list bound.
int heap_nodes(long long keys, int B) {
    long long nodes = (keys + B - 1) / B;
    int bn = 1;
    while (bn < nodes) bn <<= 1;
    return bn;
}

gh_status reset_and_run(gh_batch* b, int mode, cudaStream_t s);

}  // namespace

extern "C" {

gh_status gh_batch_create(gh_batch** out, int batch_size, int variant, int block_threads) {
    if (!out) return GH_ERR_INVALID;
    *out = nullptr;
    if (batch_size < 32 || batch_size > 1024 || (batch_size & (batch_size - 1))) return GH_ERR_INVALID;
    if (variant != GH_TOPDOWN && variant != GH_BOTTOMUP) return GH_ERR_INVALID;
    if (block_threads != 0 && block_threads != batch_size && block_threads != batch_size / 2) return GH_ERR_INVALID;
    if (block_threads > kMaxSearchThreads) return GH_ERR_INVALID;
    gh_batch* b = new (std::nothrow) gh_batch();
    if (!b) return GH_ERR_INVALID;
    b->batchSize = batch_size;
    b->variant = variant;
    b->threads = block_threads;
    if (cudaGetDevice(&b->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&b->numSMs, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess) {
        delete b;
        return GH_ERR_CUDA;
    }
    *out = b;
    return GH_OK;
}

gh_status gh_batch_destroy(gh_batch* b) {
    if (!b) return GH_ERR_INVALID;
    for (cudaEvent_t e : b->plainEv) cudaEventDestroy(e);
    free_device(b);
    if (b->graphStream) cudaStreamDestroy(b->graphStream);
    delete b;
    return GH_OK;
}

gh_status gh_batch_plain_times(gh_batch* b, float* ms_out) {
    const int count = b ? static_cast<int>(b->host.size()) : 0;
    if (!b || !ms_out || static_cast<int>(b->plainEv.size()) < count + 1 || count == 0) return GH_ERR_INVALID;
    if (cudaEventSynchronize(b->plainEv[count]) != cudaSuccess) return GH_ERR_CUDA;
    for (int i = 0; i < count; ++i)
        if (cudaEventElapsedTime(&ms_out[i], b->plainEv[i], b->plainEv[i + 1]) != cudaSuccess) return GH_ERR_CUDA;
    return GH_OK;
}

gh_status gh_batch_set_astar_blocks(gh_batch* b, long long cells_per_block, int max_blocks) {
    if (!b || cells_per_block < 1 || max_blocks < 1 || max_blocks > 64) return GH_ERR_INVALID;
    b->astarCellsPerBlock = cells_per_block;
    b->astarMaxBlocks = max_blocks;
    if (b->built) free_device(b);
    return GH_OK;
}

gh_status gh_batch_set_knapsack_order(gh_batch* b, int order, int switch_counter) {
    if (!b || order < GH_KNAP_HEAP || order > GH_KNAP_SWITCH || switch_counter < 1) return GH_ERR_INVALID;
    b->knapOrder = order;
    b->switchCounter = switch_counter;
    if (b->built) free_device(b);
    return GH_OK;
}

gh_status gh_batch_set_timeout(gh_batch* b, double seconds) {
    if (!b || !(seconds > 0) || seconds > 60.0) return GH_ERR_INVALID;
    b->timeoutNs = static_cast<long long>(seconds * 1e9);
    if (b->built) free_device(b);
    return GH_OK;
}

gh_status gh_batch_add_astar(gh_batch* b, int width, int height, const unsigned char* cost_host, int* id) {
    if (!b || !cost_host || width < 1 || height < 1 || static_cast<long long>(width) * height > (1LL << 30))
        return GH_ERR_INVALID;
    HostInst h;
    h.kind = GH_SEARCH_ASTAR;
    h.width = width;
    h.height = height;
    h.cost.assign(cost_host, cost_host + static_cast<size_t>(width) * height);
    h.work = static_cast<long long>(width) * height;
    if (id) *id = static_cast<int>(b->host.size());
    b->host.push_back(std::move(h));
    if (b->built) free_device(b);
    return GH_OK;
}

gh_status gh_batch_add_astar_bitmap(gh_batch* b, int width, int height, const unsigned char* open_host, int* id) {
    if (!b || !open_host || width < 1 || height < 1 || static_cast<long long>(width) * height > (1LL << 30))
        return GH_ERR_INVALID;
    HostInst h;
    h.kind = GH_SEARCH_ASTAR;
    h.moves = 8;
    h.width = width;
    h.height = height;
    const size_t cells = static_cast<size_t>(width) * height;
    h.cost.resize(cells);
    for (size_t i = 0; i < cells; ++i) h.cost[i] = open_host[i] ? 1 : 0;
    h.work = static_cast<long long>(cells);
    if (id) *id = static_cast<int>(b->host.size());
    b->host.push_back(std::move(h));
    if (b->built) free_device(b);
    return GH_OK;
}

gh_status gh_batch_add_knapsack(gh_batch* b, int n, const int* weight_host, const int* profit_host, long long capacity,
                                int* id) {
    if (!b || n < 1 || n > kMaxKnapItems || !weight_host || !profit_host || capacity < 0) return GH_ERR_INVALID;
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        if (weight_host[i] < 1 || profit_host[i] < 0) return GH_ERR_INVALID;
        total += profit_host[i];
    }
    if (total >= INT_MAX / 2 || capacity >= (1LL << 40)) return GH_ERR_INVALID;
    HostInst h;
    h.kind = GH_SEARCH_KNAPSACK;
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
        return static_cast<long long>(profit_host[x]) * weight_host[y] > static_cast<long long>(profit_host[y]) * weight_host[x];
    });
    h.w.resize(n);
    h.p.resize(n);
    h.W.assign(n + 1, 0);
    h.P.assign(n + 1, 0);
    long long wt = 0, pr = 0;
    for (int i = 0; i < n; ++i) {
        h.w[i] = weight_host[ord[i]];
        h.p[i] = profit_host[ord[i]];
        h.W[i + 1] = h.W[i] + h.w[i];
        h.P[i + 1] = h.P[i] + h.p[i];
        if (wt + h.w[i] <= capacity) { wt += h.w[i]; pr += h.p[i]; }
    }
    h.cap = capacity;
    h.greedy = static_cast<int>(pr);
    h.work = n;
    if (id) *id = static_cast<int>(b->host.size());
    b->host.push_back(std::move(h));
    if (b->built) free_device(b);
    return GH_OK;
}

// Lays out the arena, uploads every instance and builds the task lists.
gh_status gh_batch_build(gh_batch* b, void* stream) {
    if (!b || b->host.empty() || b->host.size() > 65535) return GH_ERR_INVALID;  // fill grid: one y-row per instance
    free_device(b);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int B = b->batchSize;
    const int count = static_cast<int>(b->host.size());
    // sizes
    struct Lay { size_t items, status, state, cost, g, w, p, W, P, pool, freeList, ring, fifo; int bn, poolCap; unsigned long long ringCap; };
    std::vector<Lay> lay(count);
    size_t off = align_up(sizeof(Inst) * count, 256);
    size_t tasksOff = 0, nextOff = 0;
    std::vector<int> blocks(count, 1);
    for (int i = 0; i < count; ++i) {
        const HostInst& h = b->host[i];
        Lay& L = lay[i];
        long long keys;
        if (h.kind == GH_SEARCH_ASTAR) {
            const long long side = std::max(h.width, h.height);
            keys = std::max<long long>(64 * side, 16LL * B);
            const long long cells = static_cast<long long>(h.width) * h.height;
            blocks[i] = static_cast<int>(std::min<long long>(b->astarMaxBlocks, std::max<long long>(1, cells / b->astarCellsPerBlock)));
        } else {
            // batched branch-and-bound explores far more nodes than a
            // sequential one; pool slots must fit the key's 20 bits
            keys = std::min<long long>(1LL << 19, std::max<long long>({1LL << 16, 64LL * B, 256LL * static_cast<long long>(h.w.size())}));
            // a breadth-first frontier can be far wider: the FIFO orders get
            // the largest pool the key's slot bits allow, and a heap that can
            // take every pooled node back at a switch
            if (b->knapOrder != GH_KNAP_HEAP) keys = 1LL << kSlotBits;
        }
        L.bn = heap_nodes(keys, B);
        L.state = off; off = align_up(off + sizeof(gh::HeapState), 256);
        L.items = off; off = align_up(off + static_cast<size_t>(L.bn + 1) * B * 8, 256);
        L.status = off; off = align_up(off + static_cast<size_t>(L.bn + 2) * 4, 256);
        if (h.kind == GH_SEARCH_ASTAR) {
            const size_t cells = static_cast<size_t>(h.width) * h.height;
            L.cost = off; off = align_up(off + cells, 256);
            L.g = off; off = align_up(off + cells * 4, 256);
        } else {
            const int n = static_cast<int>(h.w.size());
            L.poolCap = b->knapOrder != GH_KNAP_HEAP ? (1 << kSlotBits) : std::min((L.bn + 1) * B + 4 * B, 1 << kSlotBits);
            L.w = off; off = align_up(off + n * 4, 256);
            L.p = off; off = align_up(off + n * 4, 256);
            L.W = off; off = align_up(off + (n + 1) * 8, 256);
            L.P = off; off = align_up(off + (n + 1) * 8, 256);
            L.pool = off; off = align_up(off + static_cast<size_t>(L.poolCap) * 16, 256);
            L.freeList = off; off = align_up(off + static_cast<size_t>(L.poolCap + B) * 4, 256);
            L.ringCap = 0;
            if (b->knapOrder != GH_KNAP_HEAP) {
                // every live node holds a pool slot, so a ring of the pool's
                // size takes all of them at a switch
                L.ringCap = 1;
                while (L.ringCap < static_cast<unsigned long long>(L.poolCap)) L.ringCap <<= 1;
                L.fifo = off; off = align_up(off + sizeof(gh::FifoState), 256);
                L.ring = off; off = align_up(off + static_cast<size_t>(L.ringCap) * 8, 256);
            }
        }
    }
    // task order: largest instances first, each instance's blocks together
    // (they start on one heap at about the same time)
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->host[x].work > b->host[y].work; });
    std::vector<int> batched;
    for (int i : order)
        for (int r = 0; r < blocks[i]; ++r) batched.push_back(i);
    b->ntasks = static_cast<int>(batched.size());
    b->segOff.assign(count, 0);
    b->segLen.assign(count, 0);
    std::vector<int> tasks(batched);
    for (int i = 0; i < count; ++i) {
        b->segOff[i] = static_cast<int>(tasks.size());
        b->segLen[i] = blocks[i];
        for (int r = 0; r < blocks[i]; ++r) tasks.push_back(i);
    }
    tasksOff = off; off = align_up(off + tasks.size() * 4, 256);
    nextOff = off; off = align_up(off + static_cast<size_t>(count + 1) * 4, 256);
    b->arenaBytes = off;
    if (cudaMalloc(&b->arena, off) != cudaSuccess) {
        cudaGetLastError();
        b->arena = nullptr;
        return GH_ERR_CUDA;
    }
    unsigned char* A = b->arena;
    b->insts = reinterpret_cast<Inst*>(A);
    b->tasks = reinterpret_cast<int*>(A + tasksOff);
    b->next = reinterpret_cast<int*>(A + nextOff);
    b->hinst.assign(count, Inst{});
    for (int i = 0; i < count; ++i) {
        const HostInst& h = b->host[i];
        const Lay& L = lay[i];
        Inst& d = b->hinst[i];
        std::memset(&d, 0, sizeof(d));
        d.kind = h.kind;
        d.blocks = blocks[i];
        d.batchNum = L.bn;
        d.items = reinterpret_cast<u64*>(A + L.items);
        d.status = reinterpret_cast<int*>(A + L.status);
        d.state = reinterpret_cast<gh::HeapState*>(A + L.state);
        if (h.kind == GH_SEARCH_ASTAR) {
            d.width = h.width;
            d.height = h.height;
            d.moves = h.moves;
            d.start = 0;
            d.goal = h.width * h.height - 1;
            d.cost = A + L.cost;
            d.g = reinterpret_cast<unsigned*>(A + L.g);
            if (cudaMemcpyAsync(A + L.cost, h.cost.data(), h.cost.size(), cudaMemcpyHostToDevice, s) != cudaSuccess) return GH_ERR_CUDA;
        } else {
            const int n = static_cast<int>(h.w.size());
            d.n = n;
            d.cap = h.cap;
            d.poolCap = L.poolCap;
            d.w = reinterpret_cast<const int*>(A + L.w);
            d.p = reinterpret_cast<const int*>(A + L.p);
            d.W = reinterpret_cast<const long long*>(A + L.W);
            d.P = reinterpret_cast<const long long*>(A + L.P);
            d.pool = reinterpret_cast<int4*>(A + L.pool);
            d.freeList = reinterpret_cast<int*>(A + L.freeList);
            d.greedy = h.greedy;
            d.order = b->knapOrder;
            d.switchCounter = b->switchCounter;
            if (L.ringCap) {
                d.ring = reinterpret_cast<u64*>(A + L.ring);
                d.fifo = reinterpret_cast<gh::FifoState*>(A + L.fifo);
                d.ringCap = L.ringCap;
            }
            if (cudaMemcpyAsync(A + L.w, h.w.data(), n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                cudaMemcpyAsync(A + L.p, h.p.data(), n * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                cudaMemcpyAsync(A + L.W, h.W.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                cudaMemcpyAsync(A + L.P, h.P.data(), (n + 1) * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
                return GH_ERR_CUDA;
        }
    }
    if (cudaMemcpyAsync(b->insts, b->hinst.data(), sizeof(Inst) * count, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(b->tasks, tasks.data(), tasks.size() * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GH_ERR_CUDA;
    b->grid = std::min(resident_blocks(b), b->ntasks);
    b->built = true;
    return GH_OK;
}

// mode GH_BATCH_PERSISTENT: one persistent launch for every instance;
// GH_BATCH_GRAPH: the same, replayed from a captured CUDA graph;
// GH_BATCH_PLAIN: one launch per instance, back to back.
gh_status gh_batch_run(gh_batch* b, int mode, void* stream) {
    gh::trace::Range range_("gh_batch_run");
    if (!b || !b->built) return GH_ERR_INVALID;
    if (mode != GH_BATCH_PERSISTENT && mode != GH_BATCH_GRAPH && mode != GH_BATCH_PLAIN) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (mode == GH_BATCH_GRAPH) {
        if (!b->graph) {
            if (!b->graphStream && cudaStreamCreateWithFlags(&b->graphStream, cudaStreamNonBlocking) != cudaSuccess)
                return GH_ERR_CUDA;
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(b->graphStream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return GH_ERR_CUDA;
            const long long before = gh::impl::g_launches.load();
            gh_status st = reset_and_run(b, GH_BATCH_PERSISTENT, b->graphStream);
            cudaError_t e = cudaStreamEndCapture(b->graphStream, &g);
            b->graphLaunches = gh::impl::g_launches.load() - before;
            gh::impl::g_launches.fetch_sub(b->graphLaunches);  // captured, not run
            if (st != GH_OK || e != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return st != GH_OK ? st : GH_ERR_CUDA;
            }
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { b->graph = nullptr; return GH_ERR_CUDA; }
        }
        if (cudaGraphLaunch(b->graph, s) != cudaSuccess) return GH_ERR_CUDA;
        gh::impl::g_launches.fetch_add(b->graphLaunches);  // fill, seed, search, collect
        return GH_OK;
    }
    return reset_and_run(b, mode, s);
}

gh_status gh_batch_results(gh_batch* b, long long* results, int* status, unsigned long long* stats, void* stream) {
    if (!b || !b->built) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int count = static_cast<int>(b->host.size());
    if (cudaMemcpyAsync(b->hinst.data(), b->insts, sizeof(Inst) * count, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GH_ERR_CUDA;
    gh_status worst = GH_OK;
    for (int i = 0; i < count; ++i) {
        const Inst& d = b->hinst[i];
        if (results) {
            if (d.kind == GH_SEARCH_ASTAR) results[i] = static_cast<long long>(static_cast<unsigned>(d.incumbent));
            else results[i] = d.incumbent;
        }
        if (status) status[i] = d.failed;
        if (stats) {
            stats[3 * i] = d.pops;
            stats[3 * i + 1] = d.expanded;
            stats[3 * i + 2] = d.inserted;
        }
        if (d.failed && worst == GH_OK) worst = static_cast<gh_status>(d.failed);
    }
    return worst;
}

gh_status gh_batch_knapsack_switches(gh_batch* b, int* switches, void* stream) {
    if (!b || !b->built || !switches) return GH_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int count = static_cast<int>(b->host.size());
    if (cudaMemcpyAsync(b->hinst.data(), b->insts, sizeof(Inst) * count, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GH_ERR_CUDA;
    for (int i = 0; i < count; ++i) switches[i] = b->hinst[i].kind == GH_SEARCH_KNAPSACK ? b->hinst[i].switches : 0;
    return GH_OK;
}

gh_status gh_batch_info(gh_batch* b, int* count, int* tasks, int* grid, int* threads, long long* arena_bytes) {
    if (!b) return GH_ERR_INVALID;
    if (count) *count = static_cast<int>(b->host.size());
    if (tasks) *tasks = b->ntasks;
    if (grid) *grid = b->built ? b->grid : resident_blocks(b);
    if (threads) *threads = threads_for(b);
    if (arena_bytes) *arena_bytes = static_cast<long long>(b->arenaBytes);
    return GH_OK;
}

}  // extern "C"

namespace {

gh_status reset_and_run(gh_batch* b, int mode, cudaStream_t s) {
    const int count = static_cast<int>(b->host.size());
    if (cudaMemsetAsync(b->next, 0, static_cast<size_t>(count + 1) * 4, s) != cudaSuccess) return GH_ERR_CUDA;
    if (search_fill(b->insts, nullptr, count, b->batchSize, s) != cudaSuccess ||
        search_seed(b->insts, nullptr, count, s) != cudaSuccess)
        return GH_ERR_CUDA;
    if (mode == GH_BATCH_PLAIN) {
        // an event before each instance's launch and one after the last, so
        // that gh_batch_plain_times can give every instance its own time
        while (static_cast<int>(b->plainEv.size()) < count + 1) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return GH_ERR_CUDA;
            b->plainEv.push_back(e);
        }
        for (int i = 0; i < count; ++i) {
            if (cudaEventRecord(b->plainEv[i], s) != cudaSuccess) return GH_ERR_CUDA;
            if (launch(b, b->tasks + b->segOff[i], b->segLen[i], b->next + 1 + i, b->segLen[i], s) != cudaSuccess)
                return GH_ERR_CUDA;
        }
        if (cudaEventRecord(b->plainEv[count], s) != cudaSuccess) return GH_ERR_CUDA;
    } else {
        if (launch(b, b->tasks, b->ntasks, b->next, b->grid, s) != cudaSuccess) return GH_ERR_CUDA;
    }
    return search_collect(b->insts, nullptr, count, 1, b->batchSize, s) == cudaSuccess ? GH_OK : GH_ERR_CUDA;
}

}  // namespace

// ---------------------------------------------------------------------- workload generator
namespace {
inline u64 host_mix64(u64 z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
}  // namespace

extern "C" gh_status gh_gen_grid(int width, int height, unsigned long long seed, int obstacle_per_mille,
                                 unsigned char* out_host, int threads) {
    if (width < 1 || height < 1 || !out_host || obstacle_per_mille < 0 || obstacle_per_mille > 1000) return GH_ERR_INVALID;
    const long long cells = static_cast<long long>(width) * height;
    if (threads < 1) threads = 1;
    auto fill = [=](long long lo, long long hi) {
        for (long long i = lo; i < hi; ++i) {
            const u64 r = host_mix64(seed + (static_cast<u64>(i) + 1) * 0x9e3779b97f4a7c15ULL);
            const bool blocked = static_cast<int>((r >> 32) % 1000) < obstacle_per_mille;
            const unsigned char c = static_cast<unsigned char>(1 + (r & 0xffffffffu) % 9);
            out_host[i] = blocked && i != 0 && i != cells - 1 ? 0 : c;
        }
    };
    std::vector<std::thread> pool;
    const long long per = (cells + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const long long lo = t * per, hi = std::min(cells, lo + per);
        if (lo < hi) pool.emplace_back(fill, lo, hi);
    }
    for (auto& th : pool) th.join();
    return GH_OK;
}
