// Served queries: a continuous-batching loop of SSSP and grid A* queries
// over resident graphs and maps (gh_serve_*, declared in gpuheap.h).
//
// Each admitted query owns a slot in a device array of instances and one
// block of a device arena holding its heap (u64 keys, partial buffer), its
// heap words and its distance array; a host-side first-fit allocator hands
// the blocks out and takes them back when the query finishes, so admission
// is by free memory.  One step admits what fits, resets and seeds the new
// queries, runs one persistent launch over every admitted query (each block
// takes at most batches_per_step batches of a query, then moves on, so a
// query's heap carries its state into the next step), and collects the
// queries whose heaps ran empty.  The per-query work is the search loop of
// search_kernels.cuh (the reference's per-query kernels:
// applications/sssp_longfei_new/sssp.cu:19-132, artifacts/astar/
// pq_model.cuh:299-371).
//
// The device loop (gh_serve_start / gh_serve_poll / gh_serve_stop) moves
// admission, the steps and collection onto the device: the host writes
// requests into a ring in pinned host memory and reads completions from
// another; one resident launch of the search kernel admits, sets up, runs,
// collects and frees queries (search_kernels.cuh, namespace sv) and leaves
// after an idle limit or on the host's stop word.  It replaces the host
// relaunch loop of the reference's A* driver (artifacts/astar/
// astar_main.cu:127-179), which launches and synchronizes once per round.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <deque>
#include <iterator>
#include <map>
#include <new>
#include <vector>

#include "gpuheap.h"
#include "heap_kernels.cuh"
#include "search_common.cuh"
#include "trace.cuh"

using namespace gh::search;

namespace {

struct Dataset {
    int kind;  // GH_SEARCH_SSSP graph or GH_SEARCH_ASTAR map
    int n = 0, width = 0, height = 0;
    long long m = 0;  // edges of a graph
    const long long* rowptr = nullptr;
    const int* col = nullptr;
    const unsigned* w = nullptr;
    const unsigned char* cost = nullptr;
    int moves = 4;  // A* maps: 4 (cost grid) or 8 (the reference's bitmap model)
};

struct Query {
    int kind, dataset, a, b;
    int state = 0;  // 0 queued, 1 admitted, 2 finished, 3 failed
    int slot = -1;
    size_t off = 0, bytes = 0;
    int bn = 0, blocks = 1;
    unsigned long long r0 = 0, r1 = 0;
    long long finishStep = -1;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int pow2_nodes(long long keys, int B) {
    const long long nodes = (keys + B - 1) / B;
    int bn = 1;
    while (bn < nodes) bn <<= 1;
    return bn;
}

}  // namespace

struct gh_server {
    SearchConfig cfg{};
    int maxSlots = 0, batchesPerStep = 0, grid = 0;
    long long ssspPerBlock = 1 << 15, astarPerBlock = 1 << 18;
    int ssspMaxBlocks = 24, astarMaxBlocks = 8;  // more blocks on one SSSP heap only add re-expansions
    unsigned char* arena = nullptr;
    size_t arenaBytes = 0, used = 0;
    std::map<size_t, size_t> freeBlocks;  // offset -> bytes, coalesced
    unsigned char* ctlMem = nullptr;      // instances, tasks, ids, counter
    Inst* insts = nullptr;
    int* tasks = nullptr;
    int* ids = nullptr;
    int* next = nullptr;
    int maxTasks = 0;
    std::vector<Inst> hinst;
    std::vector<long long> slotQuery;
    std::vector<Dataset> data;
    std::vector<Query> queries;
    std::deque<long long> waiting;
    std::vector<long long> finished;
    long long steps = 0;
    int* hostTasks = nullptr;  // pinned
    int* hostIds = nullptr;    // pinned
    // device loop
    bool resident = false, running = false, paused = false;
    cudaStream_t loopStream = nullptr;
    cudaEvent_t loopDone = nullptr;
    long long idleNs = 100000000LL;
    int ringCap = 4096, tokensPerQuery = 1;
    unsigned char* pinned = nullptr;  // request ring, completion ring, host words (mapped)
    ServeReq* ring = nullptr;
    ServeDone* done = nullptr;
    ServeHost* hostw = nullptr;
    unsigned char* loopMem = nullptr;  // ServeDev and its arrays (device)
    ServeDev* dev = nullptr;
    unsigned long long posted = 0, consumed = 0;
    long long launches = 0;
};

namespace {

bool arena_alloc(gh_server* s, size_t bytes, size_t* off) {
    for (auto it = s->freeBlocks.begin(); it != s->freeBlocks.end(); ++it) {
        if (it->second >= bytes) {
            *off = it->first;
            const size_t rest = it->second - bytes;
            const size_t at = it->first + bytes;
            s->freeBlocks.erase(it);
            if (rest) s->freeBlocks[at] = rest;
            s->used += bytes;
            return true;
        }
    }
    return false;
}

void arena_free(gh_server* s, size_t off, size_t bytes) {
    auto it = s->freeBlocks.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != s->freeBlocks.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        s->freeBlocks.erase(nx);
    }
    if (it != s->freeBlocks.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            s->freeBlocks.erase(it);
        }
    }
    s->used -= bytes;
}

// Device bytes, heap nodes and blocks per step of a query.
void size_query(const gh_server* s, Query& q) {
    const int B = s->cfg.batchSize;
    const Dataset& d = s->data[q.dataset];
    long long keys, dist;
    if (q.kind == GH_SEARCH_SSSP) {
        // the standalone SSSP's bound: label correction can hold several
        // keys per vertex (half the edges on R-MAT graphs)
        keys = std::max({4LL * d.n, d.m / 2, 16LL * B});
        dist = d.n;
        q.blocks = static_cast<int>(std::min<long long>(s->ssspMaxBlocks, std::max<long long>(1, d.n / s->ssspPerBlock)));
    } else {
        const long long side = std::max(d.width, d.height);
        keys = std::max<long long>(64 * side, 16LL * B);
        dist = static_cast<long long>(d.width) * d.height;
        q.blocks = static_cast<int>(std::min<long long>(s->astarMaxBlocks, std::max<long long>(1, dist / s->astarPerBlock)));
    }
    q.bn = pow2_nodes(keys, B);
    q.bytes = query_layout(q.bn, B, dist).bytes;
}

// Instance record of an admitted query at arena offset q.off.
Inst make_inst(gh_server* s, const Query& q) {
    const int B = s->cfg.batchSize;
    const Dataset& d = s->data[q.dataset];
    unsigned char* p = s->arena + q.off;
    const QueryLayout L = query_layout(q.bn, B, q.kind == GH_SEARCH_SSSP ? d.n : static_cast<long long>(d.width) * d.height);
    Inst in;
    std::memset(&in, 0, sizeof(in));
    in.kind = q.kind;
    in.blocks = q.blocks;
    in.batchNum = q.bn;
    in.state = reinterpret_cast<gh::HeapState*>(p);
    in.items = reinterpret_cast<u64*>(p + L.items);
    in.status = reinterpret_cast<int*>(p + L.status);
    in.g = reinterpret_cast<unsigned*>(p + L.g);
    if (q.kind == GH_SEARCH_SSSP) {
        in.nv = d.n;
        in.source = q.a;
        in.rowptr = d.rowptr;
        in.col = d.col;
        in.wt = d.w;
    } else {
        in.width = d.width;
        in.height = d.height;
        in.cost = d.cost;
        in.moves = d.moves;
        in.start = q.a;
        in.goal = q.b;
    }
    return in;
}

#define GH_SCUDA(call)                                 \
    do {                                               \
        if ((call) != cudaSuccess) return GH_ERR_CUDA; \
    } while (0)

// ------------------------------------------------------------ device loop

// Writes waiting queries into the request ring while it has room: a record
// may be written again once its completion has been read, so at most
// ringCap queries are between posting and reading their completion (the
// device's pending array and the completion ring have ringCap entries).
void post_requests(gh_server* s) {
    const int B = s->cfg.batchSize;
    while (!s->waiting.empty() && s->posted - s->consumed < static_cast<unsigned long long>(s->ringCap)) {
        const long long id = s->waiting.front();
        s->waiting.pop_front();
        Query& q = s->queries[id];
        const Dataset& d = s->data[q.dataset];
        ServeReq* r = s->ring + (s->posted & static_cast<unsigned long long>(s->ringCap - 1));
        r->qid = id;
        r->kind = q.kind;
        r->a = q.a;
        r->b = q.b;
        r->blocks = q.blocks;
        r->bn = q.bn;
        r->n = d.n;
        r->width = d.width;
        r->height = d.height;
        r->bytes = query_layout(q.bn, B, q.kind == GH_SEARCH_SSSP ? d.n : static_cast<long long>(d.width) * d.height).bytes;
        r->off = 0;
        r->rowptr = d.rowptr;
        r->col = d.col;
        r->w = d.w;
        r->cost = d.cost;
        r->moves = d.moves;
        __atomic_store_n(&r->seq, s->posted + 1, __ATOMIC_RELEASE);
        ++s->posted;
        q.state = 1;
    }
}

gh_status launch_loop(gh_server* s) {
    GH_SCUDA(cudaMemsetAsync(&s->dev->exit, 0, sizeof(int), s->loopStream));
    GH_SCUDA(cudaMemsetAsync(&s->dev->idleSince, 0, sizeof(unsigned long long), s->loopStream));
    GH_SCUDA(cudaMemsetAsync(&s->dev->admitAt, 0, sizeof(unsigned long long), s->loopStream));
    GH_SCUDA(search_launch(s->cfg, SearchArgs{s->insts, nullptr, 0, nullptr, s->batchesPerStep, s->dev}, s->grid,
                           s->loopStream));
    GH_SCUDA(cudaEventRecord(s->loopDone, s->loopStream));
    s->running = true;
    ++s->launches;
    return GH_OK;
}

// The stop word makes the admitting block set the exit word; blocks leave
// after their current stint, with every unfinished query's tokens back in
// the queue, so a later launch resumes them.
gh_status stop_loop(gh_server* s) {
    __atomic_store_n(&s->hostw->stop, 1, __ATOMIC_RELEASE);
    const cudaError_t e = cudaEventSynchronize(s->loopDone);
    __atomic_store_n(&s->hostw->stop, 0, __ATOMIC_RELEASE);
    s->running = false;
    return e == cudaSuccess ? GH_OK : GH_ERR_CUDA;
}

gh_status loop_error(const gh_server* s) {
    const int err = __atomic_load_n(&s->hostw->err, __ATOMIC_ACQUIRE);
    return err == kServeOk ? GH_OK : err == kServeErrWait || err == kServeErrLock ? GH_ERR_TIMEOUT : GH_ERR_STATE;
}

// One-time setup of the device loop: the pinned rings and host words, the
// loop's device state (free slots, one free range over the whole arena,
// the token queue's cells at their first lap), its stream and event.
gh_status init_loop(gh_server* s) {
    const size_t ringBytes = sizeof(ServeReq) * s->ringCap, doneBytes = sizeof(ServeDone) * s->ringCap;
    if (cudaHostAlloc(&s->pinned, ringBytes + doneBytes + sizeof(ServeHost), cudaHostAllocMapped) != cudaSuccess) {
        cudaGetLastError();
        s->pinned = nullptr;
        return GH_ERR_CUDA;
    }
    std::memset(s->pinned, 0, ringBytes + doneBytes + sizeof(ServeHost));
    s->ring = reinterpret_cast<ServeReq*>(s->pinned);
    s->done = reinterpret_cast<ServeDone*>(s->pinned + ringBytes);
    s->hostw = reinterpret_cast<ServeHost*>(s->pinned + ringBytes + doneBytes);
    void* dp = nullptr;
    GH_SCUDA(cudaHostGetDevicePointer(&dp, s->pinned, 0));
    unsigned char* devPinned = static_cast<unsigned char*>(dp);

    s->tokensPerQuery = std::min(1024, s->grid);
    unsigned long long cells = 1;
    while (cells < static_cast<unsigned long long>(s->maxSlots) * s->tokensPerQuery + 1) cells <<= 1;
    const int maxRanges = s->maxSlots + 2;
    const size_t devBytes = align_up(sizeof(ServeDev), 256), pendBytes = align_up(sizeof(ServeReq) * s->ringCap, 256),
                 slotBytes = align_up(sizeof(ServeReq) * s->maxSlots, 256),
                 freeBytes = align_up(sizeof(int) * s->maxSlots, 256),
                 rangeBytes = align_up(sizeof(ServeRange) * maxRanges, 256), cellBytes = sizeof(ServeCell) * cells;
    const size_t total = devBytes + pendBytes + slotBytes + freeBytes + rangeBytes + cellBytes;
    if (cudaMalloc(&s->loopMem, total) != cudaSuccess) {
        cudaGetLastError();
        s->loopMem = nullptr;
        return GH_ERR_CUDA;
    }
    std::vector<unsigned char> img(total, 0);
    ServeDev* d = reinterpret_cast<ServeDev*>(img.data());
    unsigned char* base = s->loopMem;
    size_t at = devBytes;
    d->pend = reinterpret_cast<ServeReq*>(base + at);
    at += pendBytes;
    d->slotReq = reinterpret_cast<ServeReq*>(base + at);
    at += slotBytes;
    d->freeSlots = reinterpret_cast<int*>(base + at);
    int* hostFree = reinterpret_cast<int*>(img.data() + at);
    for (int i = 0; i < s->maxSlots; ++i) hostFree[i] = s->maxSlots - 1 - i;  // slot 0 is taken first
    at += freeBytes;
    d->ranges = reinterpret_cast<ServeRange*>(base + at);
    ServeRange* hostRanges = reinterpret_cast<ServeRange*>(img.data() + at);
    hostRanges[0].off = 0;
    hostRanges[0].len = s->arenaBytes;
    at += rangeBytes;
    d->cells = reinterpret_cast<ServeCell*>(base + at);
    ServeCell* hostCells = reinterpret_cast<ServeCell*>(img.data() + at);
    for (unsigned long long i = 0; i < cells; ++i) hostCells[i].seq = i;
    d->ring = reinterpret_cast<ServeReq*>(devPinned);
    d->done = reinterpret_cast<ServeDone*>(devPinned + ringBytes);
    d->host = reinterpret_cast<ServeHost*>(devPinned + ringBytes + doneBytes);
    d->insts = s->insts;
    d->arena = s->arena;
    d->arenaBytes = s->arenaBytes;
    d->cellMask = cells - 1;
    d->ringCap = s->ringCap;
    d->maxSlots = s->maxSlots;
    d->maxRanges = maxRanges;
    d->batchSize = s->cfg.batchSize;
    d->nfree = s->maxSlots;
    d->nranges = 1;
    d->idleNs = s->idleNs;
    d->waitNs = 2000000000LL;
    d->stallNs = 60000000000LL;
    GH_SCUDA(cudaMemcpy(s->loopMem, img.data(), total, cudaMemcpyHostToDevice));
    s->dev = reinterpret_cast<ServeDev*>(s->loopMem);
    GH_SCUDA(cudaStreamCreateWithFlags(&s->loopStream, cudaStreamNonBlocking));
    GH_SCUDA(cudaEventCreateWithFlags(&s->loopDone, cudaEventDisableTiming));
    return GH_OK;
}

}  // namespace

extern "C" {

gh_status gh_serve_create(gh_server** out, long long arena_bytes, int max_slots, int batch_size, int variant,
                          int batches_per_step) {
    if (!out) return GH_ERR_INVALID;
    *out = nullptr;
    if (batch_size < 32 || batch_size > 1024 || (batch_size & (batch_size - 1))) return GH_ERR_INVALID;
    if (variant != GH_TOPDOWN && variant != GH_BOTTOMUP) return GH_ERR_INVALID;
    if (max_slots < 1 || max_slots > 4096 || batches_per_step < 1 || arena_bytes < 0) return GH_ERR_INVALID;
    gh_server* s = new (std::nothrow) gh_server();
    if (!s) return GH_ERR_INVALID;
    auto fail = [&](gh_status st) { gh_serve_destroy(s); return st; };
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&s->cfg.numSMs, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return fail(GH_ERR_CUDA);
    s->cfg.batchSize = batch_size;
    s->cfg.variant = variant;
    s->cfg.threads = 0;
    s->cfg.timeoutNs = 2000000000LL;
    s->maxSlots = max_slots;
    s->batchesPerStep = batches_per_step;
    if (arena_bytes == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return fail(GH_ERR_CUDA);
        arena_bytes = static_cast<long long>(fr / 10 * 6);
    }
    s->arenaBytes = align_up(static_cast<size_t>(arena_bytes), 256);
    if (cudaMalloc(&s->arena, s->arenaBytes) != cudaSuccess) {
        cudaGetLastError();
        s->arena = nullptr;
        return fail(GH_ERR_CUDA);
    }
    s->freeBlocks[0] = s->arenaBytes;
    s->maxTasks = max_slots * 1024;
    const size_t instBytes = align_up(sizeof(Inst) * max_slots, 256);
    const size_t taskBytes = align_up(sizeof(int) * s->maxTasks, 256);
    const size_t idBytes = align_up(sizeof(int) * max_slots, 256);
    if (cudaMalloc(&s->ctlMem, instBytes + taskBytes + idBytes + 256) != cudaSuccess) {
        cudaGetLastError();
        s->ctlMem = nullptr;
        return fail(GH_ERR_CUDA);
    }
    s->insts = reinterpret_cast<Inst*>(s->ctlMem);
    s->tasks = reinterpret_cast<int*>(s->ctlMem + instBytes);
    s->ids = reinterpret_cast<int*>(s->ctlMem + instBytes + taskBytes);
    s->next = reinterpret_cast<int*>(s->ctlMem + instBytes + taskBytes + idBytes);
    if (cudaMallocHost(&s->hostTasks, sizeof(int) * s->maxTasks) != cudaSuccess ||
        cudaMallocHost(&s->hostIds, sizeof(int) * max_slots) != cudaSuccess)
        return fail(GH_ERR_CUDA);
    s->hinst.assign(max_slots, Inst{});
    s->slotQuery.assign(max_slots, -1);
    s->grid = search_resident_blocks(s->cfg);
    *out = s;
    return GH_OK;
}

gh_status gh_serve_destroy(gh_server* s) {
    if (!s) return GH_ERR_INVALID;
    if (s->running) stop_loop(s);
    if (s->loopDone) cudaEventDestroy(s->loopDone);
    if (s->loopStream) cudaStreamDestroy(s->loopStream);
    if (s->loopMem) cudaFree(s->loopMem);
    if (s->pinned) cudaFreeHost(s->pinned);
    if (s->arena) cudaFree(s->arena);
    if (s->ctlMem) cudaFree(s->ctlMem);
    if (s->hostTasks) cudaFreeHost(s->hostTasks);
    if (s->hostIds) cudaFreeHost(s->hostIds);
    delete s;
    return GH_OK;
}

gh_status gh_serve_set_blocks(gh_server* s, long long vertices_per_block, int sssp_max_blocks, long long cells_per_block,
                              int astar_max_blocks) {
    if (!s || vertices_per_block < 1 || cells_per_block < 1 || sssp_max_blocks < 1 || sssp_max_blocks > 1024 ||
        astar_max_blocks < 1 || astar_max_blocks > 1024)
        return GH_ERR_INVALID;
    s->ssspPerBlock = vertices_per_block;
    s->ssspMaxBlocks = sssp_max_blocks;
    s->astarPerBlock = cells_per_block;
    s->astarMaxBlocks = astar_max_blocks;
    return GH_OK;
}

gh_status gh_serve_add_graph(gh_server* s, int n, const long long* rowptr_dev, const int* col_dev,
                             const unsigned* w_dev, int* id) {
    if (!s || n < 1 || !rowptr_dev || !col_dev || !w_dev) return GH_ERR_INVALID;
    Dataset d;
    d.kind = GH_SEARCH_SSSP;
    d.n = n;
    if (cudaMemcpy(&d.m, rowptr_dev + n, sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess) return GH_ERR_CUDA;
    if (d.m < 0) return GH_ERR_INVALID;
    d.rowptr = rowptr_dev;
    d.col = col_dev;
    d.w = w_dev;
    if (id) *id = static_cast<int>(s->data.size());
    s->data.push_back(d);
    return GH_OK;
}

gh_status gh_serve_add_map(gh_server* s, int width, int height, const unsigned char* cost_dev, int* id) {
    if (!s || width < 1 || height < 1 || !cost_dev || static_cast<long long>(width) * height > (1LL << 30))
        return GH_ERR_INVALID;
    Dataset d;
    d.kind = GH_SEARCH_ASTAR;
    d.width = width;
    d.height = height;
    d.cost = cost_dev;
    if (id) *id = static_cast<int>(s->data.size());
    s->data.push_back(d);
    return GH_OK;
}

gh_status gh_serve_add_bitmap(gh_server* s, int width, int height, const unsigned char* open_dev, int* id) {
    const gh_status st = gh_serve_add_map(s, width, height, open_dev, id);
    if (st == GH_OK) s->data.back().moves = 8;
    return st;
}

gh_status gh_serve_submit(gh_server* s, int kind, int dataset, int a, int b, long long* query) {
    if (!s || dataset < 0 || dataset >= static_cast<int>(s->data.size())) return GH_ERR_INVALID;
    const Dataset& d = s->data[dataset];
    if (kind != d.kind) return GH_ERR_INVALID;
    if (kind == GH_SEARCH_SSSP && (a < 0 || a >= d.n)) return GH_ERR_INVALID;
    const long long cells = static_cast<long long>(d.width) * d.height;
    if (kind == GH_SEARCH_ASTAR && (a < 0 || a >= cells || b < 0 || b >= cells)) return GH_ERR_INVALID;
    Query q;
    q.kind = kind;
    q.dataset = dataset;
    q.a = a;
    q.b = b;
    size_query(s, q);
    if (q.bytes > s->arenaBytes) return GH_ERR_CAPACITY;
    if (s->resident) q.blocks = std::min(q.blocks, s->tokensPerQuery);
    const long long id = static_cast<long long>(s->queries.size());
    s->queries.push_back(q);
    s->waiting.push_back(id);
    if (query) *query = id;
    if (s->resident) post_requests(s);
    return GH_OK;
}

gh_status gh_serve_step(gh_server* s, void* stream, int* finished, int* active, int* queued) {
    gh::trace::Range range_("gh_serve_step");
    if (!s || s->resident) return GH_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    s->finished.clear();
    // admission, in arrival order, skipping queries that do not fit yet
    std::vector<int> fresh;
    for (auto it = s->waiting.begin(); it != s->waiting.end();) {
        int slot = -1;
        for (int i = 0; i < s->maxSlots; ++i)
            if (s->slotQuery[i] < 0) { slot = i; break; }
        if (slot < 0) break;
        Query& q = s->queries[*it];
        size_t off = 0;
        if (!arena_alloc(s, q.bytes, &off)) { ++it; continue; }
        q.off = off;
        q.slot = slot;
        q.state = 1;
        s->slotQuery[slot] = *it;
        s->hinst[slot] = make_inst(s, q);
        GH_SCUDA(cudaMemcpyAsync(s->insts + slot, &s->hinst[slot], sizeof(Inst), cudaMemcpyHostToDevice, st));
        fresh.push_back(slot);
        it = s->waiting.erase(it);
    }
    if (!fresh.empty()) {
        for (size_t i = 0; i < fresh.size(); ++i) s->hostIds[i] = fresh[i];
        GH_SCUDA(cudaMemcpyAsync(s->ids, s->hostIds, sizeof(int) * fresh.size(), cudaMemcpyHostToDevice, st));
        GH_SCUDA(search_fill(s->insts, s->ids, static_cast<int>(fresh.size()), s->cfg.batchSize, st));
        GH_SCUDA(search_seed(s->insts, s->ids, static_cast<int>(fresh.size()), st));
        GH_SCUDA(cudaStreamSynchronize(st));  // hostIds and ids are rewritten below
    }
    // one launch over every admitted query: its blocks, largest first
    std::vector<int> act;
    for (int i = 0; i < s->maxSlots; ++i)
        if (s->slotQuery[i] >= 0) act.push_back(i);
    std::stable_sort(act.begin(), act.end(), [&](int x, int y) {
        return s->queries[s->slotQuery[x]].bytes > s->queries[s->slotQuery[y]].bytes;
    });
    int nt = 0;
    for (int slot : act)
        for (int r = 0; r < s->queries[s->slotQuery[slot]].blocks && nt < s->maxTasks; ++r) s->hostTasks[nt++] = slot;
    if (nt > 0) {
        for (size_t i = 0; i < act.size(); ++i) s->hostIds[i] = act[i];
        GH_SCUDA(cudaMemcpyAsync(s->tasks, s->hostTasks, sizeof(int) * nt, cudaMemcpyHostToDevice, st));
        GH_SCUDA(cudaMemcpyAsync(s->ids, s->hostIds, sizeof(int) * act.size(), cudaMemcpyHostToDevice, st));
        GH_SCUDA(cudaMemsetAsync(s->next, 0, sizeof(int), st));
        GH_SCUDA(search_launch(s->cfg, SearchArgs{s->insts, s->tasks, nt, s->next, s->batchesPerStep, nullptr},
                               std::min(s->grid, nt), st));
        GH_SCUDA(search_collect(s->insts, s->ids, static_cast<int>(act.size()), 0, s->cfg.batchSize, st));
        GH_SCUDA(cudaMemcpyAsync(s->hinst.data(), s->insts, sizeof(Inst) * s->maxSlots, cudaMemcpyDeviceToHost, st));
        GH_SCUDA(cudaStreamSynchronize(st));
        ++s->steps;
        for (int slot : act) {
            const Inst& in = s->hinst[slot];
            if (!in.done) continue;
            Query& q = s->queries[s->slotQuery[slot]];
            q.state = in.failed ? 3 : 2;
            if (in.failed) {
                q.r0 = 0;
                q.r1 = static_cast<unsigned long long>(in.failed);
            } else if (q.kind == GH_SEARCH_SSSP) {
                q.r0 = in.reached;
                q.r1 = in.distSum;
            } else {
                q.r0 = static_cast<unsigned>(in.incumbent);
                q.r1 = 0;
            }
            q.finishStep = s->steps;
            s->finished.push_back(s->slotQuery[slot]);
            arena_free(s, q.off, q.bytes);
            s->slotQuery[slot] = -1;
        }
    }
    int nact = 0;
    for (int i = 0; i < s->maxSlots; ++i) nact += s->slotQuery[i] >= 0;
    if (finished) *finished = static_cast<int>(s->finished.size());
    if (active) *active = nact;
    if (queued) *queued = static_cast<int>(s->waiting.size());
    return GH_OK;
}

gh_status gh_serve_result(gh_server* s, long long q, int* state, unsigned long long* r0, unsigned long long* r1,
                          long long* finish_step) {
    if (!s || q < 0 || q >= static_cast<long long>(s->queries.size())) return GH_ERR_INVALID;
    const Query& x = s->queries[q];
    if (state) *state = x.state;
    if (r0) *r0 = x.r0;
    if (r1) *r1 = x.r1;
    if (finish_step) *finish_step = x.finishStep;
    return GH_OK;
}

gh_status gh_serve_finished(gh_server* s, long long* ids, int max_ids, int* count) {
    if (!s || (max_ids > 0 && !ids)) return GH_ERR_INVALID;
    const int n = std::min<int>(max_ids, static_cast<int>(s->finished.size()));
    for (int i = 0; i < n; ++i) ids[i] = s->finished[i];
    if (count) *count = static_cast<int>(s->finished.size());
    return GH_OK;
}

gh_status gh_serve_info(gh_server* s, long long* used_bytes, long long* free_bytes, int* slots_used, long long* steps) {
    if (!s) return GH_ERR_INVALID;
    if (s->resident) {
        const long long used = __atomic_load_n(&s->hostw->usedBytes, __ATOMIC_ACQUIRE);
        if (used_bytes) *used_bytes = used;
        if (free_bytes) *free_bytes = static_cast<long long>(s->arenaBytes) - used;
        if (slots_used) *slots_used = __atomic_load_n(&s->hostw->slotsUsed, __ATOMIC_ACQUIRE);
        if (steps) *steps = s->launches;
        return GH_OK;
    }
    if (used_bytes) *used_bytes = static_cast<long long>(s->used);
    if (free_bytes) *free_bytes = static_cast<long long>(s->arenaBytes - s->used);
    if (slots_used) {
        int n = 0;
        for (long long q : s->slotQuery) n += q >= 0;
        *slots_used = n;
    }
    if (steps) *steps = s->steps;
    return GH_OK;
}


gh_status gh_serve_start(gh_server* s, int idle_ms) {
    gh::trace::Range range_("gh_serve_start");
    if (!s || idle_ms < 1 || idle_ms > 600000) return GH_ERR_INVALID;
    if (s->resident) {
        if (s->running) return GH_ERR_INVALID;
        if (loop_error(s) != GH_OK) return GH_ERR_STATE;
        s->paused = false;
        return GH_OK;  // resumes: the next gh_serve_poll launches the loop when there is work
    }
    // the device loop takes over the whole arena: no query may be in the host steps
    for (long long q : s->slotQuery)
        if (q >= 0) return GH_ERR_INVALID;
    if (!s->waiting.empty()) return GH_ERR_INVALID;
    s->idleNs = static_cast<long long>(idle_ms) * 1000000LL;
    const gh_status st = init_loop(s);
    if (st != GH_OK) return st;
    s->resident = true;
    return GH_OK;
}

gh_status gh_serve_poll(gh_server* s, int* finished, int* active, int* queued) {
    gh::trace::Range range_("gh_serve_poll");
    if (!s || !s->resident) return GH_ERR_INVALID;
    s->finished.clear();
    const unsigned long long mask = static_cast<unsigned long long>(s->ringCap - 1);
    for (;;) {
        const ServeDone* r = s->done + (s->consumed & mask);
        if (__atomic_load_n(&r->seq, __ATOMIC_ACQUIRE) != s->consumed + 1) break;
        const long long id = r->qid;
        if (id >= 0 && id < static_cast<long long>(s->queries.size())) {
            Query& q = s->queries[id];
            q.state = r->state;
            q.r0 = r->r0;
            q.r1 = r->state == 3 ? static_cast<unsigned long long>(r->failed) : r->r1;
            q.finishStep = static_cast<long long>(s->consumed) + 1;  // completion order
            s->finished.push_back(id);
        }
        ++s->consumed;
    }
    post_requests(s);
    if (s->running) {
        const cudaError_t e = cudaEventQuery(s->loopDone);
        if (e == cudaSuccess) s->running = false;
        else if (e != cudaErrorNotReady) return GH_ERR_CUDA;
    }
    const gh_status err = loop_error(s);
    if (err != GH_OK) return err;
    if (!s->running && !s->paused && s->posted > s->consumed) {
        const gh_status st = launch_loop(s);
        if (st != GH_OK) return st;
    }
    if (finished) *finished = static_cast<int>(s->finished.size());
    const int act = __atomic_load_n(&s->hostw->active, __ATOMIC_ACQUIRE);
    const unsigned long long taken = __atomic_load_n(&s->hostw->reqTaken, __ATOMIC_ACQUIRE);
    if (active) *active = act;
    if (queued)
        *queued = static_cast<int>(s->waiting.size() + (s->posted - taken)) + __atomic_load_n(&s->hostw->pending, __ATOMIC_ACQUIRE);
    return GH_OK;
}

gh_status gh_serve_stop(gh_server* s) {
    gh::trace::Range range_("gh_serve_stop");
    if (!s || !s->resident) return GH_ERR_INVALID;
    s->paused = true;
    if (s->running) {
        const gh_status st = stop_loop(s);
        if (st != GH_OK) return st;
    }
    return loop_error(s);
}

}  // extern "C"
