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
#include "search_kernels.cuh"
#include "trace.cuh"

namespace {

struct Dataset {
    int kind;  // GH_SEARCH_SSSP graph or GH_SEARCH_ASTAR map
    int n = 0, width = 0, height = 0;
    const long long* rowptr = nullptr;
    const int* col = nullptr;
    const unsigned* w = nullptr;
    const unsigned char* cost = nullptr;
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
        keys = std::max<long long>(4LL * d.n, 16LL * B);
        dist = d.n;
        q.blocks = static_cast<int>(std::min<long long>(s->ssspMaxBlocks, std::max<long long>(1, d.n / s->ssspPerBlock)));
    } else {
        const long long side = std::max(d.width, d.height);
        keys = std::max<long long>(64 * side, 16LL * B);
        dist = static_cast<long long>(d.width) * d.height;
        q.blocks = static_cast<int>(std::min<long long>(s->astarMaxBlocks, std::max<long long>(1, dist / s->astarPerBlock)));
    }
    q.bn = pow2_nodes(keys, B);
    size_t b = align_up(sizeof(gh::HeapState), 256);
    b += align_up(static_cast<size_t>(q.bn + 1) * B * 8, 256);
    b += align_up(static_cast<size_t>(q.bn + 2) * 4, 256);
    b += align_up(static_cast<size_t>(dist) * 4, 256);
    q.bytes = b;
}

// Instance record of an admitted query at arena offset q.off.
Inst make_inst(gh_server* s, const Query& q) {
    const int B = s->cfg.batchSize;
    const Dataset& d = s->data[q.dataset];
    unsigned char* p = s->arena + q.off;
    Inst in;
    std::memset(&in, 0, sizeof(in));
    in.kind = q.kind;
    in.blocks = q.blocks;
    in.batchNum = q.bn;
    in.state = reinterpret_cast<gh::HeapState*>(p);
    p += align_up(sizeof(gh::HeapState), 256);
    in.items = reinterpret_cast<u64*>(p);
    p += align_up(static_cast<size_t>(q.bn + 1) * B * 8, 256);
    in.status = reinterpret_cast<int*>(p);
    p += align_up(static_cast<size_t>(q.bn + 2) * 4, 256);
    in.g = reinterpret_cast<unsigned*>(p);
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
        in.start = q.a;
        in.goal = q.b;
    }
    return in;
}

#define GH_SCUDA(call)                                 \
    do {                                               \
        if ((call) != cudaSuccess) return GH_ERR_CUDA; \
    } while (0)

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
    const long long id = static_cast<long long>(s->queries.size());
    s->queries.push_back(q);
    s->waiting.push_back(id);
    if (query) *query = id;
    return GH_OK;
}

gh_status gh_serve_step(gh_server* s, void* stream, int* finished, int* active, int* queued) {
    gh::trace::Range range_("gh_serve_step");
    if (!s) return GH_ERR_INVALID;
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
        k_search_fill<<<dim3(8, static_cast<unsigned>(fresh.size())), 256, 0, st>>>(s->insts, s->ids, s->cfg.batchSize);
        gh::impl::count_launch();
        k_search_seed<<<(static_cast<int>(fresh.size()) + 127) / 128, 128, 0, st>>>(s->insts, s->ids,
                                                                                     static_cast<int>(fresh.size()));
        gh::impl::count_launch();
        GH_SCUDA(cudaGetLastError());
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
        GH_SCUDA(search_launch(s->cfg, s->insts, s->tasks, nt, s->next, std::min(s->grid, nt), st, s->batchesPerStep));
        k_search_collect<<<static_cast<unsigned>(act.size()), 256, 0, st>>>(s->insts, s->ids, 0, s->cfg.batchSize);
        gh::impl::count_launch();
        GH_SCUDA(cudaGetLastError());
        GH_SCUDA(cudaMemcpyAsync(s->hinst.data(), s->insts, sizeof(Inst) * s->maxSlots, cudaMemcpyDeviceToHost, st));
        GH_SCUDA(cudaStreamSynchronize(st));
        ++s->steps;
        for (int slot : act) {
            const Inst& in = s->hinst[slot];
            if (!in.done) continue;
            Query& q = s->queries[s->slotQuery[slot]];
            q.state = in.failed ? 3 : 2;
            if (q.kind == GH_SEARCH_SSSP) {
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

}  // extern "C"
