// CPU oracles of the batched search workloads (grid A* and 0/1 knapsack
// branch-and-bound).
//
// TEST INFRASTRUCTURE ONLY: only tests, the smoke check and the CPU legs of
// the benchmark load this code.  It is the checker, never the thing measured
// or shipped; the product path never calls it.
//
// Grid A*: follows the closed-set A* of artifacts/astar/seq_astar.hpp:186-279
// (a std::priority_queue of f << 32 | node, stale entries skipped), restated
// for 4-connected cost grids: a move costs the u8 cost of the cell entered,
// cost 0 marks an obstacle, the heuristic is the Manhattan distance to the
// goal (every cost is at least 1, so it is consistent and the first pop of
// the goal is optimal).
//
// Knapsack: the reference ships no CPU solver.  The branching and pruning are
// those of artifacts/knapsack/knapsackKernel.cuh:4-91 (items in
// profit/weight order, a Dantzig bound: whole items while they fit, then a
// fraction of the next; take / skip the item at the node's level), run
// best-first on the bound, with integer arithmetic (the fractional part is
// floored, which keeps the bound an upper bound of any integer solution).
// A textbook dynamic program over capacities cross-checks it.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <numeric>
#include <queue>
#include <thread>
#include <vector>

#include "bgpq_oracle.h"

namespace {

struct KnapSorted {
    int n;
    int64_t cap;
    std::vector<int64_t> w, p, W, P;  // ratio-ordered items and exclusive prefix sums
};

KnapSorted knap_sort(int n, const int32_t* w, const int32_t* p, int64_t cap) {
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
        return static_cast<int64_t>(p[a]) * w[b] > static_cast<int64_t>(p[b]) * w[a];
    });
    KnapSorted k{n, cap, std::vector<int64_t>(n), std::vector<int64_t>(n), std::vector<int64_t>(n + 1, 0),
                 std::vector<int64_t>(n + 1, 0)};
    for (int i = 0; i < n; ++i) {
        k.w[i] = w[ord[i]];
        k.p[i] = p[ord[i]];
        k.W[i + 1] = k.W[i] + k.w[i];
        k.P[i + 1] = k.P[i] + k.p[i];
    }
    return k;
}

// Dantzig bound of a node deciding items level.. with (profit, weight) so far.
int64_t knap_bound(const KnapSorted& k, int level, int64_t profit, int64_t weight) {
    const int64_t rem = k.cap - weight;
    if (rem < 0) return -1;
    // largest b in [level, n] with W[b] - W[level] <= rem
    int lo = level, hi = k.n;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (k.W[mid] - k.W[level] <= rem) lo = mid;
        else hi = mid - 1;
    }
    const int b = lo;
    int64_t bound = profit + (k.P[b] - k.P[level]);
    if (b < k.n) bound += (rem - (k.W[b] - k.W[level])) * k.p[b] / k.w[b];
    return bound;
}

}  // namespace

extern "C" {

uint32_t gho_astar_grid_sg(int width, int height, const uint8_t* cost, int start, int goal, long long* expansions,
                           long long* max_open) {
    const int64_t cells = static_cast<int64_t>(width) * height;
    const int tx = goal % width, ty = goal / width;
    std::vector<uint32_t> g(cells, 0xffffffffu);
    auto h = [&](int v) { return static_cast<uint32_t>(std::abs(tx - v % width) + std::abs(ty - v / width)); };
    std::priority_queue<uint64_t, std::vector<uint64_t>, std::greater<uint64_t>> open;
    long long exp = 0, mo = 0;
    uint32_t result = 0xffffffffu;
    if (cost[start] != 0 && cost[goal] != 0) {
        g[start] = 0;
        open.push((static_cast<uint64_t>(h(start)) << 32) | static_cast<uint32_t>(start));
    }
    while (!open.empty()) {
        mo = std::max<long long>(mo, static_cast<long long>(open.size()));
        const uint64_t key = open.top();
        open.pop();
        const uint32_t f = static_cast<uint32_t>(key >> 32);
        const int v = static_cast<int>(key & 0xffffffffu);
        if (f != g[v] + h(v)) continue;  // stale entry
        if (v == goal) { result = g[v]; break; }
        ++exp;
        const int x = v % width, y = v / width;
        const int nb[4] = {x > 0 ? v - 1 : -1, x + 1 < width ? v + 1 : -1, y > 0 ? v - width : -1,
                           y + 1 < height ? v + width : -1};
        for (int u : nb) {
            if (u < 0 || cost[u] == 0) continue;
            const uint32_t ng = g[v] + cost[u];
            if (ng < g[u]) {
                g[u] = ng;
                open.push((static_cast<uint64_t>(ng + h(u)) << 32) | static_cast<uint32_t>(u));
            }
        }
    }
    if (expansions) *expansions = exp;
    if (max_open) *max_open = mo;
    return result;
}

// The reference's own move model (artifacts/astar/seq_astar.hpp:13-78,
// SeqAstarSearch :85-183), restated to pin the machinery above: a w x h
// bitmap (bit i of word i/32 set = cell i open), 8 moves in the order
// (-1,-1) (0,-1) (+1,-1) (-1,0) (+1,0) (-1,+1) (0,+1) (+1,+1) with the
// costs 3 2 2 2 1 3 1 2, the heuristic x2 - x1 + y2 - y1 to the corner
// (w-1, h-1) in 32-bit unsigned arithmetic, an entry skipped when its g is
// above the cell's best, and the search stopped as soon as a move reaches
// the corner (open or not) -- the cost then recorded there is the result,
// UINT32_MAX when the corner was never reached.
uint32_t gho_astar_ref8(int width, int height, const uint32_t* bitmap) {
    const uint32_t w = static_cast<uint32_t>(width), h = static_cast<uint32_t>(height);
    const uint64_t cells = static_cast<uint64_t>(w) * h;
    auto heur = [&](uint32_t i) { return (w - 1) - i % w + (h - 1) - i / w; };
    auto open_at = [&](uint32_t i) { return i != 0xffffffffu && ((bitmap[i / 32] >> (i % 32)) & 1u) != 0; };
    auto cell = [&](uint32_t i, int dx, int dy) -> uint32_t {
        const int x = static_cast<int>(i % w) + dx, y = static_cast<int>(i / w) + dy;
        if (x < 0 || y < 0 || x >= static_cast<int>(w) || y >= static_cast<int>(h)) return 0xffffffffu;
        return w * static_cast<uint32_t>(y) + static_cast<uint32_t>(x);
    };
    static const int kDx[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
    static const int kDy[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
    static const uint32_t kCost[8] = {3, 2, 2, 2, 1, 3, 1, 2};
    std::vector<uint32_t> best(cells, 0xffffffffu);
    best[0] = 0;
    std::priority_queue<uint64_t, std::vector<uint64_t>, std::greater<uint64_t>> open;
    open.push(static_cast<uint64_t>(heur(0)) << 32);
    const uint32_t corner = static_cast<uint32_t>(cells - 1);
    bool stop = false;
    while (!open.empty() && !stop) {
        const uint64_t item = open.top();
        open.pop();
        const uint32_t v = static_cast<uint32_t>(item);
        const uint32_t g = static_cast<uint32_t>(item >> 32) - heur(v);
        if (g > best[v]) continue;
        for (int k = 0; k < 8; ++k) {
            const uint32_t u = cell(v, kDx[k], kDy[k]);
            if (u == corner && u != 0xffffffffu) {
                best[u] = g + kCost[k];
                stop = true;
                break;
            }
            if (open_at(u) && best[u] > g + kCost[k]) {
                best[u] = g + kCost[k];
                open.push((static_cast<uint64_t>(heur(u) + g + kCost[k]) << 32) | u);
            }
        }
    }
    return best[corner];
}

// The reference's map model searched to the optimum (the result of its GPU
// A*, artifacts/astar/pq_model.cuh, which prunes on dist[target] until no
// key below it is left): open[i] != 0 marks an open cell, the eight moves
// and costs of gho_astar_ref8, the Manhattan heuristic (consistent: a
// straight move costs at least 1, a diagonal one at least 2), the goal
// (w-1, h-1) taken when popped.
uint32_t gho_astar_grid8_sg(int width, int height, const uint8_t* open_cells, int start, int goal,
                            long long* expansions) {
    const int64_t cells = static_cast<int64_t>(width) * height;
    const int tx = goal % width, ty = goal / width;
    auto heur = [&](int v) { return static_cast<uint32_t>(std::abs(tx - v % width) + std::abs(ty - v / width)); };
    static const int kDx[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
    static const int kDy[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
    static const uint32_t kCost[8] = {3, 2, 2, 2, 1, 3, 1, 2};
    std::vector<uint32_t> g(cells, 0xffffffffu);
    std::priority_queue<uint64_t, std::vector<uint64_t>, std::greater<uint64_t>> open;
    long long exp = 0;
    uint32_t result = 0xffffffffu;
    if (open_cells[start] != 0 && open_cells[goal] != 0) {
        g[start] = 0;
        open.push((static_cast<uint64_t>(heur(start)) << 32) | static_cast<uint32_t>(start));
    }
    while (!open.empty()) {
        const uint64_t key = open.top();
        open.pop();
        const int v = static_cast<int>(key & 0xffffffffu);
        if (static_cast<uint32_t>(key >> 32) != g[v] + heur(v)) continue;  // stale entry
        if (v == goal) { result = g[v]; break; }
        ++exp;
        const int x = v % width, y = v / width;
        for (int k = 0; k < 8; ++k) {
            const int nx = x + kDx[k], ny = y + kDy[k];
            if (nx < 0 || ny < 0 || nx >= width || ny >= height) continue;
            const int u = ny * width + nx;
            if (open_cells[u] == 0) continue;
            const uint32_t ng = g[v] + kCost[k];
            if (ng < g[u]) {
                g[u] = ng;
                open.push((static_cast<uint64_t>(ng + heur(u)) << 32) | static_cast<uint32_t>(u));
            }
        }
    }
    if (expansions) *expansions = exp;
    return result;
}

uint32_t gho_astar_grid8(int width, int height, const uint8_t* open_cells, long long* expansions) {
    return gho_astar_grid8_sg(width, height, open_cells, 0, static_cast<int>(static_cast<int64_t>(width) * height - 1),
                              expansions);
}

uint32_t gho_astar_grid(int width, int height, const uint8_t* cost, long long* expansions, long long* max_open) {
    return gho_astar_grid_sg(width, height, cost, 0, static_cast<int>(static_cast<int64_t>(width) * height - 1),
                             expansions, max_open);
}

void gho_astar_grid_many(int k, const int32_t* widths, const int32_t* heights, const int64_t* offsets,
                         const uint8_t* costs, int threads, uint32_t* out) {
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([=] {
            for (int i = t; i < k; i += threads)
                out[i] = gho_astar_grid(widths[i], heights[i], costs + offsets[i], nullptr, nullptr);
        });
    for (auto& th : pool) th.join();
}

long long gho_knap_bb(int n, const int32_t* w, const int32_t* p, long long cap, long long* nodes, long long* max_open) {
    const KnapSorted k = knap_sort(n, w, p, cap);
    // greedy incumbent: every item that still fits, in ratio order
    int64_t best = 0, wt = 0;
    for (int i = 0; i < n; ++i)
        if (wt + k.w[i] <= cap) { wt += k.w[i]; best += k.p[i]; }
    struct Node { int64_t bound, profit, weight; int level; };
    auto worse = [](const Node& a, const Node& b) { return a.bound < b.bound; };
    std::priority_queue<Node, std::vector<Node>, decltype(worse)> open(worse);
    open.push({knap_bound(k, 0, 0, 0), 0, 0, 0});
    long long cnt = 0, mo = 0;
    while (!open.empty()) {
        mo = std::max<long long>(mo, static_cast<long long>(open.size()));
        const Node nd = open.top();
        open.pop();
        if (nd.bound <= best) break;  // best-first: nothing left can improve
        ++cnt;
        if (nd.level == n) continue;
        const int i = nd.level;
        if (nd.weight + k.w[i] <= cap) {  // take item i
            const Node c{knap_bound(k, i + 1, nd.profit + k.p[i], nd.weight + k.w[i]), nd.profit + k.p[i],
                         nd.weight + k.w[i], i + 1};
            if (c.profit > best) best = c.profit;
            if (c.bound > best) open.push(c);
        }
        const Node c{knap_bound(k, i + 1, nd.profit, nd.weight), nd.profit, nd.weight, i + 1};  // skip item i
        if (c.bound > best) open.push(c);
    }
    if (nodes) *nodes = cnt;
    if (max_open) *max_open = mo;
    return best;
}

long long gho_knap_dp(int n, const int32_t* w, const int32_t* p, long long cap) {
    std::vector<int64_t> dp(static_cast<size_t>(cap) + 1, 0);
    for (int i = 0; i < n; ++i)
        for (int64_t c = cap; c >= w[i]; --c) dp[c] = std::max(dp[c], dp[c - w[i]] + p[i]);
    return dp[cap];
}

void gho_knap_bb_many(int k, const int32_t* sizes, const int64_t* offsets, const int32_t* w, const int32_t* p,
                      const int64_t* caps, int threads, int64_t* out) {
    if (threads < 1) threads = 1;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([=] {
            for (int i = t; i < k; i += threads)
                out[i] = gho_knap_bb(sizes[i], w + offsets[i], p + offsets[i], caps[i], nullptr, nullptr);
        });
    for (auto& th : pool) th.join();
}

}  // extern "C"
