// CPU oracle for the BGPQ hot path -- TEST INFRASTRUCTURE ONLY (see bgpq_oracle.h).
//
// The sequential model below restates the reference algorithm; each piece
// cites the reference lines it follows.  Every comparison-based step of the
// reference (swap when one batch is wholly below the other, skip when already
// ordered, full merge-path otherwise) yields the same multiset split as a full
// two-way merge, and for plain integer keys that split is unique, so the model
// uses one merge routine everywhere.
#include "bgpq_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <queue>
#include <cstdio>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- generators
// splitmix64 finaliser (Steele, Lea, Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014); key i of a stream is the finaliser applied
// to seed + (i + 1) * golden-ratio increment, so any slice can be generated
// independently (the GPU benchmark uses the same counter-based definition).
inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
inline uint64_t draw(uint64_t seed, uint64_t i) { return mix64(seed + (i + 1) * 0x9e3779b97f4a7c15ULL); }

// Uniform in [0, 2^32 - 2]: the high word scaled by (2^32 - 1) / 2^32.
inline uint32_t u32_key(uint64_t r) { return static_cast<uint32_t>(((r >> 32) * 0xffffffffULL) >> 32); }

// A bijection on 32-bit words (xor-shift / odd-multiply rounds, the
// "lowbias32" shape from C. Wellons' hash-prospector), used to scatter the
// Zipf ranks over the key space; cycle-walking keeps 0xffffffff out.
inline uint32_t scatter32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU;
    x ^= x >> 15; x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}
inline uint32_t zipf_value(uint32_t rank, uint64_t seed) {
    uint32_t x = scatter32(rank ^ static_cast<uint32_t>(mix64(seed ^ 0x5a17f00dULL)));
    while (x == 0xffffffffU) x = scatter32(x);
    return x;
}

constexpr int kZipfValues = 1 << 16;
constexpr double kZipfS = 1.2;

std::vector<double> zipf_cdf() {
    std::vector<double> cdf(kZipfValues);
    double acc = 0.0;
    for (int r = 1; r <= kZipfValues; ++r) { acc += std::pow(static_cast<double>(r), -kZipfS); cdf[r - 1] = acc; }
    for (double& c : cdf) c /= acc;
    return cdf;
}

template <typename F>
void parallel_for(uint64_t n, int threads, F&& f) {
    if (threads <= 1 || n < (1u << 16)) { f(0, n); return; }
    std::vector<std::thread> ts;
    uint64_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        uint64_t lo = t * chunk, hi = std::min(n, lo + chunk);
        if (lo >= hi) break;
        ts.emplace_back([&f, lo, hi] { f(lo, hi); });
    }
    for (auto& t : ts) t.join();
}

void gen_keys32(uint64_t seed, int dist, uint64_t n, uint32_t* out, int threads) {
    if (dist == GHO_ZIPF) {
        std::vector<double> cdf = zipf_cdf();
        parallel_for(n, threads, [&](uint64_t lo, uint64_t hi) {
            for (uint64_t i = lo; i < hi; ++i) {
                double u = static_cast<double>(draw(seed, i) >> 11) * (1.0 / 9007199254740992.0);
                uint32_t rank = static_cast<uint32_t>(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin()) + 1;
                if (rank > kZipfValues) rank = kZipfValues;
                out[i] = zipf_value(rank, seed);
            }
        });
        return;
    }
    parallel_for(n, threads, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) out[i] = u32_key(draw(seed, i));
    });
}

// ---------------------------------------------------------------- sorting
template <typename K>
void psort(K* a, uint64_t n, int threads) {
    if (threads <= 1 || n < (1u << 18)) { std::sort(a, a + n); return; }
    int parts = 1;
    while (parts * 2 <= threads) parts *= 2;
    std::vector<uint64_t> bounds(parts + 1);
    for (int p = 0; p <= parts; ++p) bounds[p] = n * p / parts;
    {
        std::vector<std::thread> ts;
        for (int p = 0; p < parts; ++p) ts.emplace_back([=] { std::sort(a + bounds[p], a + bounds[p + 1]); });
        for (auto& t : ts) t.join();
    }
    std::vector<K> tmp(n);
    K* src = a;
    K* dst = tmp.data();
    for (int width = 1; width < parts; width *= 2) {
        std::vector<std::thread> ts;
        for (int p = 0; p < parts; p += 2 * width) {
            uint64_t lo = bounds[p], mid = bounds[p + width], hi = bounds[std::min(parts, p + 2 * width)];
            ts.emplace_back([=] { std::merge(src + lo, src + mid, src + mid, src + hi, dst + lo); });
        }
        for (auto& t : ts) t.join();
        std::swap(src, dst);
    }
    if (src != a) std::memcpy(a, src, n * sizeof(K));
}

// ---------------------------------------------------------------- layout helpers
// heap/buitdd/heap.cuh:233-255: reverse the bits below the leading one.
inline uint32_t reversed_idx(uint32_t i) {
    if (i <= 1) return i;
    int msb = 31 - __builtin_clz(i);
    uint32_t r = 0;
    for (int b = 0; b < msb; ++b) r |= ((i >> b) & 1u) << (msb - 1 - b);
    return r | (1u << msb);
}
// heap/tditdd/heap.cuh:263-265: next node on the root -> target path.
inline int next_on_path(int cur, int target) {
    int shift = __builtin_clz(static_cast<unsigned>(cur)) - __builtin_clz(static_cast<unsigned>(target)) - 1;
    return target >> shift;
}

// ---------------------------------------------------------------- checker
template <typename K>
int check_heap(int variant, const K* items, const int* status, int B, int bc, int ps, char* msg, int msg_len) {
    auto fail = [&](const char* fmt, long a, long b) {
        if (msg && msg_len > 0) std::snprintf(msg, msg_len, fmt, a, b);
        return 0;
    };
    // heap/tditdd/heap.cuh:134-150
    if (status && status[0] != 0) return fail("partial buffer state %ld is not AVAIL (%ld)", status[0], 0);
    if (bc != 0 && ps != 0) {
        if (items[2 * B - 1] > items[0]) return fail("partial buffer below the root (ps=%ld, bc=%ld)", ps, bc);
        for (int i = 1; i < ps; ++i)
            if (items[i] < items[i - 1]) return fail("partial buffer unsorted at %ld (ps=%ld)", i, ps);
    }
    // heap/tditdd/heap.cuh:152-169 (top-down parent i/2), heap/buitdd/heap.cuh:147-165 (bit-reversed parent)
    for (int i = 1; i <= bc; ++i) {
        if (status && status[i] != 0) return fail("node %ld state %ld is not AVAIL", i, status[i]);
        if (i > 1) {
            int p = variant == 0 ? i / 2 : static_cast<int>(reversed_idx(reversed_idx(i) >> 1));
            if (items[static_cast<size_t>(i) * B] < items[static_cast<size_t>(p) * B + B - 1])
                return fail("node %ld starts below the end of its parent %ld", i, p);
        }
        const K* nd = items + static_cast<size_t>(i) * B;
        for (int j = 1; j < B; ++j)
            if (nd[j] < nd[j - 1]) return fail("node %ld unsorted at %ld", i, j);
    }
    return 1;
}

// ---------------------------------------------------------------- sequential model
template <typename K>
struct Model {
    int variant;  // 0 top-down insertion, 1 bottom-up insertion
    bool pb;
    int batchNum, B;
    K init;
    std::vector<K> items;  // (batchNum + 1) nodes; node 0 is the partial buffer
    int batchCount = 0, partialSize = 0, deleteCount = 0;
    std::vector<K> t1, t2;

    Model(int v, bool p, int bn, int bs, K lim)
        : variant(v), pb(p), batchNum(bn), B(bs), init(lim),
          items(static_cast<size_t>(bn + 1) * bs, lim), t1(2 * bs), t2(bs) {}

    K* node(int i) { return items.data() + static_cast<size_t>(i) * B; }

    // Two-way merge of sorted a[0,B) and b[0,B): the B smallest go to lo, the
    // rest to hi (heap/heaputil.cuh:99-158).  lo/hi may alias a/b.
    void merge(const K* a, const K* b, K* lo, K* hi) {
        std::merge(a, a + B, b, b + B, t1.data());
        if (lo) std::memcpy(lo, t1.data(), sizeof(K) * B);
        if (hi) std::memcpy(hi, t1.data() + B, sizeof(K) * B);
    }

    int parent(int i) const { return variant == 0 ? i / 2 : static_cast<int>(reversed_idx(reversed_idx(i) >> 1)); }
    int left_child(int i) const { return variant == 0 ? 2 * i : static_cast<int>(reversed_idx(reversed_idx(i) << 1)); }
    int right_child(int left) const { return variant == 0 ? left + 1 : static_cast<int>(reversed_idx(reversed_idx(left) + 1)); }

    // insertion(): heap/tditdd/heap.cuh:536-753, heap/buitdd/heap.cuh:484-690;
    // without the partial buffer: heap/tditdd_np/heap.cuh:465-684, heap/buitdd_np/heap.cuh:425-539.
    int insert(const K* in, int size) {
        std::vector<K> s1(B, init);
        std::copy(in, in + size, s1.begin());
        std::sort(s1.begin(), s1.end());  // pad + ibitonicSort (heap/tditdd/heap.cuh:557-562)
        K* n0 = node(0);
        if (pb) {
            if (batchCount == 0 && size < B) {
                if (partialSize == 0) {  // case 1.1 (:575-584)
                    std::copy(s1.begin(), s1.end(), n0);
                    partialSize = size;
                    return 0;
                }
                if (size + partialSize < B) {  // case 1.2 (:586-598)
                    merge(s1.data(), n0, n0, nullptr);
                    partialSize += size;
                    return 0;
                }
                // case 1.3 (:600-620)
                if (batchNum < 1) return -2;
                batchCount += 1;
                merge(s1.data(), n0, node(1), n0);
                partialSize += size - B;
                return 0;
            }
            if (size + partialSize < B) {  // case 2.1 (:625-648)
                merge(s1.data(), n0, s1.data(), nullptr);
                merge(s1.data(), node(1), node(1), n0);
                partialSize += size;
                return 0;
            }
            // case 2.2 (:650-662): keep the smaller B in the insert batch
            merge(s1.data(), n0, s1.data(), n0);
            partialSize += size - B;
        }
        if (batchCount + 1 > batchNum) return -2;
        int target = ++batchCount;  // (:668)
        if (variant == 0) {
            // top-down: merge along the root -> target path (:680-725)
            int cur = 1;
            while (cur != target) {
                merge(s1.data(), node(cur), node(cur), s1.data());
                cur = next_on_path(cur, target);
            }
            std::copy(s1.begin(), s1.end(), node(target));  // (:746)
        } else {
            // bottom-up: write the leaf, then bubble up (heap/buitdd/heap.cuh:627-683)
            std::copy(s1.begin(), s1.end(), node(target));
            int cur = target;
            while (cur != 1) {
                int p = parent(cur);
                merge(node(cur), node(p), node(p), node(cur));
                cur = p;
            }
        }
        return 0;
    }

    // deleteRoot + deleteUpdate with HEAP_SORT: heap/tditdd/heap.cuh:267-534,
    // heap/buitdd/heap.cuh:283-482 (and the _np copies without the partial-buffer steps).
    int erase(K* out) {
        int off = deleteCount;
        if (batchCount == 0 && partialSize == 0) return 0;
        if (pb && batchCount == 0) {  // only the partial buffer holds keys (:297-315)
            int n = partialSize;
            std::copy(node(0), node(0) + n, out + off);
            std::fill(node(0), node(0) + n, init);
            deleteCount += n;
            partialSize = 0;
            return n;
        }
        std::copy(node(1), node(1) + B, out + off);  // (:328-329)
        deleteCount += B;
        int last = batchCount--;  // (:357)
        if (last == 1) return B;
        std::vector<K> sm(node(last), node(last) + B);  // take the last node and reset it (:396)
        std::fill(node(last), node(last) + B, init);
        if (pb) merge(sm.data(), node(0), sm.data(), node(0));  // (:405-409)
        int cur = 1;
        for (;;) {
            int l = left_child(cur);
            if (l > batchNum) {  // no child inside the allocation: same result as empty children
                std::copy(sm.begin(), sm.end(), node(cur));
                return B;
            }
            int r = right_child(l);
            if (r > batchNum) {  // one child inside the allocation (:461-477)
                merge(sm.data(), node(l), node(cur), node(l));
                return B;
            }
            // two children (:479-531; bottom-up :421-479).  The larger child
            // is the one with the larger last key, the left one on a tie
            // (tditdd_np :416) -- except when both end in init_limits: then
            // the one with the larger first key.  Otherwise a padded node
            // (real keys, then init_limits) beside a node past the heap
            // (all init_limits) counts as larger, and the carried batch with
            // the padded node's real keys sinks into the node past the heap,
            // where they are lost; the reference has that tie rule, without
            // the exception.
            const K ll = node(l)[B - 1], rl = node(r)[B - 1];
            int larger = (ll < rl || (ll == rl && ll == init && node(l)[0] < node(r)[0])) ? r : l;
            int smaller = larger == r ? l : r;
            std::vector<K> low(B);
            merge(node(l), node(r), low.data(), node(larger));
            // ties: tditdd :506, tditdd_np :435 and buitdd_np :392 use <=, buitdd :451 uses <
            bool stop = (variant == 0 || !pb) ? (sm[B - 1] <= low[0]) : (sm[B - 1] < low[0]);
            if (sm[0] >= low[B - 1]) {
                std::copy(low.begin(), low.end(), node(cur));
            } else if (stop) {
                std::copy(sm.begin(), sm.end(), node(cur));
                std::copy(low.begin(), low.end(), node(smaller));
                return B;
            } else {
                merge(sm.data(), low.data(), node(cur), sm.data());
            }
            cur = smaller;
        }
    }
};

}  // namespace

// ---------------------------------------------------------------- C ABI
extern "C" {

void gho_gen_u32(uint64_t seed, int dist, uint64_t n, uint32_t* out, int threads) {
    gen_keys32(seed, dist, n, out, threads);
    if (dist == GHO_SORTED) psort(out, n, threads);
    if (dist == GHO_REVERSE) { psort(out, n, threads); std::reverse(out, out + n); }
}

void gho_gen_u64(uint64_t seed, int dist, uint64_t n, uint64_t* out, int threads) {
    std::vector<uint32_t> k(n);
    gen_keys32(seed, dist, n, k.data(), threads);
    parallel_for(n, threads, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) out[i] = (static_cast<uint64_t>(k[i]) << 32) | (i & 0xffffffffULL);
    });
    if (dist == GHO_SORTED) psort(out, n, threads);
    if (dist == GHO_REVERSE) { psort(out, n, threads); std::reverse(out, out + n); }
}

void gho_gen_i32(uint64_t seed, int dist, uint64_t n, int32_t* out, int threads) {
    gen_keys32(seed, dist, n, reinterpret_cast<uint32_t*>(out), threads);
    parallel_for(n, threads, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i)
            out[i] = static_cast<int32_t>(static_cast<int64_t>(reinterpret_cast<uint32_t*>(out)[i]) - 2147483648LL);
    });
    if (dist == GHO_SORTED) psort(out, n, threads);
    if (dist == GHO_REVERSE) { psort(out, n, threads); std::reverse(out, out + n); }
}

void gho_sort_u32(uint32_t* a, uint64_t n, int threads) { psort(a, n, threads); }
void gho_sort_u64(uint64_t* a, uint64_t n, int threads) { psort(a, n, threads); }
void gho_sort_i32(int32_t* a, uint64_t n, int threads) { psort(a, n, threads); }

uint32_t gho_reversed_idx(uint32_t i) { return reversed_idx(i); }

int gho_check_u32(int v, const uint32_t* it, const int* st, int B, int bc, int ps, char* m, int ml) { return check_heap(v, it, st, B, bc, ps, m, ml); }
int gho_check_u64(int v, const uint64_t* it, const int* st, int B, int bc, int ps, char* m, int ml) { return check_heap(v, it, st, B, bc, ps, m, ml); }
int gho_check_i32(int v, const int32_t* it, const int* st, int B, int bc, int ps, char* m, int ml) { return check_heap(v, it, st, B, bc, ps, m, ml); }

struct GhoModelBox { int kind; void* m; };

#define GHO_MODEL_FNS(T, tag, kindv)                                                                 \
    void* gho_model_create_##tag(int v, int pb, int bn, int bs, T lim) {                             \
        return new GhoModelBox{kindv, new Model<T>(v, pb != 0, bn, bs, lim)};                       \
    }                                                                                                \
    int gho_model_insert_##tag(void* m, const T* it, int sz) {                                      \
        return static_cast<Model<T>*>(static_cast<GhoModelBox*>(m)->m)->insert(it, sz);              \
    }                                                                                                \
    int gho_model_delete_##tag(void* m, T* out) {                                                   \
        return static_cast<Model<T>*>(static_cast<GhoModelBox*>(m)->m)->erase(out);                 \
    }                                                                                                \
    void gho_model_state_##tag(void* m, T* it, int* c) {                                            \
        auto* md = static_cast<Model<T>*>(static_cast<GhoModelBox*>(m)->m);                          \
        if (it) std::memcpy(it, md->items.data(), md->items.size() * sizeof(T));                     \
        if (c) { c[0] = md->batchCount; c[1] = md->partialSize; c[2] = md->deleteCount; }            \
    }

GHO_MODEL_FNS(uint32_t, u32, 0)
GHO_MODEL_FNS(uint64_t, u64, 1)
GHO_MODEL_FNS(int32_t, i32, 2)

void gho_model_destroy(void* m) {
    auto* b = static_cast<GhoModelBox*>(m);
    if (!b) return;
    if (b->kind == 0) delete static_cast<Model<uint32_t>*>(b->m);
    else if (b->kind == 1) delete static_cast<Model<uint64_t>*>(b->m);
    else delete static_cast<Model<int32_t>*>(b->m);
    delete b;
}

void gho_dijkstra(int n, const int64_t* rowptr, const int32_t* col, const uint32_t* w, int source, uint32_t* dist) {
    for (int v = 0; v < n; ++v) dist[v] = 0xffffffffu;
    if (source < 0 || source >= n) return;
    std::priority_queue<uint64_t, std::vector<uint64_t>, std::greater<uint64_t>> pq;
    dist[source] = 0;
    pq.push(static_cast<uint64_t>(source));
    while (!pq.empty()) {
        const uint64_t key = pq.top();
        pq.pop();
        const uint32_t d = static_cast<uint32_t>(key >> 32);
        const int v = static_cast<int>(key & 0xffffffffu);
        if (d != dist[v]) continue;  // stale entry
        for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e) {
            const uint64_t nd64 = static_cast<uint64_t>(d) + w[e];
            const uint32_t nd = nd64 >= 0xffffffffu ? 0xfffffffeu : static_cast<uint32_t>(nd64);
            const int u = col[e];
            if (nd < dist[u]) {
                dist[u] = nd;
                pq.push((static_cast<uint64_t>(nd) << 32) | static_cast<uint32_t>(u));
            }
        }
    }
}

void gho_dijkstra_many(int n, const int64_t* rowptr, const int32_t* col, const uint32_t* w, const int32_t* sources,
                       int k, int threads, uint32_t* dist_out) {
    std::atomic<int> next{0};
    auto worker = [&] {
        for (int i; (i = next.fetch_add(1)) < k;)
            gho_dijkstra(n, rowptr, col, w, sources[i], dist_out + static_cast<size_t>(i) * n);
    };
    std::vector<std::thread> ts;
    for (int t = 0; t < std::max(1, threads); ++t) ts.emplace_back(worker);
    for (auto& t : ts) t.join();
}

// Algorithmic node traffic of one heap-sort of n keys (bytes):
//   s * [ 2n                                   read input, write output
//       + sum_{k=1..M} 2B (floor(log2 k) + 1)  insert: read + write each node on the root->target path
//       + sum_{m=1..M} B (1 + 3 floor(log2 m)) delete: root/last + per level read 2 children, write 1
//       + (pb ? 4 B M : 0) ]                   partial buffer read + write per insert and per delete
// with M = ceil(n / B).
double gho_sort_bytes(uint64_t n, int B, int s, int pb) {
    uint64_t M = (n + B - 1) / B;
    long double sumL = 0;  // sum_{k=1..M} floor(log2 k)
    for (int l = 0; l < 63; ++l) {
        uint64_t lo = 1ULL << l;
        if (lo > M) break;
        uint64_t hi = std::min<uint64_t>(M, (lo << 1) - 1);
        sumL += static_cast<long double>(l) * static_cast<long double>(hi - lo + 1);
    }
    long double t = 2.0L * n + 2.0L * B * (sumL + M) + static_cast<long double>(B) * (M + 3.0L * sumL) +
                    (pb ? 4.0L * B * M : 0.0L);
    return static_cast<double>(t * s);
}

}  // extern "C"
