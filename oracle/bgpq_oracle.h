/* CPU oracle for the batched priority queue (BGPQ) hot path.
 *
 * TEST INFRASTRUCTURE ONLY: only tests, the smoke check and the CPU leg of the
 * benchmark load this library.  It is the checker, never the thing measured
 * or shipped; the product path (gpuheap_gb300) never calls it.
 *
 * Parity is pinned: tests/golden/ holds vectors produced by the reference's
 * own heap headers run sequentially on the host (oracle/ref_driver.cpp +
 * oracle/ref_shim.h), and the CPU tests replay them through this restatement
 * bit-exactly.
 *
 * Contents
 *   - counter-based seeded key generators (splitmix64 finaliser, Steele et al.
 *     2014) for the four key distributions of the plain heap-sort workload;
 *   - std::sort, single- and multi-threaded (the reference's own test oracle:
 *     test/heap_test.cu:118 and :163-170);
 *   - checkInsertHeap for both node layouts (heap/tditdd/heap.cuh:123-176,
 *     heap/buitdd/heap.cuh:118-172);
 *   - a sequential model of Heap<K>::insertion / deleteRoot / deleteUpdate for
 *     the four variants (heap/{tditdd,tditdd_np,buitdd,buitdd_np}/heap.cuh).
 *     With one thread block the GPU heap is deterministic, and because the keys
 *     are plain integers every merge has a unique result, so the GPU's node
 *     contents must equal this model's bit for bit.
 */
#ifndef GPUHEAP_ORACLE_H
#define GPUHEAP_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* distributions */
enum { GHO_UNIFORM = 0, GHO_SORTED = 1, GHO_REVERSE = 2, GHO_ZIPF = 3 };

/* u32 keys in [0, 2^32-2] (UINT32_MAX is reserved as init_limits). */
void gho_gen_u32(uint64_t seed, int dist, uint64_t n, uint32_t* out, int threads);
/* u64 keys = (u32 key << 32) | input index. */
void gho_gen_u64(uint64_t seed, int dist, uint64_t n, uint64_t* out, int threads);
/* i32 keys in [INT32_MIN, INT32_MAX-1]. */
void gho_gen_i32(uint64_t seed, int dist, uint64_t n, int32_t* out, int threads);

void gho_sort_u32(uint32_t* a, uint64_t n, int threads);
void gho_sort_u64(uint64_t* a, uint64_t n, int threads);
void gho_sort_i32(int32_t* a, uint64_t n, int threads);

/* Bit-reversal of the bits below the leading one (heap/buitdd/heap.cuh:238-255). */
uint32_t gho_reversed_idx(uint32_t i);

/* checkInsertHeap over a host copy.  variant: 0 top-down, 1 bottom-up.
 * status may be NULL (then the state checks are skipped).  Returns 1 when the
 * heap is valid, 0 otherwise with a reason in msg. */
int gho_check_u32(int variant, const uint32_t* items, const int* status, int batch_size,
                  int batch_count, int partial_size, char* msg, int msg_len);
int gho_check_u64(int variant, const uint64_t* items, const int* status, int batch_size,
                  int batch_count, int partial_size, char* msg, int msg_len);
int gho_check_i32(int variant, const int32_t* items, const int* status, int batch_size,
                  int batch_count, int partial_size, char* msg, int msg_len);

/* Sequential model.  variant: 0 top-down, 1 bottom-up; pb: partial buffer. */
void* gho_model_create_u32(int variant, int pb, int batch_num, int batch_size, uint32_t init_limits);
void* gho_model_create_u64(int variant, int pb, int batch_num, int batch_size, uint64_t init_limits);
void* gho_model_create_i32(int variant, int pb, int batch_num, int batch_size, int32_t init_limits);
/* One insertion(items, size) call, size <= batch_size.  Returns 0, or -2 when
 * the heap has no free node. */
int gho_model_insert_u32(void* m, const uint32_t* items, int size);
int gho_model_insert_u64(void* m, const uint64_t* items, int size);
int gho_model_insert_i32(void* m, const int32_t* items, int size);
/* deleteRoot (+ deleteUpdate) with HEAP_SORT output at out + deleteCount.
 * Returns the number of keys written (0 when empty). */
int gho_model_delete_u32(void* m, uint32_t* out);
int gho_model_delete_u64(void* m, uint64_t* out);
int gho_model_delete_i32(void* m, int32_t* out);
/* Copies (batch_num + 1) * batch_size keys and {batchCount, partialBufferSize, deleteCount}. */
void gho_model_state_u32(void* m, uint32_t* items, int* counters);
void gho_model_state_u64(void* m, uint64_t* items, int* counters);
void gho_model_state_i32(void* m, int32_t* items, int* counters);
void gho_model_destroy(void* m);

/* Single-source shortest paths with std::priority_queue on (dist << 32 | v)
 * keys (the key packing of applications/sssp_longfei_new/sssp.cu:4-6) over a
 * CSR graph with u32 weights; unreachable vertices get UINT32_MAX.  The
 * reference ships no CPU SSSP (applications/sssp/main.cpp only parses), so
 * this is textbook Dijkstra.  *_many runs `k` sources on `threads` host
 * threads, one source per task; dist_out is k * n. */
void gho_dijkstra(int n, const int64_t* rowptr, const int32_t* col, const uint32_t* w, int source, uint32_t* dist_out);
void gho_dijkstra_many(int n, const int64_t* rowptr, const int32_t* col, const uint32_t* w, const int32_t* sources,
                       int k, int threads, uint32_t* dist_out);

/* Grid A* (oracle/search_oracle.cpp): 4-connected width x height grid,
 * cost[y * width + x] in 1..9 is the cost of entering the cell, 0 an
 * obstacle; from (0, 0) to (width-1, height-1), Manhattan heuristic.
 * Returns the optimal path cost or UINT32_MAX when the goal is unreachable;
 * expansions / max_open (may be NULL) report the search's size. */
uint32_t gho_astar_grid(int width, int height, const uint8_t* cost, long long* expansions, long long* max_open);
/* The reference's 8-connected bitmap A* (artifacts/astar/seq_astar.hpp:85-183) restated. */
uint32_t gho_astar_ref8(int width, int height, const uint32_t* bitmap);
/* The reference's map model searched to the optimum (its GPU A*'s result). */
uint32_t gho_astar_grid8(int width, int height, const uint8_t* open_cells, long long* expansions);
uint32_t gho_astar_grid8_sg(int width, int height, const uint8_t* open_cells, int start, int goal,
                            long long* expansions);
/* The same between any start and goal cell (y * width + x). */
uint32_t gho_astar_grid_sg(int width, int height, const uint8_t* cost, int start, int goal, long long* expansions,
                           long long* max_open);
/* k grids, grid i at costs + offsets[i]; one grid per task on `threads` threads. */
void gho_astar_grid_many(int k, const int32_t* widths, const int32_t* heights, const int64_t* offsets,
                         const uint8_t* costs, int threads, uint32_t* out);

/* 0/1 knapsack: best-first branch-and-bound on the Dantzig bound (returns the
 * optimum; nodes / max_open may be NULL) and the capacity DP cross-check. */
long long gho_knap_bb(int n, const int32_t* w, const int32_t* p, long long cap, long long* nodes, long long* max_open);
long long gho_knap_dp(int n, const int32_t* w, const int32_t* p, long long cap);
/* k instances, instance i: sizes[i] items at w/p + offsets[i], capacity caps[i]. */
void gho_knap_bb_many(int k, const int32_t* sizes, const int64_t* offsets, const int32_t* w, const int32_t* p,
                      const int64_t* caps, int threads, int64_t* out);

/* Closed-form algorithmic byte count of one heap-sort (bytes moved by the
 * BGPQ node traffic, independent of the implementation). */
double gho_sort_bytes(uint64_t n, int batch_size, int key_bytes, int partial_buffer);

#ifdef __cplusplus
}
#endif
#endif
