/* gpuheap.h -- C ABI of the GB300 batched priority queue (BGPQ).
 *
 * Plain pointers and sizes only.  Device buffers are raw device pointers;
 * `stream` is a cudaStream_t passed as void* (NULL = the legacy default
 * stream).  Every entry point returns a gh_status.
 *
 * The reference (ruadapt/gpuheap) has no FFI: its interface is the C++ class
 * template Heap<K> in heap/{tditdd,tditdd_np,buitdd,buitdd_np}/heap.cuh, whose
 * variant is chosen by include path.  Each entry point below names the member
 * or test-driver code it replaces; the variant, partial-buffer flag and key
 * type become run-time arguments here.  Device code keeps the reference's
 * member-function shape through include/gpuheap_device.cuh.
 */
#ifndef GPUHEAP_H
#define GPUHEAP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GH_OK = 0,
    GH_ERR_INVALID = 1,   /* bad argument (size, alignment, variant ...) */
    GH_ERR_CAPACITY = 2,  /* insertion found no free node (batch_num reached) */
    GH_ERR_TIMEOUT = 3,   /* a device-side wait passed the heap's time limit */
    GH_ERR_CUDA = 4,      /* a CUDA runtime call failed */
    GH_ERR_STATE = 5      /* the heap recorded an earlier device error; reset it */
} gh_status;

typedef enum { GH_KEY_U32 = 0, GH_KEY_I32 = 1, GH_KEY_U64 = 2 } gh_key_kind;
typedef enum { GH_TOPDOWN = 0, GH_BOTTOMUP = 1 } gh_variant;

typedef struct gh_heap gh_heap;

const char* gh_status_string(gh_status s);

/* Heap<K>(batch_num, batch_size, init_limits): heap/tditdd/heap.cuh:33-67,
 * heap/buitdd/heap.cuh:34-68; variant = include path (test/Makefile:10-20).
 * batch_size: power of two in [16, 4096].  init_limits points to one key of
 * the chosen kind (NULL = the kind's maximum); every real key must be
 * strictly below it.  Nodes are filled with init_limits on the device. */
gh_status gh_heap_create(gh_heap** out, int key_kind, int variant, int partial_buffer, int batch_num,
                         int batch_size, const void* init_limits);
/* ~Heap(): heap/tditdd/heap.cuh:93-116. */
gh_status gh_heap_destroy(gh_heap* h);
/* reset(): heap/tditdd/heap.cuh:69-91 (also clears a recorded device error). */
gh_status gh_heap_reset(gh_heap* h, void* stream);

/* Time limit of every device-side wait, in (0, 60] seconds (default 2 s).
 * It turns a hang into GH_ERR_TIMEOUT.  The bulk drivers keep every wait
 * short: a bulk insert reserves its targets (no race for node 0), the blocks
 * of a bulk delete queue for node 0 by ticket, and an owner-mode delete's
 * waits last a few deletes.  Single operations and application kernels that
 * race many blocks on one heap's node 0 may need a longer limit. */
gh_status gh_heap_set_timeout(gh_heap* h, double seconds);
/* Threads per block for the bulk entry points (0 = automatic: 16-byte merge
 * runs per thread); a power of two in [32, 1024] with 2*batch_size/threads
 * in {1, 2, 4, 8}. */
gh_status gh_heap_set_block_threads(gh_heap* h, int threads);
/* Blocks for the bulk entry points (0 = one per SM). */
gh_status gh_heap_set_grid(gh_heap* h, int blocks);
/* Resident depth of the owner-mode bulk delete: -1 = automatic (the default:
 * the deepest of 2..4 whose levels fit in one block's shared memory), 0 = off
 * (the plain deleteKernel loop), 2..4 = levels 0..depth kept in the owner
 * block.  It has no counterpart in the reference.  GH_ERR_INVALID when the
 * heap has no owner mode (batch_size below 512) or the depth does not fit. */
gh_status gh_heap_set_owner_depth(gh_heap* h, int depth);

/* insertKernel (test/heap_test.cu:44-58, artifacts/synthetic/sort.cu:32-46):
 * inserts keys_dev[0, n) in insertion() calls of `chunk` keys (0 = batch_size;
 * chunk <= batch_size), spread over the heap's grid.  With chunk = batch_size
 * and the partial buffer empty, the full batches' target nodes are reserved
 * in one step before they are inserted, so they do not take node 0 one at a
 * time; the result is a heap that the same inserts could have built one by
 * one.  No other operation may use the heap during the call (the reference's
 * tests run insertKernel as a phase of its own). */
gh_status gh_heap_insert(gh_heap* h, const void* keys_dev, long long n, int chunk, void* stream);

/* deleteKernel (test/heap_test.cu:60-77): deleteRoot/deleteUpdate until the
 * heap is empty or the next deleted batch would not fit in max_keys.  Keys
 * are written in ascending order (HEAP_SORT) to out_dev[0, *n_out).  When
 * n_out is not NULL the call synchronizes the stream to read the count. */
gh_status gh_heap_delete(gh_heap* h, void* out_dev, long long max_keys, long long* n_out, void* stream);

/* deleteRoot(items, size, app_t_val) in a loop (artifacts/astar/BGPQ_B/
 * heap.cuh:260-289): as gh_heap_delete, but a delete takes nothing once
 * the heap's smallest key (the root's first, or the partial buffer's when
 * no full node is left) is not below *threshold (one key of the heap's
 * kind).  Whole batches are taken, so the output holds every key below the
 * threshold plus the rest of the last batch; the keys left stay in the heap. */
gh_status gh_heap_delete_below(gh_heap* h, void* out_dev, long long max_keys, const void* threshold,
                               long long* n_out, void* stream);

/* Garbage collection (invalidFilter, artifacts/astar/gc.cuh:77-180 and
 * artifacts/knapsack/gc.cuh:30-180): keeps the keys strictly below
 * *threshold (NULL = init_limits: every real key; a heap without the
 * partial buffer also drops its padding keys) and rebuilds the heap from
 * them by bulk insertion; the output cursor is kept.  The compaction, the
 * reset and the reinsertion run on the device back to back (one
 * synchronisation to size the scratch, like the reference's read of
 * batchCount).  *kept (may be NULL; then the call returns without waiting
 * for the device) gets the number of keys kept. */
gh_status gh_heap_gc(gh_heap* h, const void* threshold, long long* kept, void* stream);

/* concurrentKernel (test/heap_test.cu:13-38, test/partial_heap_test.cu:13-38):
 * one launch in which the first half of the grid inserts keys_dev[0, n) in
 * insertion() calls of `chunk` keys (0 = batch_size) while the second half
 * makes n / batch_size deleteRoot/deleteUpdate attempts (an attempt on an
 * empty heap writes nothing).  Deleted keys go to out_dev[0, *n_out) one
 * batch after another (each batch ascending; batches in the order their
 * deletes took the root), at most max_keys of them.  The grid is at least 2
 * blocks.  Synchronizes the stream. */
gh_status gh_heap_concurrent(gh_heap* h, const void* keys_dev, long long n, int chunk, void* out_dev,
                             long long max_keys, long long* n_out, void* stream);

/* Waits for the stream and reports the first error the heap recorded on the
 * device (the bulk entry points above return before their kernels finish). */
gh_status gh_heap_sync(gh_heap* h, void* stream);

/* One Heap::insertion(items, size, 0) by one thread block
 * (heap/tditdd/heap.cuh:536, heap/buitdd/heap.cuh:484); 0 < size <= batch_size
 * (size 0 is a no-op). */
gh_status gh_heap_insert_batch(gh_heap* h, const void* keys_dev, int size, void* stream);
/* One Heap::deleteRoot(items, size) (+ deleteUpdate when it returns true) by
 * one thread block (heap/tditdd/heap.cuh:267-534).  HEAP_SORT semantics: the
 * keys land at out_dev + (the heap's output cursor), the cursor advances, and
 * gh_heap_reset sets it back to 0.  Synchronizes the stream; *size = keys written. */
gh_status gh_heap_delete_batch(gh_heap* h, void* out_dev, int* size, void* stream);

/* retrieve(ret, *size) (applications/sssp_longfei_new/heap.cuh:79-270) by
 * one thread block: the `size` smallest keys -- at most batch_size, fewer
 * when the heap holds fewer -- into out_dev[0, *n_out), ascending.  A delete
 * takes the root batch, the rest of it goes back in through the partial
 * buffer, so heaps without the partial buffer get GH_ERR_INVALID.
 * Synchronizes the stream. */
gh_status gh_heap_retrieve(gh_heap* h, void* out_dev, int size, int* n_out, void* stream);

/* The plain heap-sort (test/partial_heap_test.cu:88-176, without the
 * concurrent phase): reset, insert in_dev[0, n) in batch_size calls, then
 * delete everything into out_dev[0, n).  out_dev must hold n keys. */
gh_status gh_heap_sort(gh_heap* h, const void* in_dev, long long n, void* out_dev, void* stream);

/* The heap-sort with host buffers: keys_host[0, n) in, out_host[0, n) in key
 * order.  The copies cross on a stream of the heap's own in eight pieces of
 * whole batches: piece i goes in while piece i - 1 is inserted, and piece j
 * comes out while piece j + 1 is deleted, so the host link hides behind the
 * inserts and deletes (pinned host memory lets the copies overlap; pageable
 * memory works without the overlap).  Device staging buffers of n keys each
 * stay with the heap for the next call.  `stream` ends after the last copy.
 * Heaps without the partial buffer need n to be a multiple of batch_size. */
gh_status gh_heap_sort_host(gh_heap* h, const void* keys_host, long long n, void* out_host, void* stream);

/* checkInsertHeap(): heap/tditdd/heap.cuh:123-176, heap/buitdd/heap.cuh:118-172,
 * run on the device over the whole heap.  *ok = 1 when valid; otherwise msg
 * (if not NULL) describes the first violation.  Synchronizes the stream. */
gh_status gh_heap_check(gh_heap* h, int* ok, char* msg, int msg_len, void* stream);

/* itemCount() / nodeCount() / isEmpty(): heap/tditdd/heap.cuh:217-235. */
gh_status gh_heap_item_count(gh_heap* h, long long* n);
gh_status gh_heap_node_count(gh_heap* h, int* n);
gh_status gh_heap_is_empty(gh_heap* h, int* empty);

/* Host copy of the heap's memory (printHeap, heap/tditdd/heap.cuh:179-208):
 * items_host gets (batch_num + 1) * batch_size keys, status_host
 * batch_num + 1 lock words, counters_host {batchCount, partialBufferSize,
 * deleteCount, err, errOp, errNode, errState}.  Any pointer may be NULL. */
gh_status gh_heap_snapshot(gh_heap* h, void* items_host, int* status_host, int* counters_host);
/* Restores a heap from a snapshot taken with no operation in flight, by
 * this heap or another of the same key kind, variant, partial-buffer flag,
 * batch_num and batch_size: items_host holds (batch_num + 1) * batch_size
 * keys, counters_host at least {batchCount, partialBufferSize,
 * deleteCount}.  Every lock word becomes AVAIL and the error record, busy
 * count and park tickets are cleared.  The reference has no counterpart
 * (its nearest is Heap::reset, heap/tditdd/heap.cuh:69-91).  Synchronous;
 * GH_ERR_INVALID when the counters do not fit this heap. */
gh_status gh_heap_restore(gh_heap* h, const void* items_host, const int* counters_host);

/* Fault injection from the host, for tests of the bounded waits: writes
 * `state` into the lock word of `node` (synchronously).  A lock word left
 * taken makes the next operation that needs it wait out the heap's time
 * limit and report GH_ERR_TIMEOUT; gh_heap_reset clears it.  The reference
 * has no counterpart (its waits are unbounded, heap/tditdd/heap.cuh:250). */
gh_status gh_heap_inject_lock(gh_heap* h, int node, int state);

/* The device view for application kernels: writes the bytes of a
 * gh::Heap<K, variant, partial_buffer> (include/gpuheap_device.cuh) to
 * view_out (view_bytes must be >= gh_heap_view_bytes()).  Replaces the
 * shallow copy of the host object to the device (test/heap_test.cu:121-129). */
size_t gh_heap_view_bytes(void);
gh_status gh_heap_device_view(gh_heap* h, void* view_out, size_t view_bytes);

/* Dynamic shared memory one block needs for the heap's operations
 * (4 * batch_size keys of node buffers plus 144 bytes of control). */
size_t gh_heap_smem_bytes(int key_kind, int batch_size);

/* The plain heap-sort of gh_heap_sort for callers that cannot allocate device
 * memory when they sort: code running under a framework whose caching
 * allocator already holds the GPU's memory, or latency-critical code that
 * cannot pay the implicit device synchronization of cudaMalloc/cudaFree.  No
 * counterpart in the reference (its Heap<K> constructor always cudaMallocs).
 * It allocates nothing: the heap lives in a fixed 16 MiB array of device
 * memory inside this library (reserved on every GPU that loads the library,
 * until the process exits); only in_dev and out_dev come from the caller.
 * Limit: the heap needs ((ceil(n / batch_size) + 1) * batch_size * key bytes,
 * rounded up to 256) + (4 * (ceil(n / batch_size) + 2), rounded up to 256) +
 * 384 bytes (the counters) <= 16 MiB, e.g. about 4.1 M u32 keys at
 * batch_size 1024; larger n returns GH_ERR_CAPACITY and prints the sizes.
 * Without the partial buffer, n must be a multiple of batch_size
 * (GH_ERR_INVALID otherwise: a padded last batch would not fit out_dev).
 * Every call looks up the array's device address on the current device
 * (cudaGetSymbolAddress); the first call on a device also loads it, so make
 * that first call before any stream capture.  Every call reuses the same
 * array (cleared at the start of each call), so calls whose work overlaps
 * on the GPU -- other streams, other host threads -- race: serialize them.
 * Synchronizes `stream` to check the result. */
gh_status gh_sort_noalloc(int key_kind, int variant, int partial_buffer, int batch_size, const void* in_dev,
                          long long n, void* out_dev, void* stream);

/* Seeded synthetic keys for the plain heap-sort workload, made on the device:
 * key i depends only on (seed, i) (splitmix64 finaliser on seed + (i+1) *
 * 0x9e3779b97f4a7c15).  zipf = 0: u32 keys uniform in [0, 2^32 - 2];
 * zipf = 1: Zipf(1.2) over 2^16 distinct values.  u64 keys are
 * (u32 key << 32) | i, i32 keys u32 key - 2^31.  Stands in for the
 * reference drivers' rand() keys (test/heap_test.cu:114-119,
 * artifacts/synthetic/sort.cu:108-119). */
gh_status gh_gen_keys(int key_kind, int zipf, unsigned long long seed, long long n, void* out_dev, void* stream);

/* R-MAT edges (Chakrabarti et al. 2004): edge e gets `scale` quadrant choices
 * with probabilities a, b, c, 1-a-b-c from counter-based draws on (seed, e),
 * and a weight uniform in [1, max_weight].  Device outputs of m entries.
 * Stands in for the reference's graph files (applications/sssp_longfei_new/
 * main.cu:24-61, which are not in the repository). */
gh_status gh_rmat_edges(int scale, long long m, double a, double b, double c, unsigned long long seed,
                        unsigned max_weight, int* src_dev, int* dst_dev, unsigned* w_dev, void* stream);

/* Single-source shortest paths driven by the heap `h` (u64 keys, partial
 * buffer on, block threads <= batch size): the caller pattern of
 * applications/sssp_longfei_new/sssp.cu:19-132 (take a batch of
 * dist << 32 | vertex keys, skip stale ones, relax their edges with
 * atomicMin, insert the improved keys) on this repository's device API.
 * CSR graph with n vertices: rowptr_dev (n + 1, int64), col_dev (int32),
 * w_dev (u32).  dist_dev (n, u32) gets the distances, UINT32_MAX where
 * unreachable.  The heap is reset first.  Synchronizes; stats_host (may be
 * NULL) gets {keys taken, edges scanned, keys inserted}.  It runs on the
 * heap's grid (gh_heap_set_grid): few blocks with large batches are fastest,
 * because blocks that take batches at the same time take keys farther from
 * the minimum and expand vertices again, and all of them contend on the root
 * (on GB300, R-MAT 18-22: batch 2048 on 24 blocks). */
gh_status gh_sssp(gh_heap* h, int n, const long long* rowptr_dev, const int* col_dev, const unsigned* w_dev,
                  int source, unsigned* dist_dev, void* stream, unsigned long long* stats_host);

/* ------------------------------------------------------------------------
 * The retrieving heap of the reference's SSSP application
 * (applications/sssp_longfei_new/heap.cuh, heap_with_aux.cuh): 0-based nodes,
 * a separate partial buffer, top-down inserts, and retrieve(), which takes
 * the `size` smallest keys and refills the root in place -- from the partial
 * buffer or the last node, or, when an insert is still on its way down to
 * the last node, from that insert's batch handed over through the root (the
 * is_taken protocol).  Device code: include/gpuheap_retrieve.cuh
 * (gh::RetHeap<K>, gh::RetHeapAux<K, Aux>).  Keys u32 or u64; batch_size a
 * power of two in [16, 2048]; every operation is one thread block.
 * ------------------------------------------------------------------------ */
typedef struct gh_rheap gh_rheap;

/* Heap<T>(batch_num, batch_size, init_limit) (heap.cuh:56-64): init_limit
 * points to one key of the kind (NULL = its maximum).  Synchronizes. */
gh_status gh_rheap_create(gh_rheap** out, int key_kind, int batch_num, int batch_size, const void* init_limit);
gh_status gh_rheap_destroy(gh_rheap* h);
/* Empties the heap (nodes and partial buffer to init_limit, counters, lock
 * and is_taken words to zero). */
gh_status gh_rheap_reset(gh_rheap* h, void* stream);
/* Time limit of every device-side wait, in (0, 60] seconds (default 2 s). */
gh_status gh_rheap_set_timeout(gh_rheap* h, double seconds);
/* insert(items, count) (heap.cuh:272-382) by one thread block; 0 <= count
 * <= batch_size.  A full heap (batch count >= batch_num - 1) takes nothing
 * and records GH_ERR_CAPACITY (gh_rheap_state counters[2]); the reference
 * flags need_gc and drops the keys. */
gh_status gh_rheap_insert(gh_rheap* h, const void* keys_dev, int count, void* stream);
/* retrieve(ret, *size) (heap.cuh:79-270) by one thread block: *size in:
 * keys wanted; out: keys written to out_dev, the smallest held, ascending
 * (at most batch_size).  Synchronizes the stream. */
gh_status gh_rheap_retrieve(gh_rheap* h, void* out_dev, int* size, void* stream);
/* One launch of inserters + retrievers blocks: the first insert keys_dev[0,
 * n) in chunks of `chunk` keys, the others retrieve `size` keys at a time
 * until the inserters are done and the heap is empty.  Retrieved runs are
 * appended to out_dev (at most max_out keys); runs_dev[2r], runs_dev[2r+1]
 * = start and length of run r (at most max_runs).  *n_out, *n_runs: keys and
 * runs retrieved.  GH_ERR_CAPACITY when out_dev or runs_dev were too small.
 * Synchronizes the stream.  It has no counterpart in the reference: it is
 * the concurrent test of the is_taken hand-over. */
gh_status gh_rheap_concurrent(gh_rheap* h, const void* keys_dev, long long n, int chunk, int inserters, int retrievers,
                              int size, void* out_dev, long long max_out, int* runs_dev, int max_runs,
                              long long* n_out, int* n_runs, void* stream);
/* Host copies: items_host (batch_num * batch_size keys), pb_host (batch_size
 * keys), counters_host[6] = {batch count, partial-buffer size, device error,
 * retrieves that took an insert's batch through the root, inserts refused
 * as full, error site}; any pointer may be NULL.  Synchronizes the device. */
gh_status gh_rheap_state(gh_rheap* h, void* items_host, void* pb_host, long long* counters_host);
/* SSSP through the retrieving heap with the auxiliary buffer (the reference's
 * ssspKernel, applications/sssp_longfei_new/sssp.cu:19-132): `blocks` blocks
 * each retrieve up to batch_size keys with their edge offsets, relax at most
 * `chunk` edges of each current key, put keys with edges left back into the
 * buffer, and insert the improved vertices.  The search ends by the
 * busy-counter protocol (the reference's term_sig check, sssp.cu:58-70, can
 * end while a block still inserts).  A heap of capacity_keys (0: max(4 n,
 * m / 2) + 16 batches) keys is allocated for the call.  CSR graph and
 * distances as in gh_sssp.  stats_host (may be NULL): {keys taken, edges
 * relaxed, keys inserted, hand-overs through the root}.  Synchronizes. */
gh_status gh_sssp_retrieve(int n, const long long* rowptr_dev, const int* col_dev, const unsigned* w_dev, int source,
                           unsigned* dist_dev, int batch_size, int chunk, int blocks, long long capacity_keys,
                           void* stream, unsigned long long* stats_host);

/* ------------------------------------------------------------------------
 * Batched searches: many independent grid A* and 0/1 knapsack instances of
 * uneven size, each with its own heap (u64 keys, partial buffer), run by one
 * persistent launch.  The reference runs one search per process and launch
 * (artifacts/astar/main.cu, artifacts/knapsack/main.cu); its per-search
 * kernels are artifacts/astar/pq_model.cuh:299-371 and
 * artifacts/knapsack/models_pq.cuh:52-137, whose caller pattern the device
 * code follows.  A batch is built once (instances uploaded into one device
 * arena) and can then be run any number of times; each run starts every
 * search from scratch.
 * ------------------------------------------------------------------------ */
typedef struct gh_batch gh_batch;
typedef enum { GH_SEARCH_ASTAR = 0, GH_SEARCH_KNAPSACK = 1, GH_SEARCH_SSSP = 2 } gh_search_kind;
typedef enum { GH_BATCH_PERSISTENT = 0, GH_BATCH_GRAPH = 1, GH_BATCH_PLAIN = 2 } gh_batch_mode;
/* The knapsack search order (artifacts/knapsack/main.cu:100-130 models):
 * best-first on the heap (models_pq.cuh), breadth-first through a FIFO
 * ring (models_fifo.cuh), or the heap/FIFO switch (models.cuh:241-440). */
typedef enum { GH_KNAP_HEAP = 0, GH_KNAP_FIFO = 1, GH_KNAP_SWITCH = 2 } gh_knapsack_order;

/* batch_size: power of two in [32, 1024]; block_threads 0 (= min(batch_size,
 * 512)), batch_size or batch_size / 2, at most 512. */
gh_status gh_batch_create(gh_batch** out, int batch_size, int variant, int block_threads);
gh_status gh_batch_destroy(gh_batch* b);
/* Time limit of every device-side wait, in (0, 60] seconds (default 2 s). */
gh_status gh_batch_set_timeout(gh_batch* b, double seconds);
/* A* instances of width * height cells get min(max_blocks,
 * max(1, cells / cells_per_block)) blocks (default 2^18 cells, 8 blocks);
 * knapsack instances get one. */
gh_status gh_batch_set_astar_blocks(gh_batch* b, long long cells_per_block, int max_blocks);
/* Search order of every knapsack instance of the batch (default
 * GH_KNAP_HEAP); for GH_KNAP_SWITCH, `switch_counter` batches in a row
 * (> 0; the reference uses 20) that insert children without raising the
 * best profit move the nodes from the heap to the FIFO, and as many that
 * raise it move them back.  The FIFO orders give each knapsack instance a
 * ring of at least its node pool.  Takes effect at the next build. */
gh_status gh_batch_set_knapsack_order(gh_batch* b, int order, int switch_counter);
/* Heap/FIFO switches each knapsack instance made in the last run (0 for
 * other instances); switches_host holds one int per instance. */
gh_status gh_batch_knapsack_switches(gh_batch* b, int* switches_host, void* stream);
/* Grid A*: cost_host[y * width + x] in 1..9 is the cost of entering the cell,
 * 0 an obstacle; the search runs from (0, 0) to (width-1, height-1) with the
 * Manhattan heuristic (artifacts/astar/astar_map.cuh:137-138 keeps start and
 * goal free the same way).  Result: the optimal path cost, UINT32_MAX if the
 * goal is unreachable.  *id (may be NULL) gets the instance index. */
gh_status gh_batch_add_astar(gh_batch* b, int width, int height, const unsigned char* cost_host, int* id);
/* Grid A* on the reference's own model (artifacts/astar/pq_model.cuh:
 * 126-190, astar_map.cuh): open_host[y * width + x] != 0 marks an open
 * cell, the eight neighbours (-1,-1) (0,-1) (+1,-1) (-1,0) (+1,0) (-1,+1)
 * (0,+1) (+1,+1) cost 3 2 2 2 1 3 1 2, from (0, 0) to (width-1, height-1)
 * with the Manhattan heuristic.  Result: the optimal path cost (the
 * reference's final dist[target]), UINT32_MAX if unreachable. */
gh_status gh_batch_add_astar_bitmap(gh_batch* b, int width, int height, const unsigned char* open_host, int* id);
/* 0/1 knapsack with n <= 1024 items (weights >= 1, profits >= 0, total
 * profit < 2^30): best-first branch-and-bound on the Dantzig bound
 * (artifacts/knapsack/knapsackKernel.cuh:4-91).  Result: the optimum. */
gh_status gh_batch_add_knapsack(gh_batch* b, int n, const int* weight_host, const int* profit_host, long long capacity,
                                int* id);
/* Lays out one device arena for every instance and uploads them
 * (synchronizes the stream). */
gh_status gh_batch_build(gh_batch* b, void* stream);
/* Runs every search once: GH_BATCH_PERSISTENT one persistent launch over all
 * instances; GH_BATCH_GRAPH the same replayed from a CUDA graph captured on
 * the first call; GH_BATCH_PLAIN one launch per instance, back to back (the
 * reference's way).  Asynchronous. */
gh_status gh_batch_run(gh_batch* b, int mode, void* stream);
/* Milliseconds of each instance's own launch in the last GH_BATCH_PLAIN run
 * (events around every launch; waits for the run).  GH_ERR_INVALID before
 * any plain run.  No counterpart in the reference (its drivers time whole
 * runs). */
gh_status gh_batch_plain_times(gh_batch* b, float* ms_out);
/* Synchronizes and copies out per-instance results (may be NULL), status
 * (gh_status per instance, may be NULL) and stats (3 per instance: keys
 * taken, keys expanded, keys inserted; may be NULL).  Returns the first
 * instance failure, GH_OK if none. */
gh_status gh_batch_results(gh_batch* b, long long* results, int* status, unsigned long long* stats, void* stream);
/* Instances, tasks (block slots), blocks of the persistent launch, block
 * threads and arena bytes (any pointer may be NULL). */
gh_status gh_batch_info(gh_batch* b, int* count, int* tasks, int* grid, int* threads, long long* arena_bytes);

/* ------------------------------------------------------------------------
 * Served queries: a continuous-batching loop for SSSP and grid A* queries
 * of different sizes over resident graphs and maps.  Each admitted query
 * gets a slot and device memory (its heap and distance array) from one
 * arena; a query is admitted when a slot and enough memory are free, and
 * its heap stays on the device between steps.  One step is one persistent
 * launch over every admitted query in which each block takes at most
 * `batches_per_step` batches of a query before moving on; queries that
 * arrive meanwhile are admitted at the next step and their work overlaps on
 * the device with the others'.  The reference has no serving loop; its
 * per-query kernels are applications/sssp_longfei_new/sssp.cu:19-132 and
 * artifacts/astar/pq_model.cuh:299-371.
 * ------------------------------------------------------------------------ */
typedef struct gh_server gh_server;

/* arena_bytes of device memory for query state (0 = 60 % of the free
 * memory), max_slots concurrent queries, batch_size (power of two in
 * [32, 1024]) / variant of every query's heap (u64 keys, partial buffer),
 * batches_per_step as above. */
gh_status gh_serve_create(gh_server** out, long long arena_bytes, int max_slots, int batch_size, int variant,
                          int batches_per_step);
gh_status gh_serve_destroy(gh_server* s);
/* Blocks a query gets in each step: SSSP min(sssp_max_blocks, max(1,
 * n / vertices_per_block)) (default 2^15 vertices, 24 blocks), A*
 * min(astar_max_blocks, max(1, cells / cells_per_block)) (default 2^18
 * cells, 8 blocks).  Applies to queries submitted afterwards. */
gh_status gh_serve_set_blocks(gh_server* s, long long vertices_per_block, int sssp_max_blocks, long long cells_per_block,
                              int astar_max_blocks);
/* Resident datasets; the device arrays stay owned by the caller and must
 * outlive the server.  CSR graph as in gh_sssp (its edge count is read from
 * rowptr_dev[n], one synchronous copy); cost grid as in gh_batch_add_astar.
 * *id gets the dataset index.  A query's heap holds max(4 n, m / 2, 16
 * batches) keys on a graph of n vertices and m edges (the bound of
 * gh_sssp's heap), 64 keys per side of the larger grid dimension on a map. */
gh_status gh_serve_add_graph(gh_server* s, int n, const long long* rowptr_dev, const int* col_dev,
                             const unsigned* w_dev, int* id);
gh_status gh_serve_add_map(gh_server* s, int width, int height, const unsigned char* cost_dev, int* id);
/* A map on the reference's own model, as in gh_batch_add_astar_bitmap:
 * open_dev[y * width + x] != 0 marks an open cell; eight moves with the
 * reference's direction costs.  A* queries on it go from cell a to cell b. */
gh_status gh_serve_add_bitmap(gh_server* s, int width, int height, const unsigned char* open_dev, int* id);
/* Queues a query: GH_SEARCH_SSSP on graph `dataset` from vertex a (b unused),
 * or GH_SEARCH_ASTAR on map `dataset` from cell a to cell b.  *query gets its
 * id.  GH_ERR_CAPACITY if the query could never fit the arena. */
gh_status gh_serve_submit(gh_server* s, int kind, int dataset, int a, int b, long long* query);
/* One step: admit queued queries into free slots and memory (in arrival
 * order, skipping any that do not fit yet), run one launch over every
 * admitted query, collect the finished ones and free their memory.
 * Synchronizes the stream.  *finished gets how many queries finished in
 * this step, *active how many are still admitted, *queued how many wait
 * (any may be NULL). */
gh_status gh_serve_step(gh_server* s, void* stream, int* finished, int* active, int* queued);
/* Results of query `q`: *state 0 queued, 1 admitted, 2 finished, 3 failed;
 * SSSP: r0 = reachable vertices, r1 = sum of their distances; A*: r0 = the
 * optimal cost (UINT32_MAX unreachable), r1 = 0; a failed query: r0 = 0,
 * r1 = the failure's gh_status; *finish_step = the step in which it
 * finished.  Any pointer may be NULL. */
gh_status gh_serve_result(gh_server* s, long long q, int* state, unsigned long long* r0, unsigned long long* r1,
                          long long* finish_step);
/* Ids of the queries the last step finished (at most max_ids; *count gets
 * how many there were). */
gh_status gh_serve_finished(gh_server* s, long long* ids, int max_ids, int* count);
/* Arena bytes in use and free, slots in use, steps run (any may be NULL).
 * With the device loop: steps = launches of the loop. */
gh_status gh_serve_info(gh_server* s, long long* used_bytes, long long* free_bytes, int* slots_used, long long* steps);

/* The device-resident request loop.  gh_serve_start switches the server to
 * it (no query may be queued or admitted by gh_serve_step; the loop takes
 * over the whole arena).  From then on gh_serve_submit writes each query
 * into a request ring in pinned host memory, and one persistent launch of
 * the search kernel, on a stream of the server's own, admits requests into
 * free slots and memory (in arrival order, skipping any that do not fit
 * yet), resets and seeds their heaps, runs them with `batches_per_step`
 * batches per block stint, collects the finished ones, frees their memory
 * and writes their results into a completion ring, with no host step in
 * between.  The launch leaves after idle_ms (1 .. 600000) with nothing
 * admitted or waiting, and every wait in it has a limit.  gh_serve_poll
 * reads the completions (their ids through gh_serve_finished, their
 * results through gh_serve_result, finish_step = completion order), posts
 * queries that did not fit into the request ring yet, and launches the loop
 * again when work is outstanding; it neither synchronizes nor blocks.
 * *active gets the queries admitted on the device, *queued those not
 * admitted yet.  gh_serve_stop pauses the loop: the launch leaves after its
 * blocks' current stints, unfinished queries keep their state, and a later
 * gh_serve_start resumes them.  GH_ERR_TIMEOUT when a wait of the loop ran
 * out.  A device-wide synchronization waits for the launch to leave.  The
 * reference's counterpart is its host relaunch loop (artifacts/astar/
 * astar_main.cu:127-179). */
gh_status gh_serve_start(gh_server* s, int idle_ms);
gh_status gh_serve_poll(gh_server* s, int* finished, int* active, int* queued);
gh_status gh_serve_stop(gh_server* s);

/* Seeded synthetic cost grid for grid A* (host memory, `threads` host
 * threads): cell i draws r = splitmix64(seed + (i + 1) * golden ratio); it is
 * an obstacle (0) when (r >> 32) % 1000 < obstacle_per_mille, else its cost
 * is 1 + (r mod 2^32) % 9; the start and goal cells are never obstacles
 * (artifacts/astar/astar_map.cuh:137-138).  Stands in for the reference's
 * map files, which are not in the repository. */
gh_status gh_gen_grid(int width, int height, unsigned long long seed, int obstacle_per_mille, unsigned char* out_host,
                      int threads);

/* The heap's block primitives on their own, one block on `stream`, for tests
 * and tuning: no Heap<K> involved.  The reference tests its counterparts
 * (imergePath, ibitonicSort, heap/heaputil.cuh:23-47,99-158) with
 * local_test/merge_path; these are not entry points there.
 * gh_merge_batches: a_dev and b_dev each hold n sorted keys (n a power of
 * two in [16, 8192]); the n smallest of both go to lo_dev, the n largest to
 * hi_dev, in order.  method 0: the merge of every insert and sift step (merge
 * path, 2n / threads keys per thread, 1..16); method 1: the owner-mode
 * delete's warp-window merge (windows of 1024 four-byte or 512 eight-byte
 * keys, so 2n at least one window).  gh_sort_batch: sorts in_dev[0, n) (n a
 * power of two in [2, 8192]) into out_dev with the insert batch's bitonic
 * network.  threads: a power of two in [32, 1024]. */
gh_status gh_merge_batches(int key_kind, int method, const void* a_dev, const void* b_dev, int n, void* lo_dev,
                           void* hi_dev, int threads, void* stream);
gh_status gh_sort_batch(int key_kind, const void* in_dev, int n, void* out_dev, int threads, void* stream);

/* Number of kernels this library has launched since it was loaded. */
long long gh_launch_count(void);

/* Counters of the last owner-mode bulk delete on this heap (gh_heap_delete
 * and gh_heap_sort run one when the heap is deep enough; it has no
 * counterpart in the reference, whose deleteKernel is the plain loop).  Up to
 * n of: [0] deletes made by the owner block, SM cycles of its delete loop
 * spent [1] waiting for the next last node, [2] waiting for a lent node to
 * come back, [3] waiting for room to lend, [4] planning paths, [5] merging;
 * [6] general sift steps; [7] cycles of the whole loop; the last-node taker's
 * cycles [8] in lock waits, [9] in bulk loads, [10] idle; [11] lends;
 * [12] lent nodes taken back.  Synchronizes the device.  All zero when the
 * heap has no owner mode (batch_size below 512) or none has run. */
gh_status gh_heap_owner_stats(gh_heap* h, unsigned long long* out, int n);

/* Properties. */
gh_status gh_heap_info(gh_heap* h, int* key_kind, int* variant, int* partial_buffer, int* batch_num,
                       int* batch_size, int* block_threads, int* grid);

#ifdef __cplusplus
}
#endif
#endif
