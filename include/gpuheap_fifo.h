/* gpuheap_fifo.h -- C ABI of the device FIFO buffer.
 *
 * Replaces the reference's Buffer<K> (artifacts/buffer/buffer.cuh:6-218) and
 * the kernels of its test driver (artifacts/buffer/bufferTest.cu:13-56).
 * Keys are u32, i32 or u64 (gh_key_kind); device pointers are raw CUDA
 * pointers, streams are cudaStream_t passed as void* (NULL = legacy stream).
 * Device-side waits are bounded: past the time limit the operation records
 * GH_ERR_TIMEOUT and every later call returns GH_ERR_STATE until
 * gh_fifo_reset.  The device form for application kernels is gh::Fifo<K>
 * (include/gpuheap_fifo.cuh).
 */
#ifndef GPUHEAP_FIFO_H
#define GPUHEAP_FIFO_H

#include <stddef.h>

#include "gpuheap.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gh_fifo gh_fifo;

/* Buffer<K>(capacity): buffer.cuh:29-51.  The ring holds `capacity` keys,
 * rounded up to a power of two (gh_fifo_info reports it); at most 2^34. */
gh_status gh_fifo_create(gh_fifo** out, int key_kind, long long capacity);
/* ~Buffer(): buffer.cuh:53-64. */
gh_status gh_fifo_destroy(gh_fifo* f);
/* Empties the ring (all four positions to 0) and clears a recorded error. */
gh_status gh_fifo_reset(gh_fifo* f, void* stream);
/* Time limit of every device-side wait, in (0, 60] seconds (default 2 s). */
gh_status gh_fifo_set_timeout(gh_fifo* f, double seconds);
/* Launch shape of the bulk calls: blocks (0 = as many as stay resident) and
 * threads per block (0 = 512; a multiple of 32 in [32, 1024]). */
gh_status gh_fifo_set_launch(gh_fifo* f, int blocks, int threads);

/* insertKernel (bufferTest.cu:39-47): appends keys_dev[0, n).
 * chunk > 0: the blocks push pieces of `chunk` keys, one insertToBuffer
 * (buffer.cuh:127-170) per piece; pieces keep their key order and enter the
 * ring whole, in the order their blocks reserved them (one block: the input
 * order).  chunk == 0: the whole call is one reservation, copied by the
 * whole grid and published once by the last block to finish, so the keys
 * enter in input order at the speed of a copy (a piece-by-piece push is
 * bound by the in-order publishing of its pieces).
 * GH_ERR_CAPACITY, before any launch, if the ring cannot hold its keys plus
 * n (nothing removes keys during this call); the keys held are bounded on
 * the host from earlier calls and read from the device only when that bound
 * does not fit, so a push does not synchronise in the common case. */
gh_status gh_fifo_push(gh_fifo* f, const void* keys_dev, long long n, int chunk, void* stream);

/* deleteKernel (bufferTest.cu:49-56): takes up to max_keys keys, in FIFO
 * order, into out_dev[0, n).  chunk > 0: the blocks call deleteFromBuffer
 * (buffer.cuh:172-214) for up to `chunk` keys at a time until max_keys were
 * taken or the ring is empty.  chunk == 0: one claim of min(max_keys, keys
 * published) for the whole call, copied by the whole grid.  *n_out (may be
 * NULL; then the call does not synchronise) gets n. */
gh_status gh_fifo_pop(gh_fifo* f, void* out_dev, long long max_keys, int chunk, long long* n_out, void* stream);

/* concurrentKernel (bufferTest.cu:13-37): in one launch half the blocks
 * push keys_dev[0, n) (each piece of `chunk` keys -- 0 = 1024, or the
 * capacity when smaller -- in two calls, its first third and then the
 * rest) while the other half take exactly max_keys keys, up to `chunk` at
 * a time, waiting while the ring is empty; out_dev as for gh_fifo_pop.  max_keys
 * must not exceed the keys already held plus n, and the keys held plus n
 * minus max_keys must fit the ring (otherwise a wait could never end:
 * GH_ERR_INVALID / GH_ERR_CAPACITY before any launch).  Synchronises. */
gh_status gh_fifo_concurrent(gh_fifo* f, const void* keys_dev, long long n, int chunk, void* out_dev,
                             long long max_keys, long long* n_out, void* stream);

/* Keys held (pushed and not yet taken); synchronises the device. */
gh_status gh_fifo_count(gh_fifo* f, long long* n);
/* printBufferPtr (buffer.cuh:88-96): the four positions
 * begin <= read <= write <= end, in keys since creation or reset. */
gh_status gh_fifo_positions(gh_fifo* f, unsigned long long* begin, unsigned long long* read,
                            unsigned long long* write, unsigned long long* end);
/* printBuffer (buffer.cuh:98-123): copies the ring (capacity keys) and the
 * four positions to host memory. */
gh_status gh_fifo_snapshot(gh_fifo* f, void* items_host, unsigned long long* positions_host);

/* Bytes of a gh::Fifo<K> for application kernels, and the view itself
 * (replaces the shallow copy of Buffer<K> to the device, bufferTest.cu:90-92). */
size_t gh_fifo_view_bytes(void);
gh_status gh_fifo_device_view(gh_fifo* f, void* view_out, size_t view_bytes);

/* Test hook: reserves n slots that are never published, as a pusher that
 * stopped between its reservation and its commit would; a later push waits
 * for it until the time limit.  Failure detection is tested with it. */
gh_status gh_fifo_inject_reservation(gh_fifo* f, long long n);

/* Properties: key kind, ring capacity, blocks and threads of the bulk calls
 * (resolved), recorded error site (0 none; 1 room, 2 publish, 3 claim,
 * 4 free, 5 empty). */
gh_status gh_fifo_info(gh_fifo* f, int* key_kind, long long* capacity, int* blocks, int* threads, int* err_site);

#ifdef __cplusplus
}
#endif

#endif /* GPUHEAP_FIFO_H */
