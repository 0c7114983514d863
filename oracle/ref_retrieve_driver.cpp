// C entry points around the reference's retrieving heap
// (applications/sssp_longfei_new/heap.cuh: Heap<T> with retrieve() and
// insert(), used by that SSSP application), compiled for the host with
// ref_shim.h and run single-threaded.
//
// TEST INFRASTRUCTURE ONLY (builds into oracle/_ref/, never shipped).
// Entry points (T in {u32, u64}):
//   rr_T_create(batchNum, batchSize, init_limit) -> handle
//   rr_T_insert(h, items, count)     Heap::insert (count <= batchSize)
//   rr_T_retrieve(h, out, *size)     Heap::retrieve; *size in: wanted, out: taken
//   rr_T_state(h, items, pb, counters)  node keys, partial buffer keys,
//                                    {curr_batch_count, curr_pb_size}
//   rr_T_destroy(h)
// Calls return 0, or -1 if the sequential run hit a lock state it cannot
// leave (ShimSpinError).  Every call starts from a cleared shared-memory
// stand-in and spin counter, so a sequence's outcome does not depend on
// what ran before it in the process.
#include "ref_shim.h"

namespace rr {
char smem[1 << 22];
#include "heap.cuh"
}  // namespace rr

namespace {

inline void fresh_call() {
    std::memset(rr::smem, 0, sizeof(rr::smem));
    g_shim_fail_streak = 0;
}

template <typename T>
void* create_t(int bn, int bs, T init) {
    return new rr::Heap<T>(bn, bs, init);
}

template <typename T>
int insert_t(void* hp, const T* items, int count) {
    auto* h = static_cast<rr::Heap<T>*>(hp);
    fresh_call();
    int need_gc = 0, rwlock_y = 0;
    try {
        h->insert(const_cast<T*>(items), count, 0, &need_gc, &rwlock_y);
    } catch (const ShimSpinError&) {
        return -1;
    }
    return need_gc ? -2 : 0;
}

template <typename T>
int retrieve_t(void* hp, T* out, int* size) {
    auto* h = static_cast<rr::Heap<T>*>(hp);
    fresh_call();
    try {
        h->retrieve(out, size, 0);
    } catch (const ShimSpinError&) {
        return -1;
    }
    return 0;
}

template <typename T>
int state_t(void* hp, T* items, T* pb, int* counters) {
    auto* h = static_cast<rr::Heap<T>*>(hp);
    const size_t n = static_cast<size_t>(h->batch_num) * h->batch_size;
    for (size_t i = 0; i < n; ++i) items[i] = h->items[i];
    for (int i = 0; i < h->batch_size; ++i) pb[i] = h->partial_buffer[i];
    counters[0] = h->curr_batch_count;
    counters[1] = h->curr_pb_size;
    return 0;
}

}  // namespace

#define RR_EXPORT(T, tag)                                                                               \
    extern "C" void* rr_##tag##_create(int bn, int bs, T init) { return create_t<T>(bn, bs, init); }  \
    extern "C" int rr_##tag##_insert(void* h, const T* it, int n) { return insert_t<T>(h, it, n); }     \
    extern "C" int rr_##tag##_retrieve(void* h, T* out, int* sz) { return retrieve_t<T>(h, out, sz); } \
    extern "C" int rr_##tag##_state(void* h, T* it, T* pb, int* c) { return state_t<T>(h, it, pb, c); } \
    extern "C" void rr_##tag##_destroy(void* h) { delete static_cast<rr::Heap<T>*>(h); }

RR_EXPORT(uint32_t, u32)
RR_EXPORT(uint64_t, u64)
