// C entry points around the reference's own Heap<K> class, compiled for the
// host with ref_shim.h and run single-threaded.
//
// TEST INFRASTRUCTURE ONLY (builds into oracle/_ref/, never shipped).  Compiled
// once per reference variant with -I<reference>/heap/<variant> and
// -DREF_NS=<variant>; each copy lives in its own namespace so the four
// different `class Heap` definitions cannot collide at link time.
//
// Entry points (per variant V and key type T in {u32, u64, i32}):
//   V_T_create(batchNum, batchSize, init_limits) -> handle
//   V_T_insert(h, items, size)      one Heap::insertion call   (heap.cuh insertion)
//   V_T_delete(h, out, *size)       Heap::deleteRoot (+ deleteUpdate when it returns true),
//                                   HEAP_SORT output at out + deleteCount
//   V_T_state(h, items, status, counters)  copy of heapItems, status, and
//                                   {batchCount, partialBufferSize, deleteCount}
//   V_T_check(h)                    Heap::checkInsertHeap
//   V_T_destroy(h)
// Every call returns 0 on success and -1 if the sequential run hit a lock
// state it cannot leave (see ShimSpinError).
#include "ref_shim.h"

#ifndef REF_NS
#error "REF_NS must name the reference variant"
#endif
#ifndef HEAP_SORT
#define HEAP_SORT
#endif

// Shared-memory stand-in: the reference addresses `extern __shared__ int s[]`
// by 4-byte word offsets; the block-scope extern declarations inside the
// namespace resolve to this array.
namespace REF_NS {
int s[1 << 21];
#include "heap.cuh"
}  // namespace REF_NS

#define GH_CAT2(a, b) a##b
#define GH_CAT(a, b) GH_CAT2(a, b)
#define GH_FN(name) GH_CAT(REF_NS, name)

namespace {

template <typename K>
struct Box {
    REF_NS::Heap<K>* h;
};

template <typename K>
void* create_t(int batchNum, int batchSize, K init) {
    auto* b = new Box<K>;
    b->h = new REF_NS::Heap<K>(batchNum, batchSize, init);
    return b;
}

// Every call starts from the same shared-memory stand-in and spin counter.
// Both are process-wide and would otherwise carry one call's leftovers into
// the next, so that a fixed operation sequence could end differently
// depending on what ran before it in the same process.
inline void fresh_call() {
    std::memset(REF_NS::s, 0, sizeof(REF_NS::s));
    g_shim_fail_streak = 0;
}

template <typename K>
int insert_t(void* hb, const K* items, int size) {
    auto* b = static_cast<Box<K>*>(hb);
    fresh_call();
    try {
        b->h->insertion(const_cast<K*>(items), size, 0);
    } catch (const ShimSpinError&) {
        return -1;
    }
    return 0;
}

template <typename K>
int delete_t(void* hb, K* out, int* size) {
    auto* b = static_cast<Box<K>*>(hb);
    int sz = 0;
    fresh_call();
    try {
        if (b->h->deleteRoot(out, sz)) b->h->deleteUpdate(0);
    } catch (const ShimSpinError&) {
        return -1;
    }
    *size = sz;
    return 0;
}

template <typename K>
int state_t(void* hb, K* items, int* status, int* counters) {
    auto* b = static_cast<Box<K>*>(hb);
    REF_NS::Heap<K>* h = b->h;
    size_t nodes = static_cast<size_t>(h->batchNum) + 1;
    if (items) std::memcpy(items, h->heapItems, sizeof(K) * nodes * h->batchSize);
    if (status) std::memcpy(status, h->status, sizeof(int) * nodes);
    if (counters) {
        counters[0] = *h->batchCount;
        counters[1] = *h->partialBufferSize;
        counters[2] = *h->deleteCount;
    }
    return 0;
}

template <typename K>
int check_t(void* hb) {
    auto* b = static_cast<Box<K>*>(hb);
    return b->h->checkInsertHeap() ? 1 : 0;
}

template <typename K>
void destroy_t(void* hb) {
    auto* b = static_cast<Box<K>*>(hb);
    delete b->h;
    delete b;
}

}  // namespace

#define GH_EXPORT_TYPE(T, tag)                                                                   \
    extern "C" void* GH_FN(_##tag##_create)(int bn, int bs, T init) { return create_t<T>(bn, bs, init); } \
    extern "C" int GH_FN(_##tag##_insert)(void* h, const T* it, int sz) { return insert_t<T>(h, it, sz); } \
    extern "C" int GH_FN(_##tag##_delete)(void* h, T* out, int* sz) { return delete_t<T>(h, out, sz); }    \
    extern "C" int GH_FN(_##tag##_state)(void* h, T* it, int* st, int* c) { return state_t<T>(h, it, st, c); } \
    extern "C" int GH_FN(_##tag##_check)(void* h) { return check_t<T>(h); }                            \
    extern "C" void GH_FN(_##tag##_destroy)(void* h) { destroy_t<T>(h); }

GH_EXPORT_TYPE(uint32_t, u32)
GH_EXPORT_TYPE(uint64_t, u64)
GH_EXPORT_TYPE(int32_t, i32)
