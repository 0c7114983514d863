// Launchers for the heap kernels, instantiated once per key type in
// heap_inst_{u32,i32,u64}.cu so the three instantiation sets compile in
// parallel.  The merge width IPT = 2 * batchSize / threads is a template
// parameter of every kernel (1, 2, 4 or 8 keys per thread per merge).
#pragma once
#include <cuda_runtime.h>

#include "heap_kernels.cuh"
#include "owner_delete.cuh"

namespace gh {
namespace impl {

struct LaunchArgs {
    const Desc* d;
    int threads;
    int grid;
    cudaStream_t stream;
    int* opSize;
    bool reserve = true;  // bulk inserts of full batches may reserve their targets (k_reserve)
};

template <typename K>
cudaError_t launch_insert(const LaunchArgs& a, const K* keys, long long n, int chunk);
template <typename K>
cudaError_t launch_erase(const LaunchArgs& a, K* out, const K* threshold = nullptr);
template <typename K>
cudaError_t launch_erase_one(const LaunchArgs& a, K* out);
template <typename K>
cudaError_t launch_retrieve(const LaunchArgs& a, K* out, int want, K* scratch);
template <typename K>
cudaError_t launch_insert_counted(const LaunchArgs& a, const K* keys, const unsigned long long* n, int chunk);
template <typename K>
cudaError_t launch_concurrent(const LaunchArgs& a, const K* keys, long long n, int chunk, K* out, long long deletes);
// Bytes of gh::Heap<K, variant, pb> (IPT chosen at run time) for application kernels.
template <typename K>
void device_view(const Desc& d, void* out, size_t* bytes);

#ifdef GH_INSTANTIATE
template <typename H>
inline cudaError_t allow_smem(const void* fn, size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
}

// At most as many blocks as the GPU holds at once.  The reserved bulk insert
// hands batch j to block j mod grid, and an insert may wait for a parent
// target that an earlier batch fills; the owner-mode delete's owner waits
// for workers.  Both make progress only if every block runs, so a grid
// larger than the resident set would wait until the time limit.
inline int resident_grid(const void* fn, int threads, size_t smem, int want) {
    int per = 0, dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem) != cudaSuccess || per < 1) {
        cudaGetLastError();
        return want;
    }
    const long long cap = static_cast<long long>(per) * sms;
    return want < cap ? want : static_cast<int>(cap);
}

// Calls f(Heap<K, V, PB, IPT>{}) for the run-time variant, pb flag and IPT.
template <typename K, typename F>
inline cudaError_t dispatch(const Desc& d, int threads, F&& f) {
    const int ipt = 2 * d.batchSize / threads;
    auto by_ipt = [&](auto v, auto pb) -> cudaError_t {
        constexpr int V = decltype(v)::value;
        constexpr bool PB = decltype(pb)::value;
        switch (ipt) {
            case 1: return f(Heap<K, V, PB, 1>{});
            case 2: return f(Heap<K, V, PB, 2>{});
            case 4: return f(Heap<K, V, PB, 4>{});
            case 8: return f(Heap<K, V, PB, 8>{});
            default: return cudaErrorInvalidValue;
        }
    };
    using TDv = std::integral_constant<int, kTopDown>;
    using BUv = std::integral_constant<int, kBottomUp>;
    using Yes = std::integral_constant<bool, true>;
    using No = std::integral_constant<bool, false>;
    if (d.variant == kTopDown) return d.pb ? by_ipt(TDv{}, Yes{}) : by_ipt(TDv{}, No{});
    return d.pb ? by_ipt(BUv{}, Yes{}) : by_ipt(BUv{}, No{});
}

template <typename H>
inline H view_of(const Desc& d, int sortOutput) {
    H h;
    h.heapItems = static_cast<typename H::key_type*>(d.items);
    h.status = d.status;
    h.state = d.state;
    __builtin_memcpy(&h.init_limits, &d.initBits, sizeof(typename H::key_type));
    h.batchNum = d.batchNum;
    h.batchSize = d.batchSize;
    h.sortOutput = sortOutput;
    h.timeoutNs = d.timeoutNs;
    return h;
}

// Full batches (chunk == batchSize) go to targets reserved up front when the
// partial buffer is empty (k_reserve, k_mark_reserved, k_insert_reserved);
// a ragged last chunk, or any other chunk size, goes through insertion().
template <typename K>
cudaError_t launch_insert(const LaunchArgs& a, const K* keys, long long n, int chunk) {
    return dispatch<K>(*a.d, a.threads, [&](auto proto) -> cudaError_t {
        using H = decltype(proto);
        const H h = view_of<H>(*a.d, 1);
        const int B = a.d->batchSize;
        const size_t smem = H::smemBytes(B);
        const long long m = (a.reserve && chunk == B) ? n / B : 0;
        if (m > 0) {
            cudaError_t e = allow_smem<H>(reinterpret_cast<const void*>(k_insert_reserved<H, K>), smem);
            if (e != cudaSuccess) return e;
            k_reserve<<<1, 1, 0, a.stream>>>(a.d->state, a.d->batchNum, m);
            count_launch();
            const int held = a.d->variant == kTopDown ? TD::TARGET : BU::INUSE;
            const long long mb = (m + 255) / 256;
            k_mark_reserved<<<static_cast<int>(mb < 1024 ? mb : 1024), 256, 0, a.stream>>>(a.d->state, a.d->status, held);
            count_launch();
            const int g = resident_grid(reinterpret_cast<const void*>(k_insert_reserved<H, K>), a.threads, smem,
                                        static_cast<int>(m < a.grid ? m : a.grid));
            k_insert_reserved<H, K><<<g, a.threads, smem, a.stream>>>(h, keys, m);
            count_launch();
            e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
        const long long rest = n - m * B;
        if (rest <= 0) return cudaSuccess;
        cudaError_t e = allow_smem<H>(reinterpret_cast<const void*>(k_insert<H, K>), smem);
        if (e != cudaSuccess) return e;
        const long long nchunks = (rest + chunk - 1) / chunk;
        const int g = static_cast<int>(nchunks < a.grid ? nchunks : a.grid);
        k_insert<H, K><<<g, a.threads, smem, a.stream>>>(h, keys + m * B, rest, chunk);
        count_launch();
        return cudaGetLastError();
    });
}

template <typename K>
cudaError_t launch_insert_counted(const LaunchArgs& a, const K* keys, const unsigned long long* n, int chunk) {
    return dispatch<K>(*a.d, a.threads, [&](auto proto) -> cudaError_t {
        using H = decltype(proto);
        const H h = view_of<H>(*a.d, 1);
        const size_t smem = H::smemBytes(a.d->batchSize);
        cudaError_t e = allow_smem<H>(reinterpret_cast<const void*>(k_insert_counted<H, K>), smem);
        if (e != cudaSuccess) return e;
        k_insert_counted<H, K><<<a.grid, a.threads, smem, a.stream>>>(h, keys, n, chunk);
        count_launch();
        return cudaGetLastError();
    });
}

// Without a threshold, a heap with a mailbox first runs the owner-mode bulk
// delete (k_delete_owner, 1024-thread blocks) while it has nodes below its
// resident levels, then deleteKernel finishes; with a threshold,
// deleteKernel alone.
template <typename K>
cudaError_t launch_erase(const LaunchArgs& a, K* out, const K* threshold) {
    const int R = a.d->ownerDepth < 0 ? owner_depth(a.d->batchSize, a.d->keyBytes) : a.d->ownerDepth;
    if (!threshold && a.d->mbox && R > 0 && a.grid >= 2) {
        cudaError_t e = cudaMemsetAsync(a.d->mbox, 0, sizeof(Mailbox), a.stream);
        if (e != cudaSuccess) return e;
        e = dispatch<K>(*a.d, 1024, [&](auto proto) -> cudaError_t {
            using H = decltype(proto);
            const H h = view_of<H>(*a.d, 1);
            const size_t smem = owner_smem(a.d->batchSize, a.d->keyBytes, R);
            cudaError_t e2 = allow_smem<H>(reinterpret_cast<const void*>(k_delete_owner<H, K>), smem);
            if (e2 != cudaSuccess) return e2;
            Mailbox* mb = static_cast<Mailbox*>(a.d->mbox);
            K* mdata = reinterpret_cast<K*>(static_cast<char*>(a.d->mbox) + sizeof(Mailbox));
            const int g = resident_grid(reinterpret_cast<const void*>(k_delete_owner<H, K>), 1024, smem, a.grid);
            k_delete_owner<H, K><<<g, 1024, smem, a.stream>>>(h, out, mb, mdata, R);
            count_launch();
            return cudaGetLastError();
        });
        if (e != cudaSuccess) return e;
    }
    return dispatch<K>(*a.d, a.threads, [&](auto proto) -> cudaError_t {
        using H = decltype(proto);
        const H h = view_of<H>(*a.d, 1);
        const size_t smem = H::smemBytes(a.d->batchSize);
        cudaError_t e = allow_smem<H>(reinterpret_cast<const void*>(k_delete<H, K>), smem);
        if (e != cudaSuccess) return e;
        k_delete<H, K><<<a.grid, a.threads, smem, a.stream>>>(h, out, threshold ? *threshold : h.init_limits,
                                                               threshold ? 1 : 0);
        count_launch();
        return cudaGetLastError();
    });
}

template <typename K>
cudaError_t launch_concurrent(const LaunchArgs& a, const K* keys, long long n, int chunk, K* out, long long deletes) {
    return dispatch<K>(*a.d, a.threads, [&](auto proto) -> cudaError_t {
        using H = decltype(proto);
        const H h = view_of<H>(*a.d, 1);
        const size_t smem = H::smemBytes(a.d->batchSize);
        cudaError_t e = allow_smem<H>(reinterpret_cast<const void*>(k_concurrent<H, K>), smem);
        if (e != cudaSuccess) return e;
        k_concurrent<H, K><<<a.grid, a.threads, smem, a.stream>>>(h, keys, n, chunk, out, deletes);
        count_launch();
        return cudaGetLastError();
    });
}

template <typename K>
cudaError_t launch_erase_one(const LaunchArgs& a, K* out) {
    return dispatch<K>(*a.d, a.threads, [&](auto proto) -> cudaError_t {
        using H = decltype(proto);
        const H h = view_of<H>(*a.d, 1);
        const size_t smem = H::smemBytes(a.d->batchSize);
        cudaError_t e = allow_smem<H>(reinterpret_cast<const void*>(k_delete_one<H, K>), smem);
        if (e != cudaSuccess) return e;
        k_delete_one<H, K><<<1, a.threads, smem, a.stream>>>(h, out, a.opSize);
        count_launch();
        return cudaGetLastError();
    });
}

template <typename K>
cudaError_t launch_retrieve(const LaunchArgs& a, K* out, int want, K* scratch) {
    return dispatch<K>(*a.d, a.threads, [&](auto proto) -> cudaError_t {
        using H = decltype(proto);
        const H h = view_of<H>(*a.d, 0);  // outputs at scratch[0]
        const size_t smem = H::smemBytes(a.d->batchSize);
        cudaError_t e = allow_smem<H>(reinterpret_cast<const void*>(k_retrieve<H, K>), smem);
        if (e != cudaSuccess) return e;
        k_retrieve<H, K><<<1, a.threads, smem, a.stream>>>(h, out, want, scratch, a.opSize);
        count_launch();
        return cudaGetLastError();
    });
}

template <typename K>
void device_view(const Desc& d, void* out, size_t* bytes) {
    auto put = [&](auto proto) {
        using H = decltype(proto);
        const H h = view_of<H>(d, 0);
        __builtin_memcpy(out, &h, sizeof(H));
        *bytes = sizeof(H);
    };
    if (d.variant == kTopDown) { if (d.pb) put(Heap<K, kTopDown, true>{}); else put(Heap<K, kTopDown, false>{}); }
    else { if (d.pb) put(Heap<K, kBottomUp, true>{}); else put(Heap<K, kBottomUp, false>{}); }
}

#define GH_INSTANTIATE_KEY(K)                                                                    \
    template cudaError_t launch_insert<K>(const LaunchArgs&, const K*, long long, int);          \
    template cudaError_t launch_erase<K>(const LaunchArgs&, K*, const K*);                       \
    template cudaError_t launch_insert_counted<K>(const LaunchArgs&, const K*, const unsigned long long*, int); \
    template cudaError_t launch_erase_one<K>(const LaunchArgs&, K*);                             \
    template cudaError_t launch_retrieve<K>(const LaunchArgs&, K*, int, K*);                     \
    template cudaError_t launch_concurrent<K>(const LaunchArgs&, const K*, long long, int, K*, long long); \
    template void device_view<K>(const Desc&, void*, size_t*);
#endif  // GH_INSTANTIATE

}  // namespace impl
}  // namespace gh
