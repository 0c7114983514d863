// Host stand-ins for the CUDA built-ins that the reference BGPQ heap headers use.
//
// TEST INFRASTRUCTURE ONLY. This header lets the reference's own heap headers
// (heap/{tditdd,tditdd_np,buitdd,buitdd_np}/heap.cuh and heap/heaputil.cuh)
// compile as plain C++ and run with ONE "thread" (blockDim = 1), so that every
// block-collective loop in them runs sequentially on the CPU.  The outputs of
// that run are what pins the project's own oracle restatement (oracle/bgpq_oracle.cpp).
// Nothing in the product links against this.
#pragma once
#include <cstdint>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <stdexcept>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __inline__ inline
#define __shared__

struct ShimDim3 { unsigned x, y, z; };
static ShimDim3 threadIdx = {0u, 0u, 0u};
static ShimDim3 blockIdx = {0u, 0u, 0u};
static ShimDim3 blockDim = {1u, 1u, 1u};
static ShimDim3 gridDim = {1u, 1u, 1u};

inline void __syncthreads() {}

inline int __clz(int x) { return x == 0 ? 32 : __builtin_clz(static_cast<unsigned>(x)); }

// __brev returns a wrapper so that a right shift by 32 or more yields 0, as
// the GPU's shr does; the reference computes `__brev(i) >> (clz(i) + 1)`,
// which is a shift by 32 for i == 1 (undefined behaviour for a plain
// 32-bit shift on the host).
struct ShimBrev { unsigned v; };
inline unsigned operator>>(ShimBrev b, int s) { return (s >= 32 || s < 0) ? 0u : (b.v >> s); }
inline ShimBrev __brev(unsigned x) {
    unsigned r = 0;
    for (int i = 0; i < 32; ++i) { r = (r << 1) | (x & 1u); x >>= 1; }
    return ShimBrev{r};
}

// A single-threaded run can never see a lock word change under it, so a CAS
// that keeps failing means the sequential schedule reached a state the lock
// protocol cannot leave.  Throw instead of spinning forever.
struct ShimSpinError : std::runtime_error {
    explicit ShimSpinError(const char* m) : std::runtime_error(m) {}
};
static thread_local long long g_shim_fail_streak = 0;

inline int atomicCAS(int* a, int cmp, int val) {
    int old = *a;
    if (old == cmp) { *a = val; g_shim_fail_streak = 0; }
    else if (++g_shim_fail_streak > (1 << 16)) {
        g_shim_fail_streak = 0;
        throw ShimSpinError("lock word never reached the expected state");
    }
    return old;
}
inline int atomicAdd(int* a, int v) { int old = *a; *a += v; return old; }
inline int atomicExch(int* a, int v) { int old = *a; *a = v; return old; }
inline void __threadfence() {}
inline int atomicSub(int* a, int v) { int old = *a; *a -= v; return old; }
inline int atomicMax(int* a, int v) {
    int old = *a;
    if (v > old) *a = v;
    if (old == v && ++g_shim_fail_streak > (1 << 16)) {
        g_shim_fail_streak = 0;
        throw ShimSpinError("atomicMax spin never saw the word released");
    }
    if (old != v) g_shim_fail_streak = 0;
    return old;
}
inline unsigned atomicCAS(unsigned* a, unsigned cmp, unsigned val) {
    unsigned old = *a; if (old == cmp) *a = val; return old;
}

typedef int cudaError_t;
enum ShimMemcpyKind { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };
// Device allocations come back zeroed, with as much room again behind them
// filled with 0x7f bytes.  On a padded node the reference's top-down sift
// without the partial buffer reads lock words past its status array
// (tditdd_np/heap.cuh:356, found with AddressSanitizer).  In that room they
// read 0x7f7f7f7f, neither AVAIL nor INUSE, which the sift takes as "no
// valid child" (:352-354).  The outcome is then the same on every run,
// instead of depending on whatever the host heap held there.
inline cudaError_t cudaMalloc(void** p, size_t n) {
    const size_t m = n ? n : 1;
    unsigned char* q = static_cast<unsigned char*>(std::malloc(2 * m + 4096));
    if (!q) return 2;
    std::memset(q, 0, m);
    std::memset(q + m, 0x7f, m + 4096);
    *p = q;
    return 0;
}
inline cudaError_t cudaFree(void* p) { std::free(p); return 0; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, int) { std::memmove(d, s, n); return 0; }
inline cudaError_t cudaMemset(void* p, int v, size_t n) { std::memset(p, v, n); return 0; }
