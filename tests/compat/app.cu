// A user program of the kind INTEGRATION.md describes: host code keeps the
// reference's Heap<K> class (gpuheap_compat.hpp, extracted from
// INTEGRATION.md by tests/test_compat_adapter.py), and its own kernels call
// insertion / deleteRoot / deleteUpdate on a gh::HeapBU<uint32_t> passed by
// value, as test/heap_test.cu:13-77 does with the reference's Heap<K>*.
// Exit code 0 and "compat ok" when the deleted keys are the sorted inputs.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "gpuheap_compat.hpp"

__global__ void user_insert(gh::HeapBU<uint32_t> heap, const uint32_t* keys, int n, int B) {
    for (int off = 0; off < n; off += B) heap.insertion(keys + off, n - off < B ? n - off : B, 0);
}

__global__ void user_delete(gh::HeapBU<uint32_t> heap, uint32_t* out, int* count) {
    int total = 0;
    for (;;) {
        int size = 0;
        if (heap.deleteRoot(out + total, size)) heap.deleteUpdate(0);
        if (size == 0) break;
        total += size;
    }
    if (threadIdx.x == 0) *count = total;
}

int main() {
    const int B = 256, n = 20 * B + 17, threads = 128;
    std::vector<uint32_t> keys(n);
    uint64_t x = 88172645463325252ull;
    for (auto& k : keys) {
        x ^= x << 13; x ^= x >> 7; x ^= x << 17;
        k = static_cast<uint32_t>(x % 0xFFFFFFFEull);
    }
    Heap<uint32_t> heap(64, B, 0xFFFFFFFFu);
    uint32_t *dk = nullptr, *dout = nullptr;
    int* dcount = nullptr;
    cudaMalloc(&dk, n * sizeof(uint32_t));
    cudaMalloc(&dout, (n + B) * sizeof(uint32_t));
    cudaMalloc(&dcount, sizeof(int));
    cudaMemcpy(dk, keys.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice);
    const size_t smem = gh_heap_smem_bytes(GH_KEY_U32, B);
    user_insert<<<1, threads, smem>>>(heap.view(), dk, n, B);
    if (cudaDeviceSynchronize() != cudaSuccess) { std::printf("insert kernel failed\n"); return 1; }
    if (!heap.checkInsertHeap() || heap.itemCount() != n) { std::printf("heap check failed\n"); return 1; }
    user_delete<<<1, threads, smem>>>(heap.view(), dout, dcount);
    if (cudaDeviceSynchronize() != cudaSuccess) { std::printf("delete kernel failed\n"); return 1; }
    int count = 0;
    std::vector<uint32_t> got(n);
    cudaMemcpy(&count, dcount, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(got.data(), dout, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    std::sort(keys.begin(), keys.end());
    const bool ok = count == n && got == keys && heap.isEmpty();
    std::printf(ok ? "compat ok\n" : "compat FAILED (count %d of %d)\n", count, n);
    cudaFree(dk);
    cudaFree(dout);
    cudaFree(dcount);
    return ok ? 0 : 1;
}
