// Transposed CSR on the device, in invertGraph order (common/global.cpp:237-277).
//
// invertGraph walks the arcs (i ascending, then j ascending), pushes i onto the list of col[j], and
// pops each list from the back, so the in-row of v lists its sources from the last arc to the
// first. Here the arcs are fed to a stable radix sort keyed by head in reverse arc order: within
// each head, the sorted arc ids then come out descending, which is exactly that order. The sort is
// CUB's (a preprocessing step; the traversal and gather kernels are this library's own).
//   t_arc[p]  = arc that transposed slot p came from
//   t_col[p]  = the tail of that arc
//   t_off     = exclusive scan of the head histogram
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "dpg_kernels.h"

namespace dpg {
namespace {

constexpr int kBlk = 256;

// keys[k] = head of arc E-1-k, vals[k] = E-1-k; counts[v] = in-degree of v.
__global__ void reverse_arcs_kernel(const int32_t* __restrict__ col, int64_t E, int32_t* __restrict__ keys,
                                    int32_t* __restrict__ vals, int32_t* counts) {
    for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < E;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t e = E - 1 - k;
        const int32_t v = __ldg(col + e);
        keys[k] = v;
        vals[k] = static_cast<int32_t>(e);
        atomicAdd(counts + v, 1);
    }
}

// tail[e] = row of arc e (warp per row).
__global__ void arc_rows_kernel(const int32_t* __restrict__ off, int32_t V, int32_t* __restrict__ tail) {
    const int lane = threadIdx.x & 31;
    const int64_t w = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t u = w; u < V; u += nw)
        for (int e = __ldg(off + u) + lane; e < __ldg(off + u + 1); e += 32) tail[e] = static_cast<int32_t>(u);
}

__global__ void gather_tails_kernel(const int32_t* __restrict__ tail, const int32_t* __restrict__ t_arc, int64_t E,
                                    int32_t* __restrict__ t_col) {
    for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < E;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x)
        t_col[p] = __ldg(tail + __ldg(t_arc + p));
}

int key_bits(int32_t V) {
    int b = 1;
    while (b < 31 && (1ll << b) < V) ++b;
    return b;
}

}  // namespace

size_t transpose_scratch_bytes(int32_t V, int64_t E) {
    size_t sort_bytes = 0, scan_bytes = 0;
    const int n = static_cast<int>(E > 0 ? E : 1);
    cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, static_cast<const int32_t*>(nullptr),
                                    static_cast<int32_t*>(nullptr), static_cast<const int32_t*>(nullptr),
                                    static_cast<int32_t*>(nullptr), n, 0, key_bits(V));
    cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, static_cast<const int32_t*>(nullptr),
                                  static_cast<int32_t*>(nullptr), V + 1);
    const size_t arrays = 4 * sizeof(int32_t) * static_cast<size_t>(n) + sizeof(int32_t) * (static_cast<size_t>(V) + 1);
    const size_t cub_bytes = sort_bytes > scan_bytes ? sort_bytes : scan_bytes;
    return arrays + cub_bytes + 2048;  // + alignment padding of the five arrays
}

cudaError_t launch_transpose(const int32_t* off, const int32_t* col, int32_t V, int64_t E, int32_t* t_off,
                             int32_t* t_col, int32_t* t_arc, void* scratch, size_t scratch_bytes, cudaStream_t s,
                             int sm_count) {
    if (V < 0 || E < 0 || E > 0x7FFFFFFF) return cudaErrorInvalidValue;
    if (scratch_bytes < transpose_scratch_bytes(V, E)) return cudaErrorInvalidValue;
    const size_t n = static_cast<size_t>(E > 0 ? E : 1);
    auto align = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
    char* p = static_cast<char*>(scratch);
    int32_t* keys_in = reinterpret_cast<int32_t*>(p);
    int32_t* keys_out = reinterpret_cast<int32_t*>(p + align(n * 4));
    int32_t* vals_in = reinterpret_cast<int32_t*>(p + 2 * align(n * 4));
    int32_t* tail = reinterpret_cast<int32_t*>(p + 3 * align(n * 4));
    int32_t* counts = reinterpret_cast<int32_t*>(p + 4 * align(n * 4));
    char* cub_tmp = p + 4 * align(n * 4) + align((static_cast<size_t>(V) + 1) * 4);
    const size_t used = static_cast<size_t>(cub_tmp - p);
    if (used > scratch_bytes) return cudaErrorInvalidValue;
    size_t cub_bytes = scratch_bytes - used;
    // t_arc doubles as the sort's value output.
    cudaError_t e = cudaMemsetAsync(counts, 0, (static_cast<size_t>(V) + 1) * 4, s);
    if (e != cudaSuccess) return e;
    const int blocks = sm_count * 8;
    if (E > 0) {
        reverse_arcs_kernel<<<blocks, kBlk, 0, s>>>(col, E, keys_in, vals_in, counts);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        e = cub::DeviceRadixSort::SortPairs(cub_tmp, cub_bytes, keys_in, keys_out, vals_in, t_arc, static_cast<int>(E),
                                            0, key_bits(V), s);
        if (e != cudaSuccess) return e;
        arc_rows_kernel<<<blocks, kBlk, 0, s>>>(off, V, tail);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        gather_tails_kernel<<<blocks, kBlk, 0, s>>>(tail, t_arc, E, t_col);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    cub_bytes = scratch_bytes - used;
    return cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, counts, t_off, V + 1, s);
}

}  // namespace dpg
