// Gather-locality layout for the row gathers: column ids renamed by descending column frequency.
//
// In a pull PageRank sweep or an SpMV, every nonzero gathers one 4-byte value at its column id. On
// R-MAT graphs the columns are extremely skewed (at scale 22 the 16 K most frequent columns take 42 %
// of all gathers; half the vertices never appear as a column), but the input ids scatter those hot
// values over the whole vector, so every gather moves its own 32-byte L2 sector. Renaming columns
// so the most frequent come first packs the hot values into a few KB that stay in L1 and share
// sectors. Only column ids change: rows, and the order of nonzeros inside each row, are untouched,
// so every sum is taken in the same order and results are bit-identical with or without the
// renaming.
//
// The order is "by frequency class, then by id": class = bit length of the column count, so the
// stable multi-split below needs 33 buckets instead of a full sort.

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "dpg_kernels.h"

namespace dpg {
namespace {

__global__ void column_histogram_kernel(const int32_t* __restrict__ col, int64_t E, int32_t* counts) {
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < E;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x)
        atomicAdd(counts + __ldg(col + e), 1);
}

__global__ void relabel_columns_kernel(const int32_t* __restrict__ col, const int32_t* __restrict__ perm, int64_t E,
                                       int32_t* __restrict__ out) {
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < E;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[e] = __ldg(perm + __ldg(col + e));
}

// The same with the range check of an unchecked upload folded in.
__global__ void relabel_check_columns_kernel(const int32_t* __restrict__ col, const int32_t* __restrict__ perm,
                                             int64_t E, int32_t V, int32_t* __restrict__ out, int* bad) {
    bool any = false;
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < E;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t c = __ldg(col + e);
        const bool ok = static_cast<uint32_t>(c) < static_cast<uint32_t>(V);
        any |= !ok;
        out[e] = ok ? __ldg(perm + c) : 0;
    }
    if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(bad, 1);
}

__global__ void gather_by_index_kernel(const float* __restrict__ x, const int32_t* __restrict__ inv, int32_t V,
                                       float* __restrict__ out) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < V;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = __ldg(x + __ldg(inv + i));
}

// Warp per row; each lane claims a slot of the target's in-row.
__global__ void transpose_scatter_kernel(const int32_t* __restrict__ off, const int32_t* __restrict__ col, int32_t V,
                                         int32_t* cursor, int32_t* __restrict__ t_col) {
    const int lane = threadIdx.x & 31;
    const int64_t w = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t u = w; u < V; u += nw) {
        const int b = __ldg(off + u), e = __ldg(off + u + 1);
        for (int k = b + lane; k < e; k += 32) {
            const int v = __ldg(col + k);
            t_col[atomicAdd(cursor + v, 1)] = static_cast<int32_t>(u);
        }
    }
}

// ---- the frequency order on the device (a stable multi-split over 33 classes) --------------------
// Vertex v's class is the bit length of its column count; the order is class descending, then id
// ascending, exactly as frequency_order() below. Blocks of kSplitBlock consecutive ids: pass 1
// counts each class per block, pass 2 turns the counts into start offsets in (class descending,
// block ascending) order, pass 3 places every id at its start plus its rank among the block's
// earlier ids of the same class.
constexpr int kSplitBlock = 1024;
constexpr int kClasses = 33;

__device__ __forceinline__ int count_class(int32_t c) { return c <= 0 ? 0 : 32 - __clz(c); }

// Per-warp class counts and each thread's rank among the earlier ids of its class in the block.
__device__ __forceinline__ int block_class_rank(int cls, bool valid, int (*s_cnt)[kClasses]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < (kSplitBlock / 32) * kClasses; i += blockDim.x) (&s_cnt[0][0])[i] = 0;
    __syncthreads();
    const int key = valid ? cls : kClasses;  // invalid lanes form their own group
    const unsigned same = __match_any_sync(0xffffffffu, key);
    const int in_warp = __popc(same & ((1u << lane) - 1u));
    if (valid && in_warp == 0) s_cnt[warp][cls] = __popc(same);
    __syncthreads();
    // Exclusive scan over warps, one class per thread.
    if (threadIdx.x < kClasses) {
        int acc = 0;
        for (int w = 0; w < kSplitBlock / 32; ++w) {
            const int t = s_cnt[w][threadIdx.x];
            s_cnt[w][threadIdx.x] = acc;
            acc += t;
        }
    }
    __syncthreads();
    return valid ? s_cnt[warp][cls] + in_warp : 0;
}

__global__ void __launch_bounds__(kSplitBlock) split_count_kernel(const int32_t* __restrict__ counts, int32_t V,
                                                                  int32_t* __restrict__ block_hist) {
    __shared__ int s_tot[kClasses];
    if (threadIdx.x < kClasses) s_tot[threadIdx.x] = 0;
    __syncthreads();
    const int64_t v = static_cast<int64_t>(blockIdx.x) * kSplitBlock + threadIdx.x;
    if (v < V) atomicAdd(&s_tot[count_class(counts[v])], 1);
    __syncthreads();
    // Column-major by class (largest class first) so that one scan gives every start.
    if (threadIdx.x < kClasses)
        block_hist[static_cast<int64_t>(kClasses - 1 - threadIdx.x) * gridDim.x + blockIdx.x] = s_tot[threadIdx.x];
}

// Exclusive scan of n ints in place by one block (n is 33 x blocks, a few hundred thousand at most).
__global__ void __launch_bounds__(1024) split_scan_kernel(int32_t* __restrict__ a, int64_t n) {
    __shared__ int32_t s_part[1024];
    __shared__ int32_t s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < n; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const int32_t x = i < n ? a[i] : 0;
        s_part[threadIdx.x] = x;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
            const int32_t t = threadIdx.x >= o ? s_part[threadIdx.x - o] : 0;
            __syncthreads();
            s_part[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < n) a[i] = s_carry + s_part[threadIdx.x] - x;
        __syncthreads();
        if (threadIdx.x == 1023) s_carry += s_part[1023];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kSplitBlock) split_place_kernel(const int32_t* __restrict__ counts, int32_t V,
                                                                  const int32_t* __restrict__ starts,
                                                                  int32_t* __restrict__ perm, int32_t* __restrict__ inv) {
    __shared__ int s_cnt[kSplitBlock / 32][kClasses];
    const int64_t v = static_cast<int64_t>(blockIdx.x) * kSplitBlock + threadIdx.x;
    const bool valid = v < V;
    const int cls = valid ? count_class(counts[v]) : 0;
    const int rank = block_class_rank(cls, valid, s_cnt);
    if (valid) {
        const int32_t pos = starts[static_cast<int64_t>(kClasses - 1 - cls) * gridDim.x + blockIdx.x] + rank;
        perm[v] = pos;
        inv[pos] = static_cast<int32_t>(v);
    }
}

}  // namespace

size_t frequency_order_scratch_bytes(int32_t V) {
    const int64_t blocks = (static_cast<int64_t>(V) + kSplitBlock - 1) / kSplitBlock;
    return static_cast<size_t>(blocks > 0 ? blocks : 1) * kClasses * sizeof(int32_t);
}

cudaError_t launch_frequency_order(const int32_t* counts, int32_t V, int32_t* scratch, int32_t* perm, int32_t* inv,
                                   cudaStream_t s) {
    if (V <= 0) return cudaSuccess;
    const int blocks = static_cast<int>((static_cast<int64_t>(V) + kSplitBlock - 1) / kSplitBlock);
    split_count_kernel<<<blocks, kSplitBlock, 0, s>>>(counts, V, scratch);
    split_scan_kernel<<<1, 1024, 0, s>>>(scratch, static_cast<int64_t>(blocks) * kClasses);
    split_place_kernel<<<blocks, kSplitBlock, 0, s>>>(counts, V, scratch, perm, inv);
    return cudaGetLastError();
}

cudaError_t launch_transpose_scatter(const int32_t* off, const int32_t* col, int32_t V, int32_t* cursor,
                                     int32_t* t_col, cudaStream_t s, int sm_count) {
    if (V > 0) transpose_scatter_kernel<<<sm_count * 8, 256, 0, s>>>(off, col, V, cursor, t_col);
    return cudaGetLastError();
}

cudaError_t launch_column_histogram(const int32_t* col, int64_t E, int32_t* counts, cudaStream_t s, int sm_count) {
    if (E > 0) column_histogram_kernel<<<sm_count * 8, 256, 0, s>>>(col, E, counts);
    return cudaGetLastError();
}

cudaError_t launch_relabel_columns(const int32_t* col, const int32_t* perm, int64_t E, int32_t* out, cudaStream_t s,
                                   int sm_count, int32_t V, int* bad) {
    if (E <= 0) return cudaGetLastError();
    if (bad) relabel_check_columns_kernel<<<sm_count * 8, 256, 0, s>>>(col, perm, E, V, out, bad);
    else relabel_columns_kernel<<<sm_count * 8, 256, 0, s>>>(col, perm, E, out);
    return cudaGetLastError();
}

cudaError_t launch_gather_by_index(const float* x, const int32_t* inv, int32_t V, float* out, cudaStream_t s,
                                   int sm_count) {
    if (V > 0) gather_by_index_kernel<<<sm_count * 4, 256, 0, s>>>(x, inv, V, out);
    return cudaGetLastError();
}

void frequency_order(const int32_t* counts, int32_t V, int32_t* perm, int32_t* inv) {
    // Stable multi-split on the bit length of the count, largest class first.
    int64_t bucket[34] = {0};
    auto cls = [](int32_t c) { return c <= 0 ? 0 : 32 - __builtin_clz(static_cast<unsigned>(c)); };
    for (int32_t v = 0; v < V; ++v) ++bucket[cls(counts[v])];
    int64_t start[34];
    int64_t acc = 0;
    for (int b = 33; b >= 0; --b) {
        start[b] = acc;
        acc += bucket[b];
    }
    for (int32_t v = 0; v < V; ++v) {
        const int32_t n = static_cast<int32_t>(start[cls(counts[v])]++);
        perm[v] = n;
        inv[n] = v;
    }
}

}  // namespace dpg
