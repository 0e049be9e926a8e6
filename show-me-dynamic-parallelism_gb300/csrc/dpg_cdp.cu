// Recursive BFS with device-side child launches (CUDA dynamic parallelism, CDP2), kept as a measured
// comparison against the persistent expansion in dpg_expand.cu; no default path uses it.
//
// The variants follow the reference's recursive traversals (apps/bfs-rec/src/bfs_rec_kernel.cu):
//   DPG_CDP_NAIVE  bfs_kernel_dp (61-89): a thread whose atomicMin lowered a child's level launches
//                  one child grid of min(degree, 64) threads over that child's arcs.
//   DPG_CDP_WARP   bfs_kernel_dp_warp_cons (158-213): children found by a warp are appended to a
//                  global buffer slice; the warp launches one child grid (<= 13 CTAs) over it.
//   DPG_CDP_BLOCK  bfs_kernel_dp_block_cons (305-352): the same per CTA.
//   DPG_CDP_GRID   bfs_kernel_dp_grid_cons (394-457): every CTA appends to one buffer; the last CTA
//                  to finish launches the next level (<= 208 CTAs) over it.
// Differences, each for correctness or CDP2:
//   * a child is launched (naive) or appended (consolidated) only when this thread's atomicMin
//     lowered its level (old > new). The reference's naive test "old == the level I read" skips a
//     real improvement when two threads race, which can leave a subtree at a stale level; its
//     consolidated variants append a child whenever they read a higher level, so a child with k
//     parents on one level is appended, and re-expanded, up to k times;
//   * the warp variant reserves each warp's exact share of the CTA's children, not half of all;
//   * CDP2 has no device-side synchronisation: warp/block/naive children are fire-and-forget
//     launches, and the grid variant's next level is a tail launch (it starts after the whole
//     launching grid has finished, which makes the level order explicit without a counter reset);
//   * every kernel carries its nesting depth and never launches past kMaxDepth (the hardware
//     allows 24 generations), and every failed or skipped launch is counted: the host reports
//     DPG_ERR_CAPACITY instead of returning levels that a missing child left unfinished.
// Launches are counted like the reference's GPU_PROFILE nested_calls.
#include <cuda_runtime.h>

#include "dpg_kernels.h"

namespace dpg {
namespace {

constexpr int kChildThreads = 64;        // THREADS_PER_BLOCK of the reference's nested kernels
constexpr unsigned kConsBlocks = 13;     // child CTAs of the warp/block variants (bfs_rec_kernel.cu:195)
constexpr unsigned kGridBlocks = 13 * 16;  // child CTAs of the grid variant (bfs_rec_kernel.cu:436)
constexpr int kMaxDepth = 23;            // generations below the host launch (hardware limit 24)

__device__ __forceinline__ void note_launch(CdpCounters* ct) {
    if (cudaGetLastError() == cudaSuccess) atomicAdd(&ct->launches, 1ull);
    else atomicAdd(&ct->failures, 1ull);
}

__global__ void cdp_naive_kernel(int node, const int32_t* __restrict__ off, const int32_t* __restrict__ col,
                                 int32_t* level, int depth, CdpCounters* ct) {
    const int b = off[node], d = off[node + 1] - b;
    for (int c = threadIdx.x; c < d; c += blockDim.x) {
        const int child = col[b + c];
        const int lv = __ldcg(level + node) + 1;
        const int cl = __ldcg(level + child);
        if (cl == DPG_UNDEFINED_LEVEL || cl > lv) {
            const int old = atomicMin(level + child, lv);
            const int gd = off[child + 1] - off[child];
            if (old > lv && gd > 0) {
                if (depth >= kMaxDepth) {
                    atomicAdd(&ct->failures, 1ull);
                } else {
                    cdp_naive_kernel<<<1, gd < kChildThreads ? gd : kChildThreads, 0, cudaStreamFireAndForget>>>(
                        child, off, col, level, depth + 1, ct);
                    note_launch(ct);
                }
            }
        }
    }
}

// Appends every child whose level this thread lowered to (node level + 1).
__device__ __forceinline__ void expand_node(int node, const int32_t* __restrict__ off, const int32_t* __restrict__ col,
                                            int32_t* level, unsigned* buffer, unsigned cap, unsigned* cursor,
                                            unsigned base, CdpCounters* ct) {
    const int b = off[node], d = off[node + 1] - b;
    for (int c = threadIdx.x; c < d; c += blockDim.x) {
        const int child = col[b + c];
        const int lv = __ldcg(level + node) + 1;
        const int cl = __ldcg(level + child);
        if ((cl == DPG_UNDEFINED_LEVEL || cl > lv) && atomicMin(level + child, lv) > lv) {
            const unsigned pos = base + atomicAdd(cursor, 1u);
            if (pos < cap) buffer[pos] = static_cast<unsigned>(child);
            else atomicAdd(&ct->failures, 1ull);
        }
    }
}

// Warp variant: each warp reserves room for the children its lanes visit (child c of a node goes to
// thread c mod 64, so warp w visits the c with (c / 32) mod 2 == w) and launches a child grid over
// what it appended.
__device__ __forceinline__ unsigned warp_share(unsigned d, int w) {
    const unsigned rem = d % kChildThreads, lo = 32u * static_cast<unsigned>(w);
    return (d / kChildThreads) * 32u + (rem > lo ? (rem - lo < 32u ? rem - lo : 32u) : 0u);
}

__global__ void cdp_warp_kernel(const int32_t* __restrict__ off, const int32_t* __restrict__ col, int32_t* level,
                                const unsigned* queue, unsigned qsize, unsigned* buffer, unsigned cap, unsigned* idx,
                                int depth, CdpCounters* ct) {
    __shared__ unsigned s_share[kChildThreads / 32];
    __shared__ unsigned s_base[kChildThreads / 32];
    __shared__ unsigned s_cnt[kChildThreads / 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        unsigned share = 0;
        for (unsigned q = blockIdx.x; q < qsize; q += gridDim.x)
            share += warp_share(static_cast<unsigned>(off[queue[q] + 1] - off[queue[q]]), warp);
        s_share[warp] = share;
        s_base[warp] = atomicAdd(idx, share);
        s_cnt[warp] = 0;
    }
    __syncthreads();
    for (unsigned q = blockIdx.x; q < qsize; q += gridDim.x)
        expand_node(static_cast<int>(queue[q]), off, col, level, buffer, cap, &s_cnt[warp], s_base[warp], ct);
    __syncthreads();
    if (lane == 0 && s_cnt[warp] > 0) {
        const unsigned n = s_cnt[warp] < s_share[warp] ? s_cnt[warp] : s_share[warp];
        if (depth >= kMaxDepth || s_base[warp] + n > cap) {
            atomicAdd(&ct->failures, 1ull);
        } else {
            cdp_warp_kernel<<<n < kConsBlocks ? n : kConsBlocks, kChildThreads, 0, cudaStreamFireAndForget>>>(
                off, col, level, buffer + s_base[warp], n, buffer, cap, idx, depth + 1, ct);
            note_launch(ct);
        }
    }
}

__global__ void cdp_block_kernel(const int32_t* __restrict__ off, const int32_t* __restrict__ col, int32_t* level,
                                 const unsigned* queue, unsigned qsize, unsigned* buffer, unsigned cap, unsigned* idx,
                                 int depth, CdpCounters* ct) {
    __shared__ unsigned s_base, s_cnt, s_total;
    if (threadIdx.x == 0) {
        unsigned total = 0;
        for (unsigned q = blockIdx.x; q < qsize; q += gridDim.x) total += off[queue[q] + 1] - off[queue[q]];
        s_total = total;
        s_base = atomicAdd(idx, total);
        s_cnt = 0;
    }
    __syncthreads();
    for (unsigned q = blockIdx.x; q < qsize; q += gridDim.x)
        expand_node(static_cast<int>(queue[q]), off, col, level, buffer, cap, &s_cnt, s_base, ct);
    __syncthreads();
    if (threadIdx.x == 0 && s_cnt > 0) {
        const unsigned n = s_cnt < s_total ? s_cnt : s_total;
        if (depth >= kMaxDepth || s_base + n > cap) {
            atomicAdd(&ct->failures, 1ull);
        } else {
            cdp_block_kernel<<<n < kConsBlocks ? n : kConsBlocks, kChildThreads, 0, cudaStreamFireAndForget>>>(
                off, col, level, buffer + s_base, n, buffer, cap, idx, depth + 1, ct);
            note_launch(ct);
        }
    }
}

// Grid variant: queue = buf[p], next level appended to buf[1-p] through cnt[1-p]; the last CTA
// tail-launches the next level over it.
__global__ void cdp_grid_kernel(const int32_t* __restrict__ off, const int32_t* __restrict__ col, int32_t* level,
                                unsigned* buf0, unsigned* buf1, unsigned cap, unsigned* cnt, unsigned* ticket, int p,
                                unsigned qsize, int depth, CdpCounters* ct) {
    const unsigned* queue = p ? buf1 : buf0;
    unsigned* next = p ? buf0 : buf1;
    for (unsigned q = blockIdx.x; q < qsize; q += gridDim.x)
        expand_node(static_cast<int>(queue[q]), off, col, level, next, cap, cnt + (1 - p), 0u, ct);
    __threadfence();
    __syncthreads();
    if (threadIdx.x != 0) return;
    if (atomicAdd(ticket, 1u) != gridDim.x - 1) return;
    __threadfence();
    *ticket = 0u;
    const unsigned n = atomicExch(cnt + (1 - p), 0u);
    if (n == 0) return;
    const unsigned m = n < cap ? n : cap;
    if (depth >= kMaxDepth) {
        atomicAdd(&ct->failures, 1ull);
        return;
    }
    cdp_grid_kernel<<<m < kGridBlocks ? m : kGridBlocks, kChildThreads, 0, cudaStreamTailLaunch>>>(
        off, col, level, buf0, buf1, cap, cnt, ticket, 1 - p, m, depth + 1, ct);
    note_launch(ct);
}

__global__ void cdp_init_kernel(int32_t* level, int32_t V, int32_t source, unsigned* buf0, unsigned* words,
                                int nwords, CdpCounters* ct) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < V;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        level[i] = i == source ? 0 : DPG_UNDEFINED_LEVEL;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        buf0[0] = static_cast<unsigned>(source);
        for (int k = 0; k < nwords; ++k) words[k] = 0u;
        ct->launches = 0ull;
        ct->failures = 0ull;
    }
}

}  // namespace

size_t cdp_buffer_entries(int64_t E, int32_t V) {
    const int64_t n = 4 * E + static_cast<int64_t>(V) + 1024;
    return static_cast<size_t>(n < 0x7FFFFFFF ? n : 0x7FFFFFFF);
}

cudaError_t launch_bfs_cdp(int variant, const int32_t* off, const int32_t* col, int32_t V, int32_t source,
                           int32_t* level, unsigned* buffer, unsigned* buffer2, size_t cap, unsigned* words,
                           CdpCounters* ct, cudaStream_t s, int sm_count) {
    // words: [0] buffer cursor, [1..2] grid-variant next-level counts, [3] grid-variant ticket.
    const int init_blocks = sm_count * 4;
    cdp_init_kernel<<<init_blocks, 256, 0, s>>>(level, V, source, buffer, words, 4, ct);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int deg_hint = 1;  // the root grid covers the source alone
    const unsigned c = static_cast<unsigned>(cap);
    switch (variant) {
        case DPG_CDP_NAIVE:
            cdp_naive_kernel<<<1, kChildThreads, 0, s>>>(source, off, col, level, 0, ct);
            break;
        case DPG_CDP_WARP:
            cdp_warp_kernel<<<deg_hint, kChildThreads, 0, s>>>(off, col, level, buffer, 1u, buffer + 1, c - 1, words, 0,
                                                               ct);
            break;
        case DPG_CDP_BLOCK:
            cdp_block_kernel<<<deg_hint, kChildThreads, 0, s>>>(off, col, level, buffer, 1u, buffer + 1, c - 1, words,
                                                                0, ct);
            break;
        case DPG_CDP_GRID:
            cdp_grid_kernel<<<1, kChildThreads, 0, s>>>(off, col, level, buffer, buffer2, c, words + 1, words + 3, 0, 1u,
                                                        0, ct);
            break;
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace dpg
