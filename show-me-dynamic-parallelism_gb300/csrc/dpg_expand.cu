// Frontier expansion for SSSP and BFS: one persistent cooperative kernel per solve.
//
// The reference runs one host-loop iteration per frontier (sssp_wrapper.cu:241-298): launch the
// relaxation kernel, memset, regenerate the queue by scanning all V update flags
// (unorder_generateQueue_kernel, sssp_kernel.cu:496-506), and copy the queue length back to the
// host. High-degree vertices go to CDP child launches consolidated per warp, block or grid
// (sssp_kernel.cu:180-387; bfs_rec_kernel.cu:158-457).
//
// Here the whole traversal is one launch. Each iteration pops a compacted frontier, relaxes with
// the reference's operator (sssp_kernel.cu:52-58: alt = cost[u] + w; if cost[v] > alt then
// atomicMin and mark v), pushes improved vertices into the next frontier with warp-aggregated
// appends and a per-vertex bitmap for de-duplication, and ends at a bounded grid barrier. The
// reference's consolidation levels become in-kernel work mappings instead of child launches:
//   DPG_SOL_THREAD  thread per vertex, serial neighbour loop            (-s 0)
//   DPG_SOL_NAIVE   degree >= threshold: a warp per vertex, right away  (-s 1)
//   DPG_SOL_WARP    degree >= threshold: consolidated per warp and expanded by the warp with a
//                   scan-based gather over all consolidated rows            (-s 2)
//   DPG_SOL_BLOCK   degree >= threshold: consolidated per CTA in shared memory and expanded by the
//                   whole CTA                                               (-s 3)
//   DPG_SOL_GRID    degree >= threshold: consolidated grid-wide at push time and expanded by every
//                   warp of the grid in 256-edge chunks                      (-s 4)
//   DPG_SOL_BINNED  warp scan-gather below the hub threshold, grid-wide chunks above (default)
// BFS uses the same machinery with level[v] set once by atomicCAS (bfs_rec_kernel.cu:76-78).

#include <cuda_runtime.h>

#include "dpg_kernels.h"

namespace dpg {
namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;

struct ExpandParams {
    const int32_t* __restrict__ off;
    const int32_t* __restrict__ col;
    const int2* __restrict__ adj;
    int32_t* label;
    int32_t V;
    int32_t threshold;
    int32_t hub_threshold;
    int32_t max_iter;
    unsigned long long timeout_ns;
    ExpandWorkspace ws;
    DevStatus* st;
};

struct SsspOp {
    static constexpr bool kDedup = true;
    __device__ __forceinline__ static void load_edge(const ExpandParams& P, int e, int du, int& v,
                                                     int& cand) {
        const int2 a = __ldg(P.adj + e);
        v = a.x;
        cand = du + a.y;
    }
    __device__ __forceinline__ static bool relax(const ExpandParams& P, int v, int cand) {
        // Read-before-atomic filter (sssp_kernel.cu:55): labels only decrease, so a stale read can
        // only cause an extra atomic, never a missed improvement.
        if (cand < __ldcg(P.label + v)) return cand < atomicMin(P.label + v, cand);
        return false;
    }
};

struct BfsOp {
    static constexpr bool kDedup = false;
    __device__ __forceinline__ static void load_edge(const ExpandParams& P, int e, int du, int& v,
                                                     int& cand) {
        v = __ldg(P.col + e);
        cand = du + 1;
    }
    __device__ __forceinline__ static bool relax(const ExpandParams& P, int v, int cand) {
        if (__ldcg(P.label + v) == DPG_UNDEFINED_LEVEL)
            return atomicCAS(P.label + v, DPG_UNDEFINED_LEVEL, cand) == DPG_UNDEFINED_LEVEL;
        return false;
    }
};

// Destination buffers of one iteration's pushes.
struct PushCtx {
    int32_t* qv;
    int2* qse;
    uint32_t* qcount;
    uint32_t* bmp;
    int32_t* hv;
    int2* hse;
    int32_t* hcpos;
    int32_t* howner;
    unsigned long long* hcount;
};

__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) {
    return *reinterpret_cast<const volatile unsigned*>(p);
}
__device__ __forceinline__ unsigned long long ld_volatile(const unsigned long long* p) {
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}

__device__ __forceinline__ void push_hub(const ExpandParams& P, const PushCtx& Q, int v, int s, int e) {
    const unsigned nch = static_cast<unsigned>((e - s + kHubChunk - 1) / kHubChunk);
    const unsigned long long old = atomicAdd(Q.hcount, (1ull << 32) | nch);
    const unsigned idx = static_cast<unsigned>(old >> 32);
    const unsigned cpos = static_cast<unsigned>(old & 0xFFFFFFFFull);
    if (idx < P.ws.cap_hub && static_cast<unsigned long long>(cpos) + nch <= static_cast<unsigned long long>(P.ws.cap_chunks)) {
        __stcg(Q.hv + idx, v);
        __stcg(Q.hse + idx, make_int2(s, e));
        __stcg(Q.hcpos + idx, static_cast<int>(cpos));
        for (unsigned c = 0; c < nch; ++c) __stcg(Q.howner + cpos + c, static_cast<int>(idx));
    } else {
        raise_error(P.st, DPG_ERR_CAPACITY, 10);
    }
}

// Called by all 32 lanes together. `ok` marks lanes whose relaxation improved vertex v.
template <class Op, bool kClassify>
__device__ __forceinline__ void push_converged(const ExpandParams& P, const PushCtx& Q, bool ok, int v) {
    if (Op::kDedup && ok) {
        const uint32_t bit = 1u << (v & 31);
        ok = (atomicOr(Q.bmp + (v >> 5), bit) & bit) == 0u;
    }
    int s = 0, e = 0;
    if (ok) {
        s = __ldg(P.off + v);
        e = __ldg(P.off + v + 1);
        ok = e > s;  // vertices without out-edges never need expanding
    }
    const bool hub = kClassify && ok && (e - s) >= P.hub_threshold;
    const bool normal = ok && !hub;
    const unsigned m = __ballot_sync(kFullMask, normal);
    if (m) {
        const int lane = lane_id();
        const int leader = __ffs(m) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(Q.qcount, static_cast<unsigned>(__popc(m)));
        base = __shfl_sync(kFullMask, base, leader);
        if (normal) {
            const unsigned pos = base + static_cast<unsigned>(__popc(m & ((1u << lane) - 1u)));
            if (pos < static_cast<unsigned long long>(P.ws.cap_v)) {
                __stcg(Q.qv + pos, v);
                __stcg(Q.qse + pos, make_int2(s, e));
            } else {
                raise_error(P.st, DPG_ERR_CAPACITY, 11);
            }
        }
    }
    if (kClassify && hub) push_hub(P, Q, v, s, e);
}

// Thread-per-vertex neighbour loops (the reference's serial loop), made warp-uniform so pushes can
// aggregate over the full warp.
template <class Op, bool kClassify>
__device__ __forceinline__ void serial_rows(const ExpandParams& P, const PushCtx& Q, bool act, int s,
                                            int d, int du) {
    const int dd = act ? d : 0;
    const int wmax = __reduce_max_sync(kFullMask, dd);
    for (int t = 0; t < wmax; ++t) {
        bool ok = false;
        int v = 0;
        if (t < dd) {
            int cand;
            Op::load_edge(P, s + t, du, v, cand);
            ok = Op::relax(P, v, cand);
        }
        push_converged<Op, kClassify>(P, Q, ok, v);
    }
}

// Scan-based gather: the warp concatenates the rows of the active lanes and relaxes 32 consecutive
// edges per step, so every step is a coalesced read whatever the per-row degrees are.
template <class Op, bool kClassify>
__device__ __forceinline__ void warp_gather(const ExpandParams& P, const PushCtx& Q, bool act, int s,
                                            int d, int du, int* sx, int* ss, int* sdu) {
    const int lane = lane_id();
    const int dd = act ? d : 0;
    const int incl = warp_inclusive_scan(dd);
    const int total = __shfl_sync(kFullMask, incl, 31);
    if (total == 0) return;
    __syncwarp();
    sx[lane] = incl - dd;
    ss[lane] = s;
    sdu[lane] = du;
    __syncwarp();
    for (int base = 0; base < total; base += 32) {
        const int k = base + lane;
        bool ok = false;
        int v = 0;
        if (k < total) {
            int r = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (sx[r + step] <= k) r += step;
            int cand;
            Op::load_edge(P, ss[r] + (k - sx[r]), sdu[r], v, cand);
            ok = Op::relax(P, v, cand);
        }
        push_converged<Op, kClassify>(P, Q, ok, v);
    }
    __syncwarp();
}

// One vertex's row expanded by the whole warp (the per-vertex child of the naive variant).
template <class Op, bool kClassify>
__device__ __forceinline__ void warp_row(const ExpandParams& P, const PushCtx& Q, int s, int d, int du) {
    const int lane = lane_id();
    for (int base = 0; base < d; base += 32) {
        const int t = base + lane;
        bool ok = false;
        int v = 0;
        if (t < d) {
            int cand;
            Op::load_edge(P, s + t, du, v, cand);
            ok = Op::relax(P, v, cand);
        }
        push_converged<Op, kClassify>(P, Q, ok, v);
    }
}

template <class Op, int POL>
__global__ void __launch_bounds__(kBlock) expand_kernel(ExpandParams P) {
    constexpr bool kClassify = (POL == DPG_SOL_GRID || POL == DPG_SOL_BINNED);
    __shared__ int s_excl[kWarps][32];
    __shared__ int s_start[kWarps][32];
    __shared__ int s_du[kWarps][32];
    // CTA consolidation buffer (DPG_SOL_BLOCK).
    __shared__ int c_start[kBlock];
    __shared__ int c_deg[kBlock];
    __shared__ int c_du[kBlock];
    __shared__ int c_excl[kBlock];
    __shared__ int c_wsum[kWarps];
    __shared__ int c_n;
    __shared__ int c_total;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const unsigned gwarp = blockIdx.x * kWarps + warp;
    const unsigned nwarps = gridDim.x * kWarps;
    unsigned long long my_edges = 0, my_pops = 0;
    if (threadIdx.x == 0) c_n = 0;
    __syncthreads();

    int j = 0;
    for (;; ++j) {
        const int p = j & 1;
        // Counters can pass the capacities only after a push has already raised DPG_ERR_CAPACITY
        // (which stops the loop at the barrier); the clamps keep every read inside its buffer anyway.
        const unsigned n = min(ld_volatile(P.ws.qcount + (j % 3)), static_cast<unsigned>(P.ws.cap_v));
        const unsigned long long hc = ld_volatile(P.ws.hcount + (j % 3));
        const unsigned nh = min(static_cast<unsigned>(hc >> 32), static_cast<unsigned>(P.ws.cap_hub));
        const unsigned nch = min(static_cast<unsigned>(hc & 0xFFFFFFFFull), static_cast<unsigned>(P.ws.cap_chunks));
        if (n == 0 && nh == 0) break;
        if (j >= P.max_iter) {
            if (blockIdx.x == 0 && threadIdx.x == 0) raise_error(P.st, DPG_ERR_CAPACITY, 2);
            break;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            P.ws.qcount[(j + 2) % 3] = 0u;
            P.ws.hcount[(j + 2) % 3] = 0ull;
        }
        // Parity selects are written as ternaries so the pointer pairs stay in registers.
        const PushCtx Q = {p ? P.ws.qv[0] : P.ws.qv[1], p ? P.ws.qse[0] : P.ws.qse[1],
                           P.ws.qcount + (j + 1) % 3, p ? P.ws.bmp[0] : P.ws.bmp[1],
                           p ? P.ws.hv[0] : P.ws.hv[1], p ? P.ws.hse[0] : P.ws.hse[1],
                           p ? P.ws.hcpos[0] : P.ws.hcpos[1], p ? P.ws.howner[0] : P.ws.howner[1],
                           P.ws.hcount + (j + 1) % 3};
        const int32_t* qv_cur = p ? P.ws.qv[1] : P.ws.qv[0];
        const int2* qse_cur = p ? P.ws.qse[1] : P.ws.qse[0];
        uint32_t* bmp_cur = p ? P.ws.bmp[1] : P.ws.bmp[0];
        const int32_t* hv_cur = p ? P.ws.hv[1] : P.ws.hv[0];
        const int2* hse_cur = p ? P.ws.hse[1] : P.ws.hse[0];
        const int32_t* hcpos_cur = p ? P.ws.hcpos[1] : P.ws.hcpos[0];
        const int32_t* howner_cur = p ? P.ws.howner[1] : P.ws.howner[0];
        const unsigned fchunks = (n + 31u) / 32u;

        if (POL == DPG_SOL_BLOCK) {
            const unsigned per_round = gridDim.x * kWarps;
            const unsigned rounds = (fchunks + per_round - 1) / per_round;
            for (unsigned r = 0; r < rounds; ++r) {
                const unsigned chunk = r * per_round + blockIdx.x * kWarps + warp;
                const unsigned i = chunk * 32u + lane;
                int u = 0, s = 0, d = 0, du = 0;
                const bool has = chunk < fchunks && i < n;
                if (has) {
                    u = __ldcg(qv_cur + i);
                    const int2 se = __ldcg(qse_cur + i);
                    s = se.x;
                    d = se.y - se.x;
                    du = __ldcg(P.label + u);
                    if (Op::kDedup) __stcg(bmp_cur + (u >> 5), 0u);
                    my_pops += 1;
                    my_edges += static_cast<unsigned long long>(d);
                }
                const bool big = has && d >= P.threshold;
                serial_rows<Op, false>(P, Q, has && !big, s, d, du);
                if (big) {
                    const int slot = atomicAdd(&c_n, 1);
                    c_start[slot] = s;
                    c_deg[slot] = d;
                    c_du[slot] = du;
                }
                __syncthreads();
                const int cn = c_n;
                if (cn > 0) {
                    // CTA-wide exclusive scan of the consolidated degrees.
                    const int dg = threadIdx.x < cn ? c_deg[threadIdx.x] : 0;
                    const int incl = warp_inclusive_scan(dg);
                    if (lane == 31) c_wsum[warp] = incl;
                    __syncthreads();
                    if (warp == 0) {
                        const int w = lane < kWarps ? c_wsum[lane] : 0;
                        const int wi = warp_inclusive_scan(w);
                        if (lane < kWarps) c_wsum[lane] = wi - w;
                        if (lane == kWarps - 1) c_total = wi;
                    }
                    __syncthreads();
                    c_excl[threadIdx.x] = incl - dg + c_wsum[warp];
                    __syncthreads();
                    const int total = c_total;
                    for (int base = 0; base < total; base += kBlock) {
                        const int k = base + static_cast<int>(threadIdx.x);
                        bool ok = false;
                        int v = 0;
                        if (k < total) {
                            int rr = 0;
#pragma unroll
                            for (int step = kBlock / 2; step > 0; step >>= 1)
                                if (rr + step < kBlock && c_excl[rr + step] <= k) rr += step;
                            int cand;
                            Op::load_edge(P, c_start[rr] + (k - c_excl[rr]), c_du[rr], v, cand);
                            ok = Op::relax(P, v, cand);
                        }
                        push_converged<Op, false>(P, Q, ok, v);
                    }
                    __syncthreads();
                    if (threadIdx.x == 0) c_n = 0;
                }
                __syncthreads();
            }
        } else {
            const unsigned hub_items = kClassify ? nch : 0u;
            const unsigned total_items = hub_items + fchunks;
            for (unsigned item = gwarp; item < total_items; item += nwarps) {
                if (kClassify && item < hub_items) {
                    // Grid-wide consolidation: one 256-edge chunk of a hub row.
                    const int c = static_cast<int>(item);
                    const int h = __ldcg(howner_cur + c);
                    if (static_cast<unsigned>(h) >= nh) {  // warp-uniform: every lane read the same c
                        if (lane == 0) raise_error(P.st, DPG_ERR_CAPACITY, 12);
                        continue;
                    }
                    const int v0 = __ldcg(hv_cur + h);
                    const int2 se = __ldcg(hse_cur + h);
                    const int cp = __ldcg(hcpos_cur + h);
                    const int du = __ldcg(P.label + v0);
                    const int k0 = se.x + (c - cp) * kHubChunk;
                    const int k1 = min(se.y, k0 + kHubChunk);
                    if (c == cp && lane == 0) {
                        if (Op::kDedup) __stcg(bmp_cur + (v0 >> 5), 0u);
                        my_pops += 1;
                    }
                    if (lane == 0) my_edges += static_cast<unsigned long long>(k1 - k0);
                    for (int base = k0; base < k1; base += 32) {
                        const int e = base + lane;
                        bool ok = false;
                        int v = 0;
                        if (e < k1) {
                            int cand;
                            Op::load_edge(P, e, du, v, cand);
                            ok = Op::relax(P, v, cand);
                        }
                        push_converged<Op, kClassify>(P, Q, ok, v);
                    }
                    continue;
                }
                const unsigned chunk = item - hub_items;
                const unsigned i = chunk * 32u + lane;
                int u = 0, s = 0, d = 0, du = 0;
                const bool has = i < n;
                if (has) {
                    u = __ldcg(qv_cur + i);
                    const int2 se = __ldcg(qse_cur + i);
                    s = se.x;
                    d = se.y - se.x;
                    du = __ldcg(P.label + u);
                    if (Op::kDedup) __stcg(bmp_cur + (u >> 5), 0u);
                    my_pops += 1;
                    my_edges += static_cast<unsigned long long>(d);
                }
                if (POL == DPG_SOL_THREAD || POL == DPG_SOL_GRID) {
                    serial_rows<Op, kClassify>(P, Q, has, s, d, du);
                } else if (POL == DPG_SOL_BINNED) {
                    warp_gather<Op, kClassify>(P, Q, has, s, d, du, s_excl[warp], s_start[warp], s_du[warp]);
                } else {
                    const bool big = has && d >= P.threshold;
                    serial_rows<Op, kClassify>(P, Q, has && !big, s, d, du);
                    if (POL == DPG_SOL_WARP) {
                        warp_gather<Op, kClassify>(P, Q, big, s, d, du, s_excl[warp], s_start[warp], s_du[warp]);
                    } else {  // DPG_SOL_NAIVE
                        unsigned bigmask = __ballot_sync(kFullMask, big);
                        while (bigmask) {
                            const int src = __ffs(bigmask) - 1;
                            bigmask &= bigmask - 1u;
                            const int bs = __shfl_sync(kFullMask, s, src);
                            const int bd = __shfl_sync(kFullMask, d, src);
                            const int bdu = __shfl_sync(kFullMask, du, src);
                            warp_row<Op, kClassify>(P, Q, bs, bd, bdu);
                        }
                    }
                }
            }
        }
        if (!grid_barrier(P.st, gridDim.x, P.timeout_ns)) break;
    }

    my_edges = warp_sum_u64(my_edges);
    my_pops = warp_sum_u64(my_pops);
    if (lane == 0) {
        if (my_edges) atomicAdd(&P.st->edges, my_edges);
        if (my_pops) atomicAdd(&P.st->pops, my_pops);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) P.st->iterations = static_cast<unsigned long long>(j);
}

__global__ void expand_init_kernel(ExpandParams P, int32_t source, int32_t init_label, int classify) {
    const int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = tid; i < P.V; i += stride) P.label[i] = (i == source) ? 0 : init_label;
    for (int64_t w = tid; w < P.ws.bmp_words; w += stride) {
        P.ws.bmp[0][w] = 0u;
        P.ws.bmp[1][w] = 0u;
    }
    if (tid == 0) {
        for (int k = 0; k < 3; ++k) {
            P.ws.qcount[k] = 0u;
            P.ws.hcount[k] = 0ull;
        }
        P.st->bar_count = 0u;
        P.st->iterations = 0ull;
        P.st->edges = 0ull;
        P.st->pops = 0ull;
        const int s = P.off[source];
        const int e = P.off[source + 1];
        if (e > s) {
            if (classify && e - s >= P.hub_threshold) {
                const int nch = (e - s + kHubChunk - 1) / kHubChunk;
                P.ws.hv[0][0] = source;
                P.ws.hse[0][0] = make_int2(s, e);
                P.ws.hcpos[0][0] = 0;
                for (int c = 0; c < nch; ++c) P.ws.howner[0][c] = 0;
                P.ws.hcount[0] = (1ull << 32) | static_cast<unsigned long long>(nch);
            } else {
                P.ws.qv[0][0] = source;
                P.ws.qse[0][0] = make_int2(s, e);
                P.ws.qcount[0] = 1u;
            }
        }
    }
}

__global__ void barrier_timeout_kernel(DevStatus* st, unsigned long long timeout_ns) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st->bar_count = 0u;
    // Only gridDim.x CTAs exist but the barrier waits for one more: every wait must time out.
    // (CTA 0 resets the counter before arriving; a late reset can only make the wait longer.)
    grid_barrier(st, gridDim.x + 1, timeout_ns);
}

template <class Op>
const void* pick_kernel(int solution) {
    switch (solution) {
        case DPG_SOL_THREAD: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_THREAD>);
        case DPG_SOL_NAIVE: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_NAIVE>);
        case DPG_SOL_WARP: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_WARP>);
        case DPG_SOL_BLOCK: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_BLOCK>);
        case DPG_SOL_GRID: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_GRID>);
        case DPG_SOL_BINNED: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_BINNED>);
        default: return nullptr;
    }
}

}  // namespace

void expand_workspace_caps(int32_t V, int64_t E, int32_t min_hub_degree, int64_t* cap_hub,
                           int64_t* cap_chunks) {
    const int64_t d = min_hub_degree < 1 ? 1 : min_hub_degree;
    int64_t hubs = E / d + 1;
    if (hubs > static_cast<int64_t>(V) + 1) hubs = static_cast<int64_t>(V) + 1;
    *cap_hub = hubs;
    *cap_chunks = E / kHubChunk + hubs + 1;
}

cudaError_t launch_expand(const ExpandLaunch& L, const ExpandWorkspace& ws, DevStatus* st,
                          cudaStream_t stream, int sm_count, int* grid_out, int* block_out,
                          LaunchHook* hook) {
    const void* fn = L.bfs ? pick_kernel<BfsOp>(L.solution) : pick_kernel<SsspOp>(L.solution);
    if (!fn) return cudaErrorInvalidValue;
    int per_sm = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBlock, 0);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int grid = per_sm * sm_count;
    ExpandParams P;
    P.off = L.off;
    P.col = L.col;
    P.adj = L.adj;
    P.label = L.label;
    P.V = L.V;
    P.threshold = L.threshold;
    P.hub_threshold = L.hub_threshold;
    P.max_iter = L.max_iter;
    P.timeout_ns = L.timeout_ns;
    P.ws = ws;
    P.st = st;
    const int classify = (L.solution == DPG_SOL_GRID || L.solution == DPG_SOL_BINNED) ? 1 : 0;
    const int32_t init_label = L.bfs ? DPG_UNDEFINED_LEVEL : DPG_INF_COST;
    int init_blocks = static_cast<int>((static_cast<int64_t>(L.V) + kBlock - 1) / kBlock);
    if (init_blocks > sm_count * 8) init_blocks = sm_count * 8;
    if (init_blocks < 1) init_blocks = 1;
    {
        HookScope hs(hook, DPG_KERNEL_INIT, stream);
        expand_init_kernel<<<init_blocks, kBlock, 0, stream>>>(P, L.source, init_label, classify);
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    void* args[] = {&P};
    {
        HookScope hs(hook, DPG_KERNEL_EXPAND, stream);
        err = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kBlock), args, 0, stream);
    }
    if (grid_out) *grid_out = grid;
    if (block_out) *block_out = kBlock;
    return err;
}

cudaError_t launch_barrier_timeout_test(DevStatus* st, unsigned long long timeout_ns, cudaStream_t stream) {
    void* args[] = {&st, &timeout_ns};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(barrier_timeout_kernel), dim3(2),
                                       dim3(32), args, 0, stream);
}

}  // namespace dpg
