// Row gathers: SpMV (y = A x over the out-edge CSR) and PageRank pull sweeps (over the in-edge CSR).
//
// Reference: csr_spmv_kernel (apps/SpMV/src/SpMV_kernel.cu:81-96) and pagerank_thread_pull_kernel
// (apps/pagerank/src/pagerank_kernel.cu:95-120) map one thread to one row, so a power-law hub row
// serialises a thread; the consolidation variants hand rows of degree >= 64 to CDP children that
// block-reduce them (SpMV_kernel.cu:196-216, pagerank_kernel.cu:357-382).
//
// Here the rows are cut (on the device, once per graph) into warp tiles of at most 256 merge items
// (rows + nonzeros):
//   - a normal tile holds whole rows of degree <= 255; one warp stages the tile's gathered
//     products in shared memory, each lane walks 8 consecutive merge items (merge-path over row
//     ends and nonzeros, from a start row and a row-end mask the plan keeps per lane), and a warp
//     segmented scan joins rows that cross lanes;
//   - a row of degree > 255 (a hub) is split into 256-nonzero segments whose partial sums are
//     combined afterwards, in segment order, by the hub fix-up kernel.
// Every sum has a fixed order, so results are bit-reproducible run to run; no float atomics.
// With renamed columns (dpg_layout.cu) `col` holds the new ids, `x` is indexed by them, and the
// PageRank epilogue writes row v's contribution at perm[v].
// PageRank folds rank/outdeg into the sweep's epilogue (contrib[v] = rank[v]/outdeg[v]), so the
// gather reads one 4-byte value per in-edge instead of the reference's rank and outdegree pair and
// divide per edge (pagerank_kernel.cu:114), and sums the dangling mass on the device (the reference
// copies every dangling rank to the host each sweep, pagerank_wrapper.cu:212-218).

#include <cuda_runtime.h>

#include <algorithm>

#include "dpg_kernels.h"

namespace dpg {
namespace {

// One CTA per SM: its dynamic shared memory holds the hot-value cache (the first `hot` renamed
// entries of x, i.e. the most gathered columns) and its warps' tile staging. DPG_GATHER_BLOCK (and
// the tile counts below) are build-time tuning knobs (DPG_NVCC_EXTRA); the defaults are measured.
#ifndef DPG_GATHER_BLOCK
#define DPG_GATHER_BLOCK 1024
#endif
constexpr int kBlock = DPG_GATHER_BLOCK;
constexpr int kWarps = kBlock / 32;
constexpr int kInitBlock = 256;
constexpr int kIpl = kRowTileItems / 32;  // merge items per lane
constexpr int kFixBlock = 256;
constexpr int kFixBatch = 8;  // loads the fix-up issues before it adds them
// Tiles a warp carries through one step (see rowgather_kernel), per mode. Measured on R-MAT scale
// 22 (PageRank sweep, 1024-thread CTAs): what limits the gathers is the L1 left beside the shared
// memory, where their sectors in flight need lines (the shared-memory budget is set with the
// hot-cache size, see hot_entries). With a 28 KB L1 one tile per step ran best (0.29 ms per sweep);
// with 92 KB, two tiles run 0.202 ms against 0.216 ms with one. Fewer warps lose at any setting
// (768 threads: 0.245 ms, 512: 0.35 ms), and three tiles would spill at 1024 threads.
#ifndef DPG_GATHER_TILES_SPMV
#define DPG_GATHER_TILES_SPMV 2
#endif
#ifndef DPG_GATHER_TILES_PR
#define DPG_GATHER_TILES_PR 2
#endif
// Shared-memory index with one pad word per 32: lane l walking items 8l.. then hits 32 distinct banks
// instead of 4 (an 8-way conflict without the pad).
constexpr int kPadded = kRowTileItems + kRowTileItems / 32;
__device__ __forceinline__ int pad(int i) { return i + (i >> 5); }

enum { kModeSpmv = 0, kModePagerank = 1 };

// Loads of the streams every tile reads once (columns, SpMV values, out-degrees, renaming slots):
// read-only for the launch (nc) and kept out of L1 (L1::no_allocate), so the L1 lines are left to
// the scattered gathers of x, which are what a sweep waits on. SpMV also marks them first for
// eviction from L2, which keeps more of x there. Measured per launch (R-MAT 22; R-MAT 24 for
// PageRank): PageRank 0.1623 -> 0.1603 ms and 0.749 -> 0.720 ms with L1::no_allocate, 0.171 and
// 0.764 ms with the L2 hint too; SpMV 0.2146 -> 0.2137 ms, and 0.2063 ms with the L2 hint.
template <int MODE>
__device__ __forceinline__ int ld_stream(const int* p) {
    int v;
    if constexpr (MODE == kModeSpmv) {
        asm("{\n\t.reg .b64 pol;\n\tcreatepolicy.fractional.L2::evict_first.b64 pol, 1.0;\n\t"
            "ld.global.nc.L1::no_allocate.L2::cache_hint.s32 %0, [%1], pol;\n\t}"
            : "=r"(v) : "l"(p));
    } else {
        asm("ld.global.nc.L1::no_allocate.s32 %0, [%1];" : "=r"(v) : "l"(p));
    }
    return v;
}
template <int MODE>
__device__ __forceinline__ float ld_stream(const float* p) {
    float v;
    if constexpr (MODE == kModeSpmv) {
        asm("{\n\t.reg .b64 pol;\n\tcreatepolicy.fractional.L2::evict_first.b64 pol, 1.0;\n\t"
            "ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], pol;\n\t}"
            : "=f"(v) : "l"(p));
    } else {
        asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
    }
    return v;
}

// PageRank epilogue of one row: new rank, next contribution, dangling mass, convergence flag.
// od / pos are the row's out-degree and contribution slot (perm[v] with renamed columns).
__device__ __forceinline__ void pr_epilogue(const RowGatherLaunch& L, int v, float sum, float base, int od, int pos,
                                            double& dang) {
    if (L.vgraph) base = __ldg(L.gbase + __ldg(L.vgraph + v));
    const float nv = fmaf(L.damping, sum, base);
    if (L.rank_out) L.rank_out[v] = nv;
    if (L.rank_prev && fabsf(nv - __ldg(L.rank_prev + v)) > L.epsilon) *L.nonstop = 1u;
    // Only vertices with out-arcs are ever gathered (they are the columns), so the contribution
    // slot of a dangling vertex is free: a batch parks its rank there for the per-graph reduction.
    // The division runs for every row (by 1 for a dangling one) so a warp's rows do not diverge
    // around it; only the stores and the dangling sum depend on the out-degree.
    const float q = nv / static_cast<float>(od > 0 ? od : 1);
    if (L.vgraph) {
        L.y[pos] = od > 0 ? q : nv;
    } else {
        if (od > 0) L.y[pos] = q;
        if (od <= 0) dang += static_cast<double>(nv);
    }
}

__device__ __forceinline__ void pr_epilogue(const RowGatherLaunch& L, int v, float sum, float base, double& dang) {
    pr_epilogue(L, v, sum, base, __ldg(L.outdeg + v), L.perm ? __ldg(L.perm + v) : v, dang);
}

__device__ __forceinline__ float pr_base(const RowGatherLaunch& L) {
    return static_cast<float>(L.base_const + L.dangling_scale * __ldg(L.dsum_in));
}

// Hub rows: the segment partials summed in segment order, then the row epilogue. Small hubs go one
// per thread, big hubs one per warp. The loads are issued in batches before they are added in the
// same order as a plain loop would, so the sums are unchanged and each batch costs one round trip.
template <int MODE>
__device__ __forceinline__ void fixup_hubs(const RowGatherLaunch& L, int tid, int nthreads, int gwarp, int nwarps,
                                           int lane, float base, double& dang) {
    // The epilogue inputs (out-degree, contribution slot) are loaded with the partials.
    for (int h = tid; h < L.plan.nhub_small; h += nthreads) {
        const int4 H = __ldg(L.plan.hubs_small + h);
        int od = 0, pos = 0;
        if (MODE == kModePagerank) {
            od = __ldg(L.outdeg + H.x);
            pos = L.perm ? __ldg(L.perm + H.x) : H.x;
        }
        float p[kSmallHubSegs];
#pragma unroll
        for (int s = 0; s < kSmallHubSegs; ++s) p[s] = s < H.z ? L.partial[H.y + s] : 0.0f;
        float acc = 0.0f;
#pragma unroll
        for (int s = 0; s < kSmallHubSegs; ++s) acc += p[s];
        if (MODE == kModeSpmv) L.y[H.x] = acc;
        else pr_epilogue(L, H.x, acc, base, od, pos, dang);
    }
    for (int h = gwarp; h < L.plan.nhub_big; h += nwarps) {
        const int4 H = __ldg(L.plan.hubs_big + h);
        int od = 0, pos = 0;
        if (MODE == kModePagerank && lane == 0) {
            od = __ldg(L.outdeg + H.x);
            pos = L.perm ? __ldg(L.perm + H.x) : H.x;
        }
        float acc = 0.0f;
        for (int s0 = lane; s0 < H.z; s0 += 32 * kFixBatch) {
            float p[kFixBatch];
#pragma unroll
            for (int q = 0; q < kFixBatch; ++q) p[q] = s0 + 32 * q < H.z ? L.partial[H.y + s0 + 32 * q] : 0.0f;
#pragma unroll
            for (int q = 0; q < kFixBatch; ++q) acc += p[q];
        }
        acc = warp_sum_f32(acc);
        if (lane == 0) {
            if (MODE == kModeSpmv) L.y[H.x] = acc;
            else pr_epilogue(L, H.x, acc, base, od, pos, dang);
        }
    }
}

// Thread t's share of a[0, n) (entries t, t + NT, ...) in index order, loads in batches.
template <int NT>
__device__ __forceinline__ double strided_sum_f64(const double* a, int n, double acc) {
    for (int i0 = threadIdx.x; i0 < n; i0 += NT * kFixBatch) {
        double p[kFixBatch];
#pragma unroll
        for (int q = 0; q < kFixBatch; ++q) p[q] = i0 + NT * q < n ? __ldcg(a + i0 + NT * q) : 0.0;
#pragma unroll
        for (int q = 0; q < kFixBatch; ++q) acc += p[q];
    }
    return acc;
}

// Sum over the block of each thread's v, warps in order; valid in thread 0.
template <int NT>
__device__ __forceinline__ double block_sum_f64(double v) {
    __shared__ double s_red[NT / 32];
    v = warp_sum_f64(v);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    double total = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < NT / 32; ++w) total += s_red[w];
    return total;
}

// One step of a warp covers KT consecutive tiles: first every column and epilogue load of all KT
// tiles, then all their gathers, then the tiles are walked one after the other through the warp's
// single staging area. A lane thus keeps KT x 8 gathers in flight instead of 8.
template <int MODE, int KT>
__global__ void __launch_bounds__(kBlock) rowgather_kernel(RowGatherLaunch L) {
    extern __shared__ __align__(16) unsigned char rg_smem[];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int gwarp = blockIdx.x * kWarps + warp;
    const int nwarps = gridDim.x * kWarps;
    float* val = reinterpret_cast<float*>(rg_smem) + warp * (2 * kPadded);
    float* out = val + kPadded;
    float* s_hot = reinterpret_cast<float*>(rg_smem) + kWarps * 2 * kPadded;
    // Hot-cache fill, loads issued in batches of 8 (one round trip each instead of one per entry).
    for (int i0 = threadIdx.x; i0 < L.hot; i0 += kBlock * 8) {
        float h[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) h[q] = i0 + kBlock * q < L.hot ? __ldg(L.x + i0 + kBlock * q) : 0.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (i0 + kBlock * q < L.hot) s_hot[i0 + kBlock * q] = h[q];
    }
    __syncthreads();
    float base = 0.0f;
    if (MODE == kModePagerank) base = pr_base(L);
    double dang = 0.0;

    const int ntiles = L.plan.ntiles;
    // Descriptors and lane walks of the next step are requested one step ahead.
    int4 Tn[KT];
    int infon[KT];
#pragma unroll
    for (int k = 0; k < KT; ++k) {
        const int t = gwarp * KT + k;
        Tn[k] = t < ntiles ? __ldg(L.plan.tiles + t) : make_int4(0, 0, 0, 0);
        infon[k] = t < ntiles ? __ldg(L.plan.lane_info + t * 32 + lane) : 0;
    }
    for (int t0 = gwarp * KT; t0 < ntiles; t0 += nwarps * KT) {
        int4 T[KT];
        int info[KT], od0[KT], pos0[KT], od1[KT], pos1[KT];
        float pv[KT][kIpl];
        // Phase 1: columns and the epilogue inputs of the first 32 rows of every tile.
        int cols[KT][kIpl];
#pragma unroll
        for (int k = 0; k < KT; ++k) {
            T[k] = Tn[k];
            info[k] = infon[k];
            const int row = T[k].x, nrows = T[k].y, nb = T[k].z, nnz = T[k].w;
#pragma unroll
            for (int i = 0; i < kIpl; ++i) {
                const int j = i * 32 + lane;
                cols[k][i] = j < nnz ? ld_stream<MODE>(L.col + nb + j) : 0;
            }
            // Predicated loads rather than branches, so they go out with the column loads.
            od0[k] = 0;
            pos0[k] = 0;
            od1[k] = 0;
            pos1[k] = 0;
            if (MODE == kModePagerank) {
                const bool in0 = lane < nrows, in1 = lane + 32 < nrows;
                od0[k] = in0 ? ld_stream<MODE>(L.outdeg + row + lane) : 0;
                od1[k] = in1 ? ld_stream<MODE>(L.outdeg + row + lane + 32) : 0;
                if (L.perm) {
                    pos0[k] = in0 ? ld_stream<MODE>(L.perm + row + lane) : 0;
                    pos1[k] = in1 ? ld_stream<MODE>(L.perm + row + lane + 32) : 0;
                } else {
                    pos0[k] = row + lane;
                    pos1[k] = row + lane + 32;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < KT; ++k) {
            const int t = t0 + nwarps * KT + k;
            Tn[k] = t < ntiles ? __ldg(L.plan.tiles + t) : make_int4(0, 0, 0, 0);
            infon[k] = t < ntiles ? __ldg(L.plan.lane_info + t * 32 + lane) : 0;
        }
        // Phase 2: the gathers of every tile. Both forms keep the hot test a select between a shared
        // and a global load (written as an if/else it became a divergent branch: PageRank 0.192 ms
        // per sweep against 0.176 ms). PageRank keeps its gathers under the (almost always warp-
        // uniform) `j < nnz` test. SpMV issues them with no branch at all, the shared-memory read
        // unconditional (entry 0 for cold columns; the launch allocates at least one) and the
        // value load predicated, so the gather and its value load go out together: 204 -> 255 GTEPS
        // on R-MAT 22. The unconditional shared read costs PageRank 1.4 %, hence the two forms.
#pragma unroll
        for (int k = 0; k < KT; ++k) {
            const int nb = T[k].z, nnz = T[k].w;
#pragma unroll
            for (int i = 0; i < kIpl; ++i) {
                const int j = i * 32 + lane;
                const int c = cols[k][i];
                if constexpr (MODE == kModeSpmv) {
                    const bool hot = c < L.hot;
                    const float hv = s_hot[hot ? c : 0];
                    float gv = 0.0f;
                    if (!hot) gv = __ldg(L.x + c);
                    const float a = j < nnz ? ld_stream<MODE>(L.vals + nb + j) : 0.0f;
                    pv[k][i] = j < nnz ? (hot ? hv : gv) * a : 0.0f;
                } else {
                    float v = 0.0f;
                    if (j < nnz) v = c < L.hot ? s_hot[c] : __ldg(L.x + c);
                    pv[k][i] = v;
                }
            }
        }

        // Phase 3: each tile through the staging area.
#pragma unroll
        for (int k = 0; k < KT; ++k) {
            if (t0 + k >= ntiles) break;
            const int row = T[k].x, nrows = T[k].y, nb = T[k].z, nnz = T[k].w;
            if (nrows < 0) {
                // Hub segment: fixed-order lane sums, then a butterfly; partial goes to the fix-up.
                // Values past the segment's end are 0 (phase 2), so every lane adds all of its own.
                float acc = 0.0f;
#pragma unroll
                for (int i = 0; i < kIpl; ++i) acc += pv[k][i];
                acc = warp_sum_f32(acc);
                if (lane == 0) L.partial[-(nrows + 1)] = acc;
                continue;
            }
            // All 8 values are staged (0 past nnz; pad(255) = 262 is inside the 264-entry row), so the
            // stores need no predicate; the walk reads only the first nnz of them as nonzeros.
#pragma unroll
            for (int i = 0; i < kIpl; ++i) val[pad(i * 32 + lane)] = pv[k][i];
            __syncwarp();
            // Merge-path: lane owns merge items [d0, d1) starting at row r0; the plan's mask says
            // which of them are row ends (emit the open row) and which are nonzeros (take one).
            // r = row ends consumed, kk = nonzeros consumed. The walk is branch-free.
            const int total = nrows + nnz;
            const int d0 = min(lane * kIpl, total);
            const int nlive = min(d0 + kIpl, total) - d0;
            const unsigned ends = static_cast<unsigned>(info[k]) >> 8;
            int r = d0 < total ? (info[k] & 0xFF) : nrows;
            int kk = d0 - r;
            float acc = 0.0f;
            // Rows advance only at row ends, so the first row the lane closes is its start row.
            const int first_emit = ends != 0u ? r : -1;
#pragma unroll
            for (int i = 0; i < kIpl; ++i) {
                const bool emit = (ends >> i) & 1u;
                const bool take = i < nlive && !emit;
                const float v = val[pad(kk)];  // kk <= nnz <= 255 stays inside the padded row
                if (emit) out[pad(r)] = acc;
                acc = take ? acc + v : (emit ? 0.0f : acc);
                kk += take ? 1 : 0;
                r += emit ? 1 : 0;
            }
            // Segmented inclusive scan of the lanes' open partials (key = row still open at lane end).
            float cv = acc;
            const int key = r;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float tv = __shfl_up_sync(kFullMask, cv, o);
                const int tk = __shfl_up_sync(kFullMask, key, o);
                if (lane >= o && tk == key) cv += tv;
            }
            const float cin = __shfl_up_sync(kFullMask, cv, 1);
            const int kin = __shfl_up_sync(kFullMask, key, 1);
            if (lane > 0 && first_emit >= 0 && kin == first_emit) out[pad(first_emit)] += cin;
            __syncwarp();
            for (int rr = lane; rr < nrows; rr += 32) {
                const float sum = out[pad(rr)];
                if (MODE == kModeSpmv) {
                    L.y[row + rr] = sum;
                } else if (rr < 32) {
                    pr_epilogue(L, row + rr, sum, base, od0[k], pos0[k], dang);
                } else if (rr < 64) {
                    pr_epilogue(L, row + rr, sum, base, od1[k], pos1[k], dang);
                } else {
                    pr_epilogue(L, row + rr, sum, base, dang);
                }
            }
            __syncwarp();
        }
    }
    if (MODE == kModePagerank) {
        dang = warp_sum_f64(dang);
        if (lane == 0) L.dpart[gwarp] = dang;
    }
}

// The hub fix-up after each gather launch (and, with no hubs, after the initial vector). For
// PageRank it also reduces the sweep's dangling mass into dsum_out.
template <int MODE>
__global__ void __launch_bounds__(kFixBlock) hub_fixup_kernel(RowGatherLaunch L, int gather_warps, DevStatus* st) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int nthreads = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int gwarp = tid >> 5;
    const int nwarps = nthreads >> 5;
    float base = 0.0f;
    if (MODE == kModePagerank) base = pr_base(L);
    double dang = 0.0;
    fixup_hubs<MODE>(L, tid, nthreads, gwarp, nwarps, lane, base, dang);
    if (MODE != kModePagerank) return;
    // Block b adds its slice of the gather warps' dangling partials to its own rows' (slices in
    // index order), leaves one partial, and the last block to finish adds those in block order.
    const int per = (gather_warps + gridDim.x - 1) / gridDim.x;
    const int lo = min(gather_warps, static_cast<int>(blockIdx.x) * per);
    const int hi = min(gather_warps, lo + per);
    double slice = 0.0;
    for (int i = lo + static_cast<int>(threadIdx.x); i < hi; i += kFixBlock) slice += __ldcg(L.dpart + i);
    const double bsum = block_sum_f64<kFixBlock>(slice + dang);
    __shared__ int s_last;
    if (threadIdx.x == 0) {
        L.dfix[blockIdx.x] = bsum;
        __threadfence();
        s_last = atomicAdd(&st->fix_count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const double total = block_sum_f64<kFixBlock>(strided_sum_f64<kFixBlock>(L.dfix, gridDim.x, 0.0));
    if (threadIdx.x == 0) {
        *L.dsum_out = total;
        st->fix_count = 0u;
    }
}

// Initial contribution vector and its dangling mass. Uses the gather grid so dpart lines up.
__global__ void __launch_bounds__(kInitBlock) pr_init_kernel(RowGatherLaunch L, float init_rank, float* rank_prev) {
    const int lane = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nthreads = gridDim.x * blockDim.x;
    double dang = 0.0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < L.V; v += nthreads) {
        const int od = __ldg(L.outdeg + v);
        const float r0 = L.vgraph ? __ldg(L.ginit + __ldg(L.vgraph + v)) : init_rank;
        const int pos = L.perm ? __ldg(L.perm + v) : v;
        if (od > 0) L.y[pos] = r0 / static_cast<float>(od);
        else if (L.vgraph) L.y[pos] = r0;
        else dang += static_cast<double>(r0);
        if (rank_prev) rank_prev[v] = r0;
    }
    dang = warp_sum_f64(dang);
    if (lane == 0) L.dpart[gwarp] = dang;
}

// Per lane of each normal tile, once per graph: the merge-path start row, i.e. the largest r with
// (row end r-1) + r <= 8 * lane (the row ends the lane's first merge item comes after), and which
// of the lane's 8 merge items are row ends rather than nonzeros. With both, the gather kernel walks
// its items without reading any row end.
// With d_ntiles the tile count is read on the device (clamped to cap), and a set bad-offsets flag
// makes the kernel do nothing: the plan it would read was built from offsets that failed the check.
__global__ void tile_lane_starts_kernel(const int4* __restrict__ tiles, int ntiles, const int64_t* d_ntiles,
                                        int64_t cap, const int* bad, const int32_t* __restrict__ off,
                                        uint16_t* __restrict__ lane_info) {
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    if (d_ntiles) {
        if (bad && (*reinterpret_cast<const volatile int*>(bad) & 4)) return;
        const int64_t n = *d_ntiles;
        ntiles = static_cast<int>(n < cap ? n : cap);
    }
    for (int t = w; t < ntiles; t += nw) {
        const int4 T = __ldg(tiles + t);
        int lo = 0;
        unsigned ends = 0;
        if (T.y > 0) {
            const int row = T.x, nrows = T.y, nb = T.z, nnz = T.w;
            const int total = nrows + nnz;
            const int d0 = min(lane * kIpl, total);
            lo = max(0, d0 - nnz);
            int hi = min(d0, nrows);
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(off + row + mid) - nb + mid <= d0) lo = mid;
                else hi = mid - 1;
            }
            // The lane's items in merge order: nonzero kk while kk < (end of row r), else the end of r.
            int r = lo, kk = d0 - lo;
            const int d1 = min(d0 + kIpl, total);
            int rend = r < nrows ? __ldg(off + row + r + 1) - nb : 0x7FFFFFFF;
            for (int i = 0; d0 + i < d1; ++i) {
                if (kk < rend) {
                    ++kk;
                } else {
                    ends |= 1u << i;
                    ++r;
                    rend = r < nrows ? __ldg(off + row + r + 1) - nb : 0x7FFFFFFF;
                }
            }
        }
        lane_info[static_cast<int64_t>(t) * 32 + lane] = static_cast<uint16_t>(lo | (ends << 8));
    }
}

}  // namespace

cudaError_t launch_tile_lane_starts(const RowPlanDev& plan, const int32_t* off, cudaStream_t s, int sm_count) {
    if (plan.ntiles > 0)
        tile_lane_starts_kernel<<<sm_count * 8, 256, 0, s>>>(plan.tiles, plan.ntiles, nullptr, 0, nullptr, off,
                                                             plan.lane_info);
    return cudaGetLastError();
}

cudaError_t launch_tile_lane_starts_dev(const int4* tiles, const int64_t* d_ntiles, int64_t cap, const int* bad,
                                        const int32_t* off, uint16_t* lane_info, cudaStream_t s, int sm_count) {
    tile_lane_starts_kernel<<<sm_count * 8, 256, 0, s>>>(tiles, 0, d_ntiles, cap, bad, off, lane_info);
    return cudaGetLastError();
}

void rowgather_grid(int sm_count, int* gather_blocks, int* fix_blocks, int* block_threads) {
    *gather_blocks = sm_count;
    *fix_blocks = sm_count * 2;
    *block_threads = kBlock;
}

size_t rowgather_staging_bytes() { return sizeof(int) * kWarps * 2 * kPadded; }

namespace {

// Sets the kernel's dynamic shared-memory limit to what this launch needs (once per size).
template <int MODE>
cudaError_t prepare_rowgather(size_t bytes) {
    static size_t configured = 0;
    if (bytes <= configured) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(rowgather_kernel<MODE, MODE == kModeSpmv ? DPG_GATHER_TILES_SPMV : DPG_GATHER_TILES_PR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(bytes));
    if (e == cudaSuccess) configured = bytes;
    return e;
}

}  // namespace

namespace {

// ---- the row plan, built on the device ------------------------------------------------------------
// Rows are tiled in fixed ranges of kPlanRange rows, one thread per range, by a greedy walk:
// consecutive rows share a tile while their merge items (rows + nonzeros) fit in kRowTileItems, and
// a row above kHubRowDegree becomes a hub cut into kRowTileItems segments (segments numbered from 0
// within the range, then offset by the earlier ranges' counts). A count pass, an exclusive scan of
// the per-range counts and a write pass produce the tiles in row order, so the plan is the same on
// every run. Offsets that are negative, decrease or pass E stop their range's walk and set bit 4 of
// the status flag; the walk never reads past off[V] and every write is checked against the capacity.
constexpr int32_t kPlanRange = 2048;
constexpr int kPlanBlock = 128;

struct PlanCount {
    int64_t tiles = 0, small = 0, big = 0, segs = 0;
    __device__ void tile(int32_t, int32_t, int32_t, int32_t) { ++tiles; }
    __device__ void hub(int32_t, int32_t, int32_t nseg) { (nseg <= kSmallHubSegs ? small : big) += 1; }
};

struct PlanWrite {
    int64_t t, hs, hb, seg_base;  // next slots, and the range's first global segment id
    int64_t cap_tiles, cap_hubs;
    int4* tiles;
    int4* hubs_small;
    int4* hubs_big;
    __device__ void tile(int32_t row, int32_t nrows_or_seg, int32_t nb, int32_t nnz) {
        // nrows_or_seg >= 0: a normal tile of that many rows; < 0: hub segment -(local id + 1).
        const int32_t y = nrows_or_seg >= 0 ? nrows_or_seg : static_cast<int32_t>(nrows_or_seg - seg_base);
        if (t < cap_tiles) tiles[t] = make_int4(row, y, nb, nnz);
        ++t;
    }
    __device__ void hub(int32_t row, int32_t first_seg, int32_t nseg) {
        const int4 h = make_int4(row, static_cast<int32_t>(seg_base + first_seg), nseg, 0);
        if (nseg <= kSmallHubSegs) {
            if (hs < cap_hubs) hubs_small[hs] = h;
            ++hs;
        } else {
            if (hb < cap_hubs) hubs_big[hb] = h;
            ++hb;
        }
    }
};

// The greedy walk over rows [r0, r1); returns the number of hub segments, or -1 on bad offsets.
template <class Sink>
__device__ int32_t plan_range(const int32_t* __restrict__ off, int32_t r0, int32_t r1, int64_t E, Sink& sk) {
    int32_t cur_row = r0, cur_rows = 0, cur_items = 0, cur_nb = 0, cur_end = 0, segs = 0;
    int32_t a = __ldg(off + r0);
    if (a < 0 || a > E) return -1;
    for (int32_t r = r0; r < r1; ++r) {
        const int32_t b = __ldg(off + r + 1);
        if (b < a || b > E) return -1;
        const int32_t d = b - a;
        if (d > kHubRowDegree) {
            if (cur_rows > 0) sk.tile(cur_row, cur_rows, cur_nb, cur_end - cur_nb);
            cur_rows = 0;
            cur_items = 0;
            const int32_t nseg = (d + kRowTileItems - 1) / kRowTileItems;
            for (int32_t k = 0; k < nseg; ++k) {
                const int32_t sb = a + k * kRowTileItems;
                sk.tile(r, -(segs + k + 1), sb, min(kRowTileItems, b - sb));
            }
            sk.hub(r, segs, nseg);
            segs += nseg;
        } else {
            if (cur_items + d + 1 > kRowTileItems) {
                sk.tile(cur_row, cur_rows, cur_nb, cur_end - cur_nb);
                cur_rows = 0;
                cur_items = 0;
            }
            if (cur_rows == 0) {
                cur_row = r;
                cur_nb = a;
            }
            ++cur_rows;
            cur_items += d + 1;
            cur_end = b;
        }
        a = b;
    }
    if (cur_rows > 0) sk.tile(cur_row, cur_rows, cur_nb, cur_end - cur_nb);
    return segs;
}

__device__ __forceinline__ int32_t range_end(int32_t r0, int32_t V) {
    const int64_t end = static_cast<int64_t>(r0) + kPlanRange;
    return static_cast<int32_t>(end < V ? end : V);
}

// counts[4][nranges]: tiles, small hubs, big hubs, segments of each range.
__global__ void __launch_bounds__(kPlanBlock) plan_count_kernel(const int32_t* __restrict__ off, int32_t V, int64_t E,
                                                                int64_t* __restrict__ counts, int32_t nranges, int* bad) {
    const int32_t k = blockIdx.x * kPlanBlock + threadIdx.x;
    if (k >= nranges) return;
    PlanCount c;
    const int32_t r0 = k * kPlanRange;
    const int32_t segs = plan_range(off, r0, range_end(r0, V), E, c);
    if (segs < 0) {
        atomicOr(bad, 4);
        c = PlanCount();
    } else {
        c.segs = segs;
    }
    counts[k] = c.tiles;
    counts[nranges + k] = c.small;
    counts[2 * static_cast<int64_t>(nranges) + k] = c.big;
    counts[3 * static_cast<int64_t>(nranges) + k] = c.segs;
}

// In-place exclusive scan of each of the four count rows; totals[0..3] receive the sums. One block.
__global__ void __launch_bounds__(1024) plan_scan_kernel(int64_t* counts, int32_t nranges, int64_t* totals) {
    __shared__ int64_t s_part[4][1024];
    const int t = threadIdx.x;
    const int32_t per = (nranges + 1023) / 1024;
    const int64_t lo = static_cast<int64_t>(t) * per;
    const int64_t hi = lo + per < nranges ? lo + per : static_cast<int64_t>(nranges);
    for (int q = 0; q < 4; ++q) {
        int64_t acc = 0;
        for (int64_t i = lo; i < hi; ++i) acc += counts[q * static_cast<int64_t>(nranges) + i];
        s_part[q][t] = acc;
    }
    __syncthreads();
    if (t < 4) {
        int64_t run = 0;
        for (int i = 0; i < 1024; ++i) {
            const int64_t v = s_part[t][i];
            s_part[t][i] = run;
            run += v;
        }
        totals[t] = run;
    }
    __syncthreads();
    for (int q = 0; q < 4; ++q) {
        int64_t run = s_part[q][t];
        for (int64_t i = lo; i < hi; ++i) {
            int64_t* p = counts + q * static_cast<int64_t>(nranges) + i;
            const int64_t v = *p;
            *p = run;
            run += v;
        }
    }
}

__global__ void __launch_bounds__(kPlanBlock) plan_write_kernel(const int32_t* __restrict__ off, int32_t V, int64_t E,
                                                                const int64_t* __restrict__ bases, int32_t nranges,
                                                                int4* tiles, int64_t cap_tiles, int4* hubs_small,
                                                                int4* hubs_big, int64_t cap_hubs) {
    const int32_t k = blockIdx.x * kPlanBlock + threadIdx.x;
    if (k >= nranges) return;
    PlanWrite w;
    w.t = bases[k];
    w.hs = bases[nranges + k];
    w.hb = bases[2 * static_cast<int64_t>(nranges) + k];
    w.seg_base = bases[3 * static_cast<int64_t>(nranges) + k];
    w.cap_tiles = cap_tiles;
    w.cap_hubs = cap_hubs;
    w.tiles = tiles;
    w.hubs_small = hubs_small;
    w.hubs_big = hubs_big;
    const int32_t r0 = k * kPlanRange;
    plan_range(off, r0, range_end(r0, V), E, w);
}

int32_t plan_ranges(int32_t V) { return V > 0 ? static_cast<int32_t>((static_cast<int64_t>(V) + kPlanRange - 1) / kPlanRange) : 0; }

}  // namespace

// Tiles of a valid CSR: consecutive normal tiles of one run (no hub or range start between them)
// hold more than kRowTileItems merge items per pair, so there are at most 2(V+E)/257 + runs of them;
// a hub of degree d >= 256 gives ceil(d/256) <= d/256 + 1 segments; hubs <= E/256 and runs <=
// hubs + ranges. Hence tiles <= (2V + 5E)/256 + ranges + 1.
RowPlanCaps row_plan_caps(int32_t V, int64_t E) {
    RowPlanCaps c;
    const int64_t ranges = plan_ranges(V);
    c.tiles = (2 * static_cast<int64_t>(V) + 5 * E) / 256 + ranges + 2;
    c.hubs = E / 256 + 1;
    c.scratch_bytes = sizeof(int64_t) * (4 * static_cast<size_t>(ranges > 0 ? ranges : 1) + 4);
    return c;
}

cudaError_t launch_build_row_plan(const int32_t* off, int32_t V, int64_t E, const RowPlanCaps& caps, int4* tiles,
                                  int4* hubs_small, int4* hubs_big, void* scratch, int64_t* totals, int* bad,
                                  cudaStream_t s) {
    const int32_t nr = plan_ranges(V);
    if (nr == 0) return cudaMemsetAsync(totals, 0, 4 * sizeof(int64_t), s);
    int64_t* counts = static_cast<int64_t*>(scratch);
    const int blocks = (nr + kPlanBlock - 1) / kPlanBlock;
    plan_count_kernel<<<blocks, kPlanBlock, 0, s>>>(off, V, E, counts, nr, bad);
    plan_scan_kernel<<<1, 1024, 0, s>>>(counts, nr, totals);
    plan_write_kernel<<<blocks, kPlanBlock, 0, s>>>(off, V, E, counts, nr, tiles, caps.tiles, hubs_small, hubs_big,
                                                    caps.hubs);
    return cudaGetLastError();
}

namespace {

// A sweep: the gather kernel, then the hub fix-up kernel (which for PageRank also reduces the
// dangling partials). Folding the fix-up into the gather behind a grid barrier (one cooperative
// launch) measured only 0.6 % faster on R-MAT 22: the fix-up's round trips stay on the critical path.
template <int MODE>
cudaError_t launch_row_sweep(const RowGatherLaunch& L, DevStatus* st, cudaStream_t stream, int sm_count,
                             LaunchHook* hook) {
    constexpr int KT = MODE == kModeSpmv ? DPG_GATHER_TILES_SPMV : DPG_GATHER_TILES_PR;
    int gb, fb, bt;
    rowgather_grid(sm_count, &gb, &fb, &bt);
    // At least one hot entry: the SpMV gather reads entry 0 for cold columns.
    const size_t smem = rowgather_staging_bytes() + sizeof(float) * static_cast<size_t>(L.hot > 0 ? L.hot : 1);
    cudaError_t err = prepare_rowgather<MODE>(smem);
    if (err != cudaSuccess) return err;
    {
        HookScope hs(hook, DPG_KERNEL_ROWGATHER, stream);
        rowgather_kernel<MODE, KT><<<gb, bt, smem, stream>>>(L);
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    if (MODE == kModeSpmv && L.plan.nhub_small + L.plan.nhub_big == 0) return cudaSuccess;
    {
        HookScope hs(hook, DPG_KERNEL_FIXUP, stream);
        hub_fixup_kernel<MODE><<<fb, kFixBlock, 0, stream>>>(L, gb * (bt / 32), st);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_spmv(const RowGatherLaunch& L, DevStatus* st, cudaStream_t stream, int sm_count,
                        LaunchHook* hook) {
    return launch_row_sweep<kModeSpmv>(L, st, stream, sm_count, hook);
}

cudaError_t launch_pagerank_sweep(const RowGatherLaunch& L, DevStatus* st, cudaStream_t stream, int sm_count,
                                  LaunchHook* hook) {
    return launch_row_sweep<kModePagerank>(L, st, stream, sm_count, hook);
}

cudaError_t launch_pagerank_init(const RowGatherLaunch& L, float init_rank, float* rank_prev, DevStatus* st,
                                 cudaStream_t stream, int sm_count, LaunchHook* hook) {
    int gb, fb, bt;
    rowgather_grid(sm_count, &gb, &fb, &bt);
    {
        HookScope hs(hook, DPG_KERNEL_INIT, stream);
        // Same number of warps as the gather grid, so dpart[] lines up one slot per warp.
        pr_init_kernel<<<gb * (bt / kInitBlock), kInitBlock, 0, stream>>>(L, init_rank, rank_prev);
    }
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    // A fix-up pass over no hubs reduces the initial dangling partials into dsum_out.
    RowGatherLaunch F = L;
    F.plan.nhub_small = 0;
    F.plan.nhub_big = 0;
    {
        HookScope hs(hook, DPG_KERNEL_INIT, stream);
        hub_fixup_kernel<kModePagerank><<<fb, kFixBlock, 0, stream>>>(F, gb * (bt / 32), st);
    }
    return cudaGetLastError();
}

}  // namespace dpg
