// Batched right-hand sides and the SpMV adjoint: Y = A X, dX = A^T G, dA[e] = <G[row(e)], X[col(e)]>.
//
// No counterpart in the reference (its SpMV, apps/SpMV/src/SpMV_kernel.cu:81-96, multiplies one
// vector). With nrhs columns stored row-major ([V][nrhs] FP32), every nonzero touches whole rows of
// 4 * nrhs bytes, so a warp reads each gathered row with coalesced loads (lane j holds columns
// j, j+32, ...). Rows are cut on the host into items of at most kSpmmSegment nonzeros; items of a
// split row write partial rows that a fix-up adds in segment order, so sums have a fixed order.
//   spmm_rows_kernel      Y[row] = sum over the item's nonzeros of val * X[col]   (Y = A X, and
//                         dX = A^T G when run over the transposed CSR with permuted values)
//   arc_dot_kernel        dA[e] = <G[row], X[col(e)]>, the warp holding G[row] in registers
// With nrhs a multiple of 32 and 16-byte aligned row blocks, the group kernels below take over:
//   spmm_group_kernel     Y = A X with float4 rows split over 8-lane groups
//   spmv_bwd_group_kernel dX and dA in one pass over the transposed CSR
#include <cuda_runtime.h>

#include <algorithm>

#include "dpg_kernels.h"

namespace dpg {
namespace {

constexpr int kBlock = 256;

template <int NV>
__device__ __forceinline__ void load_row(const float* __restrict__ M, int64_t r, int nrhs, int lane, float (&v)[NV]) {
    const float* p = M + r * nrhs;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const int j = lane + 32 * q;
        v[q] = j < nrhs ? __ldg(p + j) : 0.0f;
    }
}

// One warp per item {row, arc begin, arc end, segment or -1}; 4 nonzeros in flight.
template <int NV>
__global__ void __launch_bounds__(kBlock) spmm_rows_kernel(const int4* __restrict__ items, int nitems,
                                                           const int32_t* __restrict__ col, const float* __restrict__ val,
                                                           const float* __restrict__ X, int nrhs, float* __restrict__ Y,
                                                           float* __restrict__ partial) {
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = w; it < nitems; it += nw) {
        const int4 I = __ldg(items + it);
        float acc[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = 0.0f;
        int e = I.y;
        for (; e + 4 <= I.z; e += 4) {
            int c[4];
            float a[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                c[u] = __ldg(col + e + u);
                a[u] = __ldg(val + e + u);
            }
            float xv[4][NV];
#pragma unroll
            for (int u = 0; u < 4; ++u) load_row<NV>(X, c[u], nrhs, lane, xv[u]);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int q = 0; q < NV; ++q) acc[q] = fmaf(a[u], xv[u][q], acc[q]);
        }
        for (; e < I.z; ++e) {
            const int c = __ldg(col + e);
            const float a = __ldg(val + e);
            float xv[NV];
            load_row<NV>(X, c, nrhs, lane, xv);
#pragma unroll
            for (int q = 0; q < NV; ++q) acc[q] = fmaf(a, xv[q], acc[q]);
        }
        float* dst = I.w < 0 ? Y + static_cast<int64_t>(I.x) * nrhs : partial + static_cast<int64_t>(I.w) * nrhs;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const int j = lane + 32 * q;
            if (j < nrhs) dst[j] = acc[q];
        }
    }
}

// Split rows: Y[row] = sum of its segments' partial rows, in segment order. Warp per split row.
template <int NV>
__global__ void __launch_bounds__(kBlock) spmm_fixup_kernel(const int4* __restrict__ hubs, int nhubs,
                                                            const float* __restrict__ partial, int nrhs,
                                                            float* __restrict__ Y) {
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int h = w; h < nhubs; h += nw) {
        const int4 H = __ldg(hubs + h);
        float acc[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = 0.0f;
        for (int s = 0; s < H.z; ++s) {
            float pv[NV];
            load_row<NV>(partial, H.y + s, nrhs, lane, pv);
#pragma unroll
            for (int q = 0; q < NV; ++q) acc[q] += pv[q];
        }
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            const int j = lane + 32 * q;
            if (j < nrhs) Y[static_cast<int64_t>(H.x) * nrhs + j] = acc[q];
        }
    }
}

// dA[e] = <G[row], X[col(e)]> for the item's arcs; the warp keeps G[row] in registers.
template <int NV>
__global__ void __launch_bounds__(kBlock) arc_dot_kernel(const int4* __restrict__ items, int nitems,
                                                         const int32_t* __restrict__ col, const float* __restrict__ X,
                                                         const float* __restrict__ G, int nrhs, float* __restrict__ dA) {
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = w; it < nitems; it += nw) {
        const int4 I = __ldg(items + it);
        float g[NV];
        load_row<NV>(G, I.x, nrhs, lane, g);
        int e = I.y;
        for (; e + 4 <= I.z; e += 4) {
            float xv[4][NV];
#pragma unroll
            for (int u = 0; u < 4; ++u) load_row<NV>(X, __ldg(col + e + u), nrhs, lane, xv[u]);
            float d[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                d[u] = 0.0f;
#pragma unroll
                for (int q = 0; q < NV; ++q) d[u] = fmaf(g[q], xv[u][q], d[u]);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) d[u] = warp_sum_f32(d[u]);
            if (lane < 4) {
                const float mine = lane == 0 ? d[0] : lane == 1 ? d[1] : lane == 2 ? d[2] : d[3];
                dA[e + lane] = mine;
            }
        }
        for (; e < I.z; ++e) {
            float xv[NV];
            load_row<NV>(X, __ldg(col + e), nrhs, lane, xv);
            float d = 0.0f;
#pragma unroll
            for (int q = 0; q < NV; ++q) d = fmaf(g[q], xv[q], d);
            d = warp_sum_f32(d);
            if (lane == 0) dA[e] = d;
        }
    }
}

// One right-hand side: dA[e] = G[row] * X[col(e)], lanes across the item's arcs (coalesced).
__global__ void __launch_bounds__(kBlock) arc_dot1_kernel(const int4* __restrict__ items, int nitems,
                                                          const int32_t* __restrict__ col, const float* __restrict__ X,
                                                          const float* __restrict__ G, float* __restrict__ dA) {
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = w; it < nitems; it += nw) {
        const int4 I = __ldg(items + it);
        const float g = __ldg(G + I.x);
        for (int e = I.y + lane; e < I.z; e += 32) dA[e] = g * __ldg(X + __ldg(col + e));
    }
}

__global__ void gather_values_kernel(const float* __restrict__ v, const int32_t* __restrict__ idx, int64_t n,
                                     float* __restrict__ out) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = __ldg(v + __ldg(idx + i));
}

// ---- group kernels: nrhs a multiple of 32, rows 16-byte aligned --------------------------------------
// A warp is 4 groups of 8 lanes; a group holds one row of nrhs = 32 * QPL floats as QPL float4 per
// lane (lane l of the group holds float4 l, l + 8, ...), so each of its loads is 8 consecutive
// float4 of one row. The 4 groups take 4 different arcs of the warp's item, each group kGroupU
// arcs deep, so a warp keeps 4 * kGroupU gathered rows in flight. Each group sums its arcs in arc
// order; the 4 group partials are combined by a fixed butterfly, so sums keep a fixed order.
#ifndef DPG_GROUP_U
#define DPG_GROUP_U 4
#endif
constexpr int kGroupU = DPG_GROUP_U;

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

__device__ __forceinline__ void fma4(float4& acc, float a, const float4& x) {
    acc.x = fmaf(a, x.x, acc.x);
    acc.y = fmaf(a, x.y, acc.y);
    acc.z = fmaf(a, x.z, acc.z);
    acc.w = fmaf(a, x.w, acc.w);
}

__device__ __forceinline__ float4 shfl_xor4(const float4& v, int m) {
    return make_float4(__shfl_xor_sync(kFullMask, v.x, m), __shfl_xor_sync(kFullMask, v.y, m),
                       __shfl_xor_sync(kFullMask, v.z, m), __shfl_xor_sync(kFullMask, v.w, m));
}

__device__ __forceinline__ void add4(float4& a, const float4& b) {
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
    a.w += b.w;
}

// Y[row] = sum over the item's arcs of val * X[col].
template <int QPL>
__global__ void __launch_bounds__(kBlock) spmm_group_kernel(const int4* __restrict__ items, int nitems,
                                                            const int32_t* __restrict__ col,
                                                            const float* __restrict__ val,
                                                            const float* __restrict__ X, int nrhs,
                                                            float* __restrict__ Y, float* __restrict__ partial) {
    const int lane = threadIdx.x & 31;
    const int grp = lane >> 3;
    const int gl = lane & 7;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = w; it < nitems; it += nw) {
        const int4 I = __ldg(items + it);
        float4 acc[QPL];
#pragma unroll
        for (int q = 0; q < QPL; ++q) acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int base = I.y; base < I.z; base += 4 * kGroupU) {
            int c[kGroupU];
            float a[kGroupU];
            bool act[kGroupU];
#pragma unroll
            for (int u = 0; u < kGroupU; ++u) {
                const int t = base + 4 * u + grp;
                act[u] = t < I.z;
                c[u] = act[u] ? __ldg(col + t) : 0;
                a[u] = act[u] ? __ldg(val + t) : 0.0f;
            }
            // Slots past the item's end hold zeros (not 0 x a row, which an Inf would turn into NaN).
            float4 x[kGroupU][QPL];
#pragma unroll
            for (int u = 0; u < kGroupU; ++u)
#pragma unroll
                for (int q = 0; q < QPL; ++q)
                    x[u][q] = act[u] ? ld4(X + static_cast<int64_t>(c[u]) * nrhs + 4 * (gl + 8 * q))
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int u = 0; u < kGroupU; ++u)
#pragma unroll
                for (int q = 0; q < QPL; ++q) fma4(acc[q], a[u], x[u][q]);
        }
#pragma unroll
        for (int q = 0; q < QPL; ++q) {
            add4(acc[q], shfl_xor4(acc[q], 8));
            add4(acc[q], shfl_xor4(acc[q], 16));
        }
        if (grp == 0) {
            float* dst = I.w < 0 ? Y + static_cast<int64_t>(I.x) * nrhs : partial + static_cast<int64_t>(I.w) * nrhs;
#pragma unroll
            for (int q = 0; q < QPL; ++q) *reinterpret_cast<float4*>(dst + 4 * (gl + 8 * q)) = acc[q];
        }
    }
}

// The adjoint in one pass over the transposed CSR (item = column j of A): G[i] is gathered once per
// arc i -> j and serves both dX[j] += val * G[i] and dA[arc] = <G[i], X[j]>, with X[j] held in
// registers (every group holds it). The dot product of an arc is summed by its group (lane-local
// float4 parts, then a 3-step butterfly) and written by the group's first lane. dX or dA may be
// skipped (null). Measured on R-MAT 22 with 64 right-hand sides: 5.6 ms against 7.55 ms for the
// two general kernels (row gather over the transpose, then an arc pass gathering X as well), and
// 9.3 ms for two group kernels doing the same two passes. CTAs per SM: with 64 right-hand sides
// (QPL = 2) the kernel takes 80 registers unbounded (3 CTAs); bounded to 4 CTAs (64 registers,
// 128 bytes of spills) the call went from 5.57 to 5.30 ms on the same box. The other widths keep
// what they take unbounded (47, 106 and 128 registers).
template <int QPL>
__global__ void __launch_bounds__(kBlock, QPL == 1 ? 5 : QPL == 2 ? 4 : 2) spmv_bwd_group_kernel(const int4* __restrict__ items, int nitems,
                                                                const int32_t* __restrict__ tcol,
                                                                const int32_t* __restrict__ tarc,
                                                                const float* __restrict__ val,
                                                                const float* __restrict__ X,
                                                                const float* __restrict__ G, int nrhs,
                                                                float* __restrict__ dX, float* __restrict__ partial,
                                                                float* __restrict__ dA) {
    const int lane = threadIdx.x & 31;
    const int grp = lane >> 3;
    const int gl = lane & 7;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = w; it < nitems; it += nw) {
        const int4 I = __ldg(items + it);
        float4 xj[QPL], acc[QPL];
#pragma unroll
        for (int q = 0; q < QPL; ++q) {
            xj[q] = dA ? ld4(X + static_cast<int64_t>(I.x) * nrhs + 4 * (gl + 8 * q)) : make_float4(0.f, 0.f, 0.f, 0.f);
            acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        for (int base = I.y; base < I.z; base += 4 * kGroupU) {
            int r[kGroupU], e[kGroupU];
            bool act[kGroupU];
#pragma unroll
            for (int u = 0; u < kGroupU; ++u) {
                const int t = base + 4 * u + grp;
                act[u] = t < I.z;
                r[u] = act[u] ? __ldg(tcol + t) : 0;
                e[u] = act[u] ? __ldg(tarc + t) : 0;
            }
            float a[kGroupU];
#pragma unroll
            for (int u = 0; u < kGroupU; ++u) a[u] = act[u] ? __ldg(val + e[u]) : 0.0f;
            float4 gr[kGroupU][QPL];
#pragma unroll
            for (int u = 0; u < kGroupU; ++u)
#pragma unroll
                for (int q = 0; q < QPL; ++q)
                    gr[u][q] = act[u] ? ld4(G + static_cast<int64_t>(r[u]) * nrhs + 4 * (gl + 8 * q))
                                      : make_float4(0.f, 0.f, 0.f, 0.f);
            if (dX) {
#pragma unroll
                for (int u = 0; u < kGroupU; ++u)
#pragma unroll
                    for (int q = 0; q < QPL; ++q) fma4(acc[q], a[u], gr[u][q]);
            }
            if (dA) {
                float d[kGroupU];
#pragma unroll
                for (int u = 0; u < kGroupU; ++u) {
                    d[u] = 0.0f;
#pragma unroll
                    for (int q = 0; q < QPL; ++q) {
                        d[u] = fmaf(gr[u][q].x, xj[q].x, d[u]);
                        d[u] = fmaf(gr[u][q].y, xj[q].y, d[u]);
                        d[u] = fmaf(gr[u][q].z, xj[q].z, d[u]);
                        d[u] = fmaf(gr[u][q].w, xj[q].w, d[u]);
                    }
                }
#pragma unroll
                for (int m = 4; m > 0; m >>= 1)
#pragma unroll
                    for (int u = 0; u < kGroupU; ++u) d[u] += __shfl_xor_sync(kFullMask, d[u], m);
                if (gl == 0) {
#pragma unroll
                    for (int u = 0; u < kGroupU; ++u)
                        if (act[u]) dA[e[u]] = d[u];
                }
            }
        }
        if (!dX) continue;
#pragma unroll
        for (int q = 0; q < QPL; ++q) {
            add4(acc[q], shfl_xor4(acc[q], 8));
            add4(acc[q], shfl_xor4(acc[q], 16));
        }
        if (grp == 0) {
            float* dst = I.w < 0 ? dX + static_cast<int64_t>(I.x) * nrhs : partial + static_cast<int64_t>(I.w) * nrhs;
#pragma unroll
            for (int q = 0; q < QPL; ++q) *reinterpret_cast<float4*>(dst + 4 * (gl + 8 * q)) = acc[q];
        }
    }
}

template <int NV>
cudaError_t run_spmm(const SpmmPlanDev& P, const int32_t* col, const float* val, const float* X, int nrhs, float* Y,
                     float* partial, cudaStream_t s, int sm_count, LaunchHook* hook) {
    {
        HookScope hs(hook, DPG_KERNEL_ROWGATHER, s);
        if (P.nitems > 0) spmm_rows_kernel<NV><<<sm_count * 8, kBlock, 0, s>>>(P.items, P.nitems, col, val, X, nrhs, Y, partial);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || P.nhubs == 0) return e;
    {
        HookScope hs(hook, DPG_KERNEL_FIXUP, s);
        spmm_fixup_kernel<NV><<<sm_count * 4, kBlock, 0, s>>>(P.hubs, P.nhubs, partial, nrhs, Y);
    }
    return cudaGetLastError();
}

template <int NV>
cudaError_t run_arc_dot(const SpmmPlanDev& P, const int32_t* col, const float* X, const float* G, int nrhs, float* dA,
                        cudaStream_t s, int sm_count, LaunchHook* hook) {
    HookScope hs(hook, DPG_KERNEL_ROWGATHER, s);
    if (P.nitems > 0) arc_dot_kernel<NV><<<sm_count * 8, kBlock, 0, s>>>(P.items, P.nitems, col, X, G, nrhs, dA);
    return cudaGetLastError();
}

}  // namespace

void build_spmm_plan(const int32_t* off, int32_t V, SpmmPlanHost* plan) {
    plan->items.clear();
    plan->hubs.clear();
    plan->nseg = 0;
    for (int32_t r = 0; r < V; ++r) {
        const int32_t b = off[r], e = off[r + 1];
        if (e - b <= kSpmmSegment) {
            plan->items.push_back(make_int4(r, b, e, -1));
            continue;
        }
        const int32_t nseg = (e - b + kSpmmSegment - 1) / kSpmmSegment;
        plan->hubs.push_back(make_int4(r, plan->nseg, nseg, 0));
        for (int32_t k = 0; k < nseg; ++k) {
            const int32_t sb = b + k * kSpmmSegment;
            plan->items.push_back(make_int4(r, sb, std::min(e, sb + kSpmmSegment), plan->nseg + k));
        }
        plan->nseg += nseg;
    }
}

cudaError_t launch_spmm(const SpmmPlanDev& P, const int32_t* col, const float* val, const float* X, int nrhs, float* Y,
                        float* partial, cudaStream_t s, int sm_count, LaunchHook* hook) {
    if (nrhs <= 32) return run_spmm<1>(P, col, val, X, nrhs, Y, partial, s, sm_count, hook);
    if (nrhs <= 64) return run_spmm<2>(P, col, val, X, nrhs, Y, partial, s, sm_count, hook);
    return run_spmm<4>(P, col, val, X, nrhs, Y, partial, s, sm_count, hook);
}

cudaError_t launch_arc_dot(const SpmmPlanDev& P, const int32_t* col, const float* X, const float* G, int nrhs,
                           float* dA, cudaStream_t s, int sm_count, LaunchHook* hook) {
    if (nrhs == 1) {
        HookScope hs(hook, DPG_KERNEL_ROWGATHER, s);
        if (P.nitems > 0) arc_dot1_kernel<<<sm_count * 8, kBlock, 0, s>>>(P.items, P.nitems, col, X, G, dA);
        return cudaGetLastError();
    }
    if (nrhs <= 32) return run_arc_dot<1>(P, col, X, G, nrhs, dA, s, sm_count, hook);
    if (nrhs <= 64) return run_arc_dot<2>(P, col, X, G, nrhs, dA, s, sm_count, hook);
    return run_arc_dot<4>(P, col, X, G, nrhs, dA, s, sm_count, hook);
}

bool spmm_group_ok(int nrhs, const void* a, const void* b, const void* c, const void* d) {
    if (nrhs % 32 != 0 || nrhs > 128) return false;
    for (const void* p : {a, b, c, d})
        if (p && reinterpret_cast<uintptr_t>(p) % 16 != 0) return false;
    return true;
}

namespace {

template <int QPL>
cudaError_t run_spmm_group(const SpmmPlanDev& P, const int32_t* col, const float* val, const float* X, int nrhs,
                           float* Y, float* partial, cudaStream_t s, int sm_count, LaunchHook* hook) {
    {
        HookScope hs(hook, DPG_KERNEL_ROWGATHER, s);
        if (P.nitems > 0)
            spmm_group_kernel<QPL><<<sm_count * 8, kBlock, 0, s>>>(P.items, P.nitems, col, val, X, nrhs, Y, partial);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || P.nhubs == 0) return e;
    {
        HookScope hs(hook, DPG_KERNEL_FIXUP, s);
        spmm_fixup_kernel<QPL><<<sm_count * 4, kBlock, 0, s>>>(P.hubs, P.nhubs, partial, nrhs, Y);
    }
    return cudaGetLastError();
}

template <int QPL>
cudaError_t run_bwd_group(const SpmmPlanDev& TP, const int32_t* tcol, const int32_t* tarc, const float* val,
                          const float* X, const float* G, int nrhs, float* dX, float* partial, float* dA,
                          cudaStream_t s, int sm_count, LaunchHook* hook) {
    {
        HookScope hs(hook, DPG_KERNEL_ROWGATHER, s);
        if (TP.nitems > 0)
            spmv_bwd_group_kernel<QPL><<<sm_count * 8, kBlock, 0, s>>>(TP.items, TP.nitems, tcol, tarc, val, X, G,
                                                                       nrhs, dX, partial, dA);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || TP.nhubs == 0 || !dX) return e;
    {
        HookScope hs(hook, DPG_KERNEL_FIXUP, s);
        spmm_fixup_kernel<QPL><<<sm_count * 4, kBlock, 0, s>>>(TP.hubs, TP.nhubs, partial, nrhs, dX);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_spmm_group(const SpmmPlanDev& P, const int32_t* col, const float* val, const float* X, int nrhs,
                              float* Y, float* partial, cudaStream_t s, int sm_count, LaunchHook* hook) {
    switch (nrhs / 32) {
        case 1: return run_spmm_group<1>(P, col, val, X, nrhs, Y, partial, s, sm_count, hook);
        case 2: return run_spmm_group<2>(P, col, val, X, nrhs, Y, partial, s, sm_count, hook);
        case 3: return run_spmm_group<3>(P, col, val, X, nrhs, Y, partial, s, sm_count, hook);
        default: return run_spmm_group<4>(P, col, val, X, nrhs, Y, partial, s, sm_count, hook);
    }
}

cudaError_t launch_spmv_bwd_group(const SpmmPlanDev& TP, const int32_t* tcol, const int32_t* tarc, const float* val,
                                  const float* X, const float* G, int nrhs, float* dX, float* partial, float* dA,
                                  cudaStream_t s, int sm_count, LaunchHook* hook) {
    switch (nrhs / 32) {
        case 1: return run_bwd_group<1>(TP, tcol, tarc, val, X, G, nrhs, dX, partial, dA, s, sm_count, hook);
        case 2: return run_bwd_group<2>(TP, tcol, tarc, val, X, G, nrhs, dX, partial, dA, s, sm_count, hook);
        case 3: return run_bwd_group<3>(TP, tcol, tarc, val, X, G, nrhs, dX, partial, dA, s, sm_count, hook);
        default: return run_bwd_group<4>(TP, tcol, tarc, val, X, G, nrhs, dX, partial, dA, s, sm_count, hook);
    }
}

cudaError_t launch_gather_values(const float* v, const int32_t* idx, int64_t n, float* out, cudaStream_t s,
                                 int sm_count) {
    if (n > 0) gather_values_kernel<<<sm_count * 8, kBlock, 0, s>>>(v, idx, n, out);
    return cudaGetLastError();
}

}  // namespace dpg
