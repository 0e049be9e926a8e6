// Weighted PageRank and its gradient with respect to the edge weights.
//
// No counterpart in the reference (its PageRank, apps/pagerank/src/pagerank_kernel.cu:95-120, has
// unit arcs and no derivative). The graph is the out-adjacency: arc e = (u -> v) carries a positive
// weight w[e], W[u] = sum of u's out-weights, and u is dangling when W[u] == 0. With damping d and
// total rank T the ranks are the fixed point of
//     r[v] = (1 - d) T / V + d D / V + d * sum over arcs u->v of w[e] r[u] / W[u],
// D = sum of r over dangling vertices. For a loss L(r) with seed s = dL/dr, implicit differentiation
// at the fixed point gives the adjoint fixed point
//     lambda[u] = s[u] + d / W[u] * sum over arcs u->t of w[e] lambda[t]    (W[u] > 0)
//     lambda[u] = s[u] + d / V * sum_t lambda[t]                             (dangling u)
// and, per arc e = (u -> v), with q[u] = sum_t w[e'] lambda[t] / W[u],
//     dL/dw[e] = d * r[u] / W[u] * (lambda[v] - q[u]).
// The sweeps' gathers are the row-gather SpMV (forward over the transposed CSR with permuted
// weights, adjoint over the graph itself); the kernels here are the vector epilogues between
// sweeps and the per-arc gradient. Every reduction runs in a fixed order (per-block partials, summed
// in block order by the last block), so results are bit-reproducible.
#include <cuda_runtime.h>

#include "dpg_device.cuh"
#include "dpg_kernels.h"

namespace dpg {
namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ double block_sum_f64(double v, double* s_warp) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum_f64(v);
    if (lane == 0) s_warp[wid] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < kBlock / 32; ++i) t += s_warp[i];
    return t;  // valid in thread 0
}

// One vector pass over all V vertices (see PrVecMode). Block b handles vertices b*256+t, stepping by
// the grid; its partial of the reduced quantity goes to part[b], and the last block to finish adds
// the partials in block order into red_out.
__global__ void __launch_bounds__(kBlock) pr_vec_kernel(PrVecLaunch L) {
    __shared__ double s_warp[kBlock / 32];
    __shared__ bool s_last;
    const int mode = L.mode;
    const bool adjoint = mode == PRV_ADJ_INIT || mode == PRV_ADJ_SWEEP;
    const bool sweep = mode == PRV_FWD_SWEEP || mode == PRV_ADJ_SWEEP;
    // Forward: the uniform term (1-d)T/V + dD/V; adjoint: the dangling rows' d/V * sum(lambda).
    float uniform = 0.0f;
    if (sweep) uniform = static_cast<float>(L.base_const + L.red_scale * L.red_in[0]);
    double acc = 0.0;
    bool moved = false;
    for (int64_t v = static_cast<int64_t>(blockIdx.x) * kBlock + threadIdx.x; v < L.V;
         v += static_cast<int64_t>(gridDim.x) * kBlock) {
        const float Wv = L.W[v];
        float x;
        if (!adjoint) {
            x = sweep ? fmaf(L.damping, L.y[v], uniform) : L.init_value;
            L.contrib[v] = Wv > 0.0f ? x / Wv : 0.0f;
            if (!(Wv > 0.0f)) acc += x;
        } else {
            const float s = L.seed[v];
            if (!sweep) x = s;
            else x = Wv > 0.0f ? s + L.damping * (L.y[v] / Wv) : s + uniform;
            acc += x;
        }
        if (L.prev && fabsf(x - L.prev[v]) > L.epsilon * fabsf(x)) moved = true;
        L.out[v] = x;
    }
    if (L.nonstop && __syncthreads_or(moved) && threadIdx.x == 0) atomicOr(L.nonstop, 1u);
    const double t = block_sum_f64(acc, s_warp);
    if (threadIdx.x == 0) {
        L.part[blockIdx.x] = t;
        __threadfence();
        s_last = atomicAdd(L.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        double sum = 0.0;
        for (unsigned b = 0; b < gridDim.x; ++b) sum += static_cast<volatile double*>(L.part)[b];
        L.red_out[0] = sum;
        *L.ticket = 0u;
    }
}

// dL/dw[e] for the item's arcs e = (u -> col[e]); lanes across arcs.
__global__ void __launch_bounds__(kBlock) pr_arc_grad_kernel(const int4* __restrict__ items, int nitems,
                                                             const int32_t* __restrict__ col, const float* __restrict__ r,
                                                             const float* __restrict__ W, const float* __restrict__ y,
                                                             const float* __restrict__ lam, float damping,
                                                             float* __restrict__ grad) {
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int it = w; it < nitems; it += nw) {
        const int4 I = __ldg(items + it);
        const float Wu = __ldg(W + I.x);
        // A row with arcs and W == 0 (all weights zero) is dangling: its arcs get no gradient.
        const float c = Wu > 0.0f ? damping * __ldg(r + I.x) / Wu : 0.0f;
        const float q = Wu > 0.0f ? __ldg(y + I.x) / Wu : 0.0f;
        for (int e = I.y + lane; e < I.z; e += 32) grad[e] = c * (__ldg(lam + __ldg(col + e)) - q);
    }
}

__global__ void fill_f32_kernel(float* p, int64_t n, float v) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        p[i] = v;
}

}  // namespace

int pr_vec_blocks(int sm_count) { return sm_count * 2; }

cudaError_t launch_pr_vec(const PrVecLaunch& L, int sm_count, cudaStream_t s, LaunchHook* hook) {
    HookScope hs(hook, L.mode == PRV_FWD_INIT || L.mode == PRV_ADJ_INIT ? DPG_KERNEL_INIT : DPG_KERNEL_FIXUP, s);
    pr_vec_kernel<<<pr_vec_blocks(sm_count), kBlock, 0, s>>>(L);
    return cudaGetLastError();
}

cudaError_t launch_pr_arc_grad(const SpmmPlanDev& P, const int32_t* col, const float* r, const float* W, const float* y,
                               const float* lam, float damping, float* grad, cudaStream_t s, int sm_count,
                               LaunchHook* hook) {
    HookScope hs(hook, DPG_KERNEL_ROWGATHER, s);
    if (P.nitems > 0)
        pr_arc_grad_kernel<<<sm_count * 8, kBlock, 0, s>>>(P.items, P.nitems, col, r, W, y, lam, damping, grad);
    return cudaGetLastError();
}

cudaError_t launch_fill_f32(float* p, int64_t n, float v, cudaStream_t s, int sm_count) {
    if (n > 0) fill_f32_kernel<<<sm_count * 4, kBlock, 0, s>>>(p, n, v);
    return cudaGetLastError();
}

}  // namespace dpg
