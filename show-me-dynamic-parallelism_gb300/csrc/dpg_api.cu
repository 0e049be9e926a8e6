// C ABI of the dpg library: contexts, device graphs, and the solver entry points that replace the
// reference wrappers SSSP_GPU / BFS_REC_GPU / SpMV_GPU / PAGERANK_GPU (see include/dpg.h).
//
// Ownership: a dpg_ctx owns a device status block and a grow-only arena of scratch buffers, so
// repeated solves on graphs of the same size allocate nothing. A dpg_graph owns its device CSR and
// a host copy of the offsets used to plan row tiles.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "dpg_internal.h"
#include "dpg_kernels.h"

namespace dpg {

thread_local std::string g_last_error;

dpg_status set_error(dpg_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

}  // namespace dpg

using namespace dpg;

#include "dpg_api_internal.h"

namespace dpg_api {

dpg_status use_device(dpg_ctx* c) {
    if (!c) return set_error(DPG_ERR_INVALID_ARG, "null context");
    DPG_CUDA_TRY(cudaSetDevice(c->device));
    return DPG_OK;
}

#ifndef DPG_GRAPH_POOL
#define DPG_GRAPH_POOL 1
#endif

cudaError_t dev_alloc(dpg_ctx* c, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (DPG_GRAPH_POOL && c && c->pool) return cudaMallocFromPoolAsync(p, bytes, c->pool, c->stream);
    return cudaMalloc(p, bytes);
}

void dev_free(dpg_ctx* c, void* p) {
    if (!p) return;
    if (DPG_GRAPH_POOL && c && c->pool) cudaFreeAsync(p, c->stream);
    else cudaFree(p);
}

// A few pinned host words for flags the host reads back without a stream synchronisation.
dpg_status host_words(dpg_ctx* c, unsigned** out) {
    if (!c->host_words) {
        void* p = nullptr;
        DPG_CUDA_TRY(cudaHostAlloc(&p, 64, cudaHostAllocDefault));
        c->host_words = static_cast<unsigned*>(p);
    }
    *out = c->host_words;
    return DPG_OK;
}

void* arena(dpg_ctx* c, Slot s, size_t bytes, dpg_status* status) {
    Buf& b = c->bufs[s];
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return b.p;
    if (b.p) {
        cudaStreamSynchronize(c->stream);
        cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
    }
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        b.p = nullptr;
        *status = set_error(DPG_ERR_CAPACITY, std::string("device allocation failed: ") + cudaGetErrorString(e));
        return nullptr;
    }
    b.bytes = bytes;
    return b.p;
}

// Reads and clears the device-side error word after the stream drains.
dpg_status check_device(dpg_ctx* c) {
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    int err[2] = {0, 0};
    DPG_CUDA_TRY(cudaMemcpy(err, c->st, sizeof(err), cudaMemcpyDeviceToHost));
    if (err[0] != 0) {
        DPG_CUDA_TRY(cudaMemset(c->st, 0, sizeof(int) * 2));
        const dpg_status s = static_cast<dpg_status>(err[0]);
        return set_error(s, std::string("device reported ") + dpg_status_string(s) + " (site " + std::to_string(err[1]) + ")");
    }
    return DPG_OK;
}

__global__ void weight_sum_kernel(const int32_t* __restrict__ w, int64_t E, unsigned long long* sum) {
    unsigned long long acc = 0;
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < E;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x)
        acc += static_cast<unsigned long long>(w[e] > 0 ? w[e] : 0);
    acc = warp_sum_u64(acc);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(sum, acc);
}

__global__ void validate_interleave_kernel(const int32_t* col, const int32_t* w, int2* adj, int64_t E, int32_t V,
                                           int* bad) {
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < E;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int32_t c = col[e];
        if (c < 0 || c >= V) atomicOr(bad, 1);
        if (w) {
            const int32_t wt = w[e];
            if (wt < 0 || wt >= DPG_INF_COST) atomicOr(bad, 2);
            if (adj) adj[e] = make_int2(c, wt);
        }
    }
}

// Device-side check of a CSR given by device pointers: bad |= 4 when the offsets do not rise from 0
// to E (the columns are checked by validate_interleave_kernel).
__global__ void validate_offsets_kernel(const int32_t* off, int32_t V, int64_t E, int* bad) {
    for (int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; v < V;
         v += static_cast<int64_t>(gridDim.x) * blockDim.x)
        if (off[v + 1] < off[v]) atomicOr(bad, 4);
    if (blockIdx.x == 0 && threadIdx.x == 0 && (off[0] != 0 || static_cast<int64_t>(off[V]) != E)) atomicOr(bad, 4);
}

dpg_status validate_offsets(const int32_t* off, int32_t V, int64_t E, int32_t* max_deg) {
    if (off[0] != 0 || static_cast<int64_t>(off[V]) != E)
        return set_error(DPG_ERR_INVALID_ARG, "offsets must start at 0 and end at E");
    int32_t md = 0;
    int64_t first_bad = INT64_MAX;
#pragma omp parallel for reduction(max : md) reduction(min : first_bad) schedule(static)
    for (int32_t v = 0; v < V; ++v) {
        const int32_t d = off[v + 1] - off[v];
        if (d < 0 && v < first_bad) first_bad = v;
        if (d > md) md = d;
    }
    if (first_bad != INT64_MAX)
        return set_error(DPG_ERR_INVALID_ARG, "offsets decrease at vertex " + std::to_string(first_bad));
    *max_deg = md;
    return DPG_OK;
}

dpg_status graph_finish(dpg_ctx* c, dpg_graph* g, const int32_t* d_w_src) {
    // Range-check columns (and weights), and interleave (neighbour, weight) pairs for SSSP.
    dpg_status st = DPG_OK;
    int* bad = static_cast<int*>(arena(c, S_NONSTOP, sizeof(int) * 4, &st));
    if (!bad) return st;
    DPG_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), c->stream));
    if (g->E > 0) {
        const int blocks = c->sm_count * 4;
        validate_interleave_kernel<<<blocks, 256, 0, c->stream>>>(g->col, d_w_src, g->adj, g->E, g->V, bad);
        DPG_CUDA_TRY(cudaGetLastError());
    }
    unsigned long long* wsum = reinterpret_cast<unsigned long long*>(bad + 2);
    if (d_w_src && g->E > 0) {
        DPG_CUDA_TRY(cudaMemsetAsync(wsum, 0, sizeof(unsigned long long), c->stream));
        weight_sum_kernel<<<c->sm_count * 4, 256, 0, c->stream>>>(d_w_src, g->E, wsum);
        DPG_CUDA_TRY(cudaGetLastError());
    }
    int hbad[4] = {0, 0, 0, 0};
    DPG_CUDA_TRY(cudaMemcpyAsync(hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, c->stream));
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (hbad[0] & 1) return set_error(DPG_ERR_INVALID_ARG, "column index out of range");
    if (hbad[0] & 2) return set_error(DPG_ERR_INVALID_ARG, "weights must be in [0, 2^30)");
    if (d_w_src && g->E > 0) {
        unsigned long long sum = 0;
        memcpy(&sum, hbad + 2, sizeof(sum));
        g->mean_weight = static_cast<double>(sum) / static_cast<double>(g->E);
    }
    return DPG_OK;
}

void graph_free_device(dpg_graph* g) {
    if (g->tgraph) {
        if (g->tgraph->ctx) g->tgraph->ctx->graphs.erase(g->tgraph);
        graph_free_device(g->tgraph);
        delete g->tgraph;
        g->tgraph = nullptr;
    }
    dev_free(g->ctx, g->off);
    dev_free(g->ctx, g->col);
    dev_free(g->ctx, g->adj);
    dev_free(g->ctx, g->perm);
    dev_free(g->ctx, g->inv);
    dev_free(g->ctx, g->pcol);
    dev_free(g->ctx, g->t_off);
    dev_free(g->ctx, g->t_col);
    g->perm = g->inv = g->pcol = g->t_off = g->t_col = nullptr;
    for (SpmmPlanDev* p : {&g->spmm_plan, &g->spmm_t_plan}) {
        dev_free(g->ctx, p->items);
        dev_free(g->ctx, p->hubs);
        *p = SpmmPlanDev();
    }
    dev_free(g->ctx, g->tt_col);
    dev_free(g->ctx, g->tt_arc);
    g->tt_col = g->tt_arc = nullptr;
    g->spmm_ready = g->spmm_t_ready = false;
    g->relabel_ready = false;
    dev_free(g->ctx, g->plan.tiles);
    dev_free(g->ctx, g->plan.lane_info);
    dev_free(g->ctx, g->plan.hubs_small);
    dev_free(g->ctx, g->plan.hubs_big);
    g->off = nullptr;
    g->col = nullptr;
    g->adj = nullptr;
    g->plan = RowPlanDev();
}

cudaError_t plan_build_alloc(dpg_ctx* c, int32_t V, int64_t E, PlanBuild* pb) {
    pb->caps = row_plan_caps(V, E);
    cudaError_t e;
    if ((e = dev_alloc(c, &pb->tiles, sizeof(int4) * static_cast<size_t>(pb->caps.tiles))) != cudaSuccess ||
        (e = dev_alloc(c, &pb->hubs_small, sizeof(int4) * static_cast<size_t>(pb->caps.hubs))) != cudaSuccess ||
        (e = dev_alloc(c, &pb->hubs_big, sizeof(int4) * static_cast<size_t>(pb->caps.hubs))) != cudaSuccess)
        return e;
    return dev_alloc(c, &pb->scratch, pb->caps.scratch_bytes);
}

cudaError_t plan_build_launch(const PlanBuild& pb, const int32_t* d_off, int32_t V, int64_t E, PlanInfo* d_info,
                              cudaStream_t s) {
    return launch_build_row_plan(d_off, V, E, pb.caps, pb.tiles, pb.hubs_small, pb.hubs_big, pb.scratch,
                                 d_info->totals, &d_info->bad, s);
}

void plan_build_free(dpg_ctx* c, PlanBuild* pb) {
    dev_free(c, pb->tiles);
    dev_free(c, pb->hubs_small);
    dev_free(c, pb->hubs_big);
    dev_free(c, pb->scratch);
    *pb = PlanBuild();
}

dpg_status plan_finish(dpg_graph* g, PlanBuild* pb, const PlanInfo& info) {
    dpg_ctx* c = g->ctx;
    cudaStream_t s = c->stream;
    const int64_t nt = info.totals[0], nsm = info.totals[1], nbg = info.totals[2], nsg = info.totals[3];
    if (nt < 0 || nt > pb->caps.tiles || nsm < 0 || nsm > pb->caps.hubs || nbg < 0 || nbg > pb->caps.hubs || nsg < 0 ||
        nsg > INT32_MAX)
        return set_error(DPG_ERR_CAPACITY, "row plan exceeds its capacity");
    RowPlanDev d;
    d.ntiles = static_cast<int32_t>(nt);
    d.nhub_small = static_cast<int32_t>(nsm);
    d.nhub_big = static_cast<int32_t>(nbg);
    d.nseg = static_cast<int32_t>(nsg);
    DPG_CUDA_TRY(dev_alloc(c, &d.tiles, sizeof(int4) * static_cast<size_t>(nt + 1)));
    DPG_CUDA_TRY(dev_alloc(c, &d.lane_info, 32 * sizeof(uint16_t) * static_cast<size_t>(nt + 1)));
    DPG_CUDA_TRY(dev_alloc(c, &d.hubs_small, sizeof(int4) * static_cast<size_t>(nsm + 1)));
    DPG_CUDA_TRY(dev_alloc(c, &d.hubs_big, sizeof(int4) * static_cast<size_t>(nbg + 1)));
    if (nt > 0)
        DPG_CUDA_TRY(cudaMemcpyAsync(d.tiles, pb->tiles, sizeof(int4) * static_cast<size_t>(nt), cudaMemcpyDeviceToDevice, s));
    if (nsm > 0)
        DPG_CUDA_TRY(cudaMemcpyAsync(d.hubs_small, pb->hubs_small, sizeof(int4) * static_cast<size_t>(nsm),
                                     cudaMemcpyDeviceToDevice, s));
    if (nbg > 0)
        DPG_CUDA_TRY(cudaMemcpyAsync(d.hubs_big, pb->hubs_big, sizeof(int4) * static_cast<size_t>(nbg),
                                     cudaMemcpyDeviceToDevice, s));
    plan_build_free(c, pb);
    DPG_CUDA_TRY(launch_tile_lane_starts(d, g->off, s, c->sm_count));
    g->plan = d;
    g->plan_ready = true;
    return DPG_OK;
}

// The row plan of a graph whose offsets were validated on the host at creation.
dpg_status ensure_plan(dpg_graph* g) {
    if (g->plan_ready) return DPG_OK;
    dpg_ctx* c = g->ctx;
    dpg_status st = DPG_OK;
    PlanInfo* info = static_cast<PlanInfo*>(arena(c, S_PLANINFO, sizeof(PlanInfo), &st));
    if (!info) return st;
    PlanBuild pb;
    cudaError_t e = cudaMemsetAsync(info, 0, sizeof(PlanInfo), c->stream);
    if (e == cudaSuccess) e = plan_build_alloc(c, g->V, g->E, &pb);
    if (e == cudaSuccess) e = plan_build_launch(pb, g->off, g->V, g->E, info, c->stream);
    PlanInfo h;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, info, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        plan_build_free(c, &pb);
        return set_error(DPG_ERR_CUDA, std::string("row plan: ") + cudaGetErrorString(e));
    }
    if (h.bad & 4) {
        plan_build_free(c, &pb);
        return set_error(DPG_ERR_INVALID_ARG, "offsets are not a valid CSR");
    }
    const dpg_status fs = plan_finish(g, &pb, h);
    if (fs != DPG_OK) plan_build_free(c, &pb);
    return fs;
}

// Entries of the gathered vector kept in shared memory by the row-gather kernel: the most frequent
// (renamed) columns, as many as fit next to the tile staging within a shared-memory budget of
// DPG_GATHER_SMEM_KB per SM. The budget is below the 227 KB a CTA could take because what is left
// of the SM's 256 KB of L1/shared memory is the L1 the scattered gathers land in: their sectors in
// flight need L1 lines, and a 28 KB L1 (the 228 KB shared-memory carve-out) capped them well below
// what 32 warps issue. On R-MAT scale 22 a PageRank sweep took 0.29 ms with every free byte given
// to the hot cache (31.5 K entries) and 0.202 ms at this budget (16 K entries, 92 KB of L1).
#ifndef DPG_GATHER_SMEM_KB
#define DPG_GATHER_SMEM_KB 164
#endif
int32_t hot_entries(const dpg_ctx* c, const dpg_graph* g) {
    if (!g->relabel) return 0;
    // 1 KB of each carve-out is reserved per CTA by the system.
    const int64_t budget = std::min<int64_t>(c->smem_optin, DPG_GATHER_SMEM_KB * 1024 - 1024);
    const int64_t room = budget - static_cast<int64_t>(rowgather_staging_bytes());
    const int64_t cap = room > 0 ? room / 4 : 0;
    return static_cast<int32_t>(cap < g->V ? cap : g->V);
}

// Builds perm/inv/pcol for the row gathers: column counts, the frequency order (a 33-class stable
// multi-split) and the renamed column array, all on the device. With relabel_segments (vertex
// starts of packed graphs) each segment is ordered on its own (on the host, once per batch), so
// renamed ids stay inside their graph's range and each graph's gathers stay inside its own slice.
dpg_status ensure_relabel(dpg_graph* g) {
    if (g->relabel_ready || g->V == 0) return DPG_OK;
    dpg_ctx* c = g->ctx;
    const size_t nv = static_cast<size_t>(g->V);
    const std::vector<int32_t>& seg = g->relabel_segments;
    int32_t* counts = nullptr;
    DPG_CUDA_TRY(dev_alloc(c, &counts, nv * 4));
    cudaError_t e = dev_alloc(c, &g->perm, nv * 4);
    if (e == cudaSuccess) e = dev_alloc(c, &g->inv, nv * 4);
    if (e == cudaSuccess) e = dev_alloc(c, &g->pcol, static_cast<size_t>(g->E > 0 ? g->E : 1) * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, nv * 4, c->stream);
    if (e == cudaSuccess) e = launch_column_histogram(g->col, g->E, counts, c->stream, c->sm_count);
    if (e == cudaSuccess && seg.size() < 2) {
        // One graph: the whole order on the device.
        int32_t* scratch = nullptr;
        e = dev_alloc(c, &scratch, frequency_order_scratch_bytes(g->V));
        if (e == cudaSuccess) e = launch_frequency_order(counts, g->V, scratch, g->perm, g->inv, c->stream);
        dev_free(c, scratch);
    } else if (e == cudaSuccess) {
        // Packed graphs: each segment ordered on its own, on the host.
        std::vector<int32_t> h_counts(nv), h_perm(nv), h_inv(nv);
        e = cudaMemcpyAsync(h_counts.data(), counts, nv * 4, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e == cudaSuccess) {
            const int nseg = static_cast<int>(seg.size()) - 1;
#pragma omp parallel for schedule(dynamic, 1)
            for (int k = 0; k < nseg; ++k) {
                const int32_t lo = seg[k], n = seg[k + 1] - seg[k];
                frequency_order(h_counts.data() + lo, n, h_perm.data() + lo, h_inv.data() + lo);
                for (int32_t i = 0; i < n; ++i) {
                    h_perm[lo + i] += lo;
                    h_inv[lo + i] += lo;
                }
            }
            e = cudaMemcpyAsync(g->perm, h_perm.data(), nv * 4, cudaMemcpyHostToDevice, c->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(g->inv, h_inv.data(), nv * 4, cudaMemcpyHostToDevice, c->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        }
    }
    if (e == cudaSuccess) e = launch_relabel_columns(g->col, g->perm, g->E, g->pcol, c->stream, c->sm_count);
    dev_free(c, counts);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        dev_free(c, g->perm);
        dev_free(c, g->inv);
        dev_free(c, g->pcol);
        g->perm = g->inv = g->pcol = nullptr;
        return set_error(DPG_ERR_CUDA, std::string("column renaming: ") + cudaGetErrorString(e));
    }
    g->relabel_ready = true;
    return DPG_OK;
}

dpg_status upload_spmm_plan(dpg_ctx* c, const SpmmPlanHost& hp, SpmmPlanDev* d) {
    d->nitems = static_cast<int32_t>(hp.items.size());
    d->nhubs = static_cast<int32_t>(hp.hubs.size());
    d->nseg = hp.nseg;
    DPG_CUDA_TRY(dev_alloc(c, &d->items, sizeof(int4) * (hp.items.size() + 1)));
    DPG_CUDA_TRY(dev_alloc(c, &d->hubs, sizeof(int4) * (hp.hubs.size() + 1)));
    if (!hp.items.empty())
        DPG_CUDA_TRY(cudaMemcpyAsync(d->items, hp.items.data(), sizeof(int4) * hp.items.size(), cudaMemcpyHostToDevice,
                                     c->stream));
    if (!hp.hubs.empty())
        DPG_CUDA_TRY(cudaMemcpyAsync(d->hubs, hp.hubs.data(), sizeof(int4) * hp.hubs.size(), cudaMemcpyHostToDevice,
                                     c->stream));
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return DPG_OK;
}

dpg_status ensure_spmm_plan(dpg_graph* g) {
    if (g->spmm_ready) return DPG_OK;
    SpmmPlanHost hp;
    build_spmm_plan(g->h_off.data(), g->V, &hp);
    DPG_TRY(upload_spmm_plan(g->ctx, hp, &g->spmm_plan));
    g->spmm_ready = true;
    return DPG_OK;
}

// Deterministic transposed CSR with the arc permutation, built on the device in invertGraph order
// (dpg_transpose.cu); only its offsets come back to the host, for the batched-RHS plan. With
// need_graph the transposed CSR also becomes a graph of its own (g->tgraph).
dpg_status ensure_spmm_transpose(dpg_graph* g, bool need_graph = false) {
    if (g->spmm_t_ready && (!need_graph || g->tgraph)) return DPG_OK;
    dpg_ctx* c = g->ctx;
    const size_t nv = static_cast<size_t>(g->V), ne = static_cast<size_t>(g->E > 0 ? g->E : 1);
    int32_t* t_off = nullptr;
    DPG_CUDA_TRY(dev_alloc(c, &t_off, (nv + 1) * 4));
    cudaError_t e = cudaSuccess;
    if (!g->tt_col) e = dev_alloc(c, &g->tt_col, ne * 4);
    if (e == cudaSuccess && !g->tt_arc) e = dev_alloc(c, &g->tt_arc, ne * 4);
    dpg_status st = DPG_OK;
    const size_t scratch_bytes = transpose_scratch_bytes(g->V, g->E);
    void* scratch = e == cudaSuccess ? arena(c, S_TRANSPOSE, scratch_bytes, &st) : nullptr;
    if (e == cudaSuccess && st == DPG_OK)
        e = launch_transpose(g->off, g->col, g->V, g->E, t_off, g->tt_col, g->tt_arc, scratch, scratch_bytes,
                             c->stream, c->sm_count);
    std::vector<int32_t> h_t_off(nv + 1);
    if (e == cudaSuccess && st == DPG_OK)
        e = cudaMemcpyAsync(h_t_off.data(), t_off, (nv + 1) * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && st == DPG_OK) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess || st != DPG_OK) {
        dev_free(c, t_off);
        return st != DPG_OK ? st : set_error(DPG_ERR_CUDA, std::string("device transpose: ") + cudaGetErrorString(e));
    }
    if (!g->spmm_t_ready) {
        SpmmPlanHost hp;
        build_spmm_plan(h_t_off.data(), g->V, &hp);
        st = upload_spmm_plan(c, hp, &g->spmm_t_plan);
        if (st == DPG_OK) g->spmm_t_ready = true;
    }
    if (st == DPG_OK && need_graph && !g->tgraph) {
        st = graph_create_common(c, g->V, g->E, t_off, g->tt_col, nullptr, true, &g->tgraph);
        if (st == DPG_OK) g->tgraph->relabel = g->relabel;
    }
    dev_free(c, t_off);
    return st;
}

dpg_status check_nrhs(int32_t nrhs) {
    if (nrhs < 1 || nrhs > 128) return set_error(DPG_ERR_INVALID_ARG, "nrhs must be in [1, 128]");
    return DPG_OK;
}

// Frontier queues, bitmaps and chunk lists from the context arena.
dpg_status expand_workspace(dpg_ctx* c, int32_t V, int64_t E, int32_t min_chunked, ExpandWorkspace* wsp) {
    ExpandWorkspace& ws = *wsp;
    memset(&ws, 0, sizeof(ws));
    ws.cap_v = static_cast<int64_t>(V) + 1;
    ws.cap_chunks = expand_chunk_capacity(V, E, min_chunked);
    ws.bmp_words = (V + 31) / 32 + 1;
    dpg_status st = DPG_OK;
    const size_t nv = static_cast<size_t>(ws.cap_v);
    ws.qv[0] = static_cast<int32_t*>(arena(c, S_QV0, nv * 4, &st));
    ws.qv[1] = static_cast<int32_t*>(arena(c, S_QV1, nv * 4, &st));
    ws.qse[0] = static_cast<int2*>(arena(c, S_QSE0, nv * 8, &st));
    ws.qse[1] = static_cast<int2*>(arena(c, S_QSE1, nv * 8, &st));
    ws.bmp[0] = static_cast<uint32_t*>(arena(c, S_BMP0, static_cast<size_t>(ws.bmp_words) * 4, &st));
    ws.bmp[1] = static_cast<uint32_t*>(arena(c, S_BMP1, static_cast<size_t>(ws.bmp_words) * 4, &st));
    const size_t nc = static_cast<size_t>(ws.cap_chunks);
    ws.chunks[0] = static_cast<int4*>(arena(c, S_CH0, nc * 16, &st));
    ws.chunks[1] = static_cast<int4*>(arena(c, S_CH1, nc * 16, &st));
    ws.qcount = static_cast<uint32_t*>(arena(c, S_QCOUNT, 4 * 4, &st));
    ws.ccount = static_cast<uint32_t*>(arena(c, S_CCOUNT, 4 * 4, &st));
    return st;
}

// In-arc CSR on the device: counts by column histogram, offsets by a host scan, rows filled by an
// atomic-cursor scatter (row order unspecified, which colouring does not depend on).
dpg_status ensure_transpose(dpg_graph* g) {
    if (g->t_off) return DPG_OK;
    dpg_ctx* c = g->ctx;
    const size_t nv = static_cast<size_t>(g->V);
    int32_t* cursor = nullptr;
    DPG_CUDA_TRY(dev_alloc(c, &cursor, (nv + 1) * 4));
    std::vector<int32_t> h(nv + 1, 0);
    cudaError_t e = cudaMemsetAsync(cursor, 0, (nv + 1) * 4, c->stream);
    if (e == cudaSuccess) e = launch_column_histogram(g->col, g->E, cursor, c->stream, c->sm_count);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), cursor, nv * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        dev_free(c, cursor);
        return set_error(DPG_ERR_CUDA, std::string("transpose counts: ") + cudaGetErrorString(e));
    }
    int64_t acc = 0;
    for (size_t v = 0; v < nv; ++v) {
        const int32_t cnt = h[v];
        h[v] = static_cast<int32_t>(acc);
        acc += cnt;
    }
    h[nv] = static_cast<int32_t>(acc);
    e = dev_alloc(c, &g->t_off, (nv + 1) * 4);
    if (e == cudaSuccess) e = dev_alloc(c, &g->t_col, static_cast<size_t>(g->E > 0 ? g->E : 1) * 4);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g->t_off, h.data(), (nv + 1) * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cursor, h.data(), nv * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = launch_transpose_scatter(g->off, g->col, g->V, cursor, g->t_col, c->stream, c->sm_count);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    dev_free(c, cursor);
    if (e != cudaSuccess) {
        dev_free(c, g->t_off);
        dev_free(c, g->t_col);
        g->t_off = g->t_col = nullptr;
        return set_error(DPG_ERR_CUDA, std::string("transpose build: ") + cudaGetErrorString(e));
    }
    return DPG_OK;
}

dpg_status run_color(dpg_ctx* c, dpg_graph* g, const dpg_expand_opts* in_opts, int32_t* d_color) {
    if (!g || g->ctx != c) return set_error(DPG_ERR_INVALID_ARG, "graph does not belong to this context");
    if (g->V == 0) return DPG_OK;
    if (!d_color) return set_error(DPG_ERR_INVALID_ARG, "null output");
    dpg_expand_opts o;
    fill_expand_defaults(in_opts, &o, g);
    DPG_TRY(ensure_transpose(g));
    ExpandWorkspace ws;
    dpg_status st = expand_workspace(c, g->V, g->E, o.hub_threshold, &ws);
    int32_t* pending = static_cast<int32_t*>(arena(c, S_PENDING, static_cast<size_t>(g->V) * 4, &st));
    if (st != DPG_OK) return st;
    ExpandLaunch L;
    memset(&L, 0, sizeof(L));
    L.off = g->t_off;
    L.col = g->t_col;
    L.V = g->V;
    L.E = g->E;
    L.label = d_color;
    L.threshold = o.threshold;
    L.hub_threshold = o.hub_threshold;
    L.max_iter = o.max_iterations;
    L.timeout_ns = static_cast<unsigned long long>(o.timeout_seconds * 1e9);
    L.trace = c->trace;
    L.trace_cap = c->trace_cap;
    c->last_host_iterations = -1;
    DPG_CUDA_TRY(launch_color(L, g->off, g->col, pending, ws, c->st, c->stream, c->sm_count, &c->last_grid,
                              &c->last_block, &c->prof));
    return DPG_OK;
}

// Near-far threshold step in units of the mean arc weight (see dpg_expand.cu, DPG_SOL_NEARFAR).
// Measured (2 sources): on the 4096^2 grid (weights 1..1000) SSSP takes 120 ms at 2x the mean
// weight, 80 at 8x, 67 at 32x, 65 at 64x and 73 at 256x; on R-MAT 22 and 24 (weights 1..255) 32x
// is within 5 % of the binned expansion, and 2x is 15-50 % slower.
constexpr double kNearFarStep = 32.0;

void fill_expand_defaults(const dpg_expand_opts* in, dpg_expand_opts* o, const dpg_graph* g) {
    if (in) *o = *in;
    else {
        memset(o, 0, sizeof(*o));
        o->solution = DPG_SOL_DIROPT;  // BFS: direction-optimizing; SSSP: near-far or binned (run_expand)
    }
    if (o->threshold <= 0) o->threshold = DPG_REF_THRESHOLD;
    // Degree from which a frontier vertex is cut into grid-wide chunks. Measured on R-MAT 24 (4
    // sources): SSSP 9.06 ms at 32, 8.14 at 64, 7.81 at 128, 8.08 at 256; BFS (direction-optimizing)
    // 1.84 / 1.76 / 1.77 / 1.77 ms. At R-MAT 22, SSSP takes 2.59 / 2.28 / 2.35 / 2.36 ms.
    if (o->hub_threshold <= 0) o->hub_threshold = 128;
    if (o->solution == DPG_SOL_GRID) o->hub_threshold = o->threshold;
    if (o->max_iterations <= 0) {
        const int64_t cap = static_cast<int64_t>(g->V) + 2;
        o->max_iterations = cap > INT32_MAX ? INT32_MAX : static_cast<int32_t>(cap);
    }
    if (!(o->timeout_seconds > 0)) o->timeout_seconds = 10.0;
}

dpg_status run_expand(dpg_ctx* c, const dpg_graph* g, int32_t source, const dpg_expand_opts* in_opts,
                      int32_t* d_label, bool bfs) {
    if (!g || g->ctx != c) return set_error(DPG_ERR_INVALID_ARG, "graph does not belong to this context");
    if (!d_label && g->V > 0) return set_error(DPG_ERR_INVALID_ARG, "null output");
    if (source < 0 || source >= g->V) return set_error(DPG_ERR_INVALID_ARG, "source vertex out of range");
    if (!bfs && !g->weighted) return set_error(DPG_ERR_INVALID_ARG, "SSSP needs a weighted graph");
    dpg_expand_opts o;
    fill_expand_defaults(in_opts, &o, g);
    if (o.solution < DPG_SOL_THREAD || o.solution > DPG_SOL_NEARFAR)
        return set_error(DPG_ERR_INVALID_ARG, "unknown solution id");
    // The default id asks for the GB300 choice; for SSSP (bottom-up steps are BFS only) that is
    // near-far on graphs without hubs and of low mean degree (road-like, grids: 4096^2 grid 68 ms
    // against 167 ms binned), and the binned expansion otherwise (R-MAT: near-far only ties it).
    if (!bfs && o.solution == DPG_SOL_DIROPT)
        o.solution = (g->weighted && g->max_degree < o.hub_threshold && g->E <= 8 * static_cast<int64_t>(g->V))
                         ? DPG_SOL_NEARFAR
                         : DPG_SOL_BINNED;
    if (bfs && o.solution == DPG_SOL_NEARFAR) o.solution = DPG_SOL_DIROPT;  // the threshold is for distances
    const int32_t min_chunked = (o.solution == DPG_SOL_GRID) ? o.threshold : o.hub_threshold;
    ExpandWorkspace ws;
    dpg_status st = expand_workspace(c, g->V, g->E, min_chunked, &ws);
    if (st != DPG_OK) return st;
    ExpandLaunch L;
    L.off = g->off;
    L.col = g->col;
    L.adj = g->adj;
    L.V = g->V;
    L.E = g->E;
    L.label = d_label;
    L.source = source;
    L.bfs = bfs;
    L.solution = o.solution;
    L.wide = g->max_degree >= o.hub_threshold || g->E > 8 * static_cast<int64_t>(g->V);
    L.threshold = o.threshold;
    L.hub_threshold = o.hub_threshold;
    L.max_iter = o.max_iterations;
    L.timeout_ns = static_cast<unsigned long long>(o.timeout_seconds * 1e9);
    L.trace = c->trace;
    L.trace_cap = c->trace_cap;
    if (!bfs && o.solution == DPG_SOL_NEARFAR) {
        // Three piles of E + V {vertex, distance} pairs (at most one current entry per vertex, plus
        // stale ones; an overflow stops the solve with DPG_ERR_CAPACITY).
        const int64_t cap = g->E + g->V + 1;
        dpg_status cs = DPG_OK;
        for (int k = 0; k < 3; ++k)
            L.far[k] = static_cast<int2*>(arena(c, static_cast<Slot>(S_FAR0 + k), static_cast<size_t>(cap) * 8, &cs));
        unsigned* cnt = static_cast<unsigned*>(arena(c, S_FAR_COUNT, 64, &cs));
        if (cs != DPG_OK) return cs;
        L.far_count = cnt;
        L.far_min = reinterpret_cast<int*>(cnt + 4);
        L.far_cap = cap;
        const double mw = g->mean_weight > 0 ? g->mean_weight : 1.0;
        L.delta = o.delta > 0 ? o.delta : static_cast<int32_t>(std::max(1.0, std::min(1e9, kNearFarStep * mw)));
    }
    if (bfs && o.solution == DPG_SOL_DIROPT) {
        DPG_TRY(ensure_transpose(const_cast<dpg_graph*>(g)));
        dpg_status cs = DPG_OK;
        unsigned long long* cnt = static_cast<unsigned long long*>(arena(c, S_DO_COUNT, 64, &cs));
        if (cs != DPG_OK) return cs;
        L.t_off = g->t_off;
        L.t_col = g->t_col;
        L.do_mf = cnt;
        L.do_nf = reinterpret_cast<unsigned*>(cnt + 4);
    }
    if (c->trace) DPG_CUDA_TRY(cudaMemsetAsync(c->trace, 0, sizeof(unsigned long long) * 4 * c->trace_cap, c->stream));
    c->last_host_iterations = -1;
    DPG_CUDA_TRY(launch_expand(L, ws, c->st, c->stream, c->sm_count, &c->last_grid, &c->last_block, &c->prof));
    return DPG_OK;
}

dpg_status pr_defaults(const dpg_pr_opts* in, dpg_pr_opts* o) {
    if (in) *o = *in;
    else {
        o->damping = 0.85;
        o->total_rank = 1.0;
        o->init_zero = 0;
        o->iterations = 20;
        o->epsilon = 0.0;
    }
    if (!(o->damping >= 0.0 && o->damping <= 1.0)) return set_error(DPG_ERR_INVALID_ARG, "damping must be in [0,1]");
    if (o->iterations < 0) return set_error(DPG_ERR_INVALID_ARG, "iterations must be >= 0");
    if (o->epsilon > 0 && o->iterations == 0) o->iterations = INT32_MAX;
    return DPG_OK;
}

dpg_status run_pagerank(dpg_ctx* c, dpg_graph* g, const int32_t* d_outdeg, const dpg_pr_opts* in_opts, float* d_rank) {
    if (!g || g->ctx != c) return set_error(DPG_ERR_INVALID_ARG, "graph does not belong to this context");
    if (g->V > 0 && (!d_outdeg || !d_rank)) return set_error(DPG_ERR_INVALID_ARG, "null outdeg or rank");
    dpg_pr_opts o;
    DPG_TRY(pr_defaults(in_opts, &o));
    if (g->V == 0) return DPG_OK;
    DPG_TRY(ensure_plan(g));
    if (g->relabel) DPG_TRY(ensure_relabel(g));
    int gb, fb, bt;
    rowgather_grid(c->sm_count, &gb, &fb, &bt);
    dpg_status st = DPG_OK;
    const size_t nv = static_cast<size_t>(g->V);
    float* contrib[2] = {static_cast<float*>(arena(c, S_CONTRIB0, nv * 4, &st)),
                         static_cast<float*>(arena(c, S_CONTRIB1, nv * 4, &st))};
    float* partial = static_cast<float*>(arena(c, S_PARTIAL, static_cast<size_t>(g->plan.nseg + 1) * 4, &st));
    double* dpart = static_cast<double*>(arena(c, S_DPART, static_cast<size_t>(gb) * (bt / 32) * 8, &st));
    double* dfix = static_cast<double*>(arena(c, S_DFIX, static_cast<size_t>(fb) * (256 / 32) * 8, &st));
    double* dsum = static_cast<double*>(arena(c, S_DSUM, 2 * 8, &st));
    unsigned* nonstop = static_cast<unsigned*>(arena(c, S_NONSTOP, 16, &st));
    const bool conv = o.epsilon > 0;
    float* rk[2] = {nullptr, nullptr};
    if (conv) {
        rk[0] = static_cast<float*>(arena(c, S_RANK0, nv * 4, &st));
        rk[1] = static_cast<float*>(arena(c, S_RANK1, nv * 4, &st));
    }
    if (st != DPG_OK) return st;
    RowGatherLaunch L;
    memset(&L, 0, sizeof(L));
    L.plan = g->plan;
    L.off = g->off;
    L.col = g->relabel ? g->pcol : g->col;
    L.perm = g->relabel ? g->perm : nullptr;
    L.hot = hot_entries(c, g);
    L.vals = nullptr;
    L.partial = partial;
    L.V = g->V;
    L.outdeg = d_outdeg;
    L.damping = static_cast<float>(o.damping);
    L.base_const = (1.0 - o.damping) * o.total_rank / static_cast<double>(g->V);
    L.dangling_scale = o.damping / static_cast<double>(g->V);
    L.dpart = dpart;
    L.dfix = dfix;
    L.epsilon = static_cast<float>(o.epsilon);
    const float init_rank = o.init_zero ? 0.0f : static_cast<float>(o.total_rank / static_cast<double>(g->V));
    // Contributions of vertices without out-arcs are never written by a sweep; start them at 0 so
    // an out-degree array that disagrees with the graph still reads defined values.
    DPG_CUDA_TRY(cudaMemsetAsync(contrib[0], 0, nv * 4, c->stream));
    DPG_CUDA_TRY(cudaMemsetAsync(contrib[1], 0, nv * 4, c->stream));
    // Initial vector: contributions into contrib[0], dangling mass into dsum[0].
    L.y = contrib[0];
    L.dsum_in = dsum + 1;
    L.dsum_out = dsum;
    float* init_rank_dst = conv ? rk[0] : (o.iterations == 0 ? d_rank : nullptr);
    DPG_CUDA_TRY(launch_pagerank_init(L, init_rank, init_rank_dst, c->st, c->stream, c->sm_count, &c->prof));
    // With a tolerance the convergence test is pipelined one sweep deep: sweep it+1 is queued before
    // the host reads sweep it's flag (pinned memory, an event), so the device does not idle on the
    // read. A sweep queued after the converged one writes only buffers of the other parity (ranks,
    // contributions, dangling sum, flag), so the converged ranks stay where the count says.
    unsigned* hflags = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (conv) {
        DPG_TRY(host_words(c, &hflags));
        for (cudaEvent_t& e : ev) DPG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    struct Events {
        cudaEvent_t* e;
        ~Events() {
            if (e[0]) cudaEventDestroy(e[0]);
            if (e[1]) cudaEventDestroy(e[1]);
        }
    } ev_guard{ev};
    int64_t sweeps = 0;
    int32_t pending = -1;  // sweep whose flag is on its way to the host
    for (int32_t it = 0; it < o.iterations; ++it) {
        L.x = contrib[it & 1];
        L.y = contrib[(it + 1) & 1];
        L.dsum_in = dsum + (it & 1);
        L.dsum_out = dsum + ((it + 1) & 1);
        if (conv) {
            L.rank_prev = rk[it & 1];
            L.rank_out = rk[(it + 1) & 1];
            L.nonstop = nonstop + (it & 1);
            DPG_CUDA_TRY(cudaMemsetAsync(L.nonstop, 0, sizeof(unsigned), c->stream));
        } else {
            L.rank_prev = nullptr;
            L.nonstop = nullptr;
            L.rank_out = (it == o.iterations - 1) ? d_rank : nullptr;
        }
        DPG_CUDA_TRY(launch_pagerank_sweep(L, c->st, c->stream, c->sm_count, &c->prof));
        ++sweeps;
        if (conv) {
            DPG_CUDA_TRY(cudaMemcpyAsync(hflags + 2 + (it & 1), L.nonstop, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                         c->stream));
            DPG_CUDA_TRY(cudaEventRecord(ev[it & 1], c->stream));
            if (pending >= 0) {
                DPG_CUDA_TRY(cudaEventSynchronize(ev[pending & 1]));
                if (hflags[2 + (pending & 1)] == 0) {
                    --sweeps;  // the sweep just queued is surplus
                    break;
                }
            }
            pending = it;
        }
    }
    if (conv) {
        float* fin = rk[sweeps & 1];
        DPG_CUDA_TRY(cudaMemcpyAsync(d_rank, fin, nv * 4, cudaMemcpyDeviceToDevice, c->stream));
    }
    c->last_host_iterations = sweeps;
    c->last_grid = gb;
    c->last_block = bt;
    return DPG_OK;
}

dpg_status run_spmv(dpg_ctx* c, dpg_graph* g, const float* d_vals, const float* d_x, float* d_y) {
    if (!g || g->ctx != c) return set_error(DPG_ERR_INVALID_ARG, "graph does not belong to this context");
    if (g->V == 0) return DPG_OK;
    if (!d_x || !d_y || (g->E > 0 && !d_vals)) return set_error(DPG_ERR_INVALID_ARG, "null vals/x/y");
    DPG_TRY(ensure_plan(g));
    if (g->relabel) DPG_TRY(ensure_relabel(g));
    dpg_status st = DPG_OK;
    float* partial = static_cast<float*>(arena(c, S_PARTIAL, static_cast<size_t>(g->plan.nseg + 1) * 4, &st));
    float* xp = g->relabel ? static_cast<float*>(arena(c, S_XPERM, static_cast<size_t>(g->V) * 4, &st)) : nullptr;
    if (st != DPG_OK) return st;
    if (xp) DPG_CUDA_TRY(launch_gather_by_index(d_x, g->inv, g->V, xp, c->stream, c->sm_count));
    RowGatherLaunch L;
    memset(&L, 0, sizeof(L));
    L.plan = g->plan;
    L.off = g->off;
    L.col = g->relabel ? g->pcol : g->col;
    L.vals = d_vals;
    L.x = xp ? xp : d_x;
    L.hot = hot_entries(c, g);
    L.y = d_y;
    L.partial = partial;
    L.V = g->V;
    c->last_host_iterations = 1;
    DPG_CUDA_TRY(launch_spmv(L, c->st, c->stream, c->sm_count, &c->prof));
    return DPG_OK;
}

dpg_status graph_create_common(dpg_ctx* c, int32_t V, int64_t E, const int32_t* offsets, const int32_t* col,
                               const int32_t* weights, bool device_ptrs, dpg_graph** out) {
    if (!out) return set_error(DPG_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    DPG_TRY(use_device(c));
    if (V < 0 || E < 0 || E > INT32_MAX) return set_error(DPG_ERR_INVALID_ARG, "V must be >= 0 and 0 <= E < 2^31");
    if (!offsets || (E > 0 && !col)) return set_error(DPG_ERR_INVALID_ARG, "null offsets or columns");
    dpg_graph* g = new dpg_graph();
    g->ctx = c;
    g->device = c->device;
    g->V = V;
    g->E = E;
    g->weighted = weights != nullptr;
    g->h_off.resize(static_cast<size_t>(V) + 1);
    auto fail = [&](dpg_status s) {
        graph_free_device(g);
        delete g;
        return s;
    };
    cudaError_t e;
    if (device_ptrs) {
        e = cudaMemcpy(g->h_off.data(), offsets, sizeof(int32_t) * (static_cast<size_t>(V) + 1), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail(set_error(DPG_ERR_CUDA, std::string("offsets D2H: ") + cudaGetErrorString(e)));
    } else {
        const int64_t n = static_cast<int64_t>(V) + 1;
        int32_t* dst = g->h_off.data();
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) dst[i] = offsets[i];
    }
    dpg_status s = validate_offsets(g->h_off.data(), V, E, &g->max_degree);
    if (s != DPG_OK) return fail(s);
    const cudaMemcpyKind kind = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if ((e = dev_alloc(c, &g->off, sizeof(int32_t) * (static_cast<size_t>(V) + 1))) != cudaSuccess ||
        (e = dev_alloc(c, &g->col, sizeof(int32_t) * static_cast<size_t>(E > 0 ? E : 1))) != cudaSuccess ||
        (g->weighted && (e = dev_alloc(c, &g->adj, sizeof(int2) * static_cast<size_t>(E > 0 ? E : 1))) != cudaSuccess))
        return fail(set_error(DPG_ERR_CAPACITY, std::string("graph allocation: ") + cudaGetErrorString(e)));
    if ((e = cudaMemcpyAsync(g->off, offsets, sizeof(int32_t) * (static_cast<size_t>(V) + 1), kind, c->stream)) != cudaSuccess ||
        (E > 0 && (e = cudaMemcpyAsync(g->col, col, sizeof(int32_t) * static_cast<size_t>(E), kind, c->stream)) != cudaSuccess))
        return fail(set_error(DPG_ERR_CUDA, std::string("graph copy: ") + cudaGetErrorString(e)));
    const int32_t* d_w = nullptr;
    if (g->weighted) {
        if (device_ptrs) {
            d_w = weights;
        } else {
            dpg_status as = DPG_OK;
            int32_t* tmp = static_cast<int32_t*>(arena(c, S_VALS, sizeof(int32_t) * static_cast<size_t>(E > 0 ? E : 1), &as));
            if (!tmp) return fail(as);
            if (E > 0 && (e = cudaMemcpyAsync(tmp, weights, sizeof(int32_t) * static_cast<size_t>(E), cudaMemcpyHostToDevice,
                                              c->stream)) != cudaSuccess)
                return fail(set_error(DPG_ERR_CUDA, std::string("weights copy: ") + cudaGetErrorString(e)));
            d_w = tmp;
        }
    }
    s = graph_finish(c, g, d_w);
    if (s != DPG_OK) return fail(s);
    c->graphs.insert(g);
    *out = g;
    return DPG_OK;
}

// The pull graph of a one-shot PageRank (unweighted in-edge CSR from host arrays, V > 0, E > 0).
// Everything between the upload and the sweeps runs on the device, on the aux stream, overlapped
// with the upload of the columns; the host only issues work and waits once:
//   - the offsets and out-degrees upload first. Then the offsets are validated on the device and
//     the row plan (tiles, hub lists, each lane's start row and row-end mask) is built on the device
//     from them, into capacity-sized buffers the graph keeps;
//   - in an in-edge CSR a vertex's column count is its out-degree, so the frequency order of the
//     column renaming comes from the out-degrees. The order is only a renaming and every row keeps
//     its nonzero order, so the sums are the same with any order; out-degrees that disagree with
//     the columns only make the hot cache colder;
//   - the columns upload in kRelabelChunks pieces, and each piece is range-checked and renamed as
//     soon as it has landed (the check graph_finish would make).
// Bad offsets or columns fail the creation with graph_create_common's errors. The graph keeps no
// host copy of its offsets (h_off is empty): it serves the PageRank sweeps only.
// d_outdeg (V ints) receives the out-degrees for the sweeps.
dpg_status graph_create_pull(dpg_ctx* c, int32_t V, int64_t E, const int32_t* in_offsets, const int32_t* in_col,
                             const int32_t* h_outdeg, int32_t* d_outdeg, dpg_graph** out) {
    constexpr int kRelabelChunks = 8;
    *out = nullptr;
    dpg_graph* g = new dpg_graph();
    g->ctx = c;
    g->device = c->device;
    g->V = V;
    g->E = E;
    const size_t nv = static_cast<size_t>(V), ne = static_cast<size_t>(E);
    int32_t* scratch = nullptr;
    PlanBuild pb;
    uint16_t* lane_info = nullptr;  // capacity-sized; the graph keeps it
    cudaEvent_t ev_in = nullptr, ev_done = nullptr, ev_chunk[kRelabelChunks] = {};
    auto release = [&]() {
        if (c->aux_stream) cudaStreamSynchronize(c->aux_stream);
        dev_free(c, scratch);
        scratch = nullptr;
        dev_free(c, lane_info);
        lane_info = nullptr;
        plan_build_free(c, &pb);
        for (cudaEvent_t& ev : ev_chunk) {
            if (ev) cudaEventDestroy(ev);
            ev = nullptr;
        }
        if (ev_in) cudaEventDestroy(ev_in);
        if (ev_done) cudaEventDestroy(ev_done);
        ev_in = ev_done = nullptr;
    };
    auto fail = [&](dpg_status s) {
        release();
        graph_free_device(g);
        delete g;
        return s;
    };
    cudaError_t e = cudaSuccess;
    if (!c->aux_stream && (e = cudaStreamCreateWithFlags(&c->aux_stream, cudaStreamNonBlocking)) != cudaSuccess) {
        c->aux_stream = nullptr;
        return fail(set_error(DPG_ERR_CUDA, std::string("aux stream: ") + cudaGetErrorString(e)));
    }
    dpg_status as = DPG_OK;
    PlanInfo* info = static_cast<PlanInfo*>(arena(c, S_PLANINFO, sizeof(PlanInfo), &as));
    if (!info) return fail(as);
    cudaStream_t s0 = c->stream, s1 = c->aux_stream;
    if ((e = dev_alloc(c, &g->off, (nv + 1) * 4)) != cudaSuccess || (e = dev_alloc(c, &g->col, ne * 4)) != cudaSuccess ||
        (e = dev_alloc(c, &g->perm, nv * 4)) != cudaSuccess || (e = dev_alloc(c, &g->inv, nv * 4)) != cudaSuccess ||
        (e = dev_alloc(c, &g->pcol, ne * 4)) != cudaSuccess ||
        (e = dev_alloc(c, &scratch, frequency_order_scratch_bytes(V))) != cudaSuccess ||
        (e = plan_build_alloc(c, V, E, &pb)) != cudaSuccess ||
        (e = dev_alloc(c, &lane_info, 32 * sizeof(uint16_t) * static_cast<size_t>(pb.caps.tiles))) != cudaSuccess)
        return fail(set_error(DPG_ERR_CAPACITY, std::string("graph allocation: ") + cudaGetErrorString(e)));
    if ((e = cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ev_done, cudaEventDisableTiming)) != cudaSuccess)
        return fail(set_error(DPG_ERR_CUDA, std::string("events: ") + cudaGetErrorString(e)));
    for (cudaEvent_t& ev : ev_chunk)
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess)
            return fail(set_error(DPG_ERR_CUDA, std::string("events: ") + cudaGetErrorString(e)));
    // Everything the aux stream touches is allocated above, before ev_in is recorded on s0, so
    // waiting for ev_in also orders the aux stream after those stream-ordered allocations.
    // Upload stream: status reset, offsets, out-degrees, then the column chunks, each with an event.
    if ((e = cudaMemsetAsync(info, 0, sizeof(PlanInfo), s0)) == cudaSuccess &&
        (e = cudaMemcpyAsync(g->off, in_offsets, (nv + 1) * 4, cudaMemcpyHostToDevice, s0)) == cudaSuccess &&
        (e = cudaMemcpyAsync(d_outdeg, h_outdeg, nv * 4, cudaMemcpyHostToDevice, s0)) == cudaSuccess)
        e = cudaEventRecord(ev_in, s0);
    const int64_t step = (E + kRelabelChunks - 1) / kRelabelChunks;
    for (int k = 0; k < kRelabelChunks && e == cudaSuccess; ++k) {
        const int64_t b = std::min<int64_t>(E, k * step), n = std::min<int64_t>(E, b + step) - b;
        if (n > 0) e = cudaMemcpyAsync(g->col + b, in_col + b, static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice, s0);
        if (e == cudaSuccess) e = cudaEventRecord(ev_chunk[k], s0);
    }
    // Aux stream, once offsets and out-degrees are in: offset check, row plan, renaming order; then
    // each column chunk once it has landed.
    if (e == cudaSuccess && (e = cudaStreamWaitEvent(s1, ev_in, 0)) == cudaSuccess) {
        validate_offsets_kernel<<<c->sm_count * 4, 256, 0, s1>>>(g->off, V, E, &info->bad);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = plan_build_launch(pb, g->off, V, E, info, s1);
    if (e == cudaSuccess)
        e = launch_tile_lane_starts_dev(pb.tiles, &info->totals[0], pb.caps.tiles, &info->bad, g->off, lane_info, s1,
                                        c->sm_count);
    if (e == cudaSuccess) e = launch_frequency_order(d_outdeg, V, scratch, g->perm, g->inv, s1);
    for (int k = 0; k < kRelabelChunks && e == cudaSuccess; ++k) {
        const int64_t b = std::min<int64_t>(E, k * step), n = std::min<int64_t>(E, b + step) - b;
        if ((e = cudaStreamWaitEvent(s1, ev_chunk[k], 0)) == cudaSuccess)
            e = launch_relabel_columns(g->col + b, g->perm, n, g->pcol + b, s1, c->sm_count, V, &info->bad);
    }
    if (e == cudaSuccess && (e = cudaEventRecord(ev_done, s1)) == cudaSuccess) e = cudaStreamWaitEvent(s0, ev_done, 0);
    PlanInfo h;
    if (e == cudaSuccess && (e = cudaMemcpyAsync(&h, info, sizeof(h), cudaMemcpyDeviceToHost, s0)) == cudaSuccess)
        e = cudaStreamSynchronize(s0);
    if (e != cudaSuccess) return fail(set_error(DPG_ERR_CUDA, std::string("graph upload: ") + cudaGetErrorString(e)));
    if (h.bad & 4) {
        // The host check gives the precise message.
        int32_t md = 0;
        const dpg_status vs = validate_offsets(in_offsets, V, E, &md);
        return fail(vs != DPG_OK ? vs : set_error(DPG_ERR_INVALID_ARG, "offsets are not a valid CSR"));
    }
    if (h.bad & 1) return fail(set_error(DPG_ERR_INVALID_ARG, "column index out of range"));
    // The graph adopts the capacity-sized plan buffers as they are (it lives for one call).
    const int64_t nt = h.totals[0], nsm = h.totals[1], nbg = h.totals[2], nsg = h.totals[3];
    if (nt < 0 || nt > pb.caps.tiles || nsm < 0 || nsm > pb.caps.hubs || nbg < 0 || nbg > pb.caps.hubs || nsg < 0 ||
        nsg > INT32_MAX)
        return fail(set_error(DPG_ERR_CAPACITY, "row plan exceeds its capacity"));
    g->plan.ntiles = static_cast<int32_t>(nt);
    g->plan.nhub_small = static_cast<int32_t>(nsm);
    g->plan.nhub_big = static_cast<int32_t>(nbg);
    g->plan.nseg = static_cast<int32_t>(nsg);
    g->plan.tiles = pb.tiles;
    g->plan.hubs_small = pb.hubs_small;
    g->plan.hubs_big = pb.hubs_big;
    g->plan.lane_info = lane_info;
    pb.tiles = pb.hubs_small = pb.hubs_big = nullptr;
    lane_info = nullptr;
    g->plan_ready = true;
    release();
    g->relabel_ready = true;
    c->graphs.insert(g);
    *out = g;
    return DPG_OK;
}

// Weighted PageRank to its fixed point, the adjoint fixed point for the seed dL/dr, and the per-arc
// gradient (kernels and formulas in dpg_prgrad.cu). Sweeps stop when no entry changed by more than
// the relative tolerance times its new value (forward: opts->epsilon on r; adjoint: adjoint_epsilon
// on lambda), or after opts->iterations sweeps each; a tolerance <= 0 runs exactly that many.
dpg_status run_pagerank_grad(dpg_ctx* c, dpg_graph* g, const float* d_w, const float* d_seed, const dpg_pr_opts* in_opts,
                             double adjoint_epsilon, float* d_rank, float* d_grad) {
    if (!g || g->ctx != c) return set_error(DPG_ERR_INVALID_ARG, "graph does not belong to this context");
    dpg_pr_opts o;
    DPG_TRY(pr_defaults(in_opts, &o));
    if (g->V == 0) return DPG_OK;
    if (!d_seed || !d_rank || (g->E > 0 && (!d_w || !d_grad)))
        return set_error(DPG_ERR_INVALID_ARG, "null weights/seed/rank/grad");
    // iterations == 0 with a tolerance means "until converged"; each loop still stops at kMaxGradSweeps.
    constexpr int32_t kMaxGradSweeps = 10000;
    const int32_t fwd_iters = std::min(o.iterations, kMaxGradSweeps);
    int32_t adj_iters = fwd_iters;
    if (adjoint_epsilon > 0 && (!in_opts || in_opts->iterations == 0)) adj_iters = kMaxGradSweeps;
    DPG_TRY(ensure_spmm_transpose(g, true));
    DPG_TRY(ensure_spmm_plan(g));
    const size_t nv = static_cast<size_t>(g->V), ne = static_cast<size_t>(g->E > 0 ? g->E : 1);
    const int nb = pr_vec_blocks(c->sm_count);
    dpg_status st = DPG_OK;
    float* w_t = static_cast<float*>(arena(c, S_VALS_T, ne * 4, &st));
    float* W = static_cast<float*>(arena(c, S_PRG_W, nv * 4, &st));
    float* y = static_cast<float*>(arena(c, S_PRG_Y, nv * 4, &st));
    float* contrib = static_cast<float*>(arena(c, S_PRG_C, nv * 4, &st));
    float* vec[4] = {static_cast<float*>(arena(c, S_PRG_V0, nv * 4, &st)),
                     static_cast<float*>(arena(c, S_PRG_V1, nv * 4, &st)),
                     static_cast<float*>(arena(c, S_PRG_V2, nv * 4, &st)),
                     static_cast<float*>(arena(c, S_PRG_V3, nv * 4, &st))};
    double* part = static_cast<double*>(arena(c, S_PRG_PART, static_cast<size_t>(nb) * 8, &st));
    double* red = static_cast<double*>(arena(c, S_PRG_RED, 2 * 8, &st));
    unsigned* flags = static_cast<unsigned*>(arena(c, S_PRG_FLAGS, 16, &st));  // [0] ticket, [1..2] nonstop
    if (st != DPG_OK) return st;
    DPG_CUDA_TRY(cudaMemsetAsync(flags, 0, 16, c->stream));
    // Out-weight sums W = A 1 and the weights in transposed-slot order.
    DPG_CUDA_TRY(launch_fill_f32(y, g->V, 1.0f, c->stream, c->sm_count));
    DPG_TRY(run_spmv(c, g, d_w, y, W));
    DPG_CUDA_TRY(launch_gather_values(d_w, g->tt_arc, g->E, w_t, c->stream, c->sm_count));

    PrVecLaunch L;
    memset(&L, 0, sizeof(L));
    L.V = g->V;
    L.W = W;
    L.part = part;
    L.ticket = flags;
    L.damping = static_cast<float>(o.damping);
    // The convergence test is pipelined one sweep deep: sweep it+1 is queued before the host reads
    // sweep it's flag (copied to pinned memory, waited on with an event), so the device does not
    // idle on the read. When sweep it converged, sweep it+1 is surplus: it wrote only the other
    // vector, y, the reduction slot and flag of its own parity and (forward) the contributions,
    // none of which is read afterwards, so stepping the vector swap back restores sweep it's result.
    unsigned* hflags = nullptr;
    DPG_TRY(host_words(c, &hflags));
    cudaEvent_t ev[2] = {nullptr, nullptr};
    for (cudaEvent_t& e : ev) DPG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    struct Events {
        cudaEvent_t* e;
        ~Events() {
            cudaEventDestroy(e[0]);
            cudaEventDestroy(e[1]);
        }
    } ev_guard{ev};
    auto sweeps_until = [&](int mode, int32_t cap, double eps, float** cur, float** nxt, dpg_graph* sg,
                            const float* vals, const float* x_of_cur, int64_t* done) -> dpg_status {
        // Every loop starts from the reduction its init pass left in red[0].
        int32_t pending = -1;  // sweep whose flag is on its way to the host
        for (int32_t it = 0; it < cap; ++it) {
            unsigned* dflag = flags + 1 + (it & 1);
            DPG_TRY(run_spmv(c, sg, vals, x_of_cur ? x_of_cur : *cur, y));
            L.mode = mode;
            L.y = y;
            L.prev = eps > 0 ? *cur : nullptr;
            L.out = *nxt;
            L.red_in = red + (it & 1);
            L.red_out = red + ((it + 1) & 1);
            L.epsilon = static_cast<float>(eps);
            L.nonstop = eps > 0 ? dflag : nullptr;
            if (eps > 0) DPG_CUDA_TRY(cudaMemsetAsync(dflag, 0, 4, c->stream));
            DPG_CUDA_TRY(launch_pr_vec(L, c->sm_count, c->stream, &c->prof));
            std::swap(*cur, *nxt);
            ++*done;
            if (eps > 0) {
                DPG_CUDA_TRY(cudaMemcpyAsync(hflags + (it & 1), dflag, 4, cudaMemcpyDeviceToHost, c->stream));
                DPG_CUDA_TRY(cudaEventRecord(ev[it & 1], c->stream));
                if (pending >= 0) {
                    DPG_CUDA_TRY(cudaEventSynchronize(ev[pending & 1]));
                    if (hflags[pending & 1] == 0) {
                        std::swap(*cur, *nxt);
                        --*done;
                        pending = -1;
                        break;
                    }
                }
                pending = it;
            }
        }
        if (pending >= 0) DPG_CUDA_TRY(cudaEventSynchronize(ev[pending & 1]));
        return DPG_OK;
    };

    // Forward: r in vec[0]/vec[1], contributions r / W in contrib, dangling sum in red[0].
    float* r_cur = vec[0];
    float* r_nxt = vec[1];
    L.mode = PRV_FWD_INIT;
    L.out = r_cur;
    L.contrib = contrib;
    L.init_value = o.init_zero ? 0.0f : static_cast<float>(o.total_rank / static_cast<double>(g->V));
    L.red_out = red;
    DPG_CUDA_TRY(launch_pr_vec(L, c->sm_count, c->stream, &c->prof));
    L.base_const = (1.0 - o.damping) * o.total_rank / static_cast<double>(g->V);
    L.red_scale = o.damping / static_cast<double>(g->V);
    int64_t fwd = 0, adj = 0;
    DPG_TRY(sweeps_until(PRV_FWD_SWEEP, fwd_iters, o.epsilon, &r_cur, &r_nxt, g->tgraph, w_t, contrib, &fwd));

    // Adjoint: lambda in vec[2]/vec[3], its sum in red[0].
    float* l_cur = vec[2];
    float* l_nxt = vec[3];
    L.mode = PRV_ADJ_INIT;
    L.seed = d_seed;
    L.out = l_cur;
    L.prev = nullptr;
    L.nonstop = nullptr;
    L.red_out = red;
    DPG_CUDA_TRY(launch_pr_vec(L, c->sm_count, c->stream, &c->prof));
    L.base_const = 0.0;
    L.red_scale = o.damping / static_cast<double>(g->V);
    DPG_TRY(sweeps_until(PRV_ADJ_SWEEP, adj_iters, adjoint_epsilon, &l_cur, &l_nxt, g, d_w, nullptr, &adj));

    // q = (A lambda) / W with the final lambda, then the per-arc gradient.
    DPG_TRY(run_spmv(c, g, d_w, l_cur, y));
    DPG_CUDA_TRY(launch_pr_arc_grad(g->spmm_plan, g->col, r_cur, W, y, l_cur, static_cast<float>(o.damping), d_grad,
                                    c->stream, c->sm_count, &c->prof));
    DPG_CUDA_TRY(cudaMemcpyAsync(d_rank, r_cur, nv * 4, cudaMemcpyDeviceToDevice, c->stream));
    c->last_host_iterations = fwd + adj;
    c->last_grad_sweeps[0] = fwd;
    c->last_grad_sweeps[1] = adj;
    return DPG_OK;
}

}  // namespace dpg_api

extern "C" {

const char* dpg_status_string(dpg_status s) {
    switch (s) {
        case DPG_OK: return "DPG_OK";
        case DPG_ERR_INVALID_ARG: return "DPG_ERR_INVALID_ARG";
        case DPG_ERR_CAPACITY: return "DPG_ERR_CAPACITY";
        case DPG_ERR_TIMEOUT: return "DPG_ERR_TIMEOUT";
        case DPG_ERR_CUDA: return "DPG_ERR_CUDA";
        case DPG_ERR_NO_DEVICE: return "DPG_ERR_NO_DEVICE";
        case DPG_ERR_IO: return "DPG_ERR_IO";
        case DPG_ERR_FORMAT: return "DPG_ERR_FORMAT";
        case DPG_ERR_UNSUPPORTED: return "DPG_ERR_UNSUPPORTED";
    }
    return "DPG_ERR_UNKNOWN";
}

const char* dpg_last_error(void) { return g_last_error.c_str(); }

int dpg_version(void) { return DPG_VERSION; }

dpg_status dpg_ctx_create(int device, dpg_ctx** out) {
    if (!out) return set_error(DPG_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return set_error(DPG_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= n) return set_error(DPG_ERR_INVALID_ARG, "device index out of range");
    DPG_CUDA_TRY(cudaSetDevice(device));
    dpg_ctx* c = new dpg_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e == cudaSuccess) e = cudaMalloc(&c->st, sizeof(DevStatus));
    if (e == cudaSuccess) e = cudaMemset(c->st, 0, sizeof(DevStatus));
    int pools = 0;
    if (e == cudaSuccess && cudaDeviceGetAttribute(&pools, cudaDevAttrMemoryPoolsSupported, device) == cudaSuccess && pools) {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        if (cudaMemPoolCreate(&c->pool, &props) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;  // freed blocks stay in the pool for the next graph
            cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
        } else {
            c->pool = nullptr;
            cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        if (c->own_stream) cudaStreamDestroy(c->own_stream);
        cudaFree(c->st);
        delete c;
        return set_error(DPG_ERR_CUDA, std::string("context setup: ") + cudaGetErrorString(e));
    }
    c->stream = c->own_stream;
    *out = c;
    return DPG_OK;
}

dpg_status dpg_ctx_destroy(dpg_ctx* c) {
    if (!c) return DPG_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (dpg_graph* g : c->graphs) g->ctx = nullptr;
    for (dpg_batch* b : c->batches) batch_orphan(b);
    for (auto& b : c->bufs) cudaFree(b.p);
    cudaFree(c->st);
    cudaFree(c->trace);
    if (c->host_words) cudaFreeHost(c->host_words);
    // Blocks still held by orphaned graphs keep the pool alive until they are freed.
    if (c->pool) cudaMemPoolDestroy(c->pool);
    if (c->aux_stream) {
        cudaStreamSynchronize(c->aux_stream);
        cudaStreamDestroy(c->aux_stream);
    }
    cudaStreamDestroy(c->own_stream);
    delete c;
    return DPG_OK;
}

dpg_status dpg_ctx_set_stream(dpg_ctx* c, void* stream) {
    DPG_TRY(use_device(c));
    c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    return DPG_OK;
}

dpg_status dpg_ctx_synchronize(dpg_ctx* c) {
    DPG_TRY(use_device(c));
    return check_device(c);
}

dpg_status dpg_ctx_last_stats(dpg_ctx* c, dpg_run_stats* out) {
    DPG_TRY(use_device(c));
    if (!out) return set_error(DPG_ERR_INVALID_ARG, "null output");
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    DevStatus h;
    DPG_CUDA_TRY(cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
    out->iterations = c->last_host_iterations >= 0 ? c->last_host_iterations : static_cast<int64_t>(h.iterations);
    out->edges_scanned = static_cast<int64_t>(h.edges);
    out->vertices_popped = static_cast<int64_t>(h.pops);
    out->grid_blocks = c->last_grid;
    out->block_threads = c->last_block;
    return DPG_OK;
}

dpg_status dpg_ctx_profile_enable(dpg_ctx* c, int32_t enable) {
    DPG_TRY(use_device(c));
    c->prof.enabled = enable != 0;
    return DPG_OK;
}

dpg_status dpg_ctx_profile_reset(dpg_ctx* c) {
    DPG_TRY(use_device(c));
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->prof.reset();
    return DPG_OK;
}

dpg_status dpg_ctx_profile_read(dpg_ctx* c, int32_t kind, int64_t* launches, double* total_ms) {
    DPG_TRY(use_device(c));
    if (kind < 0 || kind >= DPG_KERNEL_KINDS) return set_error(DPG_ERR_INVALID_ARG, "unknown kernel kind");
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->prof.drain();
    if (launches) *launches = c->prof.launches[kind];
    if (total_ms) *total_ms = c->prof.ms[kind];
    return DPG_OK;
}

dpg_status dpg_ctx_trace_enable(dpg_ctx* c, int32_t max_iterations) {
    DPG_TRY(use_device(c));
    if (max_iterations < 0) return set_error(DPG_ERR_INVALID_ARG, "max_iterations must be >= 0");
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    cudaFree(c->trace);
    c->trace = nullptr;
    c->trace_cap = 0;
    if (max_iterations > 0) {
        DPG_CUDA_TRY(cudaMalloc(&c->trace, sizeof(unsigned long long) * 4 * (static_cast<size_t>(max_iterations) + 1)));
        c->trace_cap = max_iterations + 1;
    }
    return DPG_OK;
}

dpg_status dpg_ctx_trace_read(dpg_ctx* c, int64_t* out, int32_t capacity, int32_t* count) {
    DPG_TRY(use_device(c));
    if (!out || !count || capacity < 0) return set_error(DPG_ERR_INVALID_ARG, "null output");
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    const int32_t n = capacity < c->trace_cap ? capacity : c->trace_cap;
    if (n > 0) DPG_CUDA_TRY(cudaMemcpy(out, c->trace, sizeof(int64_t) * 4 * n, cudaMemcpyDeviceToHost));
    *count = n;
    return DPG_OK;
}

dpg_status dpg_ctx_sm_count(dpg_ctx* c, int32_t* out) {
    if (!c || !out) return set_error(DPG_ERR_INVALID_ARG, "null argument");
    *out = c->sm_count;
    return DPG_OK;
}

dpg_status dpg_graph_create(dpg_ctx* c, int32_t V, int64_t E, const int32_t* offsets, const int32_t* col,
                            const int32_t* weights, dpg_graph** out) {
    return graph_create_common(c, V, E, offsets, col, weights, false, out);
}

dpg_status dpg_graph_create_device(dpg_ctx* c, int32_t V, int64_t E, const int32_t* d_offsets, const int32_t* d_col,
                                   const int32_t* d_weights, dpg_graph** out) {
    return graph_create_common(c, V, E, d_offsets, d_col, d_weights, true, out);
}

dpg_status dpg_graph_destroy(dpg_graph* g) {
    if (!g) return DPG_OK;
    if (g->ctx) {
        cudaSetDevice(g->ctx->device);
        cudaStreamSynchronize(g->ctx->stream);
        g->ctx->graphs.erase(g);
    } else {
        cudaSetDevice(g->device);  // orphaned by dpg_ctx_destroy: only the memory is left to free
    }
    graph_free_device(g);
    delete g;
    return DPG_OK;
}

dpg_status dpg_graph_relabel(dpg_graph* g, int32_t enable) {
    if (!g) return set_error(DPG_ERR_INVALID_ARG, "null graph");
    g->relabel = enable != 0;
    return DPG_OK;
}

dpg_status dpg_graph_info(const dpg_graph* g, int32_t* V, int64_t* E, int32_t* weighted) {
    if (!g) return set_error(DPG_ERR_INVALID_ARG, "null graph");
    if (V) *V = g->V;
    if (E) *E = g->E;
    if (weighted) *weighted = g->weighted ? 1 : 0;
    return DPG_OK;
}

dpg_status dpg_graph_plan_info(dpg_graph* g, int32_t* tiles, int32_t* hubs_small, int32_t* hubs_big,
                               int32_t* segments) {
    if (!g || !g->ctx) return set_error(DPG_ERR_INVALID_ARG, "null graph or destroyed context");
    DPG_TRY(use_device(g->ctx));
    if (g->V > 0) DPG_TRY(ensure_plan(g));
    if (tiles) *tiles = g->plan.ntiles;
    if (hubs_small) *hubs_small = g->plan.nhub_small;
    if (hubs_big) *hubs_big = g->plan.nhub_big;
    if (segments) *segments = g->plan.nseg;
    return DPG_OK;
}

namespace {
__global__ void count_below_kernel(const int32_t* __restrict__ col, int64_t E, int32_t bound,
                                   unsigned long long* count) {
    unsigned long long c = 0;
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < E;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x)
        c += __ldg(col + e) < bound ? 1ull : 0ull;
    c = warp_sum_u64(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}
}  // namespace

dpg_status dpg_graph_hot_cache(dpg_graph* g, int32_t* hot_entries_out, int64_t* hot_arcs) {
    if (!g || !g->ctx) return set_error(DPG_ERR_INVALID_ARG, "null graph or destroyed context");
    dpg_ctx* c = g->ctx;
    DPG_TRY(use_device(c));
    const int32_t hot = hot_entries(c, g);
    if (hot_entries_out) *hot_entries_out = hot;
    if (!hot_arcs) return DPG_OK;
    *hot_arcs = 0;
    if (hot == 0 || g->E == 0) return DPG_OK;
    DPG_TRY(ensure_relabel(g));
    unsigned long long* d = nullptr;
    DPG_CUDA_TRY(cudaMalloc(&d, sizeof(unsigned long long)));
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(unsigned long long), c->stream);
    if (e == cudaSuccess) {
        count_below_kernel<<<c->sm_count * 4, 256, 0, c->stream>>>(g->pcol, g->E, hot, d);
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (e != cudaSuccess) return set_error(DPG_ERR_CUDA, std::string("hot-cache count: ") + cudaGetErrorString(e));
    *hot_arcs = static_cast<int64_t>(h);
    return DPG_OK;
}

dpg_status dpg_sssp_dev(dpg_ctx* c, const dpg_graph* g, int32_t source, const dpg_expand_opts* opts, int32_t* d_dist) {
    DPG_TRY(use_device(c));
    return run_expand(c, g, source, opts, d_dist, false);
}

dpg_status dpg_bfs_dev(dpg_ctx* c, const dpg_graph* g, int32_t source, const dpg_expand_opts* opts, int32_t* d_level) {
    DPG_TRY(use_device(c));
    return run_expand(c, g, source, opts, d_level, true);
}

static dpg_status expand_host(dpg_ctx* c, const dpg_graph* g, int32_t source, const dpg_expand_opts* opts,
                              int32_t* h_out, bool bfs) {
    DPG_TRY(use_device(c));
    if (!g) return set_error(DPG_ERR_INVALID_ARG, "null graph");
    if (!h_out && g->V > 0) return set_error(DPG_ERR_INVALID_ARG, "null output");
    dpg_status st = DPG_OK;
    int32_t* d = static_cast<int32_t*>(arena(c, S_LABEL, static_cast<size_t>(g->V) * 4, &st));
    if (!d) return st;
    DPG_TRY(run_expand(c, g, source, opts, d, bfs));
    DPG_CUDA_TRY(cudaMemcpyAsync(h_out, d, static_cast<size_t>(g->V) * 4, cudaMemcpyDeviceToHost, c->stream));
    return check_device(c);
}

dpg_status dpg_sssp(dpg_ctx* c, const dpg_graph* g, int32_t source, const dpg_expand_opts* opts, int32_t* h_dist) {
    return expand_host(c, g, source, opts, h_dist, false);
}

dpg_status dpg_bfs(dpg_ctx* c, const dpg_graph* g, int32_t source, const dpg_expand_opts* opts, int32_t* h_level) {
    return expand_host(c, g, source, opts, h_level, true);
}

dpg_status dpg_color_dev(dpg_ctx* c, const dpg_graph* g, const dpg_expand_opts* opts, int32_t* d_color) {
    DPG_TRY(use_device(c));
    return run_color(c, const_cast<dpg_graph*>(g), opts, d_color);
}

dpg_status dpg_color(dpg_ctx* c, const dpg_graph* g, const dpg_expand_opts* opts, int32_t* h_color) {
    DPG_TRY(use_device(c));
    if (!g) return set_error(DPG_ERR_INVALID_ARG, "null graph");
    if (g->V == 0) return DPG_OK;
    if (!h_color) return set_error(DPG_ERR_INVALID_ARG, "null output");
    dpg_status st = DPG_OK;
    int32_t* d = static_cast<int32_t*>(arena(c, S_LABEL, static_cast<size_t>(g->V) * 4, &st));
    if (!d) return st;
    DPG_TRY(run_color(c, const_cast<dpg_graph*>(g), opts, d));
    DPG_CUDA_TRY(cudaMemcpyAsync(h_color, d, static_cast<size_t>(g->V) * 4, cudaMemcpyDeviceToHost, c->stream));
    return check_device(c);
}

dpg_status dpg_spmm_f32_dev(dpg_ctx* c, const dpg_graph* gc, const float* d_vals, int32_t nrhs, const float* d_X,
                            float* d_Y) {
    DPG_TRY(use_device(c));
    dpg_graph* g = const_cast<dpg_graph*>(gc);
    if (!g || g->ctx != c) return set_error(DPG_ERR_INVALID_ARG, "graph does not belong to this context");
    DPG_TRY(check_nrhs(nrhs));
    if (g->V == 0) return DPG_OK;
    if (!d_X || !d_Y || (g->E > 0 && !d_vals)) return set_error(DPG_ERR_INVALID_ARG, "null vals/X/Y");
    DPG_TRY(ensure_spmm_plan(g));
    dpg_status st = DPG_OK;
    float* partial = static_cast<float*>(
        arena(c, S_SPMM_PARTIAL, static_cast<size_t>(g->spmm_plan.nseg + 1) * nrhs * 4, &st));
    if (st != DPG_OK) return st;
    c->last_host_iterations = 1;
    if (spmm_group_ok(nrhs, d_X, d_Y, partial, nullptr))
        DPG_CUDA_TRY(launch_spmm_group(g->spmm_plan, g->col, d_vals, d_X, nrhs, d_Y, partial, c->stream, c->sm_count,
                                       &c->prof));
    else
        DPG_CUDA_TRY(launch_spmm(g->spmm_plan, g->col, d_vals, d_X, nrhs, d_Y, partial, c->stream, c->sm_count,
                                 &c->prof));
    return DPG_OK;
}

dpg_status dpg_spmv_bwd_f32_dev(dpg_ctx* c, const dpg_graph* gc, const float* d_vals, int32_t nrhs, const float* d_X,
                                const float* d_G, float* d_dX, float* d_dA) {
    DPG_TRY(use_device(c));
    dpg_graph* g = const_cast<dpg_graph*>(gc);
    if (!g || g->ctx != c) return set_error(DPG_ERR_INVALID_ARG, "graph does not belong to this context");
    DPG_TRY(check_nrhs(nrhs));
    if (g->V == 0) return DPG_OK;
    if (!d_G || (d_dA && !d_X) || (g->E > 0 && !d_vals)) return set_error(DPG_ERR_INVALID_ARG, "null vals/X/G");
    c->last_host_iterations = 1;
    if (spmm_group_ok(nrhs, d_X, d_G, d_dX, nullptr) && (d_dX || d_dA)) {
        // Both outputs in one pass over the transposed CSR: each arc's row of G is gathered once.
        DPG_TRY(ensure_spmm_transpose(g));
        dpg_status st = DPG_OK;
        float* partial = static_cast<float*>(
            arena(c, S_SPMM_PARTIAL, static_cast<size_t>(g->spmm_t_plan.nseg + 1) * nrhs * 4, &st));
        if (st != DPG_OK) return st;
        if (!spmm_group_ok(nrhs, partial, nullptr, nullptr, nullptr))
            return set_error(DPG_ERR_CUDA, "misaligned workspace");
        DPG_CUDA_TRY(launch_spmv_bwd_group(g->spmm_t_plan, g->tt_col, g->tt_arc, d_vals, d_X, d_G, nrhs, d_dX, partial,
                                           d_dA, c->stream, c->sm_count, &c->prof));
        return DPG_OK;
    }
    if (d_dX) {
        DPG_TRY(ensure_spmm_transpose(g));
        dpg_status st = DPG_OK;
        float* vals_t = static_cast<float*>(arena(c, S_VALS_T, static_cast<size_t>(g->E > 0 ? g->E : 1) * 4, &st));
        float* partial = static_cast<float*>(
            arena(c, S_SPMM_PARTIAL, static_cast<size_t>(g->spmm_t_plan.nseg + 1) * nrhs * 4, &st));
        if (st != DPG_OK) return st;
        DPG_CUDA_TRY(launch_gather_values(d_vals, g->tt_arc, g->E, vals_t, c->stream, c->sm_count));
        DPG_CUDA_TRY(launch_spmm(g->spmm_t_plan, g->tt_col, vals_t, d_G, nrhs, d_dX, partial, c->stream, c->sm_count,
                                 &c->prof));
    }
    if (d_dA) {
        DPG_TRY(ensure_spmm_plan(g));
        DPG_CUDA_TRY(launch_arc_dot(g->spmm_plan, g->col, d_X, d_G, nrhs, d_dA, c->stream, c->sm_count, &c->prof));
    }
    return DPG_OK;
}

dpg_status dpg_pagerank_grad_f32_dev(dpg_ctx* c, const dpg_graph* g, const float* d_weights, const float* d_seed,
                                     const dpg_pr_opts* opts, double adjoint_epsilon, float* d_rank, float* d_grad) {
    DPG_TRY(use_device(c));
    return run_pagerank_grad(c, const_cast<dpg_graph*>(g), d_weights, d_seed, opts, adjoint_epsilon, d_rank, d_grad);
}

dpg_status dpg_ctx_grad_sweeps(const dpg_ctx* c, int64_t* forward, int64_t* adjoint) {
    if (!c) return set_error(DPG_ERR_INVALID_ARG, "null context");
    if (forward) *forward = c->last_grad_sweeps[0];
    if (adjoint) *adjoint = c->last_grad_sweeps[1];
    return DPG_OK;
}

dpg_status dpg_bfs_cdp_dev(dpg_ctx* c, const dpg_graph* g, int32_t source, int32_t variant, int32_t pending_limit,
                           int32_t* d_level, dpg_cdp_stats* stats) {
    DPG_TRY(use_device(c));
    if (!g || g->ctx != c) return set_error(DPG_ERR_INVALID_ARG, "graph does not belong to this context");
    if (source < 0 || source >= g->V || !d_level) return set_error(DPG_ERR_INVALID_ARG, "bad source or null output");
    if (variant < DPG_CDP_NAIVE || variant > DPG_CDP_GRID) return set_error(DPG_ERR_INVALID_ARG, "unknown variant");
    if (pending_limit < 0) return set_error(DPG_ERR_INVALID_ARG, "pending_limit must be >= 0");
    const size_t want = static_cast<size_t>(pending_limit > 0 ? pending_limit : 65536);
    size_t have = 0;
    DPG_CUDA_TRY(cudaDeviceGetLimit(&have, cudaLimitDevRuntimePendingLaunchCount));
    if (have != want) {
        DPG_CUDA_TRY(cudaDeviceSynchronize());
        DPG_CUDA_TRY(cudaDeviceSetLimit(cudaLimitDevRuntimePendingLaunchCount, want));
    }
    const size_t cap = cdp_buffer_entries(g->E, g->V);
    dpg_status st = DPG_OK;
    unsigned* b0 = static_cast<unsigned*>(arena(c, S_CDP_BUF0, cap * 4, &st));
    unsigned* b1 = static_cast<unsigned*>(arena(c, S_CDP_BUF1, cap * 4, &st));
    unsigned* words = static_cast<unsigned*>(arena(c, S_CDP_WORDS, 4 * 4 + sizeof(CdpCounters), &st));
    if (st != DPG_OK) return st;
    CdpCounters* ct = reinterpret_cast<CdpCounters*>(words + 4);
    c->last_host_iterations = -1;
    {
        HookScope hs(&c->prof, DPG_KERNEL_EXPAND, c->stream);
        DPG_CUDA_TRY(launch_bfs_cdp(variant, g->off, g->col, g->V, source, d_level, b0, b1, cap, words, ct, c->stream,
                                    c->sm_count));
    }
    CdpCounters h{};
    DPG_CUDA_TRY(cudaMemcpyAsync(&h, ct, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (stats) {
        stats->launches = static_cast<int64_t>(h.launches);
        stats->failed_launches = static_cast<int64_t>(h.failures);
        stats->buffer_entries = static_cast<int64_t>(cap);
    }
    if (h.failures)
        return set_error(DPG_ERR_CAPACITY, std::to_string(h.failures) +
                                               " child launches failed or were skipped (nesting depth, pending-launch "
                                               "limit or buffer); levels are incomplete");
    return DPG_OK;
}

dpg_status dpg_csr_transpose_dev(dpg_ctx* c, int32_t V, int64_t E, const int32_t* d_offsets, const int32_t* d_col,
                                 int32_t* d_in_offsets, int32_t* d_in_col, int32_t* d_in_arc) {
    DPG_TRY(use_device(c));
    if (V < 0 || E < 0 || E > INT32_MAX) return set_error(DPG_ERR_INVALID_ARG, "V must be >= 0 and 0 <= E < 2^31");
    if (!d_offsets || !d_in_offsets || (E > 0 && (!d_col || !d_in_col)))
        return set_error(DPG_ERR_INVALID_ARG, "null offsets or columns");
    dpg_status st = DPG_OK;
    int* bad = static_cast<int*>(arena(c, S_NONSTOP, sizeof(int) * 4, &st));
    if (st != DPG_OK) return st;
    DPG_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), c->stream));
    validate_offsets_kernel<<<c->sm_count * 4, 256, 0, c->stream>>>(d_offsets, V, E, bad);
    if (E > 0) validate_interleave_kernel<<<c->sm_count * 4, 256, 0, c->stream>>>(d_col, nullptr, nullptr, E, V, bad);
    DPG_CUDA_TRY(cudaGetLastError());
    int hbad = 0;
    DPG_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (hbad & 4) return set_error(DPG_ERR_INVALID_ARG, "offsets must rise from 0 to E");
    if (hbad & 1) return set_error(DPG_ERR_INVALID_ARG, "column index out of range");
    const size_t scratch_bytes = transpose_scratch_bytes(V, E);
    void* scratch = arena(c, S_TRANSPOSE, scratch_bytes, &st);
    int32_t* arc = d_in_arc ? d_in_arc
                            : static_cast<int32_t*>(arena(c, S_TRANSPOSE_ARC, static_cast<size_t>(E > 0 ? E : 1) * 4, &st));
    if (st != DPG_OK) return st;
    DPG_CUDA_TRY(launch_transpose(d_offsets, d_col, V, E, d_in_offsets, d_in_col, arc, scratch, scratch_bytes, c->stream,
                                  c->sm_count));
    return DPG_OK;
}

dpg_status dpg_spmv_f32_dev(dpg_ctx* c, const dpg_graph* g, const float* d_vals, const float* d_x, float* d_y) {
    DPG_TRY(use_device(c));
    return run_spmv(c, const_cast<dpg_graph*>(g), d_vals, d_x, d_y);
}

dpg_status dpg_spmv_f32(dpg_ctx* c, const dpg_graph* g, const float* h_vals, const float* h_x, float* h_y) {
    DPG_TRY(use_device(c));
    if (!g) return set_error(DPG_ERR_INVALID_ARG, "null graph");
    if (g->V == 0) return DPG_OK;
    if (!h_x || !h_y || (g->E > 0 && !h_vals)) return set_error(DPG_ERR_INVALID_ARG, "null vals/x/y");
    dpg_status st = DPG_OK;
    const size_t nv = static_cast<size_t>(g->V), ne = static_cast<size_t>(g->E > 0 ? g->E : 1);
    float* dv = static_cast<float*>(arena(c, S_VALS, ne * 4, &st));
    float* dx = static_cast<float*>(arena(c, S_X, nv * 4, &st));
    float* dy = static_cast<float*>(arena(c, S_Y, nv * 4, &st));
    if (st != DPG_OK) return st;
    if (g->E > 0) DPG_CUDA_TRY(cudaMemcpyAsync(dv, h_vals, static_cast<size_t>(g->E) * 4, cudaMemcpyHostToDevice, c->stream));
    DPG_CUDA_TRY(cudaMemcpyAsync(dx, h_x, nv * 4, cudaMemcpyHostToDevice, c->stream));
    DPG_TRY(run_spmv(c, const_cast<dpg_graph*>(g), dv, dx, dy));
    DPG_CUDA_TRY(cudaMemcpyAsync(h_y, dy, nv * 4, cudaMemcpyDeviceToHost, c->stream));
    return check_device(c);
}

dpg_status dpg_pagerank_f32_dev(dpg_ctx* c, const dpg_graph* g_in, const int32_t* d_outdeg, const dpg_pr_opts* opts,
                                float* d_rank) {
    DPG_TRY(use_device(c));
    return run_pagerank(c, const_cast<dpg_graph*>(g_in), d_outdeg, opts, d_rank);
}

dpg_status dpg_pagerank_f32(dpg_ctx* c, const dpg_graph* g_in, const int32_t* h_outdeg, const dpg_pr_opts* opts,
                            float* h_rank) {
    DPG_TRY(use_device(c));
    if (!g_in) return set_error(DPG_ERR_INVALID_ARG, "null graph");
    if (g_in->V == 0) return DPG_OK;
    if (!h_outdeg || !h_rank) return set_error(DPG_ERR_INVALID_ARG, "null outdeg or rank");
    dpg_status st = DPG_OK;
    const size_t nv = static_cast<size_t>(g_in->V);
    int32_t* dod = static_cast<int32_t*>(arena(c, S_OUTDEG, nv * 4, &st));
    float* dr = static_cast<float*>(arena(c, S_RANKOUT, nv * 4, &st));
    if (st != DPG_OK) return st;
    DPG_CUDA_TRY(cudaMemcpyAsync(dod, h_outdeg, nv * 4, cudaMemcpyHostToDevice, c->stream));
    DPG_TRY(run_pagerank(c, const_cast<dpg_graph*>(g_in), dod, opts, dr));
    DPG_CUDA_TRY(cudaMemcpyAsync(h_rank, dr, nv * 4, cudaMemcpyDeviceToHost, c->stream));
    return check_device(c);
}

dpg_status dpg_sssp_host(dpg_ctx* c, int32_t V, int64_t E, const int32_t* offsets, const int32_t* col,
                         const int32_t* weights, int32_t source, const dpg_expand_opts* opts, int32_t* h_dist) {
    if (!weights) return set_error(DPG_ERR_INVALID_ARG, "SSSP needs weights");
    dpg_graph* g = nullptr;
    DPG_TRY(dpg_graph_create(c, V, E, offsets, col, weights, &g));
    const dpg_status s = dpg_sssp(c, g, source, opts, h_dist);
    dpg_graph_destroy(g);
    return s;
}

dpg_status dpg_pagerank_f32_host(dpg_ctx* c, int32_t V, int64_t E, const int32_t* in_offsets, const int32_t* in_col,
                                 const int32_t* outdeg, const dpg_pr_opts* opts, float* h_rank) {
    dpg_graph* g = nullptr;
    DPG_TRY(use_device(c));
    if (V <= 0 || E <= 0 || E > INT32_MAX || !in_offsets || !in_col || !outdeg || !h_rank) {
        // Empty graphs and argument errors: the general path, which reports them.
        DPG_TRY(graph_create_common(c, V, E, in_offsets, in_col, nullptr, false, &g));
        const dpg_status s = dpg_pagerank_f32(c, g, outdeg, opts, h_rank);
        dpg_graph_destroy(g);
        return s;
    }
    dpg_status st = DPG_OK;
    const size_t nv = static_cast<size_t>(V);
    int32_t* dod = static_cast<int32_t*>(arena(c, S_OUTDEG, nv * 4, &st));
    float* dr = static_cast<float*>(arena(c, S_RANKOUT, nv * 4, &st));
    if (st != DPG_OK) return st;
    DPG_TRY(graph_create_pull(c, V, E, in_offsets, in_col, outdeg, dod, &g));
    dpg_status s = run_pagerank(c, g, dod, opts, dr);
    if (s == DPG_OK) {
        const cudaError_t e = cudaMemcpyAsync(h_rank, dr, nv * 4, cudaMemcpyDeviceToHost, c->stream);
        s = e == cudaSuccess ? check_device(c) : set_error(DPG_ERR_CUDA, cudaGetErrorString(e));
    }
    dpg_graph_destroy(g);
    return s;
}

dpg_status dpg_selftest_barrier_timeout(dpg_ctx* c, double timeout_seconds) {
    DPG_TRY(use_device(c));
    if (!(timeout_seconds > 0) || timeout_seconds > 30) return set_error(DPG_ERR_INVALID_ARG, "timeout must be in (0, 30] s");
    DPG_TRY(check_device(c));  // start from a clean status word
    DPG_CUDA_TRY(launch_barrier_timeout_test(c->st, static_cast<unsigned long long>(timeout_seconds * 1e9), c->stream));
    return check_device(c);
}

}  // extern "C"
