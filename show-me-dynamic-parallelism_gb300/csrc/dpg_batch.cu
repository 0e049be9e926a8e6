// Batches: many graphs of uneven size, many SSSP sources per graph and one PageRank per graph, run
// as one CUDA-graph launch.
//
// No counterpart in the reference, whose apps solve one graph from one source per process
// (sssp_wrapper.cu:241-298, pagerank_wrapper.cu:147-241). The graphs are packed into one union CSR:
// graph g owns vertices [vstart[g], vstart[g+1]) and its arcs keep inside that range.
//   SSSP       all sources of all graphs in one persistent multi-source expansion (MaskSsspOp,
//              dpg_expand.cu): a frontier vertex carries the mask of its sources whose distance
//              changed, so one scan of its arcs serves all of them, the frontier of an iteration
//              holds the work of every graph, and the launch takes as many iterations as the
//              deepest single search instead of their sum.
//   PageRank   one row-gather sweep over the union's in-CSR serves every graph; the uniform term
//              of each graph, (1-d) T / V_g + d D_g / V_g, comes from a per-graph dangling sum
//              reduced over fixed pieces of the graph-major dangling list in a fixed order.
//   CUDA graph both solves captured once (kernels and memsets only) and replayed per call.
//   Autotuner  picks the hub threshold and chunk size of the SSSP binning per graph: graphs fall into
//              size classes by arc count, each class's candidates are timed on one source per
//              graph of the class, and every graph takes its class's fastest. Graphs of one setting
//              form one multi-source launch; the launches of the groups run one after another
//              (labels filled once, by the first), and their graphs' vertices are disjoint. The
//              gather's shared-memory hot-cache size is timed for the batch as a whole: one sweep
//              serves every graph, and the hot cache is a per-launch resource.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "dpg_api_internal.h"

using namespace dpg_api;

namespace {

constexpr int kPiece = 4096;  // dangling entries per reduction piece
constexpr int kBlk = 256;

__global__ void gather_i32_kernel(const int32_t* __restrict__ src, const int32_t* __restrict__ idx, int64_t n,
                                  int32_t* __restrict__ out) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = __ldg(src + __ldg(idx + i));
}

// ginit[g] = initial rank of graph g's vertices.
__global__ void batch_pr_setup_kernel(const int32_t* __restrict__ vstart, int n, double total, int init_zero,
                                      float* __restrict__ ginit) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
        const int vg = vstart[g + 1] - vstart[g];
        ginit[g] = (init_zero || vg == 0) ? 0.0f : static_cast<float>(total / static_cast<double>(vg));
    }
}

// Per-graph dangling mass of the ranks parked in the contribution slots, then each graph's uniform
// term for the next sweep. Warp per piece (lanes stride the piece, fixed-order warp sum); the last
// block to finish adds each graph's piece partials in piece order.
__global__ void __launch_bounds__(kBlk) batch_dangling_kernel(const int4* __restrict__ pieces, int npieces,
                                                              const int32_t* __restrict__ dslot,
                                                              const float* __restrict__ y,
                                                              const int32_t* __restrict__ gpiece,
                                                              const int32_t* __restrict__ vstart, int n, double damping,
                                                              double total, double* gpart, float* gbase,
                                                              unsigned* ticket) {
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int p = w; p < npieces; p += nw) {
        const int4 P = __ldg(pieces + p);
        double acc = 0.0;
        for (int k = P.y + lane; k < P.z; k += 32) acc += static_cast<double>(__ldcg(y + __ldg(dslot + k)));
        acc = warp_sum_f64(acc);
        if (lane == 0) gpart[p] = acc;
    }
    __threadfence();
    __syncthreads();
    __shared__ bool s_last;
    if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int g = threadIdx.x; g < n; g += blockDim.x) {
        double D = 0.0;
        for (int p = gpiece[g]; p < gpiece[g + 1]; ++p) D += __ldcg(gpart + p);
        const double vg = static_cast<double>(vstart[g + 1] - vstart[g]);
        if (vg > 0) gbase[g] = static_cast<float>((1.0 - damping) * total / vg + (damping / vg) * D);
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

}  // namespace

struct dpg_batch {
    dpg_ctx* ctx = nullptr;  // null once the context was destroyed
    int device = 0;
    int32_t n = 0;
    int32_t V = 0;
    int64_t E = 0;
    std::vector<int32_t> h_vstart;
    int32_t* vstart = nullptr;
    dpg_graph* out = nullptr;  // union out-adjacency with weights (SSSP)
    dpg_graph* in = nullptr;   // union in-adjacency in invertGraph order per graph (PageRank)
    int32_t* outdeg = nullptr;
    int32_t* vgraph = nullptr;
    int32_t* dang = nullptr;   // vertices without out-arcs, ascending
    int32_t* dslot = nullptr;  // their contribution slots in `in`
    int64_t ndang = 0;
    bool dslot_ready = false;
    int4* pieces = nullptr;
    int32_t npieces = 0;
    int32_t* gpiece = nullptr;
    double* gpart = nullptr;
    float* gbase = nullptr;
    float* ginit = nullptr;
    unsigned* ticket = nullptr;
    // Sources as label indices v * nsrc + k, k = source number within its graph.
    std::vector<int32_t> h_src;
    int32_t nsrc = 0;
    int32_t* d_src = nullptr;
    int64_t src_version = 0;
    dpg_batch_tuning tune{32, 256, -1};
    // Per-graph SSSP binning (empty: every graph uses tune.hub_threshold and tune.chunk).
    std::vector<int32_t> g_hub, g_chunk;
    int64_t tuning_version = 0;
    // Graphs grouped by SSSP setting, each group with its sources as label indices; rebuilt when the
    // sources or the settings change.
    struct Group {
        int32_t hub;
        int32_t chunk;
        int32_t* d_src;
        int32_t nsources;
    };
    std::vector<Group> groups;
    int64_t groups_src_version = -1;
    int64_t groups_tuning_version = -1;
    // Captured solve: recorded on a private stream (the context stream may be the legacy default
    // stream, which cannot be captured) and launched on the context stream.
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<unsigned char> key;
    int64_t replay_launches = 0;
};

namespace {

void free_groups(dpg_batch* b) {
    for (auto& gr : b->groups) cudaFree(gr.d_src);
    b->groups.clear();
    b->groups_src_version = b->groups_tuning_version = -1;
}

void batch_free(dpg_batch* b) {
    free_groups(b);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    b->cap_stream = nullptr;
    if (b->out) dpg_graph_destroy(b->out);
    if (b->in) dpg_graph_destroy(b->in);
    b->out = b->in = nullptr;
    for (void* p : {static_cast<void*>(b->vstart), static_cast<void*>(b->outdeg), static_cast<void*>(b->vgraph),
                    static_cast<void*>(b->dang), static_cast<void*>(b->dslot), static_cast<void*>(b->pieces),
                    static_cast<void*>(b->gpiece), static_cast<void*>(b->gpart), static_cast<void*>(b->gbase),
                    static_cast<void*>(b->ginit), static_cast<void*>(b->ticket), static_cast<void*>(b->d_src)})
        cudaFree(p);
}

template <class T>
dpg_status upload(dpg_ctx* c, T** dst, const T* src, size_t count) {
    DPG_CUDA_TRY(cudaMalloc(dst, sizeof(T) * (count > 0 ? count : 1)));
    if (count > 0) DPG_CUDA_TRY(cudaMemcpyAsync(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice, c->stream));
    return DPG_OK;
}

// Slots of the dangling vertices in the renamed contribution vector (built with the PageRank plan).
dpg_status ensure_dslot(dpg_batch* b) {
    if (b->dslot_ready) return DPG_OK;
    dpg_ctx* c = b->ctx;
    DPG_TRY(ensure_plan(b->in));
    if (b->in->relabel) DPG_TRY(ensure_relabel(b->in));
    DPG_CUDA_TRY(cudaMalloc(&b->dslot, sizeof(int32_t) * (b->ndang > 0 ? b->ndang : 1)));
    if (b->ndang > 0) {
        if (b->in->relabel) {
            gather_i32_kernel<<<c->sm_count * 4, kBlk, 0, c->stream>>>(b->in->perm, b->dang, b->ndang, b->dslot);
            DPG_CUDA_TRY(cudaGetLastError());
        } else {
            DPG_CUDA_TRY(cudaMemcpyAsync(b->dslot, b->dang, sizeof(int32_t) * b->ndang, cudaMemcpyDeviceToDevice,
                                         c->stream));
        }
    }
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    b->dslot_ready = true;
    return DPG_OK;
}

// Everything the PageRank solve needs that allocates, done before any capture.
struct PrBuffers {
    float* contrib[2];
    float* partial;
    double* dpart;
    double* dfix;
    double* dsum;
};

dpg_status pr_buffers(dpg_batch* b, PrBuffers* pb) {
    dpg_ctx* c = b->ctx;
    DPG_TRY(ensure_dslot(b));
    int gb, fb, bt;
    rowgather_grid(c->sm_count, &gb, &fb, &bt);
    const size_t nv = static_cast<size_t>(b->V);
    dpg_status st = DPG_OK;
    pb->contrib[0] = static_cast<float*>(arena(c, S_CONTRIB0, nv * 4, &st));
    pb->contrib[1] = static_cast<float*>(arena(c, S_CONTRIB1, nv * 4, &st));
    pb->partial = static_cast<float*>(arena(c, S_PARTIAL, static_cast<size_t>(b->in->plan.nseg + 1) * 4, &st));
    pb->dpart = static_cast<double*>(arena(c, S_DPART, static_cast<size_t>(gb) * (bt / 32) * 8, &st));
    pb->dfix = static_cast<double*>(arena(c, S_DFIX, static_cast<size_t>(fb) * (256 / 32) * 8, &st));
    pb->dsum = static_cast<double*>(arena(c, S_DSUM, 2 * 8, &st));
    if (st == DPG_OK) DPG_CUDA_TRY(cudaMemsetAsync(pb->dsum, 0, 2 * 8, c->stream));
    return st;
}

int32_t pr_hot(const dpg_batch* b) {
    const int32_t cap = hot_entries(b->ctx, b->in);
    if (b->tune.pr_hot < 0) return cap;
    return std::min(cap, b->tune.pr_hot);
}

int64_t pr_launches(int32_t iterations) { return 1 + 2 + 1 + 3 * static_cast<int64_t>(iterations) - 1; }

// Fixed-sweep PageRank of every graph; kernels and memsets only, so it can be captured.
dpg_status run_batch_pagerank(dpg_batch* b, const PrBuffers& pb, const dpg_pr_opts& o, float* d_rank,
                              LaunchHook* hook) {
    dpg_ctx* c = b->ctx;
    dpg_graph* g = b->in;
    cudaStream_t s = c->stream;
    RowGatherLaunch L;
    memset(&L, 0, sizeof(L));
    L.plan = g->plan;
    L.off = g->off;
    L.col = g->relabel ? g->pcol : g->col;
    L.perm = g->relabel ? g->perm : nullptr;
    L.hot = pr_hot(b);
    L.partial = pb.partial;
    L.V = g->V;
    L.outdeg = b->outdeg;
    L.damping = static_cast<float>(o.damping);
    L.dpart = pb.dpart;
    L.dfix = pb.dfix;
    L.vgraph = b->vgraph;
    L.gbase = b->gbase;
    L.ginit = b->ginit;
    L.dsum_in = pb.dsum + 1;
    L.dsum_out = pb.dsum;
    const int dang_blocks = std::max(1, std::min(c->sm_count * 4, (b->npieces + 7) / 8));
    auto dangling = [&](const float* y) -> cudaError_t {
        HookScope hs(hook, DPG_KERNEL_FIXUP, s);
        batch_dangling_kernel<<<dang_blocks, kBlk, 0, s>>>(b->pieces, b->npieces, b->dslot, y, b->gpiece, b->vstart,
                                                           b->n, o.damping, o.total_rank, b->gpart, b->gbase,
                                                           b->ticket);
        return cudaGetLastError();
    };
    {
        HookScope hs(hook, DPG_KERNEL_INIT, s);
        batch_pr_setup_kernel<<<(b->n + kBlk - 1) / kBlk, kBlk, 0, s>>>(b->vstart, b->n, o.total_rank, o.init_zero,
                                                                         b->ginit);
    }
    DPG_CUDA_TRY(cudaGetLastError());
    L.y = pb.contrib[0];
    DPG_CUDA_TRY(launch_pagerank_init(L, 0.0f, o.iterations == 0 ? d_rank : nullptr, c->st, s, c->sm_count, hook));
    if (o.iterations > 0) DPG_CUDA_TRY(dangling(pb.contrib[0]));
    for (int32_t it = 0; it < o.iterations; ++it) {
        L.x = pb.contrib[it & 1];
        L.y = pb.contrib[(it + 1) & 1];
        L.rank_out = (it == o.iterations - 1) ? d_rank : nullptr;
        DPG_CUDA_TRY(launch_pagerank_sweep(L, c->st, s, c->sm_count, hook));
        if (it + 1 < o.iterations) DPG_CUDA_TRY(dangling(L.y));
    }
    return DPG_OK;
}

struct GroupLaunch {
    int32_t hub;
    int32_t chunk;
    const int32_t* d_src;  // label indices of the group's sources
    int32_t nsources;
};

struct SsspPlan {
    ExpandWorkspace ws;  // shared by the groups' launches, sized for the largest need
    std::vector<MultiExpandLaunch> L;
};

// Workspace and launches of the multi-source expansion, one launch per group; allocates, so it runs
// before capture. An explicit in->hub_threshold overrides every group's.
dpg_status sssp_plan(dpg_batch* b, int32_t nsrc, const std::vector<GroupLaunch>& groups, const dpg_expand_opts* in,
                     int32_t* d_dist, SsspPlan* sp) {
    dpg_ctx* c = b->ctx;
    dpg_expand_opts o;
    fill_expand_defaults(in, &o, b->out);
    if (nsrc < 1 || nsrc > 32) return set_error(DPG_ERR_INVALID_ARG, "1 to 32 sources per graph");
    if (static_cast<int64_t>(b->V) * nsrc > INT32_MAX - 64)
        return set_error(DPG_ERR_CAPACITY, "sources x vertices must stay below 2^31");
    auto hub_of = [&](const GroupLaunch& g) { return (in && in->hub_threshold > 0) ? in->hub_threshold : g.hub; };
    ExpandWorkspace& ws = sp->ws;
    memset(&ws, 0, sizeof(ws));
    ws.cap_v = static_cast<int64_t>(b->V) + 1;
    ws.cap_chunks = 1;
    for (const GroupLaunch& g : groups)
        ws.cap_chunks = std::max(ws.cap_chunks, expand_chunk_capacity(b->V, b->E, hub_of(g), g.chunk));
    ws.bmp_words = 1;
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
    unsigned long long* d0 = static_cast<unsigned long long*>(arena(c, S_DIRTY0, static_cast<size_t>(b->V) * 8, &st));
    unsigned long long* d1 = static_cast<unsigned long long*>(arena(c, S_DIRTY1, static_cast<size_t>(b->V) * 8, &st));
    if (st != DPG_OK) return st;
    sp->L.clear();
    for (size_t k = 0; k < groups.size(); ++k) {
        MultiExpandLaunch L;
        memset(&L, 0, sizeof(L));
        L.off = b->out->off;
        L.adj = b->out->adj;
        L.V = b->V;
        L.nsrc = nsrc;
        L.dirty[0] = d0;
        L.dirty[1] = d1;
        L.label = d_dist;
        L.sources = groups[k].d_src;
        L.nsources = groups[k].nsources;
        L.hub_threshold = hub_of(groups[k]);
        L.chunk = groups[k].chunk;
        L.max_iter = o.max_iterations;
        L.timeout_ns = static_cast<unsigned long long>(o.timeout_seconds * 1e9);
        L.skip_fill = k > 0 ? 1 : 0;  // the first launch fills every label and mark
        sp->L.push_back(L);
    }
    return DPG_OK;
}

dpg_status run_batch_sssp(dpg_batch* b, const SsspPlan& sp, LaunchHook* hook) {
    dpg_ctx* c = b->ctx;
    int grid = 0;
    for (const MultiExpandLaunch& L : sp.L)
        DPG_CUDA_TRY(launch_expand_multi(L, sp.ws, c->st, c->stream, c->sm_count, &grid, hook));
    c->last_grid = grid;
    c->last_block = 256;
    c->last_host_iterations = -1;
    return DPG_OK;
}

int32_t graph_hub(const dpg_batch* b, int32_t g) { return b->g_hub.empty() ? b->tune.hub_threshold : b->g_hub[g]; }
int32_t graph_chunk(const dpg_batch* b, int32_t g) { return b->g_chunk.empty() ? b->tune.chunk : b->g_chunk[g]; }

// The groups of graphs that share an SSSP setting, with their sources (after set_sources).
dpg_status ensure_groups(dpg_batch* b) {
    if (b->groups_src_version == b->src_version && b->groups_tuning_version == b->tuning_version) return DPG_OK;
    free_groups(b);
    std::vector<std::pair<std::pair<int32_t, int32_t>, std::vector<int32_t>>> sets;
    for (int32_t g = 0; g < b->n; ++g) {
        const std::pair<int32_t, int32_t> key(graph_hub(b, g), graph_chunk(b, g));
        auto it = std::find_if(sets.begin(), sets.end(), [&](const auto& x) { return x.first == key; });
        if (it == sets.end()) {
            sets.push_back({key, {}});
            it = sets.end() - 1;
        }
        for (int32_t k = 0; k < b->nsrc; ++k) it->second.push_back(b->h_src[static_cast<size_t>(g) * b->nsrc + k]);
    }
    std::sort(sets.begin(), sets.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
    for (const auto& set : sets) {
        dpg_batch::Group gr{set.first.first, set.first.second, nullptr, static_cast<int32_t>(set.second.size())};
        dpg_status st = upload(b->ctx, &gr.d_src, set.second.data(), set.second.size());
        if (st != DPG_OK) {
            free_groups(b);
            return st;
        }
        b->groups.push_back(gr);
    }
    DPG_CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
    b->groups_src_version = b->src_version;
    b->groups_tuning_version = b->tuning_version;
    return DPG_OK;
}

std::vector<GroupLaunch> group_launches(const dpg_batch* b) {
    std::vector<GroupLaunch> v;
    for (const auto& gr : b->groups) v.push_back({gr.hub, gr.chunk, gr.d_src, gr.nsources});
    return v;
}

// Sources of every graph as label indices (copy c = source number within its graph).
dpg_status set_sources(dpg_batch* b, int32_t nsrc, const int32_t* h_sources) {
    if (nsrc < 1 || nsrc > 32) return set_error(DPG_ERR_INVALID_ARG, "1 to 32 sources per graph");
    if (!h_sources) return set_error(DPG_ERR_INVALID_ARG, "null sources");
    if (static_cast<int64_t>(b->V) * nsrc > INT32_MAX - 64)
        return set_error(DPG_ERR_CAPACITY, "sources x vertices must stay below 2^31");
    std::vector<int32_t> x(static_cast<size_t>(b->n) * nsrc);
    for (int32_t g = 0; g < b->n; ++g) {
        const int32_t vg = b->h_vstart[g + 1] - b->h_vstart[g];
        for (int32_t k = 0; k < nsrc; ++k) {
            const int32_t s = h_sources[static_cast<size_t>(g) * nsrc + k];
            if (vg == 0) return set_error(DPG_ERR_INVALID_ARG, "graph " + std::to_string(g) + " has no vertices");
            if (s < 0 || s >= vg)
                return set_error(DPG_ERR_INVALID_ARG, "source " + std::to_string(s) + " out of range in graph " +
                                                          std::to_string(g));
            x[static_cast<size_t>(g) * nsrc + k] = (b->h_vstart[g] + s) * nsrc + k;
        }
    }
    if (nsrc == b->nsrc && x == b->h_src) return DPG_OK;
    dpg_ctx* c = b->ctx;
    cudaFree(b->d_src);
    b->d_src = nullptr;
    DPG_TRY(upload(c, &b->d_src, x.data(), x.size()));
    DPG_CUDA_TRY(cudaStreamSynchronize(c->stream));
    b->h_src.swap(x);
    b->nsrc = nsrc;
    ++b->src_version;
    return DPG_OK;
}

dpg_status check_batch(dpg_ctx* c, const dpg_batch* b) {
    if (!b || b->ctx != c) return set_error(DPG_ERR_INVALID_ARG, "batch does not belong to this context");
    return DPG_OK;
}

float time_ms(dpg_ctx* c, const std::function<dpg_status()>& fn, int reps, dpg_status* st) {
    cudaEvent_t a, z;
    cudaEventCreate(&a);
    cudaEventCreate(&z);
    float best = 1e30f;
    for (int r = 0; r < reps && *st == DPG_OK; ++r) {
        cudaEventRecord(a, c->stream);
        *st = fn();
        cudaEventRecord(z, c->stream);
        if (*st != DPG_OK) break;
        if (cudaEventSynchronize(z) != cudaSuccess) {
            *st = set_error(DPG_ERR_CUDA, "autotune timing failed");
            break;
        }
        *st = check_device(c);
        float t = 0.f;
        cudaEventElapsedTime(&t, a, z);
        best = std::min(best, t);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(z);
    return best;
}

}  // namespace

namespace dpg_api {
void batch_orphan(dpg_batch* b) { b->ctx = nullptr; }
}  // namespace dpg_api

extern "C" {

dpg_status dpg_batch_create(dpg_ctx* c, int32_t ngraphs, const int32_t* vstart, int64_t E, const int32_t* offsets,
                            const int32_t* col, const int32_t* weights, dpg_batch** out) {
    if (!out) return set_error(DPG_ERR_INVALID_ARG, "null output handle");
    *out = nullptr;
    DPG_TRY(use_device(c));
    if (ngraphs < 1 || !vstart || !offsets || (E > 0 && (!col || !weights)))
        return set_error(DPG_ERR_INVALID_ARG, "need >= 1 graph, vertex starts, offsets, columns and weights");
    if (vstart[0] != 0) return set_error(DPG_ERR_INVALID_ARG, "vstart[0] must be 0");
    for (int32_t g = 0; g < ngraphs; ++g)
        if (vstart[g + 1] < vstart[g]) return set_error(DPG_ERR_INVALID_ARG, "vstart decreases at graph " + std::to_string(g));
    const int32_t V = vstart[ngraphs];
    if (offsets[0] != 0 || static_cast<int64_t>(offsets[V]) != E)
        return set_error(DPG_ERR_INVALID_ARG, "offsets must start at 0 and end at E");
    // Arcs stay inside their graph (checked per graph, in parallel).
    int bad_graph = -1;
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t g = 0; g < ngraphs; ++g) {
        const int32_t lo = vstart[g], hi = vstart[g + 1];
        for (int32_t v = lo; v < hi; ++v) {
            bool bad = offsets[v + 1] < offsets[v];
            for (int32_t e = offsets[v]; !bad && e < offsets[v + 1]; ++e) bad = col[e] < lo || col[e] >= hi;
            if (bad) {
#pragma omp critical
                bad_graph = (bad_graph < 0 || g < bad_graph) ? g : bad_graph;
                break;
            }
        }
    }
    if (bad_graph >= 0)
        return set_error(DPG_ERR_INVALID_ARG, "graph " + std::to_string(bad_graph) +
                                                  " has an arc leaving its vertex range (or decreasing offsets)");
    dpg_batch* b = new dpg_batch();
    b->ctx = c;
    b->device = c->device;
    b->n = ngraphs;
    b->V = V;
    b->E = E;
    b->h_vstart.assign(vstart, vstart + ngraphs + 1);
    auto fail = [&](dpg_status s) {
        batch_free(b);
        delete b;
        return s;
    };
    dpg_status st = graph_create_common(c, V, E, offsets, col, weights, false, &b->out);
    if (st != DPG_OK) return fail(st);
    // In-adjacency per graph, in invertGraph order (sources ascending within each in-row).
    std::vector<int32_t> in_off(static_cast<size_t>(V) + 1), in_col(static_cast<size_t>(E > 0 ? E : 1));
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t g = 0; g < ngraphs; ++g) {
        // Graph g writes in_off[lo, hi) only; in_off[hi] is the next graph's start (or E).
        const int32_t lo = vstart[g], hi = vstart[g + 1];
        std::vector<int32_t> cur(static_cast<size_t>(hi - lo) + 1, 0);
        for (int64_t e = offsets[lo]; e < offsets[hi]; ++e) ++cur[col[e] - lo + 1];
        cur[0] = offsets[lo];
        for (int32_t k = 0; k < hi - lo; ++k) cur[k + 1] += cur[k];
        for (int32_t v = lo; v < hi; ++v) in_off[v] = cur[v - lo];
        for (int32_t u = lo; u < hi; ++u)
            for (int32_t e = offsets[u]; e < offsets[u + 1]; ++e) in_col[cur[col[e] - lo]++] = u;
    }
    in_off[V] = static_cast<int32_t>(E);
    st = graph_create_common(c, V, E, in_off.data(), in_col.data(), nullptr, false, &b->in);
    if (st != DPG_OK) return fail(st);
    b->in->relabel_segments.assign(vstart, vstart + ngraphs + 1);
    std::vector<int32_t>().swap(in_col);
    std::vector<int32_t> od(static_cast<size_t>(V > 0 ? V : 1)), vg(static_cast<size_t>(V > 0 ? V : 1));
    std::vector<int32_t> dang, gpiece(static_cast<size_t>(ngraphs) + 1, 0);
    std::vector<int4> pieces;
    for (int32_t g = 0; g < ngraphs; ++g) {
        gpiece[g] = static_cast<int32_t>(pieces.size());
        const int64_t d0 = static_cast<int64_t>(dang.size());
        for (int32_t v = vstart[g]; v < vstart[g + 1]; ++v) {
            od[v] = offsets[v + 1] - offsets[v];
            vg[v] = g;
            if (od[v] == 0) dang.push_back(v);
        }
        const int64_t d1 = static_cast<int64_t>(dang.size());
        for (int64_t k = d0; k < d1; k += kPiece)
            pieces.push_back(make_int4(g, static_cast<int32_t>(k), static_cast<int32_t>(std::min(d1, k + kPiece)), 0));
    }
    gpiece[ngraphs] = static_cast<int32_t>(pieces.size());
    b->ndang = static_cast<int64_t>(dang.size());
    b->npieces = static_cast<int32_t>(pieces.size());
    if ((st = upload(c, &b->vstart, vstart, static_cast<size_t>(ngraphs) + 1)) != DPG_OK) return fail(st);
    if ((st = upload(c, &b->outdeg, od.data(), static_cast<size_t>(V))) != DPG_OK) return fail(st);
    if ((st = upload(c, &b->vgraph, vg.data(), static_cast<size_t>(V))) != DPG_OK) return fail(st);
    if ((st = upload(c, &b->dang, dang.data(), dang.size())) != DPG_OK) return fail(st);
    if ((st = upload(c, &b->pieces, pieces.data(), pieces.size())) != DPG_OK) return fail(st);
    if ((st = upload(c, &b->gpiece, gpiece.data(), gpiece.size())) != DPG_OK) return fail(st);
    cudaError_t e = cudaMalloc(&b->gpart, sizeof(double) * (pieces.size() + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->gbase, sizeof(float) * ngraphs);
    if (e == cudaSuccess) e = cudaMalloc(&b->ginit, sizeof(float) * ngraphs);
    if (e == cudaSuccess) e = cudaMalloc(&b->ticket, sizeof(unsigned) * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->ticket, 0, sizeof(unsigned) * 4, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail(set_error(DPG_ERR_CUDA, std::string("batch buffers: ") + cudaGetErrorString(e)));
    c->batches.insert(b);
    *out = b;
    return DPG_OK;
}

dpg_status dpg_batch_destroy(dpg_batch* b) {
    if (!b) return DPG_OK;
    if (b->ctx) {
        cudaSetDevice(b->ctx->device);
        cudaStreamSynchronize(b->ctx->stream);
        b->ctx->batches.erase(b);
    } else {
        cudaSetDevice(b->device);  // orphaned by dpg_ctx_destroy: only the memory is left to free
    }
    batch_free(b);
    delete b;
    return DPG_OK;
}

dpg_status dpg_batch_info(const dpg_batch* b, int32_t* ngraphs, int32_t* V, int64_t* E) {
    if (!b) return set_error(DPG_ERR_INVALID_ARG, "null batch");
    if (ngraphs) *ngraphs = b->n;
    if (V) *V = b->V;
    if (E) *E = b->E;
    return DPG_OK;
}

dpg_status dpg_batch_set_tuning(dpg_batch* b, const dpg_batch_tuning* t) {
    if (!b || !t) return set_error(DPG_ERR_INVALID_ARG, "null batch or tuning");
    if (t->hub_threshold < 1) return set_error(DPG_ERR_INVALID_ARG, "hub_threshold must be >= 1");
    if (t->chunk != 128 && t->chunk != 256 && t->chunk != 512)
        return set_error(DPG_ERR_INVALID_ARG, "chunk must be 128, 256 or 512");
    b->tune = *t;
    b->g_hub.clear();  // the batch-wide setting applies to every graph again
    b->g_chunk.clear();
    ++b->tuning_version;
    return DPG_OK;
}

dpg_status dpg_batch_get_tuning(const dpg_batch* b, dpg_batch_tuning* t) {
    if (!b || !t) return set_error(DPG_ERR_INVALID_ARG, "null batch or tuning");
    *t = b->tune;
    return DPG_OK;
}

dpg_status dpg_batch_set_graph_tuning(dpg_batch* b, const int32_t* hub_threshold, const int32_t* chunk) {
    if (!b) return set_error(DPG_ERR_INVALID_ARG, "null batch");
    if (!hub_threshold && !chunk) {
        b->g_hub.clear();
        b->g_chunk.clear();
        ++b->tuning_version;
        return DPG_OK;
    }
    if (!hub_threshold || !chunk) return set_error(DPG_ERR_INVALID_ARG, "give both per-graph arrays, or neither");
    for (int32_t g = 0; g < b->n; ++g) {
        if (hub_threshold[g] < 1)
            return set_error(DPG_ERR_INVALID_ARG, "hub_threshold of graph " + std::to_string(g) + " must be >= 1");
        if (chunk[g] != 128 && chunk[g] != 256 && chunk[g] != 512)
            return set_error(DPG_ERR_INVALID_ARG, "chunk of graph " + std::to_string(g) + " must be 128, 256 or 512");
    }
    b->g_hub.assign(hub_threshold, hub_threshold + b->n);
    b->g_chunk.assign(chunk, chunk + b->n);
    ++b->tuning_version;
    return DPG_OK;
}

dpg_status dpg_batch_get_graph_tuning(const dpg_batch* b, int32_t* hub_threshold, int32_t* chunk) {
    if (!b || !hub_threshold || !chunk) return set_error(DPG_ERR_INVALID_ARG, "null batch or output");
    for (int32_t g = 0; g < b->n; ++g) {
        hub_threshold[g] = graph_hub(b, g);
        chunk[g] = graph_chunk(b, g);
    }
    return DPG_OK;
}

dpg_status dpg_batch_sssp_dev(dpg_ctx* c, dpg_batch* b, int32_t nsrc, const int32_t* h_sources,
                              const dpg_expand_opts* opts, int32_t* d_dist) {
    DPG_TRY(use_device(c));
    DPG_TRY(check_batch(c, b));
    if (!d_dist) return set_error(DPG_ERR_INVALID_ARG, "null output");
    DPG_TRY(set_sources(b, nsrc, h_sources));
    DPG_TRY(ensure_groups(b));
    SsspPlan sp;
    DPG_TRY(sssp_plan(b, nsrc, group_launches(b), opts, d_dist, &sp));
    return run_batch_sssp(b, sp, &c->prof);
}

dpg_status dpg_batch_pagerank_dev(dpg_ctx* c, dpg_batch* b, const dpg_pr_opts* opts, float* d_rank) {
    DPG_TRY(use_device(c));
    DPG_TRY(check_batch(c, b));
    if (!d_rank) return set_error(DPG_ERR_INVALID_ARG, "null output");
    dpg_pr_opts o;
    DPG_TRY(pr_defaults(opts, &o));
    if (o.epsilon > 0) return set_error(DPG_ERR_UNSUPPORTED, "batched PageRank runs a fixed number of sweeps");
    PrBuffers pb;
    DPG_TRY(pr_buffers(b, &pb));
    c->last_host_iterations = o.iterations;
    return run_batch_pagerank(b, pb, o, d_rank, &c->prof);
}

dpg_status dpg_batch_run(dpg_ctx* c, dpg_batch* b, int32_t nsrc, const int32_t* h_sources,
                         const dpg_expand_opts* sssp_opts, int32_t* d_dist, const dpg_pr_opts* pr_opts, float* d_rank) {
    DPG_TRY(use_device(c));
    DPG_TRY(check_batch(c, b));
    if (!d_dist || !d_rank) return set_error(DPG_ERR_INVALID_ARG, "null output");
    dpg_pr_opts o;
    DPG_TRY(pr_defaults(pr_opts, &o));
    if (o.epsilon > 0) return set_error(DPG_ERR_UNSUPPORTED, "batched PageRank runs a fixed number of sweeps");
    DPG_TRY(set_sources(b, nsrc, h_sources));
    // Everything that allocates or synchronises happens here, outside the capture.
    DPG_TRY(ensure_groups(b));
    SsspPlan sp;
    DPG_TRY(sssp_plan(b, nsrc, group_launches(b), sssp_opts, d_dist, &sp));
    PrBuffers pb;
    DPG_TRY(pr_buffers(b, &pb));
    // The captured graph is reused while the launch arguments are unchanged.
    std::vector<unsigned char> key;
    auto put = [&key](const void* p, size_t n) {
        const unsigned char* q = static_cast<const unsigned char*>(p);
        key.insert(key.end(), q, q + n);
    };
    for (const MultiExpandLaunch& L : sp.L) put(&L, sizeof(L));
    put(&sp.ws, sizeof(sp.ws));
    put(&pb, sizeof(pb));
    put(&o, sizeof(o));
    put(&d_rank, sizeof(d_rank));
    put(&b->tune, sizeof(b->tune));
    put(&b->src_version, sizeof(b->src_version));
    if (!b->exec || key != b->key) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        if (!b->cap_stream) DPG_CUDA_TRY(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
        const cudaStream_t user_stream = c->stream;
        DPG_CUDA_TRY(cudaStreamSynchronize(user_stream));
        DPG_CUDA_TRY(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeRelaxed));
        c->stream = b->cap_stream;  // the solves launch on c->stream
        dpg_status s1 = run_batch_sssp(b, sp, nullptr);
        dpg_status s2 = s1 == DPG_OK ? run_batch_pagerank(b, pb, o, d_rank, nullptr) : s1;
        c->stream = user_stream;
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(b->cap_stream, &graph);
        if (s2 != DPG_OK) {
            if (graph) cudaGraphDestroy(graph);
            return s2;
        }
        if (ec != cudaSuccess) return set_error(DPG_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(ec));
        const cudaError_t ei = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            b->exec = nullptr;
            return set_error(DPG_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(ei));
        }
        b->key.swap(key);
        b->replay_launches = 3 * static_cast<int64_t>(sp.L.size()) + pr_launches(o.iterations);
    }
    DPG_CUDA_TRY(cudaGraphLaunch(b->exec, c->stream));
    c->last_host_iterations = -1;
    return DPG_OK;
}

dpg_status dpg_batch_launches(const dpg_batch* b, int64_t* kernels_per_run) {
    if (!b || !kernels_per_run) return set_error(DPG_ERR_INVALID_ARG, "null batch or output");
    *kernels_per_run = b->replay_launches;
    return DPG_OK;
}

dpg_status dpg_batch_autotune(dpg_ctx* c, dpg_batch* b, int32_t nsrc, const int32_t* h_sources,
                              dpg_batch_tuning* chosen) {
    DPG_TRY(use_device(c));
    DPG_TRY(check_batch(c, b));
    DPG_TRY(set_sources(b, nsrc, h_sources));
    // SSSP binning per graph. Graphs fall into size classes by arc count (below 2^17, below 2^21,
    // the rest); each class's candidates are timed on the first source of each of its graphs alone
    // (one launch, best of two after a warm-up), and every graph of the class takes the fastest.
    int32_t* dist = nullptr;
    DPG_CUDA_TRY(cudaMalloc(&dist, sizeof(int32_t) * (b->V > 0 ? b->V : 1)));
    const dpg_batch_tuning saved = b->tune;
    dpg_batch_tuning best = saved;
    std::vector<int32_t> hub(static_cast<size_t>(b->n), saved.hub_threshold), chunk(static_cast<size_t>(b->n), saved.chunk);
    const std::vector<int32_t>& h_off = b->out->h_off;
    auto arcs_of = [&](int32_t g) {
        return static_cast<int64_t>(h_off[b->h_vstart[g + 1]]) - h_off[b->h_vstart[g]];
    };
    auto class_of = [&](int32_t g) { return arcs_of(g) < (1 << 17) ? 0 : arcs_of(g) < (1 << 21) ? 1 : 2; };
    int64_t class_arcs[3] = {0, 0, 0};
    dpg_status st = DPG_OK;
    for (int cls = 0; cls < 3 && st == DPG_OK; ++cls) {
        std::vector<int32_t> first;
        for (int32_t g = 0; g < b->n; ++g)
            if (class_of(g) == cls) {
                first.push_back(b->h_src[static_cast<size_t>(g) * nsrc] / nsrc);  // label index of nsrc = 1
                class_arcs[cls] += arcs_of(g);
            }
        if (first.empty()) continue;
        int32_t* d_first = nullptr;
        st = upload(c, &d_first, first.data(), first.size());
        float best_ms = 1e30f;
        int32_t best_hub = saved.hub_threshold, best_chunk = saved.chunk;
        for (int32_t h : {16, 32, 64, 128}) {
            for (int32_t ch : {128, 256, 512}) {
                if (st != DPG_OK) break;
                SsspPlan sp;
                st = sssp_plan(b, 1, {{h, ch, d_first, static_cast<int32_t>(first.size())}}, nullptr, dist, &sp);
                if (st == DPG_OK) {
                    run_batch_sssp(b, sp, nullptr);  // warm-up
                    st = check_device(c);
                }
                const float t = st == DPG_OK ? time_ms(c, [&] { return run_batch_sssp(b, sp, nullptr); }, 2, &st) : 1e30f;
                if (st == DPG_OK && t < best_ms) {
                    best_ms = t;
                    best_hub = h;
                    best_chunk = ch;
                }
            }
        }
        cudaStreamSynchronize(c->stream);
        cudaFree(d_first);
        for (int32_t g = 0; g < b->n; ++g)
            if (class_of(g) == cls) {
                hub[g] = best_hub;
                chunk[g] = best_chunk;
            }
    }
    cudaFree(dist);
    if (st != DPG_OK) {
        b->tune = saved;
        return st;
    }
    // The batch-wide summary is the setting of the class holding the most arcs.
    const int big = static_cast<int>(std::max_element(class_arcs, class_arcs + 3) - class_arcs);
    for (int32_t g = 0; g < b->n; ++g)
        if (class_of(g) == big) {
            best.hub_threshold = hub[g];
            best.chunk = chunk[g];
            break;
        }
    // Gather hot-cache size: three sweeps per candidate.
    PrBuffers pb;
    st = pr_buffers(b, &pb);
    float* rank = nullptr;
    if (st == DPG_OK && cudaMalloc(&rank, sizeof(float) * (b->V > 0 ? b->V : 1)) != cudaSuccess)
        st = set_error(DPG_ERR_CAPACITY, "autotune rank buffer");
    dpg_pr_opts o;
    pr_defaults(nullptr, &o);
    o.iterations = 3;
    float best_pr = 1e30f;
    const int32_t cap = hot_entries(c, b->in);
    for (int32_t hot : {0, 4096, 16384, -1}) {
        if (st != DPG_OK) break;
        if (hot > cap) continue;
        b->tune.pr_hot = hot;
        run_batch_pagerank(b, pb, o, rank, nullptr);
        st = check_device(c);
        const float t = st == DPG_OK ? time_ms(c, [&] { return run_batch_pagerank(b, pb, o, rank, nullptr); }, 2, &st)
                                     : 1e30f;
        if (st == DPG_OK && t < best_pr) {
            best_pr = t;
            best.pr_hot = hot;
        }
    }
    cudaFree(rank);
    if (st != DPG_OK) {
        b->tune = saved;
        return st;
    }
    b->tune = best;
    b->g_hub.swap(hub);
    b->g_chunk.swap(chunk);
    ++b->tuning_version;
    if (chosen) *chosen = best;
    return DPG_OK;
}

}  // extern "C"
