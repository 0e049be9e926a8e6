// Host-side internals of the C ABI shared by dpg_api.cu and dpg_batch.cu: the context (stream,
// status word, scratch arena, launch profiler), the device graph, and the helpers both use.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <unordered_set>
#include <vector>

#include "dpg_internal.h"
#include "dpg_kernels.h"

using namespace dpg;

#define DPG_CUDA_TRY(call)                                                                       \
    do {                                                                                         \
        cudaError_t _e = (call);                                                                 \
        if (_e != cudaSuccess)                                                                   \
            return set_error(DPG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

#define DPG_TRY(expr)                  \
    do {                               \
        dpg_status _s = (expr);        \
        if (_s != DPG_OK) return _s;   \
    } while (0)

namespace dpg_api {

enum Slot {
    S_QV0, S_QV1, S_QSE0, S_QSE1, S_BMP0, S_BMP1, S_CH0, S_CH1, S_QCOUNT, S_CCOUNT, S_LABEL, S_CONTRIB0, S_CONTRIB1, S_RANK0, S_RANK1,
    S_PARTIAL, S_DPART, S_DFIX, S_DSUM, S_NONSTOP, S_VALS, S_X, S_Y, S_OUTDEG, S_RANKOUT, S_XPERM, S_PENDING, S_SPMM_PARTIAL, S_VALS_T,
    S_PRG_W, S_PRG_Y, S_PRG_C, S_PRG_V0, S_PRG_V1, S_PRG_V2, S_PRG_V3, S_PRG_PART, S_PRG_RED, S_PRG_FLAGS,
    S_DIRTY0, S_DIRTY1,
    S_CDP_BUF0, S_CDP_BUF1, S_CDP_WORDS,
    S_TRANSPOSE, S_TRANSPOSE_ARC, S_DO_COUNT, S_FAR0, S_FAR1, S_FAR2, S_FAR_COUNT, S_PLANINFO,
    S_COUNT_SLOTS
};

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
};

// Counts every kernel launch by kind; when enabled, brackets each launch with a CUDA event pair on
// the launching stream so the device time of each kind can be summed afterwards.
struct Profiler : LaunchHook {
    bool enabled = false;
    int64_t launches[DPG_KERNEL_KINDS] = {};
    double ms[DPG_KERNEL_KINDS] = {};
    struct Pending {
        cudaEvent_t a, b;
        int kind;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t open = nullptr;

    cudaEvent_t take() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    void begin(int kind, cudaStream_t s) override {
        if (kind >= 0 && kind < DPG_KERNEL_KINDS) ++launches[kind];
        if (!enabled) return;
        open = take();
        cudaEventRecord(open, s);
    }
    void end(int kind, cudaStream_t s) override {
        if (!enabled || !open) return;
        cudaEvent_t b = take();
        cudaEventRecord(b, s);
        pending.push_back({open, b, kind});
        open = nullptr;
        if (pending.size() > 65536) drain();
    }
    // Accumulates finished pairs; synchronises on their end events.
    void drain() {
        for (auto& p : pending) {
            float t = 0.f;
            cudaEventSynchronize(p.b);
            if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess && p.kind >= 0 && p.kind < DPG_KERNEL_KINDS)
                ms[p.kind] += t;
            pool.push_back(p.a);
            pool.push_back(p.b);
        }
        pending.clear();
    }
    void reset() {
        drain();
        for (auto& x : launches) x = 0;
        for (auto& x : ms) x = 0.0;
    }
    ~Profiler() override {
        for (auto& p : pending) {
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

}  // namespace dpg_api

using namespace dpg_api;

struct dpg_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    int smem_optin = 0;  // max dynamic shared memory per CTA (bytes)
    DevStatus* st = nullptr;
    Buf bufs[S_COUNT_SLOTS];
    int last_grid = 0;
    int last_block = 0;
    int64_t last_grad_sweeps[2] = {0, 0};  // forward and adjoint sweeps of the last PageRank gradient
    int64_t last_host_iterations = -1;  // PageRank sweeps (host-counted); -1: read from the device
    Profiler prof;
    unsigned long long* trace = nullptr;  // per-iteration expansion trace (dpg_ctx_trace_enable)
    int32_t trace_cap = 0;
    // Graphs and batches created on this context. Destroying the context orphans them (their ctx
    // becomes null) so that destroying them afterwards frees their memory without touching it.
    std::unordered_set<dpg_graph*> graphs;
    std::unordered_set<dpg_batch*> batches;
    // Stream-ordered pool for graph-owned memory (CSR, plans, renaming, transposes). It keeps freed
    // blocks, so graphs created and destroyed per call (the one-shot entry points) reuse them.
    cudaMemPool_t pool = nullptr;
    // Second stream, created on first use: work that overlaps an upload on `stream` (event-ordered).
    cudaStream_t aux_stream = nullptr;
    unsigned* host_words = nullptr;  // pinned, 16 words (host_words())
};

struct dpg_graph {
    dpg_ctx* ctx = nullptr;  // null once the context was destroyed
    int device = 0;
    int32_t V = 0;
    int64_t E = 0;
    bool weighted = false;
    int32_t* off = nullptr;
    int32_t* col = nullptr;
    int2* adj = nullptr;
    std::vector<int32_t> h_off;
    int32_t max_degree = 0;
    double mean_weight = 0.0;  // weighted graphs: mean arc weight (the near-far step default)
    bool plan_ready = false;
    RowPlanDev plan;
    // Column renaming by frequency for the row gathers (dpg_layout.cu); built on first use.
    bool relabel = true;
    bool relabel_ready = false;
    int32_t* perm = nullptr;  // old column id -> new
    int32_t* inv = nullptr;   // new -> old
    int32_t* pcol = nullptr;  // col[e] renamed
    std::vector<int32_t> relabel_segments;  // optional vertex starts: rename within each segment
    // Transposed CSR (in-arcs), built on first use by colouring.
    int32_t* t_off = nullptr;
    int32_t* t_col = nullptr;
    // Batched-RHS plans: over the graph's rows, and over the transposed CSR in invertGraph order
    // (tt_*, with tt_arc[p] = the arc that transposed slot p came from), built on first use.
    bool spmm_ready = false;
    SpmmPlanDev spmm_plan;
    bool spmm_t_ready = false;
    SpmmPlanDev spmm_t_plan;
    int32_t* tt_col = nullptr;
    int32_t* tt_arc = nullptr;
    // The same transposed CSR as a graph of its own (row-gather plan, column renaming), for pull
    // sweeps over in-arcs with permuted arc values; built on first use by the weighted PageRank.
    dpg_graph* tgraph = nullptr;
};

namespace dpg_api {

dpg_status use_device(dpg_ctx* c);
// Graph-owned device memory: from the context's pool on its stream; freed stream-ordered, or
// synchronously when the context is gone (orphaned graphs).
cudaError_t dev_alloc(dpg_ctx* c, void** p, size_t bytes);
template <class T>
cudaError_t dev_alloc(dpg_ctx* c, T** p, size_t bytes) {
    return dev_alloc(c, reinterpret_cast<void**>(p), bytes);
}
void dev_free(dpg_ctx* c, void* p);
void* arena(dpg_ctx* c, Slot s, size_t bytes, dpg_status* status);
dpg_status host_words(dpg_ctx* c, unsigned** out);
dpg_status check_device(dpg_ctx* c);
dpg_status graph_create_common(dpg_ctx* c, int32_t V, int64_t E, const int32_t* offsets, const int32_t* col,
                               const int32_t* weights, bool device_ptrs, dpg_graph** out);
dpg_status graph_create_pull(dpg_ctx* c, int32_t V, int64_t E, const int32_t* in_offsets, const int32_t* in_col,
                             const int32_t* h_outdeg, int32_t* d_outdeg, dpg_graph** out);
dpg_status ensure_plan(dpg_graph* g);
// Device row-plan build: capacity buffers and the asynchronous build, then (with the totals read
// back) exact buffers, the lane starts and the release of the build buffers.
struct PlanInfo {
    int64_t totals[4];  // tiles, small hubs, big hubs, segments
    int bad;            // 1: column out of range, 4: bad offsets
    int pad[3];
};
struct PlanBuild {
    RowPlanCaps caps;
    int4* tiles = nullptr;
    int4* hubs_small = nullptr;
    int4* hubs_big = nullptr;
    void* scratch = nullptr;
};
cudaError_t plan_build_alloc(dpg_ctx* c, int32_t V, int64_t E, PlanBuild* pb);
cudaError_t plan_build_launch(const PlanBuild& pb, const int32_t* d_off, int32_t V, int64_t E, PlanInfo* d_info,
                              cudaStream_t s);
dpg_status plan_finish(dpg_graph* g, PlanBuild* pb, const PlanInfo& info);
void plan_build_free(dpg_ctx* c, PlanBuild* pb);
dpg_status ensure_relabel(dpg_graph* g);
int32_t hot_entries(const dpg_ctx* c, const dpg_graph* g);
dpg_status pr_defaults(const dpg_pr_opts* in, dpg_pr_opts* o);
void batch_orphan(dpg_batch* b);
dpg_status expand_workspace(dpg_ctx* c, int32_t V, int64_t E, int32_t min_chunked, ExpandWorkspace* wsp);
void fill_expand_defaults(const dpg_expand_opts* in, dpg_expand_opts* o, const dpg_graph* g);

}  // namespace dpg_api
