// Host-side launch interface between the C ABI layer (dpg_api.cu) and the kernel translation
// units (dpg_expand.cu, dpg_rowgather.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "dpg_device.cuh"

namespace dpg {

// Optional per-launch hook: the C ABI layer records CUDA events around each kernel when profiling.
struct LaunchHook {
    virtual void begin(int kind, cudaStream_t s) = 0;
    virtual void end(int kind, cudaStream_t s) = 0;
    virtual ~LaunchHook() = default;
};

struct HookScope {
    LaunchHook* h;
    int kind;
    cudaStream_t s;
    HookScope(LaunchHook* hook, int k, cudaStream_t st) : h(hook), kind(k), s(st) {
        if (h) h->begin(kind, s);
    }
    ~HookScope() {
        if (h) h->end(kind, s);
    }
};

// ---- frontier expansion (SSSP / BFS) ------------------------------------------------------------

// Edges per grid-wide hub chunk: hubs are split into chunks of this many adjacency entries and the
// chunks are spread over every warp of the persistent grid.
constexpr int kHubChunk = 256;

// Device buffers of one expansion. Index [p] is the frontier parity (iteration & 1).
struct ExpandWorkspace {
    int32_t* qv[2];        // frontier vertex ids
    int2* qse[2];          // frontier (row start, row end) so the pop needs no offsets lookup
    uint32_t* bmp[2];      // "already queued this iteration" bit per vertex (SSSP)
    int32_t* hv[2];        // hub vertices (degree >= hub threshold), grid-wide consolidation buffer
    int2* hse[2];          // hub (row start, row end)
    int32_t* hcpos[2];     // first chunk index of each hub in the iteration's chunk space
    int32_t* howner[2];    // chunk -> hub index
    uint32_t* qcount;      // [3] frontier lengths, rotated so resets never race with pushes
    unsigned long long* hcount;  // [3] packed (hub count << 32 | chunk count)
    int64_t cap_v;
    int64_t cap_hub;
    int64_t cap_chunks;
    int32_t bmp_words;
};

struct ExpandLaunch {
    const int32_t* off;
    const int32_t* col;   // unweighted adjacency (BFS)
    const int2* adj;      // interleaved (neighbour, weight) adjacency (SSSP)
    int32_t V;
    int64_t E;
    int32_t* label;       // distances or levels, written in place
    int32_t source;
    bool bfs;
    int32_t solution;
    int32_t threshold;
    int32_t hub_threshold;
    int32_t max_iter;
    unsigned long long timeout_ns;
};

// Bytes of every workspace buffer for a graph of V vertices and E arcs with the given minimum hub
// degree; used to size the context arena.
void expand_workspace_caps(int32_t V, int64_t E, int32_t min_hub_degree, int64_t* cap_hub,
                           int64_t* cap_chunks);

cudaError_t launch_expand(const ExpandLaunch& L, const ExpandWorkspace& ws, DevStatus* st,
                          cudaStream_t stream, int sm_count, int* grid_out, int* block_out,
                          LaunchHook* hook);

// Grid barrier with one CTA missing: its bounded waits must run out (failure-detection test).
cudaError_t launch_barrier_timeout_test(DevStatus* st, unsigned long long timeout_ns,
                                        cudaStream_t stream);

// ---- row gather (SpMV / PageRank pull) ----------------------------------------------------------

constexpr int kRowTileItems = 256;  // merge items (rows + nonzeros) per warp tile
constexpr int kHubRowDegree = 255;  // rows above this are split into hub segments
constexpr int kSmallHubSegs = 8;    // hubs with at most this many segments are fixed up per thread

// Tile {row, nrows, nnz_begin, nnz}: nrows > 0 covers whole rows [row, row+nrows) and exactly their
// nonzeros; nrows < 0 is segment -(nrows+1) of hub row `row`, nonzeros [nnz_begin, nnz_begin+nnz).
// Hub {row, first segment, segment count, 0}.
struct RowPlanHost {
    std::vector<int4> tiles;
    std::vector<int4> hubs_small;
    std::vector<int4> hubs_big;
    int32_t nseg = 0;
};

void build_row_plan(const int32_t* offsets, int32_t V, RowPlanHost* plan);

struct RowPlanDev {
    int4* tiles = nullptr;
    int32_t ntiles = 0;
    int4* hubs_small = nullptr;
    int32_t nhub_small = 0;
    int4* hubs_big = nullptr;
    int32_t nhub_big = 0;
    int32_t nseg = 0;
};

struct RowGatherLaunch {
    RowPlanDev plan;
    const int32_t* off;
    const int32_t* col;
    const float* vals;      // SpMV values; nullptr for PageRank
    const float* x;         // SpMV x / PageRank contribution in
    float* y;               // SpMV y / PageRank contribution out
    float* partial;         // [plan.nseg] hub-segment partial sums
    int32_t V;
    // PageRank only
    const int32_t* outdeg;
    float* rank_out;        // nullable: written when this sweep's ranks are needed
    const float* rank_prev; // nullable: convergence check against it
    float damping;
    double base_const;      // (1-d) * total / V
    double dangling_scale;  // d / V
    const double* dsum_in;  // dangling rank mass of the previous sweep
    double* dsum_out;
    double* dpart;          // [gather warps] dangling partials
    double* dfix;           // [fix-up warps] dangling partials
    float epsilon;
    unsigned* nonstop;      // nullable: set to 1 when some |new-old| > epsilon
};

// Grid shape used by the row-gather kernels (needed to size dpart/dfix).
void rowgather_grid(int sm_count, int* gather_blocks, int* fix_blocks, int* block_threads);

cudaError_t launch_spmv(const RowGatherLaunch& L, DevStatus* st, cudaStream_t stream, int sm_count,
                        LaunchHook* hook);
// One PageRank sweep: gather + hub fix-up + dangling reduction into dsum_out.
cudaError_t launch_pagerank_sweep(const RowGatherLaunch& L, DevStatus* st, cudaStream_t stream,
                                  int sm_count, LaunchHook* hook);
// contrib[v] = init / outdeg[v] (0 for dangling), rank_prev[v] = init (nullable), and the
// dangling mass of the initial vector into dsum_out.
cudaError_t launch_pagerank_init(const RowGatherLaunch& L, float init_rank, float* rank_prev,
                                 DevStatus* st, cudaStream_t stream, int sm_count, LaunchHook* hook);

}  // namespace dpg
