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

// Arcs per grid-wide chunk: every vertex at or above the chunking degree is cut into chunks of this
// many adjacency entries at push time, and the chunks are spread over every warp of the grid.
constexpr int kHubChunk = 256;

// Device buffers of one expansion. Index [p] is the frontier parity (iteration & 1).
struct ExpandWorkspace {
    int32_t* qv[2];        // small-degree frontier: vertex ids
    int2* qse[2];          // small-degree frontier: (row start, row end), so a pop needs no offsets lookup
    uint32_t* bmp[2];      // "already queued this iteration" bit per vertex (SSSP)
    int4* chunks[2];       // chunked frontier: {vertex, arc begin, arc end, 1 on a vertex's first chunk}
    uint32_t* qcount;      // [3] small-frontier lengths, rotated so resets never race with pushes
    uint32_t* ccount;      // [3] chunk counts, rotated the same way
    int64_t cap_v;
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
    unsigned long long* trace = nullptr;  // nullable: [trace_cap][4] {t_ns, small frontier, chunks, 2 if bottom-up}
    int32_t trace_cap = 0;
    // Direction-optimizing BFS only: in-arc CSR and the frontier statistics (3 + 3 counters).
    const int32_t* t_off = nullptr;
    const int32_t* t_col = nullptr;
    unsigned long long* do_mf = nullptr;
    unsigned* do_nf = nullptr;
    // Near-far SSSP only: three piles of far_cap {vertex, distance} pairs, 3 counts, 3 minima.
    int2* far[3] = {nullptr, nullptr, nullptr};
    unsigned* far_count = nullptr;
    int* far_min = nullptr;
    int64_t far_cap = 0;
    int32_t delta = 0;
    // A graph with hubs or more than 8 arcs per vertex: the binned and direction-optimizing kernels
    // run their build for more CTAs per SM (kWideBlocks in dpg_expand.cu).
    bool wide = false;
};

// Chunk capacity per parity for a graph of V vertices and E arcs when vertices of degree >=
// min_chunked_degree are chunked: sum of ceil(deg/256) over distinct vertices of one iteration.
int64_t expand_chunk_capacity(int32_t V, int64_t E, int32_t min_chunked_degree, int32_t chunk = kHubChunk);

cudaError_t launch_expand(const ExpandLaunch& L, const ExpandWorkspace& ws, DevStatus* st,
                          cudaStream_t stream, int sm_count, int* grid_out, int* block_out,
                          LaunchHook* hook);

// SSSP from nsrc <= 32 sources per graph at once over a union of graphs (label[v * nsrc + k]; the
// marks dirty[2][V] are scratch); sources[i] = v * nsrc + k. Binned policy, chunk in {128, 256, 512}.
struct MultiExpandLaunch {
    const int32_t* off;
    const int2* adj;
    int32_t V;
    int32_t nsrc;
    int32_t* label;
    unsigned long long* dirty[2];
    const int32_t* sources;
    int32_t nsources;
    int32_t hub_threshold;
    int32_t chunk;
    int32_t max_iter;
    unsigned long long timeout_ns;
    // Non-zero: the labels and marks were filled by an earlier launch of the same solve (another
    // group of graphs with other settings, over disjoint vertices); only the counters are reset.
    int32_t skip_fill;
};
cudaError_t launch_expand_multi(const MultiExpandLaunch& L, const ExpandWorkspace& ws, DevStatus* st,
                                cudaStream_t stream, int sm_count, int* grid_out, LaunchHook* hook);

// Greedy colouring over the transposed graph (L.off / L.col = in-CSR) with the persistent kernel;
// out_off/out_col is the graph itself, pending a V-int scratch array, L.label the colours.
cudaError_t launch_color(const ExpandLaunch& L, const int32_t* out_off, const int32_t* out_col, int32_t* pending,
                         const ExpandWorkspace& ws, DevStatus* st, cudaStream_t stream, int sm_count, int* grid_out,
                         int* block_out, LaunchHook* hook);

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
// The plan is built on the device (dpg_rowgather.cu) into buffers of the capacities below, which
// bound any valid CSR with V rows and E nonzeros; totals[0..3] receive the tile, small-hub, big-hub
// and segment counts, and bad offsets set *bad |= 4 (the plan is then unusable).
struct RowPlanCaps {
    int64_t tiles = 0;
    int64_t hubs = 0;  // per hub list
    size_t scratch_bytes = 0;
};
RowPlanCaps row_plan_caps(int32_t V, int64_t E);
cudaError_t launch_build_row_plan(const int32_t* off, int32_t V, int64_t E, const RowPlanCaps& caps, int4* tiles,
                                  int4* hubs_small, int4* hubs_big, void* scratch, int64_t* totals, int* bad,
                                  cudaStream_t s);

struct RowPlanDev {
    int4* tiles = nullptr;
    // [ntiles][32] per lane of a normal tile: merge-path start row (low byte) and the mask of its
    // merge items that are row ends (high byte, bit i = item 8*lane + i).
    uint16_t* lane_info = nullptr;
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
    int32_t hot;            // x[0, hot) is staged in shared memory (the most gathered renamed columns)
    float* y;               // SpMV y / PageRank contribution out
    float* partial;         // [plan.nseg] hub-segment partial sums
    int32_t V;
    // PageRank only
    const int32_t* outdeg;
    const int32_t* perm;    // nullable: contribution of row v goes to y[perm[v]] (renamed columns)
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
    // Batches of graphs (nullable): row v belongs to graph vgraph[v], whose uniform term this sweep
    // is gbase[g] and whose initial rank is ginit[g]. A dangling row then stores its rank in its
    // (never gathered) contribution slot, where the per-graph dangling reduction reads it.
    const int32_t* vgraph;
    const float* gbase;
    const float* ginit;
};

// ---- batched right-hand sides / SpMV adjoint (dpg_adjoint.cu) -----------------------------------
constexpr int kSpmmSegment = 512;  // nonzeros per item; longer rows are split and fixed up in order

// Items {row, arc begin, arc end, segment index or -1}; hubs {row, first segment, segments, 0}.
struct SpmmPlanHost {
    std::vector<int4> items;
    std::vector<int4> hubs;
    int32_t nseg = 0;
};
struct SpmmPlanDev {
    int4* items = nullptr;
    int32_t nitems = 0;
    int4* hubs = nullptr;
    int32_t nhubs = 0;
    int32_t nseg = 0;
};
void build_spmm_plan(const int32_t* off, int32_t V, SpmmPlanHost* plan);
// The group kernels (8 lanes per row piece, float4 loads) take nrhs a multiple of 32 (up to 128)
// and 16-byte aligned row blocks; spmm_group_ok says whether the given pointers qualify.
bool spmm_group_ok(int nrhs, const void* a, const void* b, const void* c, const void* d);
cudaError_t launch_spmm_group(const SpmmPlanDev& P, const int32_t* col, const float* val, const float* X, int nrhs,
                              float* Y, float* partial, cudaStream_t s, int sm_count, LaunchHook* hook);
// One pass over the transposed CSR (plan TP, columns tcol, arc permutation tarc): dX = A^T G and
// dA[e] = <G[row(e)], X[col(e)]>; either output may be null.
cudaError_t launch_spmv_bwd_group(const SpmmPlanDev& TP, const int32_t* tcol, const int32_t* tarc, const float* val,
                                  const float* X, const float* G, int nrhs, float* dX, float* partial, float* dA,
                                  cudaStream_t s, int sm_count, LaunchHook* hook);
// Y[row][:] = sum over the row's arcs of val[e] * X[col[e]][:] (row-major [*][nrhs], nrhs <= 128);
// partial holds nseg rows of nrhs.
cudaError_t launch_spmm(const SpmmPlanDev& P, const int32_t* col, const float* val, const float* X, int nrhs, float* Y,
                        float* partial, cudaStream_t s, int sm_count, LaunchHook* hook);
// dA[e] = <G[row(e)][:], X[col[e]][:]>.
cudaError_t launch_arc_dot(const SpmmPlanDev& P, const int32_t* col, const float* X, const float* G, int nrhs,
                           float* dA, cudaStream_t s, int sm_count, LaunchHook* hook);
// out[i] = v[idx[i]].
cudaError_t launch_gather_values(const float* v, const int32_t* idx, int64_t n, float* out, cudaStream_t s,
                                 int sm_count);

// ---- transposed CSR on the device in invertGraph order (dpg_transpose.cu) ------------------------
size_t transpose_scratch_bytes(int32_t V, int64_t E);
cudaError_t launch_transpose(const int32_t* off, const int32_t* col, int32_t V, int64_t E, int32_t* t_off,
                             int32_t* t_col, int32_t* t_arc, void* scratch, size_t scratch_bytes, cudaStream_t s,
                             int sm_count);

// ---- recursive BFS with device-side launches (dpg_cdp.cu, relocatable device code) --------------
struct CdpCounters {
    unsigned long long launches;  // child grids launched
    unsigned long long failures;  // launches that failed or were skipped (depth, buffer)
};
// Append-buffer entries the consolidated variants get for a graph of V vertices and E arcs.
size_t cdp_buffer_entries(int64_t E, int32_t V);
// Runs variant DPG_CDP_* from source; buffer and buffer2 hold cap entries each, words 4 unsigned.
cudaError_t launch_bfs_cdp(int variant, const int32_t* off, const int32_t* col, int32_t V, int32_t source,
                           int32_t* level, unsigned* buffer, unsigned* buffer2, size_t cap, unsigned* words,
                           CdpCounters* ct, cudaStream_t s, int sm_count);

// ---- weighted PageRank and its edge-weight gradient (dpg_prgrad.cu) ------------------------------

enum PrVecMode {
    PRV_FWD_INIT = 0,   // r = init_value; contrib = r / W; red_out = sum of r over dangling vertices
    PRV_FWD_SWEEP = 1,  // r = (base_const + red_scale * red_in) + damping * y; contrib, red_out as above
    PRV_ADJ_INIT = 2,   // lambda = seed; red_out = sum of lambda
    PRV_ADJ_SWEEP = 3,  // lambda = seed + (W > 0 ? damping * y / W : red_scale * red_in); red_out = sum
};

struct PrVecLaunch {
    int mode;
    int32_t V;
    const float* y;       // gathered sums of this sweep
    const float* W;       // out-weight sums
    const float* seed;    // dL/dr (adjoint)
    const float* prev;    // previous vector for the change test, or null
    float* out;           // new vector
    float* contrib;       // forward: out / W, 0 where W == 0
    const double* red_in; // reduction of the previous vector
    double* red_out;
    double* part;         // pr_vec_blocks(sm_count) partials
    unsigned* ticket;     // zero before the first launch; the last block resets it
    float damping;
    float init_value;
    double base_const;
    double red_scale;
    float epsilon;
    unsigned* nonstop;    // set to 1 when some |out - prev| > epsilon * |out| (null: no test)
};

int pr_vec_blocks(int sm_count);
cudaError_t launch_pr_vec(const PrVecLaunch& L, int sm_count, cudaStream_t s, LaunchHook* hook);
cudaError_t launch_pr_arc_grad(const SpmmPlanDev& P, const int32_t* col, const float* r, const float* W, const float* y,
                               const float* lam, float damping, float* grad, cudaStream_t s, int sm_count,
                               LaunchHook* hook);
cudaError_t launch_fill_f32(float* p, int64_t n, float v, cudaStream_t s, int sm_count);

// Column renaming by frequency (dpg_layout.cu).
cudaError_t launch_column_histogram(const int32_t* col, int64_t E, int32_t* counts, cudaStream_t s, int sm_count);
// out[e] = perm[col[e]] for e < E. With `bad`, columns are range-checked against V on the way
// (an out-of-range one sets *bad |= 1 and writes 0) for uploads whose columns were not yet checked.
cudaError_t launch_relabel_columns(const int32_t* col, const int32_t* perm, int64_t E, int32_t* out, cudaStream_t s,
                                   int sm_count, int32_t V = 0, int* bad = nullptr);
cudaError_t launch_gather_by_index(const float* x, const int32_t* inv, int32_t V, float* out, cudaStream_t s,
                                   int sm_count);
// Transposed CSR on the device: t_col[t_off[v] .. t_off[v+1]) lists the u with v in row u (order
// within a row unspecified); cursor is V ints of scratch holding t_off[0..V).
cudaError_t launch_transpose_scatter(const int32_t* off, const int32_t* col, int32_t V, int32_t* cursor,
                                     int32_t* t_col, cudaStream_t s, int sm_count);
// perm[old] = new, inv[new] = old; most frequent columns first (by bit length of the count), ties by id.
void frequency_order(const int32_t* counts, int32_t V, int32_t* perm, int32_t* inv);
// The same order computed on the device: scratch holds frequency_order_scratch_bytes(V).
size_t frequency_order_scratch_bytes(int32_t V);
cudaError_t launch_frequency_order(const int32_t* counts, int32_t V, int32_t* scratch, int32_t* perm, int32_t* inv,
                                   cudaStream_t s);

// Fills plan.lane_info from the tiles and the offsets (once per graph).
cudaError_t launch_tile_lane_starts(const RowPlanDev& plan, const int32_t* off, cudaStream_t s, int sm_count);
// The same over a plan whose tile count is on the device (*d_ntiles, at most cap), skipped when
// *bad has bit 4 (offsets failed their check).
cudaError_t launch_tile_lane_starts_dev(const int4* tiles, const int64_t* d_ntiles, int64_t cap, const int* bad,
                                        const int32_t* off, uint16_t* lane_info, cudaStream_t s, int sm_count);

// Grid shape used by the row-gather kernels (needed to size dpart/dfix).
void rowgather_grid(int sm_count, int* gather_blocks, int* fix_blocks, int* block_threads);
// Shared memory the gather kernel needs besides the hot-value cache.
size_t rowgather_staging_bytes();

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
