/*
 * dpg.h — C ABI of the GB300-native irregular CSR neighbour-expansion library.
 *
 * The reference (show-me-dynamic-parallelism) has no plugin or FFI API: each app's main() calls a
 * zero-argument wrapper that talks through globals:
 *     void SSSP_GPU();        apps/sssp/src/sssp.h:32
 *     void SpMV_GPU();        apps/SpMV/src/SpMV.h:38
 *     void PAGERANK_GPU();    apps/pagerank/src/pagerank.h:36
 *     void BFS_REC_GPU();     apps/bfs-rec/src/bfs_rec.h:34
 *     void GRAPH_COLOR_GPU(); apps/graph-color/src/graph_color.h:24
 * Their inputs are the globals of common/global.h:28-58 (graph.vertexArray, graph.edgeArray,
 * graph.weightArray, graph.childVertexArray, graph.rEdgeArray, graph.outdegreeArray, noNodeTotal,
 * noEdgeTotal, source, config.solution, config.device_num). Their outputs are written in place into
 * graph.costArray / y / graph.rankArray / graph.levelArray / graph.colorArray.
 *
 * Every entry point below replaces one of those calls (or one phase of it) with explicit pointers
 * and sizes. The conventions are:
 *   - every function returns dpg_status and never calls exit();
 *   - host-pointer entry points ("e2e" calls) copy inputs to the GPU, run, and copy results back,
 *     synchronously, like the reference wrappers;
 *   - *_dev entry points take device pointers and are stream-ordered on the context's stream;
 *     errors raised inside a kernel (timeout, capacity) are reported by dpg_ctx_synchronize();
 *   - one context per host thread.
 */
#ifndef DPG_H
#define DPG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DPG_VERSION 1

/* Unreachable SSSP distance: INF in apps/sssp/src/sssp_wrapper.cu:5 and common/global.h:19. */
#define DPG_INF_COST 1073741824
/* Unreached BFS level: UNDEFINED in apps/bfs-rec/src/bfs_rec.h:13. */
#define DPG_UNDEFINED_LEVEL 0x7FFFFFFF
/* Degree threshold of the reference's consolidation kernels (THRESHOLD, sssp_kernel.cu:7). */
#define DPG_REF_THRESHOLD 64

typedef enum dpg_status {
    DPG_OK = 0,
    DPG_ERR_INVALID_ARG = 1, /* bad pointer, size, vertex id or option */
    DPG_ERR_CAPACITY = 2,    /* a worklist or buffer would overflow, or the iteration cap was hit */
    DPG_ERR_TIMEOUT = 3,     /* a bounded device-side wait (grid barrier) ran out */
    DPG_ERR_CUDA = 4,        /* a CUDA runtime call failed; see dpg_last_error() */
    DPG_ERR_NO_DEVICE = 5,   /* no usable CUDA device */
    DPG_ERR_IO = 6,          /* file could not be opened / read / written */
    DPG_ERR_FORMAT = 7,      /* malformed graph file */
    DPG_ERR_UNSUPPORTED = 8  /* option combination not implemented */
} dpg_status;

/* Work-mapping strategy for the frontier expansion (the reference's -s/--solution flag).
 * 0-4 keep the meaning of apps/sssp/src/sssp.cpp:65-70; 5 is the GB300 default. */
typedef enum dpg_solution {
    DPG_SOL_THREAD = 0, /* thread per frontier vertex, serial neighbour loop (unorder_threadQueue_kernel) */
    DPG_SOL_NAIVE = 1,  /* degree >= threshold: one warp per vertex, launched per vertex (naive DP) */
    DPG_SOL_WARP = 2,   /* degree >= threshold: consolidated per warp, expanded by the warp */
    DPG_SOL_BLOCK = 3,  /* degree >= threshold: consolidated per CTA in shared memory, expanded by the CTA */
    DPG_SOL_GRID = 4,   /* degree >= threshold: consolidated grid-wide, expanded by every CTA */
    DPG_SOL_BINNED = 5, /* warp scan-gather below hub_threshold, grid-wide edge chunks above */
    DPG_SOL_DIROPT = 6, /* BFS: binned top-down steps, bottom-up steps over in-arcs while the frontier
                           is large (direction-optimizing); SSSP runs DPG_SOL_NEARFAR on graphs without
                           vertices of degree >= hub_threshold and E <= 8V, else DPG_SOL_BINNED */
    DPG_SOL_NEARFAR = 7 /* SSSP: binned steps over the vertices below a distance threshold, the rest
                           deferred to a far pile (near-far); BFS runs DPG_SOL_DIROPT */
} dpg_solution;

typedef struct dpg_ctx dpg_ctx;
typedef struct dpg_graph dpg_graph;

typedef struct dpg_expand_opts {
    int32_t solution;        /* dpg_solution; DPG_SOL_DIROPT when the struct pointer is NULL */
    int32_t threshold;       /* consolidation degree threshold; 0 -> DPG_REF_THRESHOLD */
    int32_t hub_threshold;   /* BINNED: degree at which a vertex is expanded grid-wide; 0 -> auto */
    int32_t max_iterations;  /* 0 -> V + 2 (label-correcting never needs more) */
    double timeout_seconds;  /* limit of each grid-barrier wait; 0 -> 10 s */
    int32_t delta;           /* NEARFAR: threshold step; 0 -> 32 x the mean arc weight */
} dpg_expand_opts;

typedef struct dpg_pr_opts {
    double damping;          /* 0.85 (workload) ; 0.5 in the reference (pagerank_wrapper.cu:7) */
    double total_rank;       /* 1.0 (workload) ; 1000 in the reference (pagerank.h:15) */
    int32_t init_zero;       /* 1: start from rank 0 (pagerank_wrapper.cu:115); 0: total/V */
    int32_t iterations;      /* fixed iteration count when epsilon <= 0 ; cap otherwise */
    double epsilon;          /* > 0: iterate until every |new-old| <= epsilon (wrapper.cu:8, kernel.cu:72-81) */
} dpg_pr_opts;

typedef struct dpg_run_stats {
    int64_t iterations;      /* frontier iterations (SSSP/BFS) or PageRank sweeps */
    int64_t edges_scanned;   /* adjacency entries read by the expansion (>= E for label-correcting) */
    int64_t vertices_popped; /* frontier entries processed */
    int32_t grid_blocks;     /* CTAs of the persistent launch */
    int32_t block_threads;
} dpg_run_stats;

/* ---- errors / version ------------------------------------------------------------------------ */
const char* dpg_status_string(dpg_status s);
const char* dpg_last_error(void); /* thread-local detail of the last failing call */
int dpg_version(void);

/* ---- context (replaces prepare_gpu's cudaSetDevice, e.g. sssp_wrapper.cu:54-68) --------------- */
dpg_status dpg_ctx_create(int device, dpg_ctx** out);
dpg_status dpg_ctx_destroy(dpg_ctx* ctx);
/* Use an existing cudaStream_t (passed as void*) for every later call; NULL restores the own stream. */
dpg_status dpg_ctx_set_stream(dpg_ctx* ctx, void* cuda_stream);
/* Waits for the context's stream and returns the first device-side error raised since the last call. */
dpg_status dpg_ctx_synchronize(dpg_ctx* ctx);
/* Statistics of the last SSSP/BFS/PageRank call (synchronises). */
dpg_status dpg_ctx_last_stats(dpg_ctx* ctx, dpg_run_stats* out);
dpg_status dpg_ctx_sm_count(dpg_ctx* ctx, int32_t* out);

/* ---- device graphs (replaces the cudaMalloc + H2D half of prepare_gpu, sssp_wrapper.cu:94-111) -- */
/* Copies a host CSR (offsets[V+1], col[E], optional weights[E]) into the device layout. */
dpg_status dpg_graph_create(dpg_ctx* ctx, int32_t V, int64_t E, const int32_t* offsets,
                            const int32_t* col, const int32_t* weights, dpg_graph** out);
/* Same from device pointers (copied device-to-device into the library layout). */
dpg_status dpg_graph_create_device(dpg_ctx* ctx, int32_t V, int64_t E, const int32_t* d_offsets,
                                   const int32_t* d_col, const int32_t* d_weights, dpg_graph** out);
dpg_status dpg_graph_destroy(dpg_graph* g);
/* Gather-locality layout for SpMV / PageRank (on by default): column ids are renamed once, by
 * descending frequency, so hot gathered values share cache sectors. Rows and the order of nonzeros in
 * each row are unchanged, so results are bit-identical either way; enable = 0 turns it off. No
 * counterpart in the reference. */
dpg_status dpg_graph_relabel(dpg_graph* g, int32_t enable);
dpg_status dpg_graph_info(const dpg_graph* g, int32_t* V, int64_t* E, int32_t* weighted);
/* Row-gather plan of the graph (built on first use, on the device): warp tiles (normal tiles plus
 * hub segments), hub rows fixed up per thread (<= 8 segments) and per warp, and hub segments.
 * No counterpart in the reference. */
dpg_status dpg_graph_plan_info(dpg_graph* g, int32_t* tiles, int32_t* hubs_small, int32_t* hubs_big,
                               int32_t* segments);
/* Shared-memory hot cache of the row gathers (no counterpart in the reference): the number of
 * renamed columns each CTA keeps in shared memory, and how many of the graph's arcs gather from
 * them (builds the column renaming when needed; synchronises). The other arcs' gathers are the
 * random reads that dpg_calibrate_random_reads bounds. */
dpg_status dpg_graph_hot_cache(dpg_graph* g, int32_t* hot_entries, int64_t* hot_arcs);

/* ---- SSSP (replaces SSSP_GPU, apps/sssp/src/sssp_wrapper.cu:304-341) --------------------------- */
/* dist[v] = shortest distance from source, DPG_INF_COST when unreachable. Weights must be >= 0. */
dpg_status dpg_sssp(dpg_ctx* ctx, const dpg_graph* g, int32_t source, const dpg_expand_opts* opts,
                    int32_t* h_dist);
dpg_status dpg_sssp_dev(dpg_ctx* ctx, const dpg_graph* g, int32_t source,
                        const dpg_expand_opts* opts, int32_t* d_dist);

/* ---- BFS (replaces BFS_REC_GPU, apps/bfs-rec/src/bfs_rec_wrapper.cu:240-280) ------------------- */
/* level[v] = hop count from source, DPG_UNDEFINED_LEVEL when unreachable. */
dpg_status dpg_bfs(dpg_ctx* ctx, const dpg_graph* g, int32_t source, const dpg_expand_opts* opts,
                   int32_t* h_level);
dpg_status dpg_bfs_dev(dpg_ctx* ctx, const dpg_graph* g, int32_t source,
                       const dpg_expand_opts* opts, int32_t* d_level);

/* ---- graph colouring (replaces GRAPH_COLOR_GPU, apps/graph-color/src/graph_color_wrapper.cu:210-238) */
/* color[v] = the round in which the reference's gclr_bitmap_kernel (graph_color_kernel.cu:28-49)
 * colours v: 1 + the largest colour among out-neighbours u < v (1 when there is none). Runs as one
 * persistent level-by-level pass over the transposed graph (built on the device on first use). Only
 * the timeout/iteration fields of opts are used. */
dpg_status dpg_color(dpg_ctx* ctx, const dpg_graph* g, const dpg_expand_opts* opts, int32_t* h_color);
dpg_status dpg_color_dev(dpg_ctx* ctx, const dpg_graph* g, const dpg_expand_opts* opts, int32_t* d_color);

/* ---- SpMV (replaces SpMV_GPU / csr_spmv_kernel, apps/SpMV/src/SpMV_kernel.cu:81-96) ------------ */
/* y[r] = sum over row r of vals[e] * x[col[e]]; FP32 in and out, deterministic summation order. */
dpg_status dpg_spmv_f32(dpg_ctx* ctx, const dpg_graph* g, const float* h_vals, const float* h_x,
                        float* h_y);
dpg_status dpg_spmv_f32_dev(dpg_ctx* ctx, const dpg_graph* g, const float* d_vals,
                            const float* d_x, float* d_y);

/* ---- batched right-hand sides and the SpMV adjoint (no counterpart in the reference) ------------ */
/* Row-major blocks of nrhs columns (1 <= nrhs <= 128): X, G, Y, dX are [V][nrhs] FP32.
 *   dpg_spmm_f32_dev:      Y = A X, A = g with values vals[E] in CSR order
 *   dpg_spmv_bwd_f32_dev:  dX = A^T G and dA[e] = sum_j G[row(e)][j] * X[col(e)][j]
 * Sums run in a fixed order (A^T through the transposed CSR in invertGraph order, built once per
 * graph on first use), so results are bit-reproducible. d_dX or d_dA may be NULL to skip one. */
dpg_status dpg_spmm_f32_dev(dpg_ctx* ctx, const dpg_graph* g, const float* d_vals, int32_t nrhs, const float* d_X,
                            float* d_Y);
dpg_status dpg_spmv_bwd_f32_dev(dpg_ctx* ctx, const dpg_graph* g, const float* d_vals, int32_t nrhs,
                                const float* d_X, const float* d_G, float* d_dX, float* d_dA);

/* ---- weighted PageRank and its gradient w.r.t. the edge weights (no counterpart in the reference) */
/* g is the out-adjacency; arc e = (u -> col[e]) has weight w[e] >= 0 and W[u] = sum of u's weights
 * (u dangling when W[u] == 0). r is the fixed point of
 *     r[v] = (1-d) T / V + d D / V + d * sum_{u->v} w[e] r[u] / W[u],   D = sum of dangling r,
 * with d = opts->damping and T = opts->total_rank, run from T / V (0 with init_zero) until no rank
 * changes by more than opts->epsilon times its new value (a relative test; with epsilon <= 0 for
 * exactly opts->iterations sweeps). d_seed = dL/dr (V floats). The adjoint
 * lambda = s + d P lambda (dangling rows d/V * sum lambda) is solved the same way with relative
 * tolerance adjoint_epsilon, and
 *     d_grad[e] = dL/dw[e] = d * r[u] / W[u] * (lambda[col[e]] - sum_t w[e'] lambda[t] / W[u]).
 * opts->iterations caps each of the two loops (0 with a tolerance: 10000 sweeps at most).
 * Outputs: d_rank (V), d_grad (E). The pull sweeps use the transposed CSR, built once per graph. */
dpg_status dpg_pagerank_grad_f32_dev(dpg_ctx* ctx, const dpg_graph* g, const float* d_weights, const float* d_seed,
                                     const dpg_pr_opts* opts, double adjoint_epsilon, float* d_rank, float* d_grad);
/* Forward and adjoint sweeps of the last dpg_pagerank_grad_f32_dev call on ctx. */
dpg_status dpg_ctx_grad_sweeps(const dpg_ctx* ctx, int64_t* forward, int64_t* adjoint);

/* ---- PageRank pull (replaces PAGERANK_GPU / pg_pull_gpu, pagerank_wrapper.cu:199-244,366-400) -- */
/* g_in is the transposed CSR (childVertexArray/rEdgeArray of invertGraph, global.cpp:237-277);
 * outdeg[v] is the out-degree in the original graph (outdegreeArray, pagerank.cpp:108-113). */
dpg_status dpg_pagerank_f32(dpg_ctx* ctx, const dpg_graph* g_in, const int32_t* h_outdeg,
                            const dpg_pr_opts* opts, float* h_rank);
dpg_status dpg_pagerank_f32_dev(dpg_ctx* ctx, const dpg_graph* g_in, const int32_t* d_outdeg,
                                const dpg_pr_opts* opts, float* d_rank);

/* ---- batches of graphs (no counterpart in the reference) ---------------------------------------- */
/* n graphs packed as one union CSR: graph g owns vertices [vstart[g], vstart[g+1]) and the union
 * out-adjacency (offsets[V+1], col[E], weights[E], global vertex ids) keeps every arc inside its
 * graph. The batch builds the union in-adjacency (invertGraph order per graph) for PageRank. */
typedef struct dpg_batch dpg_batch;
typedef struct dpg_batch_tuning {
    int32_t hub_threshold; /* SSSP: out-degree from which a frontier vertex is cut into chunks (default 32) */
    int32_t chunk;         /* SSSP: arcs per chunk, 128 / 256 / 512 (default 256) */
    int32_t pr_hot;        /* PageRank: gathered entries kept in shared memory, -1 = as many as fit */
} dpg_batch_tuning;
dpg_status dpg_batch_create(dpg_ctx* ctx, int32_t ngraphs, const int32_t* vstart, int64_t E, const int32_t* offsets,
                            const int32_t* col, const int32_t* weights, dpg_batch** out);
dpg_status dpg_batch_destroy(dpg_batch* b);
dpg_status dpg_batch_info(const dpg_batch* b, int32_t* ngraphs, int32_t* V, int64_t* E);
/* Batch-wide tuning; setting it also drops any per-graph SSSP setting. */
dpg_status dpg_batch_set_tuning(dpg_batch* b, const dpg_batch_tuning* t);
dpg_status dpg_batch_get_tuning(const dpg_batch* b, dpg_batch_tuning* t);
/* Per-graph SSSP binning: hub_threshold[g] (>= 1) and chunk[g] (128 / 256 / 512) for each of the n
 * graphs. The graphs that share a setting are solved by one multi-source launch; the launches of
 * the settings run one after another in the same solve. Both NULL: every graph uses the batch-wide
 * tuning again. Results never depend on these settings. dpg_batch_get_graph_tuning fills n entries
 * each with the setting every graph runs with. */
dpg_status dpg_batch_set_graph_tuning(dpg_batch* b, const int32_t* hub_threshold, const int32_t* chunk);
dpg_status dpg_batch_get_graph_tuning(const dpg_batch* b, int32_t* hub_threshold, int32_t* chunk);
/* SSSP from nsrc (1..32) sources of every graph in one persistent launch: h_sources[g * nsrc + k] is
 * a vertex of graph g (local id); d_dist[v * nsrc + k] = distance of union vertex v from source k of
 * v's graph (DPG_INF_COST when unreachable). Distances are exactly those of dpg_sssp on each graph
 * alone. */
dpg_status dpg_batch_sssp_dev(dpg_ctx* ctx, dpg_batch* b, int32_t nsrc, const int32_t* h_sources,
                              const dpg_expand_opts* opts, int32_t* d_dist);
/* opts->iterations sweeps of pull PageRank on every graph at once (opts->epsilon must be 0); each
 * graph is normalised on its own (teleport and dangling mass over its V_g vertices), as dpg_pagerank
 * on that graph alone with its out-degrees. d_rank[v] for union vertex v. */
dpg_status dpg_batch_pagerank_dev(dpg_ctx* ctx, dpg_batch* b, const dpg_pr_opts* opts, float* d_rank);
/* Both solves as one CUDA graph on the context stream: captured on the first call (and whenever an
 * argument, the tuning or a scratch buffer changes), replayed on later calls. */
dpg_status dpg_batch_run(dpg_ctx* ctx, dpg_batch* b, int32_t nsrc, const int32_t* h_sources,
                         const dpg_expand_opts* sssp_opts, int32_t* d_dist, const dpg_pr_opts* pr_opts, float* d_rank);
/* Kernel launches in one replay of the captured graph. */
dpg_status dpg_batch_launches(const dpg_batch* b, int64_t* kernels_per_run);
/* Tunes the batch and keeps the result in it. SSSP binning per graph: the graphs fall into size
 * classes by arc count (below 2^17, below 2^21, the rest); each class's 12 candidate settings
 * (hub_threshold 16/32/64/128 x chunk 128/256/512) are timed on one source per graph of the class,
 * and every graph takes its class's fastest (dpg_batch_get_graph_tuning). PageRank's shared-memory
 * hot-cache size is timed on three sweeps of the whole batch (one gather serves every graph).
 * `chosen` gets the batch-wide summary: the setting of the class holding the most arcs, and the
 * hot-cache size. Results never depend on the tuning. */
dpg_status dpg_batch_autotune(dpg_ctx* ctx, dpg_batch* b, int32_t nsrc, const int32_t* h_sources,
                              dpg_batch_tuning* chosen);

/* Shards a batch over `parts` ranks for the multi-GPU batched workload (no exchange step): owner[i]
 * of unit i (a graph, with cost = arcs x tasks) by longest-processing-time-first; load[parts] gets
 * each part's total cost (nullable). Deterministic: every rank computes the same owners. */
dpg_status dpg_partition_lpt(int32_t n, const int64_t* cost, int32_t parts, int32_t* owner, int64_t* load);

/* ---- recursive BFS with device-side launches (a measured comparison; replaces nothing) ---------- */
/* The reference's recursive traversals (bfs_rec_kernel.cu: bfs_kernel_dp 61-89, warp 158-213,
 * block 305-352, grid 394-457) as CUDA dynamic-parallelism (CDP2) child launches, to be timed
 * against dpg_bfs. Synchronous. Child launches are limited to 23 generations below the first and
 * to pending_limit outstanding launches (0: 65536; set as the context's device-runtime limit); a
 * launch that fails or is skipped makes the call return DPG_ERR_CAPACITY, since its subtree may be
 * unfinished. Levels are exact when the call succeeds. */
enum { DPG_CDP_NAIVE = 1, DPG_CDP_WARP = 2, DPG_CDP_BLOCK = 3, DPG_CDP_GRID = 4 };
typedef struct dpg_cdp_stats {
    int64_t launches;        /* child grids launched (the reference's nested_calls) */
    int64_t failed_launches; /* launches that failed or were skipped */
    int64_t buffer_entries;  /* append-buffer capacity of the consolidated variants */
} dpg_cdp_stats;
dpg_status dpg_bfs_cdp_dev(dpg_ctx* ctx, const dpg_graph* g, int32_t source, int32_t variant, int32_t pending_limit,
                           int32_t* d_level, dpg_cdp_stats* stats);

/* ---- one-shot host calls: the whole reference wrapper in one call (upload, solve, download) ----
 * dpg_pagerank_f32_host validates the offsets and columns, plans the row gathers and renames the
 * columns on the device while the columns upload; errors are those of dpg_graph_create, and the
 * ranks are bitwise those of dpg_graph_create + dpg_pagerank_f32 on the same arrays. */
dpg_status dpg_sssp_host(dpg_ctx* ctx, int32_t V, int64_t E, const int32_t* offsets,
                         const int32_t* col, const int32_t* weights, int32_t source,
                         const dpg_expand_opts* opts, int32_t* h_dist);
dpg_status dpg_pagerank_f32_host(dpg_ctx* ctx, int32_t V, int64_t E, const int32_t* in_offsets,
                                 const int32_t* in_col, const int32_t* outdeg,
                                 const dpg_pr_opts* opts, float* h_rank);

/* ---- SSSP without allocation (no counterpart in the reference) -------------------------------- */
/* For callers that must not allocate device memory, nor let a library do it: a serving engine
 * that reserves the whole device pool at start-up for its own arena (cudaMalloc would find nothing
 * left, and cudaMalloc/cudaFree can synchronise the device under its other streams), or a plugin
 * host that gives its plugins only buffers it owns. Runs the binned SSSP kernel on caller-owned
 * device inputs and output, with its workspace in a fixed 7 MiB __device__ array inside libdpg.so
 * (held by every GPU that loads the library until exit). Limits: V <= 262144 and E <= 4194304,
 * else DPG_ERR_CAPACITY.
 *   d_offsets[V+1]      CSR offsets, rising from 0 to E
 *   d_adj_pairs[2*E]    interleaved (neighbour, weight) int32 pairs, 8-byte aligned, neighbours in
 *                       [0, V), weights in [0, 2^30)
 *   d_dist[V]           output distances (DPG_INF_COST when unreachable)
 *   stream              cudaStream_t (NULL = legacy default stream); the call synchronises it
 * The graph is checked on the device before anything is relaxed: a violation of the ranges above
 * returns DPG_ERR_INVALID_ARG. Every call shares the array and clears what must start at zero;
 * calls whose GPU work overlaps (two threads or streams) race on it. The first call on a device
 * looks up the array's address (cudaGetSymbolAddress) and keeps it; reload the library after a
 * cudaDeviceReset of that device. Calls no cudaMalloc, cudaFree or other allocating routine. */
dpg_status dpg_sssp_noalloc_dev(int32_t V, int64_t E, const int32_t* d_offsets, const int32_t* d_adj_pairs,
                                int32_t source, int32_t* d_dist, void* stream);

/* ---- launch accounting (no counterpart in the reference; its GPU_PROFILE counter,
 *      sssp_kernel.cu:14-25, counts CDP launches only) ------------------------------------------- */
typedef enum dpg_kernel_kind {
    DPG_KERNEL_EXPAND = 0,    /* persistent SSSP/BFS frontier kernel */
    DPG_KERNEL_ROWGATHER = 1, /* SpMV / PageRank warp-tile gather */
    DPG_KERNEL_FIXUP = 2,     /* hub-row fix-up and dangling reduction */
    DPG_KERNEL_INIT = 3,      /* initialisation kernels */
    DPG_KERNEL_KINDS = 4
} dpg_kernel_kind;
/* Launch counts are always kept; enable != 0 also brackets every launch with a pair of CUDA events
 * recorded on the launching stream, so per-kind device time can be read back. */
dpg_status dpg_ctx_profile_enable(dpg_ctx* ctx, int32_t enable);
dpg_status dpg_ctx_profile_reset(dpg_ctx* ctx);
/* Synchronises; launches and summed event time (ms) of one kind since the last reset. */
dpg_status dpg_ctx_profile_read(dpg_ctx* ctx, int32_t kind, int64_t* launches, double* total_ms);

/* Per-iteration trace of the SSSP/BFS persistent kernel: max_iterations > 0 records, for each
 * frontier iteration j, {global ns at its start, small-frontier length, chunk count, 0}, then an end
 * entry {ns, 0, 0, 1}; 0 turns it off. dpg_ctx_trace_read copies up to `capacity` entries of
 * 4 int64 each (synchronises) and reports how many slots exist. */
dpg_status dpg_ctx_trace_enable(dpg_ctx* ctx, int32_t max_iterations);
dpg_status dpg_ctx_trace_read(dpg_ctx* ctx, int64_t* out, int32_t capacity, int32_t* count);

/* ---- random-read ceiling (no counterpart in the reference) -------------------------------------- */
/* Measures how many random 4-byte reads per second the device sustains from an array of n_floats
 * floats (two 1024-thread CTAs per SM, 8 independent loads in flight per thread, `iters` rounds):
 * the ceiling of the row gathers' and the expansion's scattered reads, beside HBM bandwidth. An
 * array of 16 MB stays in L2; one of several GB is read from HBM. Allocates the array, synchronises. */
dpg_status dpg_calibrate_random_reads(dpg_ctx* ctx, int64_t n_floats, int32_t iters, double* loads_per_second);

/* ---- failure-detection self test --------------------------------------------------------------- */
/* Runs the persistent kernel's grid barrier with one block missing, so its bounded wait must run
 * out after timeout_seconds; returns DPG_ERR_TIMEOUT when the device reported it and left the
 * context usable. */
dpg_status dpg_selftest_barrier_timeout(dpg_ctx* ctx, double timeout_seconds);

/* ---- host graph I/O and construction (common/global.cpp) -------------------------------------- */
typedef struct dpg_host_graph {
    int32_t V;
    int64_t E;
    int32_t source;    /* from the DIMACS9 's' line, 0-based; 0 when absent (global.cpp:10,43-46) */
    int32_t* offsets;  /* [V+1] vertexArray */
    int32_t* col;      /* [E]   edgeArray   */
    int32_t* weights;  /* [E]   weightArray */
} dpg_host_graph;

/* format: 0 DIMACS9 (.gr), 1 DIMACS10 (.graph), 2 SLNDC edge list — the -f flag of every app.
 * Semantics of readInputDIMACS9/10/SLNDC + convertCSR (global.cpp:29-235): 1-based ids, each
 * vertex's neighbour order reversed with respect to the file, DIMACS10/SLNDC weights drawn with
 * srand(7); rand()%1000+1. */
dpg_status dpg_read_graph(const char* path, int32_t format, dpg_host_graph* out);
/* The same with an explicit thread count: DIMACS9 files are parsed in parallel over line-aligned
 * chunks (threads = 0: all OpenMP threads; 1: the serial reader). Results, including the first
 * error reported, are identical either way. */
dpg_status dpg_read_graph_ex(const char* path, int32_t format, int32_t threads, dpg_host_graph* out);
/* Binary CSR cache of a loaded graph ("DPGCSR01", V, E, source, offsets, col, weights): a reload
 * skips parsing and CSR construction. */
dpg_status dpg_write_graph_cache(const char* path, const dpg_host_graph* g);
dpg_status dpg_read_graph_cache(const char* path, dpg_host_graph* out);
void dpg_host_graph_free(dpg_host_graph* g);
/* convertCSR on an in-memory arc list in file order (global.cpp:192-235). Outputs are caller-owned. */
dpg_status dpg_csr_from_arcs(int32_t V, int64_t E, const int32_t* src, const int32_t* dst,
                             const int32_t* w, int32_t* offsets, int32_t* col, int32_t* weights);
/* invertGraph (global.cpp:237-277): transposed CSR in the reference's neighbour order. */
dpg_status dpg_csr_transpose(int32_t V, int64_t E, const int32_t* offsets, const int32_t* col,
                             int32_t* in_offsets, int32_t* in_col);
/* The same on the device (replaces invertGraph, global.cpp:237-277): identical arrays, built with a
 * stable radix sort of the arcs by head; d_in_arc (nullable) receives the arc permutation. The input
 * is checked on the device first (offsets rising from 0 to E, columns in [0, V)), so the call
 * synchronises once; the transpose itself is stream-ordered on the context's stream. */
dpg_status dpg_csr_transpose_dev(dpg_ctx* ctx, int32_t V, int64_t E, const int32_t* d_offsets, const int32_t* d_col,
                                 int32_t* d_in_offsets, int32_t* d_in_col, int32_t* d_in_arc);
/* Same, and in_arc[p] = index in col of the arc that transposed slot p came from. */
dpg_status dpg_csr_transpose_perm(int32_t V, int64_t E, const int32_t* offsets, const int32_t* col,
                                  int32_t* in_offsets, int32_t* in_col, int32_t* in_arc);
/* Writes a DIMACS9 .gr file: "p sp V E", optional "s", then "a u v w" lines in arc order. */
dpg_status dpg_write_dimacs9(const char* path, int32_t V, int64_t E, const int32_t* src,
                             const int32_t* dst, const int32_t* w, int32_t source);
/* outputCost / outputLevel / outputRank / outputColor text formats (global.cpp:361-399). */
dpg_status dpg_write_cost(const char* path, int32_t V, int32_t source, const int32_t* dist);
dpg_status dpg_write_level(const char* path, int32_t V, const int32_t* level);
dpg_status dpg_write_rank(const char* path, int32_t V, const float* rank);
dpg_status dpg_write_color(const char* path, int32_t V, const int32_t* color);

/* ---- seeded synthetic graphs (counter-based; any arc range is reproducible on its own) --------- */
/* R-MAT: arc e in [0,E) draws `scale` quadrant choices with probabilities a,b,c,(1-a-b-c), then a
 * weight uniform in [wmin,wmax]; permute != 0 relabels vertices by a seeded bijection of
 * [0, 2^scale). Arcs with an endpoint >= V are redrawn (for V not a power of two). */
dpg_status dpg_rmat_arcs(int32_t scale, int32_t V, int64_t E, uint64_t seed, double a, double b,
                         double c, int32_t wmin, int32_t wmax, int32_t permute, int32_t* src,
                         int32_t* dst, int32_t* w);
/* rows x cols 4-neighbour grid, every undirected adjacency as two arcs, weights uniform in
 * [wmin,wmax]; E = 2*(rows*(cols-1) + cols*(rows-1)). */
dpg_status dpg_grid_arcs(int32_t rows, int32_t cols, uint64_t seed, int32_t wmin, int32_t wmax,
                         int32_t* src, int32_t* dst, int32_t* w);

#ifdef __cplusplus
}
#endif
#endif /* DPG_H */
