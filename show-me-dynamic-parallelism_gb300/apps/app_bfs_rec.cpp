// gpu-bfs-rec: drop-in for the reference's apps/bfs-rec (main bfs_rec.cpp:143-219, BFS_REC_GPU
// bfs_rec_wrapper.cu:240-280). Same flags and messages; like the reference it always validates the
// GPU levels against a CPU FIFO BFS (bfs_cpu, bfs_rec.cpp:102-121) and prints PASS/ERROR.
// Solution ids keep their bfs-rec meaning: 0 flat, 1 naive recursive, 2 hierarchical recursive,
// 3 warp, 4 block, 5 grid consolidation; 6 selects the library's binned kernel.
#include <cstdint>
#include <vector>

#include "app_common.h"

static void usage() {
    app_usage_common("gpu-bfs-synth");
    fprintf(stderr, "    --solution,-s <number>             specify the solution\n");
    fprintf(stderr, "                 0 - GPU flat\n");
    fprintf(stderr, "                 1 - GPU naive dynamic parallelism\n");
    fprintf(stderr, "                 2 - GPU hierachical dynamic parallelism\n");
    fprintf(stderr, "                 3 - warp-level consolidation\n");
    fprintf(stderr, "                 4 - block-level consolidation\n");
    fprintf(stderr, "                 5 - grid-level consolidation\n");
    fprintf(stderr, "                 6 - degree-binned persistent kernel\n");
    app_usage_tail();
}

static void bfs_cpu(const dpg_host_graph& g, int32_t src, int32_t* level) {
    for (int32_t v = 0; v < g.V; ++v) level[v] = DPG_UNDEFINED_LEVEL;
    level[src] = 0;
    std::vector<int32_t> q;
    q.reserve(g.V);
    q.push_back(src);
    for (size_t h = 0; h < q.size(); ++h) {
        const int32_t node = q[h];
        const unsigned next_level = static_cast<unsigned>(level[node]) + 1u;
        for (int32_t e = g.offsets[node]; e < g.offsets[node + 1]; ++e) {
            const int32_t nb = g.col[e];
            if (level[nb] == DPG_UNDEFINED_LEVEL || static_cast<unsigned>(level[nb]) > next_level) {
                level[nb] = static_cast<int32_t>(next_level);
                q.push_back(nb);
            }
        }
    }
}

int main(int argc, char** argv) {
    AppConf c;
    if (!app_parse(argc, argv, &c, usage)) return 0;
    app_print_conf(c, true);
    if (!c.graph_file) return 0;
    static const int kMap[7] = {DPG_SOL_THREAD, DPG_SOL_NAIVE, DPG_SOL_NAIVE, DPG_SOL_WARP,
                                DPG_SOL_BLOCK,  DPG_SOL_GRID,  DPG_SOL_BINNED};
    if (c.solution < 0 || c.solution > 6) {
        printf("Unsopported solutions\n");
        return 0;
    }
    dpg_host_graph g;
    double read_s = 0;
    if (int rc = app_load(c, &g, false, &read_s)) return rc;
    if (c.verbose) {
        fprintf(stderr, "Import graph:\t\t%lf\n", read_s);
        fprintf(stderr, "AdjList to CSR:\t\t%lf\n", 0.0);
    }
    printf("\n===MAIN=== :: [num_nodes,num_edges] = %u, %u\n", static_cast<unsigned>(g.V), static_cast<unsigned>(g.E));
    double t0 = app_gettime();
    dpg_ctx* ctx = nullptr;
    APP_CHECK(dpg_ctx_create(c.device_num, &ctx));
    const double init_ms = (app_gettime() - t0) * 1e3;
    t0 = app_gettime();
    dpg_graph* dg = nullptr;
    APP_CHECK(dpg_graph_create(ctx, g.V, g.E, g.offsets, g.col, nullptr, &dg));
    const double h2d_ms = (app_gettime() - t0) * 1e3;
    dpg_expand_opts o = {kMap[c.solution], DPG_REF_THRESHOLD, 0, 0, 0.0};
    std::vector<int32_t> level(g.V > 0 ? g.V : 1), level_cpu(g.V > 0 ? g.V : 1);
    APP_CHECK(dpg_ctx_profile_enable(ctx, 1));
    APP_CHECK(dpg_ctx_profile_reset(ctx));
    t0 = app_gettime();
    APP_CHECK(dpg_bfs(ctx, dg, g.source, &o, level.data()));
    const double total_ms = (app_gettime() - t0) * 1e3;
    double k_ms = 0, i_ms = 0;
    int64_t n = 0;
    APP_CHECK(dpg_ctx_profile_read(ctx, DPG_KERNEL_EXPAND, &n, &k_ms));
    APP_CHECK(dpg_ctx_profile_read(ctx, DPG_KERNEL_INIT, &n, &i_ms));
    bfs_cpu(g, g.source, level_cpu.data());
    // validateArrays (bfs_rec.cpp:130-141)
    int flag = 1;
    for (int32_t node = 0; node < g.V; ++node) {
        if (level[node] != level_cpu[node]) {
            printf("ERROR: validation error at %d: %s !\n", node, "GPU bfs rec");
            printf("Node %d : %d v.s. %d\n", node, level[node], level_cpu[node]);
            flag = 0;
            break;
        }
    }
    if (flag) printf("PASS: %s !\n", "GPU bfs rec");
    if (c.verbose) {
        fprintf(stdout, "===MAIN=== :: CUDA runtime init:\t\t%.2lf ms.\n", init_ms);
        fprintf(stdout, "===MAIN=== :: CUDA device cudaMalloc:\t\t%.2lf ms.\n", 0.0);
        fprintf(stdout, "===MAIN=== :: CUDA H2D cudaMemcpy:\t\t%.2lf ms.\n", h2d_ms);
        fprintf(stdout, "===MAIN=== :: CUDA kernel execution:\t\t%.2lf ms.\n", k_ms + i_ms);
        fprintf(stdout, "===MAIN=== :: CUDA D2H cudaMemcpy:\t\t%.2lf ms.\n",
                total_ms > k_ms + i_ms ? total_ms - k_ms - i_ms : 0.0);
    }
    if (c.debug)
        for (int32_t i = 0; i < g.V; ++i) printf("Node %d is in level %d\n", i + 1, level[i]);
    if (c.out_file) APP_CHECK(dpg_write_level(c.out_file, g.V, level.data()));
    dpg_graph_destroy(dg);
    dpg_ctx_destroy(ctx);
    dpg_host_graph_free(&g);
    return flag ? 0 : 3;
}
