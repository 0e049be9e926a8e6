// gpu-graph-color: drop-in for the reference's apps/graph-color (main graph_color.cpp,
// GRAPH_COLOR_GPU graph_color_wrapper.cu:210-238). Same flags; prints "Execution time" like the
// wrapper (line 232) and, with -d, the colour of every vertex in outputColor's format
// (global.cpp:393-399). The colouring is the reference's round rule computed level by level in one
// persistent launch; solution ids 0-4 are accepted and all run it.
#include <cstdint>
#include <vector>

#include "app_common.h"

static void usage() {
    app_usage_common("gpu-graph-color");
    fprintf(stderr, "    --solution,-s <number>             specify the solution (0-4, all map to the level pass)\n");
    app_usage_tail();
}

int main(int argc, char** argv) {
    AppConf c;
    if (!app_parse(argc, argv, &c, usage)) return 0;
    app_print_conf(c, false);
    if (!c.graph_file) return 0;
    if (c.solution < 0 || c.solution > 4) {
        printf("Unsupported solution\n");
        return 0;
    }
    dpg_host_graph g;
    double read_s = 0;
    if (int rc = app_load(c, &g, false, &read_s)) return rc;
    if (c.verbose) {
        fprintf(stderr, "Import graph:\t\t%lf\n", read_s);
        fprintf(stderr, "AdjList to CSR:\t\t%lf\n", 0.0);
    }
    dpg_ctx* ctx = nullptr;
    APP_CHECK(dpg_ctx_create(c.device_num, &ctx));
    dpg_graph* dg = nullptr;
    double t0 = app_gettime();
    APP_CHECK(dpg_graph_create(ctx, g.V, g.E, g.offsets, g.col, nullptr, &dg));
    if (c.verbose) fprintf(stderr, "cudaMemcpy:\t\t%lf\n", app_gettime() - t0);
    std::vector<int32_t> color(g.V > 0 ? g.V : 1);
    t0 = app_gettime();
    APP_CHECK(dpg_color(ctx, dg, nullptr, color.data()));
    fprintf(stderr, "Execution time:\t\t%lf\n", app_gettime() - t0);
    dpg_run_stats st;
    APP_CHECK(dpg_ctx_last_stats(ctx, &st));
    int32_t max_color = 0;
    for (int32_t v = 0; v < g.V; ++v) max_color = color[v] > max_color ? color[v] : max_color;
    if (c.debug) {
        fprintf(stderr, "Graph Coloring ends in %d iterations.\n", max_color);
        fprintf(stderr, "------- Color value ------\n");
        for (int32_t i = 0; i < g.V; ++i) fprintf(stdout, "Node %d: %d\n", i + 1, color[i]);
    }
    if (c.out_file) APP_CHECK(dpg_write_color(c.out_file, g.V, color.data()));
    dpg_graph_destroy(dg);
    dpg_ctx_destroy(ctx);
    dpg_host_graph_free(&g);
    return 0;
}
