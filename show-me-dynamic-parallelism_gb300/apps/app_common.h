// Shared host-side plumbing of the command-line apps (gpu-sssp, gpu-bfs-rec, gpu-SpMV, gpu-pg,
// gpu-graph-color). They keep the reference apps' flags, messages and output formats
// (apps/sssp/src/sssp.cpp:51-188 and its siblings) and call libdpg.so through include/dpg.h instead
// of the CUDA wrappers.
//
// Flags (sssp.cpp:59-98): -h/--help, -v/--verbose, -d/--debug, -f/--format N (0 DIMACS9, 1 DIMACS10,
// 2 SLNDC), -s/--solution N, -e/--device N, -i/--import FILE. Additions, all optional:
// --source N (1-based; default: the file's `s` line, else 1), --out FILE (write the result in the
// reference's text format), --verify (check against a CPU restatement and print PASS/ERROR the way
// apps/bfs-rec/src/bfs_rec.cpp:130-141 does).
#pragma once

#include <sys/stat.h>

#include <string>

#include <sys/time.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "dpg.h"

struct AppConf {
    bool verbose = false;
    bool debug = false;
    int data_set_format = 0;
    int solution = 0;
    int device_num = 0;
    const char* graph_file = nullptr;
    int source_1based = 0;  // 0: from the file
    const char* out_file = nullptr;
    bool verify = false;
    bool cache = false;  // --cache: reuse <graph file>.dpgcsr when newer than the file
    double damping = -1.0;  // PageRank overrides (< 0: reference default)
    int iterations = -1;
};

inline double app_gettime() {
    struct timeval t;
    gettimeofday(&t, nullptr);
    return t.tv_sec + t.tv_usec * 1e-6;
}

// Same walk over argv as parse_arguments (sssp.cpp:59-98): unknown words are skipped; returns 0
// when the program should stop after printing usage.
inline int app_parse(int argc, char** argv, AppConf* c, void (*usage)()) {
    if (argc < 2) {
        usage();
        return 0;
    }
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        auto next = [&]() -> const char* { return (i + 1 < argc) ? argv[++i] : nullptr; };
        if (!strcmp(a, "-h") || !strcmp(a, "--help")) {
            usage();
            return 0;
        } else if (!strcmp(a, "-v") || !strcmp(a, "--verbose")) {
            c->verbose = true;
        } else if (!strcmp(a, "-d") || !strcmp(a, "--debug")) {
            c->debug = true;
        } else if (!strcmp(a, "-f") || !strcmp(a, "--format")) {
            const char* v = next();
            c->data_set_format = v ? atoi(v) : 0;
        } else if (!strcmp(a, "-s") || !strcmp(a, "--solution")) {
            const char* v = next();
            c->solution = v ? atoi(v) : 0;
        } else if (!strcmp(a, "-e") || !strcmp(a, "--device")) {
            const char* v = next();
            c->device_num = v ? atoi(v) : 0;
        } else if (!strcmp(a, "-i") || !strcmp(a, "--import")) {
            const char* v = next();
            if (!v) fprintf(stderr, "Graph file name missing.\n");
            c->graph_file = v;
        } else if (!strcmp(a, "--source")) {
            const char* v = next();
            c->source_1based = v ? atoi(v) : 0;
        } else if (!strcmp(a, "--out")) {
            c->out_file = next();
        } else if (!strcmp(a, "--verify")) {
            c->verify = true;
        } else if (!strcmp(a, "--cache")) {
            c->cache = true;
        } else if (!strcmp(a, "--damping")) {
            const char* v = next();
            c->damping = v ? atof(v) : -1.0;
        } else if (!strcmp(a, "--iters")) {
            const char* v = next();
            c->iterations = v ? atoi(v) : -1;
        }
    }
    return 1;
}

inline void app_print_conf(const AppConf& c, bool with_device) {
    fprintf(stderr, "\nCONFIGURATION:\n");
    if (c.graph_file) {
        fprintf(stderr, "- Graph file: %s\n", c.graph_file);
        fprintf(stderr, "- Graph format: %d\n", c.data_set_format);
    }
    fprintf(stderr, "- Solution: %d\n", c.solution);
    if (with_device) fprintf(stderr, "- GPU Device: %d\n", c.device_num);
    if (c.verbose && c.debug) fprintf(stderr, "- verbose mode\n");
    if (c.debug) fprintf(stderr, "- debug mode\n");
}

inline void app_usage_common(const char* name) {
    fprintf(stderr, "\n");
    fprintf(stderr, "Usage:  %s [option]\n", name);
    fprintf(stderr, "\nOptions:\n");
    fprintf(stderr, "    --help,-h      print this message\n");
    fprintf(stderr, "    --verbose,-v   basic verbosity level\n");
    fprintf(stderr, "    --debug,-d     enhanced verbosity level\n");
    fprintf(stderr, "\nOther:\n");
    fprintf(stderr, "    --import,-i <graph_file>           import graph file\n");
    fprintf(stderr, "    --format,-f <number>               specify the input format\n");
    fprintf(stderr, "                 0 - DIMACS9\n");
    fprintf(stderr, "                 1 - DIMACS10\n");
    fprintf(stderr, "                 2 - SLNDC\n");
}

inline void app_usage_tail() {
    fprintf(stderr, "    --device,-e <number>               select the device\n");
    fprintf(stderr, "    --source <number>                  source vertex (1-based; default: the file's s line)\n");
    fprintf(stderr, "    --out <file>                       write the result in the reference's text format\n");
    fprintf(stderr, "    --verify                           check against a CPU restatement (PASS/ERROR)\n");
    fprintf(stderr, "    --cache                            keep a binary CSR next to the input and reuse it\n");
}

// Loads the graph with the reference reader semantics and prints the reference's progress lines.
// Returns 0 on success, 1 when the file cannot be opened (sssp.cpp:141-147), 2 on a parse error.
inline int app_load(const AppConf& c, dpg_host_graph* g, bool print_source, double* read_s) {
    FILE* probe = fopen(c.graph_file, "r");
    if (!probe) {
        fprintf(stderr, "Error: NULL file pointer.\n");
        return 1;
    }
    fclose(probe);
    const double t0 = app_gettime();
    dpg_status s = DPG_ERR_IO;
    std::string cache_path = std::string(c.graph_file) + ".dpgcsr";
    bool from_cache = false;
    if (c.cache) {
        struct stat sf, sc;
        if (stat(c.graph_file, &sf) == 0 && stat(cache_path.c_str(), &sc) == 0 && sc.st_mtime >= sf.st_mtime) {
            s = dpg_read_graph_cache(cache_path.c_str(), g);
            from_cache = s == DPG_OK;
        }
    }
    if (!from_cache) s = dpg_read_graph(c.graph_file, c.data_set_format, g);
    if (c.cache && !from_cache && s == DPG_OK && dpg_write_graph_cache(cache_path.c_str(), g) != DPG_OK)
        fprintf(stderr, "Warning: %s\n", dpg_last_error());
    const double t1 = app_gettime();
    if (s != DPG_OK) {
        fprintf(stderr, "Error: %s\n", dpg_last_error());
        return 2;
    }
    if (c.source_1based > 0) g->source = c.source_1based - 1;
    if (g->V > 0 && (g->source < 0 || g->source >= g->V)) {
        fprintf(stderr, "Error: source vertex out of range\n");
        return 2;
    }
    *read_s = t1 - t0;
    if (c.verbose) {
        if (print_source) fprintf(stderr, "Source node is: %d\n", g->source + 1);
        fprintf(stderr, "Node no: %d\n", g->V);
        fprintf(stderr, "Edge no: %lld\n", static_cast<long long>(g->E));
    }
    return 0;
}

#define APP_CHECK(call)                                                 \
    do {                                                                \
        dpg_status _s = (call);                                         \
        if (_s != DPG_OK) {                                             \
            printf("Error: %s (%s)\n", dpg_status_string(_s), dpg_last_error()); \
            exit(1);                                                    \
        }                                                               \
    } while (0)
