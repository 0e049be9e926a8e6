// ref_driver.cpp — C entry points over the reference's own host code, for checking the oracle and
// the library's loader against the reference itself.
//
// TEST INFRASTRUCTURE ONLY. This file is compiled together with the reference sources
// common/global.cpp and apps/bfs-rec/src/bfs_rec.cpp (main renamed) by oracle/Makefile into
// oracle/_ref/libref.so; nothing here is shipped in libdpg.so.
//
// The reference talks through globals (common/global.h:48-58); these wrappers set `fp`, call the
// reader + convertCSR (+ invertGraph), and copy the arrays out.
#include <cstdio>
#include <cstring>

#include "bfs_rec.h"

// bfs_rec.cpp calls this from its (renamed) main; the driver never runs that main.
void BFS_REC_GPU() {}
void bfs_cpu(int* levelArray);  // bfs_rec.cpp:102
int outputCost(FILE* file);     // global.cpp:369
int outputRank(FILE* file);     // global.cpp:385
int outputColor(FILE* file);    // global.cpp:393

extern "C" {

// Loads a graph with the reference reader (format 0 DIMACS9, 1 DIMACS10, 2 SLNDC) and converts it
// to CSR, then builds the transposed CSR. Returns 0 on success.
int ref_load(const char* path, int format, int* V, long long* E, int* src) {
    fp = fopen(path, "r");
    if (!fp) return -1;
    source = 0;
    graph.childVertexArray = nullptr;
    graph.rEdgeArray = nullptr;
    switch (format) {
        case 0: readInputDIMACS9(); break;
        case 1: readInputDIMACS10(); break;
        case 2: readInputSLNDC(); break;
        default: fclose(fp); return -2;
    }
    fclose(fp);
    fp = nullptr;
    convertCSR();
    invertGraph();
    *V = noNodeTotal;
    *E = noEdgeTotal;
    *src = source;
    return 0;
}

void ref_get_csr(int* off, int* col, int* w) {
    memcpy(off, graph.vertexArray, sizeof(int) * (noNodeTotal + 1));
    memcpy(col, graph.edgeArray, sizeof(int) * noEdgeTotal);
    memcpy(w, graph.weightArray, sizeof(int) * noEdgeTotal);
}

void ref_get_transpose(int* in_off, int* in_col) {
    memcpy(in_off, graph.childVertexArray, sizeof(int) * (noNodeTotal + 1));
    memcpy(in_col, graph.rEdgeArray, sizeof(int) * noEdgeTotal);
}

// bfs_cpu on the loaded graph from `src`, as bfs_rec.cpp:197-200 sets it up.
void ref_bfs_cpu(int src, int* level) {
    source = src;
    for (int i = 0; i < noNodeTotal; ++i) level[i] = UNDEFINED;
    level[src] = 0;
    bfs_cpu(level);
}

// outputCost of the given distances into `path` (global.cpp:369-375).
int ref_output_cost(const char* path, int src, const int* dist) {
    FILE* f = fopen(path, "w");
    if (!f) return -1;
    source = src;
    int* saved = graph.costArray;
    graph.costArray = const_cast<int*>(dist);
    outputCost(f);
    graph.costArray = saved;
    fclose(f);
    return 0;
}

int ref_output_rank(const char* path, const float* rank) {
    FILE* f = fopen(path, "w");
    if (!f) return -1;
    float* saved = graph.rankArray;
    graph.rankArray = const_cast<float*>(rank);
    outputRank(f);
    graph.rankArray = saved;
    fclose(f);
    return 0;
}

int ref_output_color(const char* path, const int* color) {
    FILE* f = fopen(path, "w");
    if (!f) return -1;
    int* saved = graph.colorArray;
    graph.colorArray = const_cast<int*>(color);
    outputColor(f);
    graph.colorArray = saved;
    fclose(f);
    return 0;
}

}  // extern "C"
