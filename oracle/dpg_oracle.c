/*
 * dpg_oracle.c — CPU oracle for the irregular CSR neighbour-expansion path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs
 * may load this code, and only as the checker or the timed CPU baseline; the library under
 * test (libdpg.so) never calls it.
 *
 * Each function restates the reference algorithm it names (paths relative to the reference repo):
 *   oracle_sssp_dijkstra      SSSP fixed point of unorder_threadQueue_kernel + host loop
 *                             (apps/sssp/src/sssp_kernel.cu:40-61, sssp_wrapper.cu:147-187);
 *                             distances >= INF (2^30) stay INF exactly as the int relaxation does.
 *   oracle_sssp_worklist      the reference's own label-correcting schedule, sequentially:
 *                             update flags -> queue (sssp_kernel.cu:496-506) -> relax pass.
 *   oracle_sssp_bf_omp        OpenMP frontier Bellman-Ford (timed CPU baseline, all cores).
 *   oracle_bfs                bfs_cpu (apps/bfs-rec/src/bfs_rec.cpp:102-121), UNDEFINED=0x7FFFFFFF.
 *   oracle_bfs_omp            OpenMP level-synchronous BFS (timed CPU baseline).
 *   oracle_spmv_*             csr_spmv_kernel (apps/SpMV/src/SpMV_kernel.cu:81-96) in FP64.
 *   oracle_pagerank_f64       pull PageRank (pagerank_kernel.cu:95-120 + pagerank_wrapper.cu:147-241)
 *                             in FP64, with damping / total / initial vector / convergence options.
 *   oracle_pagerank_ref_f32   the same loop in the reference's FP32 arithmetic order (per-edge
 *                             divide, damping multiplied per edge, epsilon test of check_delta_kernel).
 *   oracle_pagerank_omp_f32   OpenMP FP32 pull PageRank (timed CPU baseline).
 *   oracle_color              gclr_bitmap_kernel rounds (apps/graph-color/src/graph_color_kernel.cu:28-49,
 *                             graph_color_wrapper.cu:113-130).
 *
 * Pinning: oracle_bfs is checked against the reference's own bfs_cpu (compiled into
 * oracle/_ref/libref.so, recorded in tests/golden/); oracle_sssp_* against the known distances of the
 * reference's datasets/data_test.gr and against each other. SpMV and PageRank: parity unpinned by the
 * reference, which has no CPU implementation of them; they are restated from the kernel sources and
 * checked in the reference's exact FP64 known-answer mode (data[e] = e%13+0.5, x[i] = i%17+0.5).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_INF 1073741824
#define ORACLE_UNDEFINED 0x7FFFFFFF

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------------------------------------------------------- SSSP: Dijkstra, binary heap -- */
typedef struct {
    int64_t key;
    int32_t v;
} heap_item;

static void heap_push(heap_item* h, int64_t* n, int64_t key, int32_t v) {
    int64_t i = (*n)++;
    while (i > 0) {
        int64_t p = (i - 1) / 2;
        if (h[p].key <= key) break;
        h[i] = h[p];
        i = p;
    }
    h[i].key = key;
    h[i].v = v;
}

static heap_item heap_pop(heap_item* h, int64_t* n) {
    heap_item top = h[0];
    heap_item last = h[--(*n)];
    int64_t i = 0;
    for (;;) {
        int64_t c = 2 * i + 1;
        if (c >= *n) break;
        if (c + 1 < *n && h[c + 1].key < h[c].key) ++c;
        if (h[c].key >= last.key) break;
        h[i] = h[c];
        i = c;
    }
    if (*n > 0) h[i] = last;
    return top;
}

/* Returns 0 on success, -1 on allocation failure, -2 on a negative weight. */
int oracle_sssp_dijkstra(int32_t V, const int32_t* off, const int32_t* col, const int32_t* w, int32_t src,
                         int32_t* dist) {
    int64_t E = off[V];
    for (int64_t e = 0; e < E; ++e)
        if (w[e] < 0) return -2;
    int64_t* d = (int64_t*)malloc(sizeof(int64_t) * (size_t)(V > 0 ? V : 1));
    heap_item* h = (heap_item*)malloc(sizeof(heap_item) * (size_t)(E + 2));
    if (!d || !h) {
        free(d);
        free(h);
        return -1;
    }
    for (int32_t v = 0; v < V; ++v) d[v] = INT64_MAX;
    int64_t n = 0;
    d[src] = 0;
    heap_push(h, &n, 0, src);
    while (n > 0) {
        heap_item it = heap_pop(h, &n);
        if (it.key != d[it.v]) continue;
        /* The reference relaxes alt = cost[u] + w only from vertices whose cost is below INF;
         * a path of length >= INF can never lower an INF label, so it stops here too. */
        if (it.key >= ORACLE_INF) continue;
        for (int32_t e = off[it.v]; e < off[it.v + 1]; ++e) {
            int64_t nd = it.key + w[e];
            if (nd < d[col[e]]) {
                d[col[e]] = nd;
                heap_push(h, &n, nd, col[e]);
            }
        }
    }
    for (int32_t v = 0; v < V; ++v) dist[v] = (d[v] >= ORACLE_INF) ? ORACLE_INF : (int32_t)d[v];
    free(d);
    free(h);
    return 0;
}

/* The reference's schedule, run sequentially: all flagged vertices form the queue, then each queued
 * vertex relaxes its row (alt = cost[u] + w; if cost[v] > alt: cost[v] = alt, update[v] = 1).
 * Returns the number of passes (the reference's `iteration` counter, sssp_wrapper.cu:182). */
int64_t oracle_sssp_worklist(int32_t V, const int32_t* off, const int32_t* col, const int32_t* w, int32_t src,
                             int32_t* cost) {
    char* update = (char*)calloc((size_t)(V > 0 ? V : 1), 1);
    int32_t* queue = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V > 0 ? V : 1));
    if (!update || !queue) {
        free(update);
        free(queue);
        return -1;
    }
    for (int32_t v = 0; v < V; ++v) cost[v] = ORACLE_INF;
    cost[src] = 0;
    update[src] = 1;
    int64_t passes = 0;
    for (;;) {
        int32_t q = 0;
        for (int32_t v = 0; v < V; ++v)
            if (update[v]) {
                update[v] = 0;
                queue[q++] = v;
            }
        if (q == 0) break;
        for (int32_t i = 0; i < q; ++i) {
            int32_t u = queue[i];
            int32_t cu = cost[u];
            for (int32_t e = off[u]; e < off[u + 1]; ++e) {
                int32_t alt = cu + w[e];
                if (cost[col[e]] > alt) {
                    cost[col[e]] = alt;
                    update[col[e]] = 1;
                }
            }
        }
        ++passes;
    }
    free(update);
    free(queue);
    return passes;
}

/* OpenMP frontier Bellman-Ford with atomic min: the all-cores CPU baseline for SSSP. */
int oracle_sssp_bf_omp(int32_t V, const int32_t* off, const int32_t* col, const int32_t* w, int32_t src,
                       int32_t* dist, int32_t nthreads) {
    int32_t* q0 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V + 1));
    int32_t* q1 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V + 1));
    unsigned char* inq = (unsigned char*)calloc((size_t)(V + 1), 1);
    if (!q0 || !q1 || !inq) {
        free(q0);
        free(q1);
        free(inq);
        return -1;
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int32_t v = 0; v < V; ++v) dist[v] = ORACLE_INF;
    dist[src] = 0;
    int64_t n = 1, n1;
    q0[0] = src;
    while (n > 0) {
        n1 = 0;
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < n; ++i) {
            int32_t u = q0[i];
            /* Clear u's queued flag, then read its distance. Both sequentially consistent, as are
             * the compare-and-swap and the exchange of a relaxer: otherwise the clear can wait in a
             * store buffer while the read goes first, a concurrent improvement of u sees the flag
             * still set and does not queue u, and that improvement is never relaxed. */
            __atomic_store_n(&inq[u], (unsigned char)0, __ATOMIC_SEQ_CST);
            int32_t du = __atomic_load_n(&dist[u], __ATOMIC_SEQ_CST);
            for (int32_t e = off[u]; e < off[u + 1]; ++e) {
                int32_t v = col[e];
                int32_t nd = du + w[e];
                int32_t cur;
#pragma omp atomic read
                cur = dist[v];
                while (nd < cur) {
                    if (__atomic_compare_exchange_n(&dist[v], &cur, nd, 0, __ATOMIC_SEQ_CST, __ATOMIC_RELAXED)) {
                        if (!__atomic_exchange_n(&inq[v], (unsigned char)1, __ATOMIC_SEQ_CST)) {
                            int64_t pos = __atomic_fetch_add(&n1, 1, __ATOMIC_RELAXED);
                            q1[pos] = v;
                        }
                        break;
                    }
                }
            }
        }
        int32_t* t = q0;
        q0 = q1;
        q1 = t;
        n = n1;
    }
    free(q0);
    free(q1);
    free(inq);
    return 0;
}

/* ------------------------------------------------------------------------------------- BFS ---- */
/* bfs_cpu, bfs_rec.cpp:102-121: FIFO queue; a neighbour is (re)visited when it is UNDEFINED or has a
 * larger level. level[] must come in filled with UNDEFINED except level[src] = 0 (bfs_rec.cpp:190-192,
 * 197-199); this function does that itself. Returns the number of pops. */
int64_t oracle_bfs(int32_t V, const int32_t* off, const int32_t* col, int32_t src, int32_t* level) {
    int64_t cap = (int64_t)V + 1, head = 0, tail = 0, pops = 0;
    int32_t* q = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
    if (!q) return -1;
    for (int32_t v = 0; v < V; ++v) level[v] = ORACLE_UNDEFINED;
    level[src] = 0;
    q[tail] = src;
    tail = (tail + 1) % cap;
    int64_t size = 1;
    while (size > 0) {
        int32_t node = q[head];
        head = (head + 1) % cap;
        --size;
        ++pops;
        unsigned next_level = (unsigned)level[node] + 1u;
        for (int32_t e = off[node]; e < off[node + 1]; ++e) {
            int32_t nb = col[e];
            if (level[nb] == ORACLE_UNDEFINED || (unsigned)level[nb] > next_level) {
                level[nb] = (int32_t)next_level;
                /* In FIFO order a vertex is never lowered after its first visit, so the queue never
                 * holds more than V entries; guard anyway. */
                if (size == cap) {
                    free(q);
                    return -1;
                }
                q[tail] = nb;
                tail = (tail + 1) % cap;
                ++size;
            }
        }
    }
    free(q);
    return pops;
}

int oracle_bfs_omp(int32_t V, const int32_t* off, const int32_t* col, int32_t src, int32_t* level,
                   int32_t nthreads) {
    int32_t* q0 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V + 1));
    int32_t* q1 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V + 1));
    if (!q0 || !q1) {
        free(q0);
        free(q1);
        return -1;
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int32_t v = 0; v < V; ++v) level[v] = ORACLE_UNDEFINED;
    level[src] = 0;
    int64_t n = 1, n1;
    q0[0] = src;
    int32_t lvl = 0;
    while (n > 0) {
        n1 = 0;
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t i = 0; i < n; ++i) {
            int32_t u = q0[i];
            for (int32_t e = off[u]; e < off[u + 1]; ++e) {
                int32_t v = col[e];
                int32_t expect = ORACLE_UNDEFINED;
                if (__atomic_load_n(&level[v], __ATOMIC_RELAXED) == ORACLE_UNDEFINED &&
                    __atomic_compare_exchange_n(&level[v], &expect, lvl + 1, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                    int64_t pos = __atomic_fetch_add(&n1, 1, __ATOMIC_RELAXED);
                    q1[pos] = v;
                }
            }
        }
        int32_t* t = q0;
        q0 = q1;
        q1 = t;
        n = n1;
        ++lvl;
    }
    free(q0);
    free(q1);
    return 0;
}

/* ------------------------------------------------------------------------------------ SpMV ---- */
/* y[r] = sum_e data[e] * x[col[e]] in FP64 (csr_spmv_kernel); FLOAT_T is double in the reference.
 * `dot += data[i] * x[indices[i]]` is one fused multiply-add per nonzero as nvcc compiles it (its
 * default contracts a*b+c), so the restatement uses fma() and matches the kernel's output bit for
 * bit (checked against the reference kernel's own output in tests/golden/refgpu.npz). */
void oracle_spmv_f64(int32_t V, const int32_t* off, const int32_t* col, const double* data, const double* x,
                     double* y) {
    for (int32_t r = 0; r < V; ++r) {
        double dot = 0.0;
        for (int32_t e = off[r]; e < off[r + 1]; ++e) dot = fma(data[e], x[col[e]], dot);
        y[r] = dot;
    }
}

/* FP32 inputs, FP64 accumulation; absy[r] = sum |data * x| gives the row's conditioning scale. */
void oracle_spmv_f32in(int32_t V, const int32_t* off, const int32_t* col, const float* data, const float* x,
                       double* y, double* absy, int32_t nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1024)
    for (int32_t r = 0; r < V; ++r) {
        double dot = 0.0, a = 0.0;
        for (int32_t e = off[r]; e < off[r + 1]; ++e) {
            double p = (double)data[e] * (double)x[col[e]];
            dot += p;
            a += fabs(p);
        }
        y[r] = dot;
        if (absy) absy[r] = a;
    }
}

/* FP32 SpMV with FP32 accumulation, all threads: the timed CPU baseline. */
void oracle_spmv_omp_f32(int32_t V, const int32_t* off, const int32_t* col, const float* data, const float* x,
                         float* y, int32_t nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1024)
    for (int32_t r = 0; r < V; ++r) {
        float dot = 0.0f;
        for (int32_t e = off[r]; e < off[r + 1]; ++e) dot += data[e] * x[col[e]];
        y[r] = dot;
    }
}

/* -------------------------------------------------------------------------------- PageRank ---- */
/* Pull PageRank over the transposed CSR (in_off/in_col = childVertexArray/rEdgeArray), FP64:
 *   new[v] = d * sum_{p in in(v)} rank[p]/outdeg[p] + (1-d)*total/V + d*dangling/V
 * with dangling = sum of rank over vertices of out-degree 0 (pagerank_wrapper.cu:207-227).
 * epsilon > 0: stop after the first sweep whose max |new-old| <= epsilon (check_delta_kernel),
 * at most `iterations` sweeps; epsilon <= 0: exactly `iterations` sweeps.
 * Returns the number of sweeps. */
int64_t oracle_pagerank_f64(int32_t V, const int32_t* in_off, const int32_t* in_col, const int32_t* outdeg,
                            double damping, double total, int32_t init_zero, int32_t iterations, double epsilon,
                            double* rank, int32_t nthreads) {
    double* nr = (double*)malloc(sizeof(double) * (size_t)(V > 0 ? V : 1));
    double* contrib = (double*)malloc(sizeof(double) * (size_t)(V > 0 ? V : 1));
    if (!nr || !contrib) {
        free(nr);
        free(contrib);
        return -1;
    }
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int32_t v = 0; v < V; ++v) rank[v] = init_zero ? 0.0 : total / (double)V;
    int64_t sweeps = 0;
    for (int32_t it = 0; it < iterations; ++it) {
        double dang = 0.0;
        for (int32_t v = 0; v < V; ++v) {
            if (outdeg[v] == 0) dang += rank[v];
            contrib[v] = outdeg[v] > 0 ? rank[v] / (double)outdeg[v] : 0.0;
        }
        const double base = (1.0 - damping) * total / (double)V + damping * dang / (double)V;
        double maxd = 0.0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(max : maxd)
        for (int32_t v = 0; v < V; ++v) {
            double s = 0.0;
            for (int32_t e = in_off[v]; e < in_off[v + 1]; ++e) s += contrib[in_col[e]];
            nr[v] = damping * s + base;
            double dd = fabs(nr[v] - rank[v]);
            if (dd > maxd) maxd = dd;
        }
        memcpy(rank, nr, sizeof(double) * (size_t)V);
        ++sweeps;
        if (epsilon > 0 && !(maxd > epsilon)) break;
    }
    free(nr);
    free(contrib);
    return sweeps;
}

/* The reference's FP32 arithmetic, in its order: per in-edge new = fma(damping, rank[p]/outdeg[p], new)
 * (pagerank_kernel.cu:112-115; nvcc contracts `new_rank_tid += damping * rank` into one fused
 * multiply-add), then + rank_random_walk + rank_dangling_node (:117). On the host:
 * rank_random_walk = (1-damping)*TOTAL_RANK/V with float (1-damping) and the double TOTAL_RANK,
 * rounded to float (pagerank_wrapper.cu:183); the dangling ranks summed in FP32 in vertex order and
 * rank_dangling_node = damping * dangling / V in float (:210-221); continue while some
 * |rank - new| (float) exceeds the double EPSILON (check_delta_kernel, pagerank_kernel.cu:72-81).
 * epsilon < 0 runs exactly max_iterations sweeps. Matches the reference kernels' output bit for bit
 * (tests/golden/refgpu.npz). */
int64_t oracle_pagerank_ref_f32(int32_t V, const int32_t* in_off, const int32_t* in_col, const int32_t* outdeg,
                                float damping, double total, int32_t init_zero, int32_t max_iterations,
                                double epsilon, float* rank) {
    float* nr = (float*)malloc(sizeof(float) * (size_t)(V > 0 ? V : 1));
    if (!nr) return -1;
    for (int32_t v = 0; v < V; ++v) rank[v] = init_zero ? 0.0f : (float)total / (float)V;
    const float rank_random_walk = (float)((double)(1.0f - damping) * total / (double)V);
    int64_t sweeps = 0;
    int nonstop = 1;
    while (nonstop && sweeps < max_iterations) {
        float dangling_rank = 0.0f;
        for (int32_t v = 0; v < V; ++v)
            if (outdeg[v] == 0) dangling_rank += rank[v];
        const float rank_dangling_node = damping * dangling_rank / (float)V;
        nonstop = epsilon < 0;
        for (int32_t v = 0; v < V; ++v) {
            float s = 0.0f;
            for (int32_t e = in_off[v]; e < in_off[v + 1]; ++e) {
                int32_t p = in_col[e];
                float r = rank[p] / (float)outdeg[p];
                s = fmaf(damping, r, s);
            }
            s = s + rank_random_walk + rank_dangling_node;
            nr[v] = s;
        }
        for (int32_t v = 0; v < V; ++v) {
            if ((double)fabsf(rank[v] - nr[v]) > epsilon) nonstop = 1;
            rank[v] = nr[v];
        }
        ++sweeps;
    }
    free(nr);
    return sweeps;
}

/* FP32 pull PageRank on all threads with contributions precomputed: the timed CPU baseline. */
int64_t oracle_pagerank_omp_f32(int32_t V, const int32_t* in_off, const int32_t* in_col, const int32_t* outdeg,
                                float damping, float total, int32_t iterations, float* rank, int32_t nthreads) {
    float* contrib = (float*)malloc(sizeof(float) * (size_t)(V > 0 ? V : 1));
    if (!contrib) return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    for (int32_t v = 0; v < V; ++v) rank[v] = total / (float)V;
    for (int32_t it = 0; it < iterations; ++it) {
        double dang = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : dang)
        for (int32_t v = 0; v < V; ++v) {
            if (outdeg[v] == 0) dang += rank[v];
            contrib[v] = outdeg[v] > 0 ? rank[v] / (float)outdeg[v] : 0.0f;
        }
        const float base = (float)((1.0 - damping) * total / V + damping * dang / V);
#pragma omp parallel for schedule(dynamic, 1024)
        for (int32_t v = 0; v < V; ++v) {
            float s = 0.0f;
            for (int32_t e = in_off[v]; e < in_off[v + 1]; ++e) s += contrib[in_col[e]];
            rank[v] = damping * s + base;
        }
    }
    free(contrib);
    return iterations;
}

/* ---------------------------------------------------------------------------- colouring ---- */
/* Round k = 1, 2, ...: an uncoloured v takes colour k iff no out-neighbour u < v has color[u] in
 * {0, k} (gclr_bitmap_kernel). Within a round the kernel's reads race with writes of the same
 * round; whether a neighbour u < v coloured k in this round is seen as 0 or k, v is blocked either
 * way, so the result is schedule-independent. Returns the number of rounds. */
int64_t oracle_color(int32_t V, const int32_t* off, const int32_t* col, int32_t* color) {
    for (int32_t v = 0; v < V; ++v) color[v] = 0;
    int64_t rounds = 0;
    int nonstop = 1;
    int32_t k = 1;
    while (nonstop) {
        nonstop = 0;
        for (int32_t v = 0; v < V; ++v) {
            if (color[v] != 0) continue;
            int ok = 1;
            for (int32_t e = off[v]; e < off[v + 1]; ++e) {
                int32_t u = col[e];
                if (u < v && (color[u] == 0 || color[u] == k)) {
                    ok = 0;
                    break;
                }
            }
            if (ok) {
                color[v] = k;
                nonstop = 1;
            }
        }
        ++k;
        ++rounds;
    }
    return rounds;
}

/* ------------------------------------------------------- synthetic graphs and CSR construction -- */
/* These let the CPU arms of bench.py build the benchmark graph without the library under test.
 *
 * oracle_rmat_arcs restates the seeded counter-based R-MAT generator the benchmark uses (the
 * library's dpg_rmat_arcs): arc e draws its 64-bit words from splitmix64(splitmix64(seed ^ e*K) +
 * counter), four 16-bit quadrant draws per word, rejection of endpoints >= V, then a seeded
 * bijection of the vertex ids; weight = wmin + draw(e, 2^32-1) % (wmax-wmin+1). The same seed thus
 * gives the same arc list as the library, which the CPU-only tests check.
 * oracle_csr_from_arcs restates convertCSR (common/global.cpp:192-235): a vertex's arcs appear in
 * the reverse of their order in the input, as convertCSR pops each adjacency list from its back.
 * oracle_csr_transpose restates invertGraph (common/global.cpp:237-277): in-row v lists the
 * sources of v's in-arcs in descending source order (push_back over ascending sources, then
 * popped from the back). */
static uint64_t orc_mix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

static uint64_t orc_draw(uint64_t seed, uint64_t stream, uint64_t counter) {
    return orc_mix(orc_mix(seed ^ (stream * 0xD1B54A32D192ED03ull)) + counter);
}

static uint32_t orc_permute(uint32_t x, int bits, uint64_t seed) {
    if (bits <= 0) return x;
    const uint64_t mask = bits >= 32 ? 0xFFFFFFFFull : ((1ull << bits) - 1ull);
    const int sh = bits / 2 + 1;
    uint64_t y = x;
    for (int round = 0; round < 3; ++round) {
        const uint64_t k = orc_draw(seed, 0xA5A5ull + (uint64_t)round, 0);
        y = (y ^ (k >> 40)) & mask;
        y = (y * ((k & 0xFFFFFFFFull) | 1ull)) & mask;
        if (sh < bits) y = (y ^ (y >> sh)) & mask;
    }
    return (uint32_t)y;
}

/* Returns 0, or -1 on bad arguments, or -2 when rejection sampling did not converge. */
int oracle_rmat_arcs(int32_t scale, int32_t V, int64_t E, uint64_t seed, double a, double b, double c,
                     int32_t wmin, int32_t wmax, int32_t permute, int32_t* src, int32_t* dst, int32_t* w) {
    if (scale < 1 || scale > 30 || V < 1 || (int64_t)V > (1ll << scale) || E < 0) return -1;
    const uint32_t ta = (uint32_t)llround(a * 65536.0);
    const uint32_t tab = (uint32_t)llround((a + b) * 65536.0);
    const uint32_t tabc = (uint32_t)llround((a + b + c) * 65536.0);
    const uint64_t span = w ? (uint64_t)((int64_t)wmax - wmin + 1) : 1;
    int failed = 0;
#pragma omp parallel for schedule(static) reduction(| : failed)
    for (int64_t e = 0; e < E; ++e) {
        uint32_t u = 0, v = 0;
        int ok = 0;
        for (uint64_t attempt = 0; attempt <= 4097 && !ok; ++attempt) {
            uint64_t word = 0;
            u = v = 0;
            for (int lvl = 0; lvl < scale; ++lvl) {
                if (lvl % 4 == 0) word = orc_draw(seed, (uint64_t)e, attempt * 64 + (uint64_t)(lvl / 4));
                const uint32_t r = (uint32_t)(word & 0xFFFFu);
                word >>= 16;
                u = 2 * u + (r >= tab);
                v = 2 * v + ((r >= ta && r < tab) || r >= tabc);
            }
            if (permute) {
                u = orc_permute(u, scale, seed);
                v = orc_permute(v, scale, seed);
            }
            ok = (int64_t)u < V && (int64_t)v < V;
        }
        if (!ok) failed = 1;
        src[e] = (int32_t)u;
        dst[e] = (int32_t)v;
        if (w) w[e] = wmin + (int32_t)(orc_draw(seed, (uint64_t)e, 0xFFFFFFFFull) % span);
    }
    return failed ? -2 : 0;
}

/* off[V+1], col[E] (and wout[E] when w and wout are given). Returns 0, or -1 on an id out of range. */
int oracle_csr_from_arcs(int32_t V, int64_t E, const int32_t* src, const int32_t* dst, const int32_t* w,
                         int32_t* off, int32_t* col, int32_t* wout) {
    int64_t* fill = (int64_t*)calloc((size_t)V + 1, sizeof(int64_t));
    if (!fill) return -2;
    for (int64_t e = 0; e < E; ++e) {
        if (src[e] < 0 || src[e] >= V || dst[e] < 0 || dst[e] >= V) {
            free(fill);
            return -1;
        }
        ++fill[src[e] + 1];
    }
    for (int32_t v = 0; v < V; ++v) fill[v + 1] += fill[v];
    for (int32_t v = 0; v <= V; ++v) off[v] = (int32_t)fill[v];
    /* Fill each row from its end, so the last arc of the input lands first. */
    for (int32_t v = 0; v < V; ++v) fill[v] = off[v + 1];
    for (int64_t e = 0; e < E; ++e) {
        const int64_t p = --fill[src[e]];
        col[p] = dst[e];
        if (w && wout) wout[p] = w[e];
    }
    free(fill);
    return 0;
}

int oracle_csr_transpose(int32_t V, const int32_t* off, const int32_t* col, int32_t* in_off, int32_t* in_col) {
    const int64_t E = off[V];
    int64_t* fill = (int64_t*)calloc((size_t)V + 1, sizeof(int64_t));
    if (!fill) return -2;
    for (int64_t e = 0; e < E; ++e) {
        if (col[e] < 0 || col[e] >= V) {
            free(fill);
            return -1;
        }
        ++fill[col[e] + 1];
    }
    for (int32_t v = 0; v < V; ++v) fill[v + 1] += fill[v];
    for (int32_t v = 0; v <= V; ++v) in_off[v] = (int32_t)fill[v];
    for (int32_t v = 0; v < V; ++v) fill[v] = in_off[v + 1];
    /* Ascending sources, each in-row filled from its end: the largest source ends up first. */
    for (int32_t u = 0; u < V; ++u)
        for (int32_t e = off[u]; e < off[u + 1]; ++e) in_col[--fill[col[e]]] = u;
    free(fill);
    return 0;
}
