// ref_gpu_driver.cpp — runs the reference's own kernels (oracle/_ref/ref_<app>.cubin, built by
// `make -C oracle refgpu` from oracle/ref_kernels.cu) on a GPU, to generate golden vectors.
//
// TEST INFRASTRUCTURE ONLY: used by tests/golden/make_golden_gpu.py; libdpg.so never loads it.
//
// The kernels are the reference's, loaded through the CUDA driver API. The host loops around them
// restate the reference wrappers' solution-0 paths (its wrappers cannot be built without its host
// program): the launch shapes, the initial values, the per-iteration order of launches, memsets
// and copies, and the host-side arithmetic are theirs:
//   refgpu_sssp      sssp_wrapper.cu:54-136 (prepare_gpu), 147-183 (sssp_tqueue_gpu)
//   refgpu_color     graph_color_wrapper.cu:60-100 (prepare_gpu), 113-130 (gclr_nopruning_gpu)
//   refgpu_spmv_f64  SpMV_wrapper.cu:60-120 (prepare_gpu), 144-150 (spmv_gpu)
//   refgpu_pagerank  pagerank_wrapper.cu:80-184 (prepare_gpu, prepare_dangling_node), 199-244
//                    (pg_pull_gpu)
// Differences, all outside the kernels: errors return a negative code instead of exit(); every
// loop has an iteration cap (the reference loops until its flag clears); refgpu_pagerank can run
// a fixed number of sweeps and start from a given uniform rank (the reference memsets the ranks to
// 0 and stops on its epsilon test) so that the kernels can also be run with other parameters.
#include <cuda.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

constexpr int kThreads = 128;           // THREADS_PER_BLOCK / maxDegreeT of the wrappers
constexpr unsigned kQueueMax = 10240000;  // QMAXLENGTH
constexpr unsigned kMaxGrid = 65535;      // MAXDIMGRID
constexpr int kInf = 1073741824;          // INF, sssp_wrapper.cu:5

#define CK(call)                                                                      \
    do {                                                                              \
        CUresult r_ = (call);                                                         \
        if (r_ != CUDA_SUCCESS) {                                                     \
            const char* s_ = nullptr;                                                 \
            cuGetErrorString(r_, &s_);                                                \
            fprintf(stderr, "ref_gpu_driver: %s failed: %s\n", #call, s_ ? s_ : "?"); \
            return -100 - static_cast<int>(r_);                                       \
        }                                                                             \
    } while (0)

struct Session {
    CUdevice dev = 0;
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    std::vector<CUdeviceptr> bufs;
    ~Session() {
        for (CUdeviceptr p : bufs) cuMemFree(p);
        if (mod) cuModuleUnload(mod);
        if (ctx) cuDevicePrimaryCtxRelease(dev);
    }
    int open(const char* cubin) {
        CK(cuInit(0));
        CK(cuDeviceGet(&dev, 0));
        CK(cuDevicePrimaryCtxRetain(&ctx, dev));
        CK(cuCtxSetCurrent(ctx));
        CK(cuModuleLoad(&mod, cubin));
        return 0;
    }
    int alloc(CUdeviceptr* p, size_t bytes) {
        CK(cuMemAlloc(p, bytes ? bytes : 16));
        bufs.push_back(*p);
        return 0;
    }
    int upload(CUdeviceptr* p, const void* h, size_t bytes) {
        int rc = alloc(p, bytes);
        if (rc) return rc;
        if (bytes) CK(cuMemcpyHtoD(*p, h, bytes));
        return 0;
    }
    int fn(CUfunction* f, const char* mangled) {
        CK(cuModuleGetFunction(f, mod, mangled));
        return 0;
    }
};

int launch(CUfunction f, unsigned grid, unsigned block, void** args) {
    CK(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, nullptr, args, nullptr));
    CK(cuCtxSynchronize());
    return 0;
}

// dimGrid/dimBlock of the wrappers' thread+bitmap configuration for n items; the SpMV and
// PageRank wrappers round a single block up to whole warps, the SSSP and colouring ones do not.
void bitmap_shape(int n, bool warp_round, unsigned* grid, unsigned* block) {
    if (n > kThreads) {
        *grid = static_cast<unsigned>(n / kThreads + 1);
        *block = kThreads;
    } else {
        *grid = 1;
        *block = warp_round ? static_cast<unsigned>(32 * (n / 32 + 1)) : static_cast<unsigned>(n);
    }
}

}  // namespace

extern "C" {

// Distances from src by unorder_generateQueue_kernel + unorder_threadQueue_kernel (solution 0).
// Returns the number of relaxation iterations, or < 0 on error.
int refgpu_sssp(const char* cubin, int V, long long E, const int* off, const int* col, const int* w, int src,
                int* dist) {
    if (V < 1 || E < 0 || src < 0 || src >= V) return -1;
    Session s;
    int rc = s.open(cubin);
    if (rc) return rc;
    CUfunction gen, relax;
    if ((rc = s.fn(&gen, "_Z28unorder_generateQueue_kernelPciPiPjj"))) return rc;
    if ((rc = s.fn(&relax, "_Z26unorder_threadQueue_kernelPiS_S_S_PciS_Pj"))) return rc;
    std::vector<int> cost(V, kInf);
    std::vector<char> update(V, 0);
    cost[src] = 0;
    update[src] = 1;
    CUdeviceptr d_off, d_col, d_w, d_cost, d_update, d_queue, d_qlen;
    if ((rc = s.upload(&d_off, off, sizeof(int) * (V + 1))) || (rc = s.upload(&d_col, col, sizeof(int) * E)) ||
        (rc = s.upload(&d_w, w, sizeof(int) * E)) || (rc = s.upload(&d_cost, cost.data(), sizeof(int) * V)) ||
        (rc = s.upload(&d_update, update.data(), V)) || (rc = s.alloc(&d_queue, sizeof(int) * kQueueMax)) ||
        (rc = s.alloc(&d_qlen, sizeof(unsigned))))
        return rc;
    CK(cuMemsetD32(d_qlen, 0, 1));
    unsigned grid, block;
    bitmap_shape(V, false, &grid, &block);
    int n = V;
    unsigned qmax = kQueueMax;
    void* gen_args[] = {&d_update, &n, &d_queue, &d_qlen, &qmax};
    if ((rc = launch(gen, grid, block, gen_args))) return rc;
    unsigned qlen = 0;
    CK(cuMemcpyDtoH(&qlen, d_qlen, sizeof(unsigned)));
    int iterations = 0;
    const long long cap = 4ll * V + 16;  // each iteration lowers some label; the fixed point ends it
    while (qlen != 0) {
        if (iterations >= cap) return -2;
        unsigned tgrid = qlen <= static_cast<unsigned>(kThreads) ? 1u : qlen / kThreads + 1;
        if (qlen > static_cast<unsigned>(kThreads) * kMaxGrid) return -3;
        void* relax_args[] = {&d_off, &d_col, &d_cost, &d_w, &d_update, &n, &d_queue, &d_qlen};
        if ((rc = launch(relax, tgrid, kThreads, relax_args))) return rc;
        CK(cuMemsetD32(d_qlen, 0, 1));
        if ((rc = launch(gen, grid, block, gen_args))) return rc;
        CK(cuMemcpyDtoH(&qlen, d_qlen, sizeof(unsigned)));
        ++iterations;
    }
    CK(cuMemcpyDtoH(dist, d_cost, sizeof(int) * V));
    return iterations;
}

// Colours by gclr_bitmap_kernel rounds (solution 0). Returns the number of rounds, or < 0.
int refgpu_color(const char* cubin, int V, long long E, const int* off, const int* col, int* color) {
    if (V < 1 || E < 0) return -1;
    Session s;
    int rc = s.open(cubin);
    if (rc) return rc;
    CUfunction k;
    if ((rc = s.fn(&k, "_Z18gclr_bitmap_kernelPiS_S_Pjii"))) return rc;
    std::vector<int> zero(V, 0);
    CUdeviceptr d_off, d_col, d_color, d_nonstop;
    if ((rc = s.upload(&d_off, off, sizeof(int) * (V + 1))) || (rc = s.upload(&d_col, col, sizeof(int) * E)) ||
        (rc = s.upload(&d_color, zero.data(), sizeof(int) * V)) || (rc = s.alloc(&d_nonstop, sizeof(unsigned))))
        return rc;
    unsigned grid, block;
    bitmap_shape(V, false, &grid, &block);
    unsigned nonstop = 1;
    int color_type = 1;
    int n = V;
    while (nonstop) {
        if (color_type > V + 1) return -2;
        CK(cuMemsetD32(d_nonstop, 0, 1));
        void* args[] = {&d_off, &d_col, &d_color, &d_nonstop, &color_type, &n};
        if ((rc = launch(k, grid, block, args))) return rc;
        ++color_type;
        CK(cuMemcpyDtoH(&nonstop, d_nonstop, sizeof(unsigned)));
    }
    CK(cuMemcpyDtoH(color, d_color, sizeof(int) * V));
    return color_type - 1;
}

// y = A x by csr_spmv_kernel, FP64 (FLOAT_T is double in the SpMV app). Returns 0, or < 0.
int refgpu_spmv_f64(const char* cubin, int V, long long E, const int* off, const int* col, const double* data,
                    const double* x, double* y) {
    if (V < 1 || E < 0) return -1;
    Session s;
    int rc = s.open(cubin);
    if (rc) return rc;
    CUfunction k;
    if ((rc = s.fn(&k, "_Z15csr_spmv_kernelPiS_PdS0_S0_i"))) return rc;
    CUdeviceptr d_off, d_col, d_data, d_x, d_y;
    if ((rc = s.upload(&d_off, off, sizeof(int) * (V + 1))) || (rc = s.upload(&d_col, col, sizeof(int) * E)) ||
        (rc = s.upload(&d_data, data, sizeof(double) * E)) || (rc = s.upload(&d_x, x, sizeof(double) * V)) ||
        (rc = s.alloc(&d_y, sizeof(double) * V)))
        return rc;
    CK(cuMemsetD8(d_y, 0, sizeof(double) * V));
    unsigned grid, block;
    bitmap_shape(V, true, &grid, &block);
    int n = V;
    void* args[] = {&d_off, &d_col, &d_data, &d_x, &d_y, &n};
    if ((rc = launch(k, grid, block, args))) return rc;
    CK(cuMemcpyDtoH(y, d_y, sizeof(double) * V));
    return 0;
}

// Pull PageRank by update_danglingrankarray_kernel + pagerank_thread_pull_kernel +
// check_delta_kernel over the transposed CSR (FLOAT_T float). outdeg comes from the out-CSR
// (graph.outdegreeArray); the dangling vertices are those of out-degree 0, ascending.
// init_uniform = 0: ranks start at 0 (prepare_gpu's memset); 1: at (float)total / V.
// fixed_sweeps = 0: stop when check_delta_kernel leaves the flag clear (or at max_sweeps);
// 1: run exactly max_sweeps sweeps. Returns the number of sweeps, or < 0.
int refgpu_pagerank(const char* cubin, int V, long long E, const int* in_off, const int* in_col, const int* outdeg,
                    float damping, double total, int init_uniform, int max_sweeps, int fixed_sweeps, float* rank) {
    if (V < 1 || E < 0 || max_sweeps < 0) return -1;
    Session s;
    int rc = s.open(cubin);
    if (rc) return rc;
    CUfunction kd, kp, kc;
    if ((rc = s.fn(&kd, "_Z31update_danglingrankarray_kernelPfS_Pii"))) return rc;
    if ((rc = s.fn(&kp, "_Z27pagerank_thread_pull_kernelPiS_S_PfS0_fffi"))) return rc;
    if ((rc = s.fn(&kc, "_Z18check_delta_kernelPfS_Pji"))) return rc;
    std::vector<int> dangling;
    for (int v = 0; v < V; ++v)
        if (outdeg[v] == 0) dangling.push_back(v);
    int nd = static_cast<int>(dangling.size());
    std::vector<float> r0(V, init_uniform ? static_cast<float>(total) / V : 0.0f);
    CUdeviceptr d_in_off, d_in_col, d_od, d_rank, d_new, d_dvert, d_drank, d_nonstop;
    if ((rc = s.upload(&d_in_off, in_off, sizeof(int) * (V + 1))) ||
        (rc = s.upload(&d_in_col, in_col, sizeof(int) * E)) || (rc = s.upload(&d_od, outdeg, sizeof(int) * V)) ||
        (rc = s.upload(&d_rank, r0.data(), sizeof(float) * V)) || (rc = s.alloc(&d_new, sizeof(float) * V)) ||
        (rc = s.upload(&d_dvert, dangling.data(), sizeof(int) * nd)) ||
        (rc = s.alloc(&d_drank, sizeof(float) * nd)) || (rc = s.alloc(&d_nonstop, sizeof(unsigned))))
        return rc;
    CK(cuMemsetD32(d_new, 0, V));
    unsigned grid, block, dgrid = 1, dblock = 1;
    bitmap_shape(V, true, &grid, &block);
    if (nd > kThreads) {
        dgrid = static_cast<unsigned>(nd / kThreads + 1);
        dblock = kThreads;
    } else if (nd > 0) {
        dblock = static_cast<unsigned>(nd);
    }
    // rank_random_walk = (1-damping)*TOTAL_RANK/noNodeTotal: float (1-d), then double arithmetic
    // with the double TOTAL_RANK, stored to float (pagerank_wrapper.cu:183).
    float rank_random_walk = static_cast<float>(static_cast<double>(1 - damping) * total / V);
    std::vector<float> drank(nd);
    unsigned nonstop = 1;
    int sweeps = 0;
    int n = V;
    while (fixed_sweeps ? sweeps < max_sweeps : (nonstop && sweeps < max_sweeps)) {
        float dangling_rank = 0.0f;
        if (nd != 0) {
            void* a[] = {&d_rank, &d_drank, &d_dvert, &nd};
            if ((rc = launch(kd, dgrid, dblock, a))) return rc;
            CK(cuMemcpyDtoH(drank.data(), d_drank, sizeof(float) * nd));
            for (int i = 0; i < nd; ++i) dangling_rank += drank[i];
        }
        float rank_dangling_node = damping * dangling_rank / V;
        void* ap[] = {&d_in_off, &d_in_col, &d_od, &d_rank, &d_new, &rank_random_walk, &rank_dangling_node, &damping, &n};
        if ((rc = launch(kp, grid, block, ap))) return rc;
        CK(cuMemsetD32(d_nonstop, 0, 1));
        void* ac[] = {&d_rank, &d_new, &d_nonstop, &n};
        if ((rc = launch(kc, grid, block, ac))) return rc;
        CK(cuMemcpyDtoH(&nonstop, d_nonstop, sizeof(unsigned)));
        CUdeviceptr t = d_rank;
        d_rank = d_new;
        d_new = t;
        ++sweeps;
    }
    CK(cuMemcpyDtoH(rank, d_rank, sizeof(float) * V));
    return sweeps;
}

}  // extern "C"
