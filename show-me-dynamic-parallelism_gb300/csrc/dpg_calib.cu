// Random-read ceilings of the GPU, the second roofline of the gather and expansion kernels.
//
// The row gathers and the frontier expansion read 4-byte values at random addresses (x[col],
// dist[head]); a warp's such load touches 32 different sectors. Their ceiling is the rate at which
// the SMs can issue and retire those sector misses, well below HBM bandwidth / 32 bytes. This
// kernel measures it: every thread of two 1024-thread CTAs per SM keeps 8 independent random loads
// of a float array in flight (a 64-bit LCG per thread picks the indices, all inside the array),
// for `iters` rounds. An array of 16 MB stays in L2; one of several GB is read from HBM.
#include <cuda_runtime.h>

#include "dpg_api_internal.h"

using namespace dpg_api;

namespace {

constexpr int kCalibBlock = 1024;

__global__ void __launch_bounds__(kCalibBlock, 2) random_read_kernel(const float* __restrict__ a, uint64_t n,
                                                                     int iters, float* sink) {
    uint64_t x = (static_cast<uint64_t>(blockIdx.x) * kCalibBlock + threadIdx.x) * 0x9E3779B97F4A7C15ull + 1ull;
    float acc = 0.0f;
    for (int it = 0; it < iters; ++it) {
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            x = x * 6364136223846793005ull + 1442695040888963407ull;
            v[q] = __ldg(a + (x >> 24) % n);
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) acc += v[q];
    }
    if (acc == -1.0f) *sink = acc;  // keeps the loads; the array holds no negative values
}

__global__ void fill_kernel(float* a, uint64_t n) {
    for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        a[i] = static_cast<float>(i & 1023);
}

}  // namespace

extern "C" dpg_status dpg_calibrate_random_reads(dpg_ctx* c, int64_t n_floats, int32_t iters,
                                                 double* loads_per_second) {
    DPG_TRY(use_device(c));
    if (n_floats < 1024 || iters < 1 || !loads_per_second)
        return set_error(DPG_ERR_INVALID_ARG, "need n_floats >= 1024, iters >= 1 and an output");
    float* a = nullptr;
    float* sink = nullptr;
    DPG_CUDA_TRY(cudaMalloc(&a, sizeof(float) * static_cast<size_t>(n_floats)));
    cudaError_t e = cudaMalloc(&sink, sizeof(float));
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    const int grid = c->sm_count * 2;
    float ms = 0.0f;
    if (e == cudaSuccess) {
        fill_kernel<<<c->sm_count * 8, 256, 0, c->stream>>>(a, static_cast<uint64_t>(n_floats));
        random_read_kernel<<<grid, kCalibBlock, 0, c->stream>>>(a, static_cast<uint64_t>(n_floats), iters, sink);
        cudaEventRecord(t0, c->stream);
        random_read_kernel<<<grid, kCalibBlock, 0, c->stream>>>(a, static_cast<uint64_t>(n_floats), iters, sink);
        cudaEventRecord(t1, c->stream);
        e = cudaEventSynchronize(t1);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    cudaFree(sink);
    cudaFree(a);
    if (e != cudaSuccess) return set_error(DPG_ERR_CUDA, std::string("random-read calibration: ") + cudaGetErrorString(e));
    *loads_per_second = 8.0 * iters * kCalibBlock * static_cast<double>(grid) / (ms * 1e-3);
    return DPG_OK;
}
