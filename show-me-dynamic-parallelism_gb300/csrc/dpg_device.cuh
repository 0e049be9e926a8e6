// Device-side building blocks shared by the dpg kernels: the per-context status block, the
// bounded grid barrier of the persistent kernels, and warp helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dpg.h"

namespace dpg {

constexpr unsigned kFullMask = 0xFFFFFFFFu;

// One per context, in device memory. `error` keeps the first device-side failure until the host
// reads and clears it (dpg_ctx_synchronize).
struct DevStatus {
    int error;                     // dpg_status raised on the device
    int error_site;                // small code telling which check fired
    unsigned bar_count;            // grid-barrier word (see grid_barrier); 0 when a launch starts
    unsigned bar_gen;              // unused
    unsigned fix_count;            // last-block ticket of the hub fix-up kernel
    unsigned pad0;
    unsigned long long iterations; // statistics of the last persistent launch
    unsigned long long edges;
    unsigned long long pops;
    unsigned long long pad1[4];
};

__device__ __forceinline__ unsigned long long global_timer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void raise_error(DevStatus* st, int code, int site) {
    if (atomicCAS(&st->error, 0, code) == 0) st->error_site = site;
}

__device__ __forceinline__ int load_error(const DevStatus* st) {
    return *reinterpret_cast<const volatile int*>(&st->error);
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier for a cooperative (co-resident) launch, one atomic per CTA on one word: CTA 0 adds
// 2^31 - (expected - 1), every other CTA adds 1, so the word's top bit flips exactly when the last
// of `expected` CTAs arrives (the low 31 bits of a partial sum stay below 2^31, and each complete
// generation adds exactly 2^31). The word must be 0 when the launch starts. Waiters poll it with
// acquire loads. Measured with 456 CTAs: 2.0 us per barrier, against 3.2 us for a counter plus a
// separate generation word with sleeping waits.
// Every wait is bounded: after `timeout_ns` of global time (or a spin cap derived from it) the
// waiting CTA records DPG_ERR_TIMEOUT and leaves. Returns false when the grid must stop (any error
// recorded). `expected` is the number of CTAs that take part (gridDim.x in normal use).
__device__ __forceinline__ bool grid_barrier(DevStatus* st, unsigned expected,
                                             unsigned long long timeout_ns) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned inc = blockIdx.x == 0 ? (0x80000000u - (expected - 1u)) : 1u;
        __threadfence();
        const unsigned old = atomicAdd(&st->bar_count, inc);
        const unsigned long long t0 = global_timer_ns();
        // The spin cap bounds the loop even if the timer were to stall (each pass is a round trip to
        // L2 of a few hundred ns at least).
        const unsigned long long max_spins = timeout_ns / 256 + 4096;
        unsigned long long spins = 0;
        while (((old ^ ld_acquire_gpu(&st->bar_count)) & 0x80000000u) == 0u) {
            ++spins;
            if ((spins & 63) == 0) {
                if (load_error(st) != 0) break;
                if (global_timer_ns() - t0 > timeout_ns || spins > max_spins) {
                    raise_error(st, DPG_ERR_TIMEOUT, 1);
                    break;
                }
            }
        }
        __threadfence();
        s_ok = load_error(st) == 0;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ int warp_inclusive_scan(int v) {
    const int lane = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFullMask, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ float warp_sum_f32(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
    return v;
}

__device__ __forceinline__ double warp_sum_f64(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
    return v;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
    return v;
}

}  // namespace dpg
