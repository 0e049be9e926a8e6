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
    unsigned bar_count;            // grid-barrier arrivals in the current generation
    unsigned bar_gen;              // grid-barrier generation
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

// Sense-counting grid barrier for a cooperative (co-resident) launch. Every wait is bounded: after
// `timeout_ns` of global time (or a spin cap derived from it) the waiting CTA records
// DPG_ERR_TIMEOUT and leaves. Returns false when the grid must stop (any error recorded).
// `expected` is the number of CTAs that take part (gridDim.x in normal use).
__device__ __forceinline__ bool grid_barrier(DevStatus* st, unsigned expected,
                                             unsigned long long timeout_ns) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = &st->bar_gen;
        const unsigned g = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(&st->bar_count, 1u);
        if (arrived == expected - 1) {
            atomicExch(&st->bar_count, 0u);
            __threadfence();
            atomicAdd(&st->bar_gen, 1u);
        } else {
            const unsigned long long t0 = global_timer_ns();
            // The spin cap bounds the loop even if the timer were to stall: each pass sleeps.
            const unsigned long long max_spins = timeout_ns / 8 + 1024;
            unsigned long long spins = 0;
            while (*gen == g) {
                if (load_error(st) != 0) break;
                ++spins;
                if ((spins & 31) == 0 && (global_timer_ns() - t0 > timeout_ns || spins > max_spins)) {
                    raise_error(st, DPG_ERR_TIMEOUT, 1);
                    break;
                }
                __nanosleep(32);
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
