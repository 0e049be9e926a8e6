// ref_kernels.cu — the reference's own CUDA kernels, compiled from the reference tree into
// device-only modules (oracle/_ref/ref_<app>.cubin) for generating golden vectors.
//
// TEST INFRASTRUCTURE ONLY. Nothing here is part of libdpg.so. oracle/Makefile (`make refgpu
// REF=<reference tree>`) compiles this file once per app with -DREF_APP_<APP>, with the app's
// source directory on the include path, so that each module holds exactly the kernels of one
// reference kernel file, compiled where it lies:
//   REF_APP_SSSP      apps/sssp/src/sssp_kernel.cu          (unorder_generateQueue_kernel 496-506,
//                                                            unorder_threadQueue_kernel 40-61)
//   REF_APP_COLOR     apps/graph-color/src/graph_color_kernel.cu (gclr_bitmap_kernel 28-49)
//   REF_APP_SPMV      apps/SpMV/src/SpMV_kernel.cu          (csr_spmv_kernel 81-96)
//   REF_APP_PAGERANK  apps/pagerank/src/pagerank_kernel.cu  (check_delta_kernel 72-81,
//                                                            update_danglingrankarray_kernel 84-92,
//                                                            pagerank_thread_pull_kernel 95-120)
// Before each kernel file come the app header and the macros its wrapper defines before including
// it (sssp_wrapper.cu:1-16, graph_color_wrapper.cu:1-13, SpMV_wrapper.cu:1-14,
// pagerank_wrapper.cu:1-16), so the kernels see what they see in the reference build.
//
// All four are compiled with -DBUFFER_ALLOCATOR=2, the value the reference's Makefiles pass
// (apps/sssp/src/Makefile:28, apps/SpMV/src/Makefile:21; other values need device-side
// synchronisation, which CDP2 removed). SpMV and PageRank still do not compile under CUDA 13 as
// shipped. Three compile-only shims make them build; none touches a kernel that
// oracle/ref_gpu_driver.cpp launches:
//   * their own atomicAdd(double*, double) clashes with the builtin: every atomicAdd in the file is
//     routed to ref_atomic_add, which forwards the builtin overloads (their CAS loop keeps its
//     body, under the new name);
//   * legacy __shfl_down (no mask) becomes __shfl_down_sync over the full warp, used only by the
//     CDP block reductions;
//   * device-side cudaDeviceSynchronize, removed by CDP2, becomes a no-op in PageRank's
//     pg_multidp_kernel (pagerank_kernel.cu:349), which is never launched from this module.
// The module keeps the file's CDP kernels, so it is device-linked with cudadevrt (nvlink).

#include <cstdio>
#include <cuda.h>

#if defined(REF_APP_SSSP)
#include "sssp.h"
#define INF 1073741824
#define QMAXLENGTH 10240000
#define GM_BUFF_SIZE 10240000
#define WARP_SIZE 32
#define THREADS_PER_BLOCK 128
#define CONSOLIDATE_LEVEL 0
#include "sssp_kernel.cu"

#elif defined(REF_APP_COLOR)
#include "graph_color.h"
#define QMAXLENGTH 10240000
#define GM_BUFF_SIZE 10240000
#define WARP_SIZE 32
#define CONSOLIDATE_LEVEL 0
#include "graph_color_kernel.cu"

#elif defined(REF_APP_SPMV) || defined(REF_APP_PAGERANK)
#if defined(REF_APP_SPMV)
#include "SpMV.h"
#else
#include "pagerank.h"
#define DAMPING_FACTOR 0.5
#define EPSILON 1.0e-13
#endif
#define QMAXLENGTH 10240000
#define GM_BUFF_SIZE 10240000
#define THREADS_PER_BLOCK 128
#define CONSOLIDATE_LEVEL 0
__device__ __forceinline__ float ref_atomic_add(float* p, float v) { return atomicAdd(p, v); }
__device__ __forceinline__ int ref_atomic_add(int* p, int v) { return atomicAdd(p, v); }
__device__ __forceinline__ unsigned ref_atomic_add(unsigned* p, unsigned v) { return atomicAdd(p, v); }
#define atomicAdd ref_atomic_add
#define __shfl_down(v, d) __shfl_down_sync(0xffffffffu, (v), (d))
#if defined(REF_APP_SPMV)
#include "SpMV_kernel.cu"
#else
#define cudaDeviceSynchronize() (cudaSuccess)
#include "pagerank_kernel.cu"
#endif

#else
#error "define one of REF_APP_SSSP, REF_APP_COLOR, REF_APP_SPMV, REF_APP_PAGERANK"
#endif
