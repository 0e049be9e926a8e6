// SSSP entry point that allocates nothing: dpg_sssp_noalloc_dev (declared in include/dpg.h).
//
// Why it exists: some callers of this library must not allocate device memory, nor let a library
// do it for them. A serving engine that reserves the whole device pool at start-up and hands out
// slices of its own arena has nothing left for cudaMalloc, and its other streams would stall on
// the device-wide synchronisation that cudaMalloc/cudaFree can imply. A plugin host that gives its
// plugins only the buffers it owns, and audits every allocation, forbids them outright. The
// regular entry points need a dpg_ctx and a dpg_graph, and both allocate (status block, stream,
// frontier arena, device CSR). This one runs the same persistent SSSP kernel (binned work mapping)
// on caller-owned inputs and outputs, with its frontier queues, bitmaps, chunk lists and status
// words carved out of one file-scope __device__ array.
//
// Limits and sharing rules:
//   * at most kNoAllocMaxVertices vertices and kNoAllocMaxArcs arcs; larger graphs are rejected
//     with DPG_ERR_CAPACITY before anything is launched;
//   * the array (kNoAllocScratchBytes, 7 MiB) lives in every GPU that loads the library, until the
//     process exits;
//   * every call on a device uses the same array and leaves its contents behind; each call clears
//     what must start at zero, but calls whose GPU work overlaps (two host threads, two streams)
//     race on it, so callers must not let calls overlap;
//   * the caller's CSR is checked on the device before the expansion runs (offsets rise from 0 to
//     E, neighbour ids in [0, V), weights in [0, 2^30)); a bad graph returns DPG_ERR_INVALID_ARG
//     and nothing is relaxed;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress, which
//     may load the module) and keeps it for later calls on that device. The kept address belongs
//     to the device's primary context as it was at that call: after cudaDeviceReset the library
//     must be reloaded before this entry point is used again on that device.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "dpg_internal.h"
#include "dpg_kernels.h"

namespace dpg {
namespace {

constexpr int32_t kNoAllocMaxVertices = 1 << 18;  // 262,144
constexpr int64_t kNoAllocMaxArcs = 1 << 22;      // 4,194,304
constexpr int32_t kNoAllocHubDegree = 1024;
constexpr size_t kNoAllocScratchBytes = size_t(7) << 20;  // 7 MiB
constexpr int kMaxDevices = 64;

constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

struct NoAllocLayout {
    size_t qv, qse, bmp, chunks, qcount, ccount, status, check, total;
};

constexpr NoAllocLayout layout_for(int64_t V, int64_t E) {
    NoAllocLayout L{};
    const int64_t cap_v = V + 1;
    const int64_t chunked_raw = E / kNoAllocHubDegree + 1;
    const int64_t chunked = chunked_raw < V + 1 ? chunked_raw : V + 1;
    const int64_t cap_chunks = E / kHubChunk + chunked + 1;
    const int64_t words = (V + 31) / 32 + 1;
    L.qv = align256(sizeof(int32_t) * size_t(cap_v));
    L.qse = align256(sizeof(int2) * size_t(cap_v));
    L.bmp = align256(sizeof(uint32_t) * size_t(words));
    L.chunks = align256(sizeof(int4) * size_t(cap_chunks));
    L.qcount = align256(sizeof(uint32_t) * 4);
    L.ccount = align256(sizeof(uint32_t) * 4);
    L.status = align256(sizeof(DevStatus));
    L.check = align256(sizeof(int));
    L.total = 2 * (L.qv + L.qse + L.bmp + L.chunks) + L.qcount + L.ccount + L.status + L.check;
    return L;
}

static_assert(layout_for(kNoAllocMaxVertices, kNoAllocMaxArcs).total <= kNoAllocScratchBytes,
              "the no-alloc scratch array must hold the workspace of the largest accepted graph");

// The scratch itself. In host code this name is only a handle for cudaGetSymbolAddress; the kernels
// receive the device address obtained below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The caller's CSR, checked before anything is relaxed: *bad |= 1 for a neighbour id outside
// [0, V), 2 for a weight outside [0, 2^30) (sums of two stay below 2^31), 4 for offsets that do
// not rise from 0 to E. The reads stay inside the arrays the caller declared: offsets [0, V],
// pairs [0, E).
__global__ void noalloc_check_kernel(const int32_t* __restrict__ off, const int2* __restrict__ adj, int32_t V,
                                     int64_t E, int* bad) {
    const int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    int flags = 0;
    for (int64_t v = tid; v < V; v += stride)
        if (off[v + 1] < off[v]) flags |= 4;
    if (tid == 0 && (off[0] != 0 || static_cast<int64_t>(off[V]) != E)) flags |= 4;
    for (int64_t e = tid; e < E; e += stride) {
        const int2 a = adj[e];
        if (a.x < 0 || a.x >= V) flags |= 1;
        if (a.y < 0 || a.y >= DPG_INF_COST) flags |= 2;
    }
    if (flags) atomicOr(bad, flags);
}

std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

dpg_status scratch_address(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices) return set_error(DPG_ERR_INVALID_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_error(DPG_ERR_CUDA, std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
        g_scratch_addr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch_addr[device]);
    return DPG_OK;
}

}  // namespace
}  // namespace dpg

using namespace dpg;

extern "C" dpg_status dpg_sssp_noalloc_dev(int32_t V, int64_t E, const int32_t* d_offsets, const int32_t* d_adj_pairs,
                                           int32_t source, int32_t* d_dist, void* stream) {
    if (V < 1 || E < 0) return set_error(DPG_ERR_INVALID_ARG, "dpg_sssp_noalloc_dev: need V >= 1 and E >= 0");
    if (V > kNoAllocMaxVertices || E > kNoAllocMaxArcs)
        return set_error(DPG_ERR_CAPACITY, "dpg_sssp_noalloc_dev: graph exceeds the no-alloc scratch limit of " +
                                               std::to_string(kNoAllocMaxVertices) + " vertices and " +
                                               std::to_string(kNoAllocMaxArcs) + " arcs");
    if (!d_offsets || !d_dist || (E > 0 && !d_adj_pairs))
        return set_error(DPG_ERR_INVALID_ARG, "dpg_sssp_noalloc_dev: null device pointer");
    if (reinterpret_cast<uintptr_t>(d_adj_pairs) % alignof(int2) != 0)
        return set_error(DPG_ERR_INVALID_ARG, "dpg_sssp_noalloc_dev: adjacency pairs must be 8-byte aligned");
    if (source < 0 || source >= V) return set_error(DPG_ERR_INVALID_ARG, "dpg_sssp_noalloc_dev: source out of range");
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return set_error(DPG_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    unsigned char* base = nullptr;
    dpg_status s = scratch_address(device, &base);
    if (s != DPG_OK) return s;
    int sm_count = 0;
    e = cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return set_error(DPG_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));

    const NoAllocLayout Lo = layout_for(V, E);
    ExpandWorkspace ws;
    memset(&ws, 0, sizeof(ws));
    ws.cap_v = int64_t(V) + 1;
    ws.cap_chunks = expand_chunk_capacity(V, E, kNoAllocHubDegree);
    ws.bmp_words = (V + 31) / 32 + 1;
    unsigned char* p = base;
    for (int k = 0; k < 2; ++k) {
        ws.qv[k] = reinterpret_cast<int32_t*>(p); p += Lo.qv;
        ws.qse[k] = reinterpret_cast<int2*>(p); p += Lo.qse;
        ws.bmp[k] = reinterpret_cast<uint32_t*>(p); p += Lo.bmp;
        ws.chunks[k] = reinterpret_cast<int4*>(p); p += Lo.chunks;
    }
    ws.qcount = reinterpret_cast<uint32_t*>(p); p += Lo.qcount;
    ws.ccount = reinterpret_cast<uint32_t*>(p); p += Lo.ccount;
    DevStatus* st = reinterpret_cast<DevStatus*>(p); p += Lo.status;
    int* bad = reinterpret_cast<int*>(p);

    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    // The status and check words keep the previous call's contents: start this call from clean
    // ones. The expansion's init kernel clears the queues' counters and both bitmaps.
    e = cudaMemsetAsync(st, 0, sizeof(DevStatus), cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), cs);
    if (e != cudaSuccess) return set_error(DPG_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    // The expansion trusts its graph (an out-of-range id would make it write outside d_dist), so the
    // check completes before it is launched.
    int check_blocks = static_cast<int>((std::max<int64_t>(V, E) + 255) / 256);
    if (check_blocks > sm_count * 4) check_blocks = sm_count * 4;
    noalloc_check_kernel<<<check_blocks, 256, 0, cs>>>(d_offsets, reinterpret_cast<const int2*>(d_adj_pairs), V, E,
                                                       bad);
    int flags = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, bad, sizeof(int), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) return set_error(DPG_ERR_CUDA, std::string("no-alloc graph check: ") + cudaGetErrorString(e));
    if (flags & 4) return set_error(DPG_ERR_INVALID_ARG, "dpg_sssp_noalloc_dev: offsets must rise from 0 to E");
    if (flags & 1) return set_error(DPG_ERR_INVALID_ARG, "dpg_sssp_noalloc_dev: neighbour id outside [0, V)");
    if (flags & 2) return set_error(DPG_ERR_INVALID_ARG, "dpg_sssp_noalloc_dev: weight outside [0, 2^30)");

    ExpandLaunch L;
    L.off = d_offsets;
    L.col = nullptr;
    L.adj = reinterpret_cast<const int2*>(d_adj_pairs);
    L.V = V;
    L.E = E;
    L.label = d_dist;
    L.source = source;
    L.bfs = false;
    L.solution = DPG_SOL_BINNED;
    L.threshold = DPG_REF_THRESHOLD;
    L.hub_threshold = kNoAllocHubDegree;
    L.max_iter = V + 2;
    L.timeout_ns = 10ull * 1000000000ull;
    e = launch_expand(L, ws, st, cs, sm_count, nullptr, nullptr, nullptr);
    if (e != cudaSuccess) return set_error(DPG_ERR_CUDA, std::string("no-alloc SSSP launch: ") + cudaGetErrorString(e));
    int err[2] = {0, 0};
    e = cudaMemcpyAsync(err, st, sizeof(err), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) return set_error(DPG_ERR_CUDA, std::string("no-alloc SSSP status: ") + cudaGetErrorString(e));
    if (err[0] != 0) {
        const dpg_status ds = static_cast<dpg_status>(err[0]);
        return set_error(ds, std::string("device reported ") + dpg_status_string(ds) + " (site " + std::to_string(err[1]) + ")");
    }
    return DPG_OK;
}
