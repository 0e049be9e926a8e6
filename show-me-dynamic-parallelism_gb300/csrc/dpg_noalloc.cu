// SSSP entry point that allocates nothing: dpg_sssp_noalloc_dev (declared in include/dpg.h).
//
// Why it exists: some callers of this library cannot allocate device memory themselves or let a
// library do it. Examples are code running inside a CUDA-graph capture, and engines that own the
// whole device pool (a serving runtime with a fixed arena, an allocator-less plugin host) and
// forbid cudaMalloc/cudaFree behind their back. The regular entry points need a dpg_ctx and a
// dpg_graph, and both allocate (status block, stream, frontier arena, device CSR). This one runs
// the same persistent SSSP kernel (binned work mapping) on caller-owned inputs and outputs, with
// its frontier queues, bitmaps, chunk lists and status word carved out of one file-scope
// __device__ array.
//
// Limits and sharing rules:
//   * at most kNoAllocMaxVertices vertices and kNoAllocMaxArcs arcs; larger graphs are rejected
//     with DPG_ERR_CAPACITY before anything is launched;
//   * the array (kNoAllocScratchBytes, 7 MiB) lives in every GPU that loads the library, until the
//     process exits;
//   * every call on a device uses the same array and leaves its contents behind; each call clears
//     what must start at zero, but calls whose GPU work overlaps (two host threads, two streams)
//     race on it, so callers must not let calls overlap;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress, which
//     may load the module); make that first call before any stream capture.

#include <cuda_runtime.h>

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
    size_t qv, qse, bmp, chunks, qcount, ccount, status, total;
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
    L.total = 2 * (L.qv + L.qse + L.bmp + L.chunks) + L.qcount + L.ccount + L.status;
    return L;
}

static_assert(layout_for(kNoAllocMaxVertices, kNoAllocMaxArcs).total <= kNoAllocScratchBytes,
              "the no-alloc scratch array must hold the workspace of the largest accepted graph");

// The scratch itself. In host code this name is only a handle for cudaGetSymbolAddress; the kernels
// receive the device address obtained below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

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
    DevStatus* st = reinterpret_cast<DevStatus*>(p);

    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    // The status word keeps the previous call's contents: start this call from a clean one. The
    // expansion's init kernel clears the queues' counters and both bitmaps.
    e = cudaMemsetAsync(st, 0, sizeof(DevStatus), cs);
    if (e != cudaSuccess) return set_error(DPG_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));

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
