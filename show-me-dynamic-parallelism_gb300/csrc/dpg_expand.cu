// Frontier expansion for SSSP and BFS: one persistent cooperative kernel per solve.
//
// The reference runs one host-loop iteration per frontier (sssp_wrapper.cu:241-298): launch the
// relaxation kernel, memset, regenerate the queue by scanning all V update flags
// (unorder_generateQueue_kernel, sssp_kernel.cu:496-506), and copy the queue length back to the
// host. High-degree vertices go to CDP child launches consolidated per warp, block or grid
// (sssp_kernel.cu:180-387; bfs_rec_kernel.cu:158-457).
//
// Here the whole traversal is one launch. Each iteration pops a compacted frontier, relaxes with
// the reference's operator (sssp_kernel.cu:52-58: alt = cost[u] + w; if cost[v] > alt then
// atomicMin and mark v), pushes improved vertices into the next frontier with warp-aggregated
// appends and a per-vertex bitmap for de-duplication, and ends at a bounded grid barrier. The
// reference's consolidation levels become in-kernel work mappings instead of child launches:
//   DPG_SOL_THREAD  thread per vertex, serial neighbour loop            (-s 0)
//   DPG_SOL_NAIVE   degree >= threshold: a warp per vertex, right away  (-s 1)
//   DPG_SOL_WARP    degree >= threshold: consolidated per warp and expanded by the warp with a
//                   scan-based gather over all consolidated rows            (-s 2)
//   DPG_SOL_BLOCK   degree >= threshold: consolidated per CTA in shared memory and expanded by the
//                   whole CTA                                               (-s 3)
//   DPG_SOL_GRID    degree >= threshold: consolidated grid-wide at push time and expanded by every
//                   warp of the grid in 256-arc chunks                       (-s 4)
//   DPG_SOL_BINNED  binned at push time: below hub_threshold (default 32) into the small queue,
//                   expanded by warp scan-gathers over 32 vertices; at or above it cut into 256-arc
//                   chunks over every warp, so no work item exceeds 8 warp steps (default)
// BFS uses the same machinery with level[v] set once by atomicCAS (bfs_rec_kernel.cu:76-78).

#include <cuda_runtime.h>

#include <cstring>
#include <type_traits>

#include "dpg_kernels.h"

namespace dpg {
namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;

struct ExpandParams {
    const int32_t* __restrict__ off;
    const int32_t* __restrict__ col;
    const int2* __restrict__ adj;
    int32_t* label;
    int32_t V;
    int32_t threshold;
    int32_t hub_threshold;
    int32_t max_iter;
    unsigned long long timeout_ns;
    ExpandWorkspace ws;
    DevStatus* st;
    unsigned long long* trace;
    int32_t trace_cap;
    int32_t* aux;  // colouring: pending lower-neighbour count per vertex
    // Multi-source SSSP (MaskSsspOp): label[v * nsrc + k] is v's distance from source k of v's
    // graph; dirty[p][v] = (iteration tag << 32) | mask of the sources whose label of v changed.
    int32_t nsrc;
    unsigned long long* dirty[2];
    // Direction-optimizing BFS (DPG_SOL_DIROPT): in-arcs, and per rotating parity the out-degree sum
    // (mf) and the size (nf) of the frontier pushed into it.
    const int32_t* t_off;
    const int32_t* t_col;
    unsigned long long* mf;
    unsigned* nf;
    int64_t E;
    // Near-far SSSP (DPG_SOL_NEARFAR): three rotating piles of deferred {vertex, distance} pairs.
    int2* far[3];
    unsigned* far_count;  // [3]
    int* far_min;         // [3] smallest distance pushed into each pile
    int64_t far_cap;
    int32_t delta;
    // Multi-source SSSP: non-zero when nsrc is a multiple of 4 and the labels are 16-byte aligned,
    // so a vertex's labels can be read four at a time (relax_mask_vec4).
    int32_t label_vec4;
};

// Operator interface of the expansion:
//   RV                     type of the value carried with a popped vertex
//   row_value(u)           that value (its label, or its id)
//   load_edge(e, rv)       label index v, adjacency row r and candidate value of arc e's head
//   want(v, cand, cur)     cheap filter before the atomic (cur = label[v] when kPeek)
//   commit(v, cand)        the atomic update; true when v must be pushed
//   min_blocks(CH)         CTAs per SM the kernel is compiled for (its register budget). A bound is
//                          always given: without one the compiler picks its own, and an explicit 1
//                          lets it spend up to 110 registers where it would otherwise use 64.
//                          Single-source SSSP on R-MAT scale 24 took 8.6-9.1 ms at 3 CTAs (80
//                          registers) against 9.3 ms at 2. The binned and direction-optimizing
//                          kernels also have a kWideBlocks build for graphs with hubs.
struct SsspOp {
    using RV = int;
    static constexpr bool kDedup = true;
    static constexpr bool kPeek = true;
    static constexpr bool kMask = false;
    static constexpr int min_blocks(int) { return 3; }
    __device__ __forceinline__ static int row_value(const ExpandParams& P, int u, int) { return __ldcg(P.label + u); }
    __device__ __forceinline__ static void load_edge(const ExpandParams& P, int e, int du, int& v, int& r,
                                                     int& cand) {
        const int2 a = __ldg(P.adj + e);
        v = a.x;
        r = a.x;
        cand = du + a.y;
    }
    // Read-before-atomic filter (sssp_kernel.cu:55): labels only decrease, so a stale read can only
    // cause an extra atomic, never a missed improvement.
    __device__ __forceinline__ static bool want(int, int cand, int cur) { return cand < cur; }
    __device__ __forceinline__ static bool commit(const ExpandParams& P, int v, int cand) {
        return cand < atomicMin(P.label + v, cand);
    }
};

struct BfsOp {
    using RV = int;
    static constexpr bool kDedup = false;
    static constexpr bool kPeek = true;
    static constexpr bool kMask = false;
    static constexpr int min_blocks(int) { return 3; }
    // Levels are claimed once, level-synchronously (top-down pushes and bottom-up claims of
    // iteration j both set j + 1), so a vertex popped in iteration j has level j: no load needed.
    __device__ __forceinline__ static int row_value(const ExpandParams&, int, int j) { return j; }
    __device__ __forceinline__ static void load_edge(const ExpandParams& P, int e, int du, int& v, int& r,
                                                     int& cand) {
        v = __ldg(P.col + e);
        r = v;
        cand = du + 1;
    }
    __device__ __forceinline__ static bool want(int, int, int cur) { return cur == DPG_UNDEFINED_LEVEL; }
    __device__ __forceinline__ static bool commit(const ExpandParams& P, int v, int cand) {
        return atomicCAS(P.label + v, DPG_UNDEFINED_LEVEL, cand) == DPG_UNDEFINED_LEVEL;
    }
};

// Greedy colouring (graph_color_kernel.cu:28-49): colour(v) = 1 + max colour of its out-neighbours
// u < v. The expansion runs over the transposed graph: a coloured u decrements the pending count of
// every in-neighbour v > u, and the decrement that reaches zero colours v and pushes it.
struct ColorOp {
    using RV = int;
    static constexpr bool kDedup = false;
    static constexpr bool kPeek = false;
    static constexpr bool kMask = false;
    static constexpr int min_blocks(int) { return 3; }
    __device__ __forceinline__ static int row_value(const ExpandParams&, int u, int) { return u; }
    __device__ __forceinline__ static void load_edge(const ExpandParams& P, int e, int u, int& v, int& r, int& cand) {
        v = __ldg(P.col + e);
        r = v;
        cand = u;
    }
    __device__ __forceinline__ static bool want(int v, int u, int) { return v > u; }
    __device__ __forceinline__ static bool commit(const ExpandParams& P, int v, int u) {
        if (atomicSub(P.aux + v, 1) != 1) return false;
        P.label[v] = __ldcg(P.label + u) + 1;
        return true;
    }
};

// SSSP from up to 32 sources per graph at once (a batch of graphs packed as one union CSR), in the
// manner of multi-source traversal (Then et al., "The More the Merrier: Efficient Multi-Source
// Graph Traversal", VLDB 2014): a frontier entry is a vertex with the mask of the sources whose
// label of it changed, its labels label[v * nsrc + k] sit side by side, and one scan of its arcs
// serves every source in the mask. The marks for the next frontier are 64-bit words
// (iteration tag << 32 | mask) in a parity-indexed array: a tag other than the current iteration's
// reads as an empty mask, so no clearing pass is needed.
struct MaskSsspOp {
    using RV = int2;  // {vertex, source mask}
    static constexpr bool kDedup = false;
    static constexpr bool kMask = true;
    // 64 registers (4 CTAs) with 128- and 256-arc chunks, 128 (2 CTAs) with 512: the batch autotuner
    // compares the three.
    static constexpr int min_blocks(int ch) { return ch >= 512 ? 2 : 4; }
    __device__ __forceinline__ static int2 row_value(const ExpandParams& P, int u, int j) {
        const unsigned long long w = __ldcg(P.dirty[j & 1] + u);
        const unsigned mask = (w >> 32) == static_cast<unsigned long long>(static_cast<unsigned>(j))
                                  ? static_cast<unsigned>(w) : 0u;
        return make_int2(u, static_cast<int>(mask));
    }
};

// Adds `bits` to v's mark for the iteration `tag`; true when this call made the first mark of the
// iteration (v must be pushed). A word changes at most nsrc + 1 times per iteration, so the loop
// ends after at most that many failed compare-and-swaps.
__device__ __forceinline__ bool tag_or(unsigned long long* w, unsigned tag, unsigned bits) {
    const unsigned long long tg = static_cast<unsigned long long>(tag) << 32;
    unsigned long long old = __ldcg(w);
    for (;;) {
        const bool fresh = (old >> 32) == static_cast<unsigned long long>(tag);
        const unsigned long long want = fresh ? (old | bits) : (tg | bits);
        if (want == old) return false;
        const unsigned long long prev = atomicCAS(w, old, want);
        if (prev == old) return !fresh;
        old = prev;
    }
}

// Multi-source relaxation of one arc (tail labels lu, head labels lv, weight w) for the sources in
// mask m, eight sources at a time: two 16-byte loads of the tail's labels and two of the head's,
// then an atomicMin for every source whose candidate beats the head's label, all issued before any
// result is used. Source by source, each needed a load and then its atomic, and an atomic keeps
// the next source's loads from being issued ahead of it: two round trips per source in the mask
// instead of two per eight. Returns the mask of the sources whose label of the head this call
// lowered. Needs nsrc % 4 == 0 and 16-byte aligned labels; a group's upper four labels are read
// only when the mask has a bit there, so nsrc = 4 (mod 8) reads nothing past the vertex.
__device__ __forceinline__ unsigned relax_mask_vec4(int nsrc, const int32_t* lu, int32_t* lv, int w, unsigned m) {
    unsigned bits = 0;
    for (int g0 = 0; g0 < nsrc; g0 += 8) {
        const unsigned mm = (m >> g0) & 0xFFu;
        if (mm == 0u) continue;
        const int4* tl = reinterpret_cast<const int4*>(lu + g0);
        const int4* hl = reinterpret_cast<const int4*>(lv + g0);
        int4 t0 = make_int4(0, 0, 0, 0), t1 = t0, h0 = t0, h1 = t0;
        if (mm & 0x0Fu) {
            t0 = __ldcg(tl);
            h0 = __ldcg(hl);
        }
        if (mm & 0xF0u) {
            t1 = __ldcg(tl + 1);
            h1 = __ldcg(hl + 1);
        }
        const int t[8] = {t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z, t1.w};
        const int h[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
        int cand[8], old[8];
        unsigned want = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            cand[q] = t[q] + w;
            if (((mm >> q) & 1u) && cand[q] < h[q]) want |= 1u << q;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) old[q] = ((want >> q) & 1u) ? atomicMin(lv + g0 + q, cand[q]) : 0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (((want >> q) & 1u) && cand[q] < old[q]) bits |= 1u << (g0 + q);
    }
    return bits;
}

// tag_or starting from a value of the word read earlier (`seen`): the first compare-and-swap goes out
// at once, and a stale `seen` only costs a retry. Each failed swap means the word changed after
// `seen` was read, at most nsrc + 1 times in an iteration, so the loop ends.
__device__ __forceinline__ bool tag_or_from(unsigned long long* w, unsigned tag, unsigned bits,
                                            unsigned long long seen) {
    const unsigned long long tg = static_cast<unsigned long long>(tag) << 32;
    unsigned long long old = seen;
    for (;;) {
        const bool fresh = (old >> 32) == static_cast<unsigned long long>(tag);
        const unsigned long long want = fresh ? (old | bits) : (tg | bits);
        if (want == old) return false;
        const unsigned long long prev = atomicCAS(w, old, want);
        if (prev == old) return !fresh;
        old = prev;
    }
}

// Up to 8 sources (nsrc <= 8, labels 16-byte aligned), G arcs at a time in three phases: the
// tail's and head's labels of every arc (16-byte loads), then the atomicMin of every improving
// source of every arc together with a read of each improved head's mark word, then the marks'
// compare-and-swaps. A chain of three round trips per G arcs.
template <int G>
__device__ __forceinline__ void relax_mask8_group(const ExpandParams& P, unsigned long long* dirty, unsigned tag,
                                                  const unsigned (&m)[G], const int (&tail)[G],
                                                  const int (&head)[G], const int (&w)[G], bool (&ok)[G]) {
    int4 t0[G], t1[G], h0[G], h1[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
        const int4* tl = reinterpret_cast<const int4*>(P.label + static_cast<int64_t>(tail[g]) * P.nsrc);
        const int4* hl = reinterpret_cast<const int4*>(P.label + static_cast<int64_t>(head[g]) * P.nsrc);
        t0[g] = make_int4(0, 0, 0, 0);
        t1[g] = t0[g];
        h0[g] = t0[g];
        h1[g] = t0[g];
        if (m[g] & 0x0Fu) {
            t0[g] = __ldcg(tl);
            h0[g] = __ldcg(hl);
        }
        if (m[g] & 0xF0u) {
            t1[g] = __ldcg(tl + 1);
            h1[g] = __ldcg(hl + 1);
        }
    }
    unsigned want[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
        const int t[8] = {t0[g].x, t0[g].y, t0[g].z, t0[g].w, t1[g].x, t1[g].y, t1[g].z, t1[g].w};
        const int h[8] = {h0[g].x, h0[g].y, h0[g].z, h0[g].w, h1[g].x, h1[g].y, h1[g].z, h1[g].w};
        want[g] = 0u;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (((m[g] >> q) & 1u) && t[q] + w[g] < h[q]) want[g] |= 1u << q;
    }
    int old[G][8];
    unsigned long long seen[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
        const int t[8] = {t0[g].x, t0[g].y, t0[g].z, t0[g].w, t1[g].x, t1[g].y, t1[g].z, t1[g].w};
        int32_t* lv = P.label + static_cast<int64_t>(head[g]) * P.nsrc;
#pragma unroll
        for (int q = 0; q < 8; ++q) old[g][q] = ((want[g] >> q) & 1u) ? atomicMin(lv + q, t[q] + w[g]) : 0;
        seen[g] = want[g] ? __ldcg(dirty + head[g]) : 0ull;
    }
#pragma unroll
    for (int g = 0; g < G; ++g) {
        const int t[8] = {t0[g].x, t0[g].y, t0[g].z, t0[g].w, t1[g].x, t1[g].y, t1[g].z, t1[g].w};
        unsigned bits = 0u;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (((want[g] >> q) & 1u) && t[q] + w[g] < old[g][q]) bits |= 1u << q;
        ok[g] = bits != 0u && tag_or_from(dirty + head[g], tag, bits, seen[g]);
    }
}

__device__ __forceinline__ int shfl_rv(int v, int src) { return __shfl_sync(kFullMask, v, src); }
__device__ __forceinline__ int2 shfl_rv(int2 v, int src) {
    return make_int2(__shfl_sync(kFullMask, v.x, src), __shfl_sync(kFullMask, v.y, src));
}

// Destination buffers of one iteration's pushes.
struct PushCtx {
    int32_t* qv;
    int2* qse;
    uint32_t* qcount;
    uint32_t* bmp;
    int4* chunks;
    uint32_t* ccount;
    unsigned long long* dirty;  // MaskSsspOp: marks of the next frontier
    unsigned tag;               // MaskSsspOp: iteration of the next frontier
    unsigned long long* mf;     // direction-optimizing BFS: out-degree sum of the next frontier
    unsigned* nf;               // direction-optimizing BFS: size of the next frontier
    int2* far;                  // near-far SSSP: pile receiving distances >= threshold (null: off)
    unsigned* far_count;
    int* far_min;
    int threshold;
    // Small iterations (latency-bound): each candidate head's row range is loaded with its label
    // peek, so a push needs no further round trip.
    bool early_rows;
    // The warp's push buffer in shared memory (see flush_pushes) and its share of the frontier
    // statistics, added to mf / nf once per iteration.
    int* buf_v;
    int2* buf_se;
    unsigned* buf_n;
    unsigned long long* buf_mf;
    unsigned* buf_nf;
};

// Frontier vertices a warp collects in shared memory before it reserves their queue slots with one
// atomic: every warp appending to the same global counter serialised on that address (R-MAT 24:
// about 3 M appends per SSSP solve, 0.5 M in one bottom-up BFS step).
constexpr int kPushBuf = 256;
constexpr unsigned long long kPushBufferWork = 65536;  // arcs per iteration from which pushes are buffered

__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) {
    return *reinterpret_cast<const volatile unsigned*>(p);
}
// The warp's buffered frontier vertices go to the global queue behind one reservation, and its
// frontier statistics to mf / nf. All 32 lanes call it; every warp calls it before the iteration's
// grid barrier, so the next iteration sees the whole frontier.
__device__ __forceinline__ void flush_pushes(const ExpandParams& P, const PushCtx& Q) {
    if (!Q.buf_n) return;  // this iteration pushes straight to the queue
    const int lane = lane_id();
    const unsigned n = *reinterpret_cast<volatile unsigned*>(Q.buf_n);
    if (n) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(Q.qcount, n);
        base = __shfl_sync(kFullMask, base, 0);
        for (unsigned i = lane; i < n; i += 32) {
            const unsigned pos = base + i;
            if (pos < static_cast<unsigned long long>(P.ws.cap_v)) {
                __stcg(Q.qv + pos, Q.buf_v[i]);
                __stcg(Q.qse + pos, Q.buf_se[i]);
            } else {
                raise_error(P.st, DPG_ERR_CAPACITY, 11);
            }
        }
    }
    __syncwarp();
    if (lane == 0) {
        *Q.buf_n = 0u;
        if (Q.mf && *Q.buf_nf) {
            atomicAdd(Q.mf, *Q.buf_mf);
            atomicAdd(Q.nf, *Q.buf_nf);
            *Q.buf_mf = 0ull;
            *Q.buf_nf = 0u;
        }
    }
    __syncwarp();
}

// Called by all 32 lanes together with U candidate slots each; ok[u] marks slots whose relaxation
// improved vertex v[u]. Vertices below the chunking degree go to the small queue with one
// warp-aggregated append for all U slots; chunked vertices get their chunk range from one
// warp-aggregated atomic per slot and the warp writes every chunk descriptor.
template <class Op, bool kClassify, int CH, int U>
__device__ __forceinline__ void push_batch(const ExpandParams& P, const PushCtx& Q, bool (&ok)[U],
                                           const int (&v)[U], const int (&row)[U], const int2* se_pre = nullptr) {
    bool any = false;
#pragma unroll
    for (int u = 0; u < U; ++u) any |= ok[u];
    if (!__any_sync(kFullMask, any)) return;
    // Row ranges: passed in by a caller that fetched them ahead (se_pre[u]), or loaded here, issued
    // together with the de-duplication atomics so the two share one round trip (a head that the
    // bitmap then drops wasted its two loads).
    int s[U], e[U];
    unsigned old[U];
#pragma unroll
    for (int u = 0; u < U; ++u) old[u] = (Op::kDedup && ok[u]) ? atomicOr(Q.bmp + (v[u] >> 5), 1u << (v[u] & 31)) : 0u;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        s[u] = 0;
        e[u] = 0;
        if (se_pre) {
            s[u] = ok[u] ? se_pre[u].x : 0;
            e[u] = ok[u] ? se_pre[u].y : 0;
        } else if (ok[u]) {
            s[u] = __ldg(P.off + row[u]);
            e[u] = __ldg(P.off + row[u] + 1);
        }
    }
    if (Op::kDedup) {
#pragma unroll
        for (int u = 0; u < U; ++u) ok[u] = ok[u] && (old[u] & (1u << (v[u] & 31))) == 0u;
    }
    const int lane = lane_id();
    const unsigned lt = (1u << lane) - 1u;
    bool chunked[U];
    unsigned m[U];
    unsigned cnt = 0;
    unsigned long long degs = 0;
    unsigned pushed = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        ok[u] = ok[u] && e[u] > s[u];  // vertices without out-arcs never need expanding
        chunked[u] = kClassify && ok[u] && (e[u] - s[u]) >= P.hub_threshold;
        m[u] = __ballot_sync(kFullMask, ok[u] && !chunked[u]);
        cnt += static_cast<unsigned>(__popc(m[u]));
        degs += ok[u] ? static_cast<unsigned long long>(e[u] - s[u]) : 0ull;
        pushed += ok[u] ? 1u : 0u;
    }
    if (Q.mf) {  // frontier statistics for the direction choice (added up per warp when buffering)
        degs = warp_sum_u64(degs);
        pushed = static_cast<unsigned>(warp_sum_u64(pushed));
        if (lane == 0 && pushed) {
            if (Q.buf_n) {
                *Q.buf_mf += degs;
                *Q.buf_nf += pushed;
            } else {
                atomicAdd(Q.mf, degs);
                atomicAdd(Q.nf, pushed);
            }
        }
    }
    if (cnt > static_cast<unsigned>(kPushBuf) || !Q.buf_n) {
        // A batch larger than the buffer (512-arc chunks), or a caller without one: its own
        // reservation.
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(Q.qcount, cnt);
        base = __shfl_sync(kFullMask, base, 0);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (ok[u] && !chunked[u]) {
                const unsigned pos = base + static_cast<unsigned>(__popc(m[u] & lt));
                if (pos < static_cast<unsigned long long>(P.ws.cap_v)) {
                    __stcg(Q.qv + pos, v[u]);
                    __stcg(Q.qse + pos, make_int2(s[u], e[u]));
                } else {
                    raise_error(P.st, DPG_ERR_CAPACITY, 11);
                }
            }
            base += static_cast<unsigned>(__popc(m[u]));
        }
    } else if (cnt) {
        unsigned n0 = *reinterpret_cast<volatile unsigned*>(Q.buf_n);
        if (n0 + cnt > static_cast<unsigned>(kPushBuf)) {
            flush_pushes(P, Q);
            n0 = 0;
        }
        unsigned base = n0;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (ok[u] && !chunked[u]) {
                const unsigned pos = base + static_cast<unsigned>(__popc(m[u] & lt));
                Q.buf_v[pos] = v[u];
                Q.buf_se[pos] = make_int2(s[u], e[u]);
            }
            base += static_cast<unsigned>(__popc(m[u]));
        }
        __syncwarp();
        if (lane == 0) *Q.buf_n = n0 + cnt;
        __syncwarp();
    }
    if (kClassify) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            unsigned hm = __ballot_sync(kFullMask, chunked[u]);
            if (!hm) continue;
            const int nch = chunked[u] ? (e[u] - s[u] + CH - 1) / CH : 0;
            const int incl = warp_inclusive_scan(nch);
            const int total = __shfl_sync(kFullMask, incl, 31);
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(Q.ccount, static_cast<unsigned>(total));
            base = __shfl_sync(kFullMask, base, 0);
            const unsigned my_first = base + static_cast<unsigned>(incl - nch);
            if (static_cast<unsigned long long>(base) + total > static_cast<unsigned long long>(P.ws.cap_chunks)) {
                if (lane == 0) raise_error(P.st, DPG_ERR_CAPACITY, 10);
                hm = 0u;
            }
            while (hm) {  // the whole warp writes one chunked vertex's descriptors at a time
                const int src = __ffs(hm) - 1;
                hm &= hm - 1u;
                const int hv = __shfl_sync(kFullMask, v[u], src);
                const int hs = __shfl_sync(kFullMask, s[u], src);
                const int he = __shfl_sync(kFullMask, e[u], src);
                const unsigned first = __shfl_sync(kFullMask, my_first, src);
                const int hn = (he - hs + CH - 1) / CH;
                for (int c = lane; c < hn; c += 32) {
                    const int k0 = hs + c * CH;
                    __stcg(Q.chunks + first + c, make_int4(hv, k0, min(he, k0 + CH), c == 0 ? 1 : 0));
                }
            }
        }
    }
}

// Near-far: appends the slots with ok[u] to the far pile as {vertex, distance} (warp-aggregated),
// and lowers the pile's minimum distance.
template <int U>
__device__ __forceinline__ void far_push(const ExpandParams& P, const PushCtx& Q, const bool (&ok)[U],
                                         const int (&v)[U], const int (&c)[U]) {
    const int lane = lane_id();
    const unsigned lt = (1u << lane) - 1u;
    unsigned m[U];
    unsigned cnt = 0;
    int cmin = 0x7FFFFFFF;
#pragma unroll
    for (int u = 0; u < U; ++u) {
        m[u] = __ballot_sync(kFullMask, ok[u]);
        cnt += static_cast<unsigned>(__popc(m[u]));
        if (ok[u]) cmin = min(cmin, c[u]);
    }
    if (cnt == 0) return;
    cmin = __reduce_min_sync(kFullMask, cmin);
    unsigned base = 0;
    if (lane == 0) {
        base = atomicAdd(Q.far_count, cnt);
        atomicMin(Q.far_min, cmin);
    }
    base = __shfl_sync(kFullMask, base, 0);
#pragma unroll
    for (int u = 0; u < U; ++u) {
        if (ok[u]) {
            const unsigned pos = base + static_cast<unsigned>(__popc(m[u] & lt));
            if (static_cast<int64_t>(pos) < P.far_cap) __stcg(Q.far + pos, make_int2(v[u], c[u]));
            else raise_error(P.st, DPG_ERR_CAPACITY, 14);
        }
        base += static_cast<unsigned>(__popc(m[u]));
    }
}

// U independent relaxations per lane, issued phase by phase (U adjacency loads, U label loads, U
// atomics, one batched push) so each warp keeps U memory operations in flight instead of one.
template <class Op, bool kClassify, int CH, int U>
__device__ __forceinline__ void relax_batch(const ExpandParams& P, const PushCtx& Q, const bool (&act)[U],
                                            const int (&e)[U], const typename Op::RV (&du)[U]) {
    int v[U], row[U];
    bool ok[U];
    if constexpr (Op::kMask) {
        // One adjacency read per arc; then, per source in the tail's mask, the reference's
        // relaxation (sssp_kernel.cu:52-58) on that source's label of the head.
        int w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            v[u] = 0;
            w[u] = 0;
            if (act[u]) {
                const int2 a = __ldg(P.adj + e[u]);
                v[u] = a.x;
                w[u] = a.y;
            }
            row[u] = v[u];
        }
        if (P.label_vec4 && P.nsrc <= 8) {
            constexpr int G = (U >= 2 && Op::min_blocks(CH) <= 2) ? 2 : 1;
#pragma unroll
            for (int u0 = 0; u0 < U; u0 += G) {
                unsigned m[G];
                int tail[G], head[G], wg[G];
                bool okg[G];
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    m[g] = act[u0 + g] ? static_cast<unsigned>(du[u0 + g].y) : 0u;
                    tail[g] = du[u0 + g].x;
                    head[g] = v[u0 + g];
                    wg[g] = w[u0 + g];
                }
                relax_mask8_group<G>(P, Q.dirty, Q.tag, m, tail, head, wg, okg);
#pragma unroll
                for (int g = 0; g < G; ++g) ok[u0 + g] = okg[g];
            }
        } else {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            unsigned m = act[u] ? static_cast<unsigned>(du[u].y) : 0u;
            const int32_t* lu = P.label + static_cast<int64_t>(du[u].x) * P.nsrc;
            int32_t* lv = P.label + static_cast<int64_t>(v[u]) * P.nsrc;
            unsigned bits = 0;
            if (P.label_vec4) {
                if (m) bits = relax_mask_vec4(P.nsrc, lu, lv, w[u], m);
            } else {
                while (m) {
                    const int k = __ffs(m) - 1;
                    m &= m - 1u;
                    const int cand = __ldcg(lu + k) + w[u];
                    if (cand < __ldcg(lv + k) && cand < atomicMin(lv + k, cand)) bits |= 1u << k;
                }
            }
            ok[u] = bits != 0u && tag_or(Q.dirty + v[u], Q.tag, bits);
        }
        }
    } else {
        // Inactive lanes load arc 0 (the adjacency always holds at least one entry) and the label of
        // its head, so the loads need no branch; only the atomic depends on act.
        int cand[U], cur[U];
#pragma unroll
        for (int u = 0; u < U; ++u) Op::load_edge(P, act[u] ? e[u] : 0, du[u], v[u], row[u], cand[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) cur[u] = Op::kPeek ? __ldcg(P.label + v[u]) : 0;
        if constexpr (U <= 4) {
            if (Q.early_rows) {
                // Row ranges of every candidate head, issued with the peeks (extra loads for heads
                // that are not pushed; worth it only while an iteration is latency-bound).
                int2 se[U];
#pragma unroll
                for (int u = 0; u < U; ++u) se[u] = make_int2(__ldg(P.off + row[u]), __ldg(P.off + row[u] + 1));
#pragma unroll
                for (int u = 0; u < U; ++u)
                    ok[u] = act[u] && Op::want(v[u], cand[u], cur[u]) && Op::commit(P, v[u], cand[u]);
                if (Q.far) {
                    bool far[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        far[u] = ok[u] && cand[u] >= Q.threshold;
                        ok[u] = ok[u] && !far[u];
                    }
                    far_push<U>(P, Q, far, v, cand);
                }
                push_batch<Op, kClassify, CH, U>(P, Q, ok, v, row, se);
                return;
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            ok[u] = act[u] && Op::want(v[u], cand[u], cur[u]) && Op::commit(P, v[u], cand[u]);
        if (Q.far) {  // near-far: improvements at or above the threshold wait in the far pile
            bool far[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                far[u] = ok[u] && cand[u] >= Q.threshold;
                ok[u] = ok[u] && !far[u];
            }
            far_push<U>(P, Q, far, v, cand);
        }
    }
    push_batch<Op, kClassify, CH, U>(P, Q, ok, v, row);
}

// Push of vertices whose label index is their row (single-source operators).
template <class Op, bool kClassify, int CH>
__device__ __forceinline__ void push_converged(const ExpandParams& P, const PushCtx& Q, bool ok, int v,
                                               const int2* se_pre = nullptr) {
    bool okb[1] = {ok};
    const int vb[1] = {v};
    push_batch<Op, kClassify, CH, 1>(P, Q, okb, vb, vb, se_pre);
}

// Relaxation of one candidate per lane (all lanes call it together).
template <class Op, bool kClassify, int CH>
__device__ __forceinline__ void relax_one(const ExpandParams& P, const PushCtx& Q, bool act, int e,
                                          typename Op::RV du) {
    const bool a[1] = {act};
    const int ee[1] = {e};
    const typename Op::RV dd[1] = {du};
    relax_batch<Op, kClassify, CH, 1>(P, Q, a, ee, dd);
}

// Thread-per-vertex neighbour loops (the reference's serial loop), made warp-uniform so pushes can
// aggregate over the full warp.
template <class Op, bool kClassify, int CH>
__device__ __forceinline__ void serial_rows(const ExpandParams& P, const PushCtx& Q, bool act, int s,
                                            int d, typename Op::RV du) {
    const int dd = act ? d : 0;
    const int wmax = __reduce_max_sync(kFullMask, dd);
    for (int t = 0; t < wmax; ++t) relax_one<Op, kClassify, CH>(P, Q, t < dd, s + t, du);
}

// Scan-based gather: the warp concatenates the rows of the active lanes and relaxes 32 consecutive
// edges per step, so every step is a coalesced read whatever the per-row degrees are.
template <class Op, bool kClassify, int CH>
__device__ __forceinline__ void warp_gather(const ExpandParams& P, const PushCtx& Q, bool act, int s,
                                            int d, typename Op::RV du, int* sx, int* ss,
                                            typename Op::RV* sdu) {
    const int lane = lane_id();
    const int dd = act ? d : 0;
    const int incl = warp_inclusive_scan(dd);
    const int total = __shfl_sync(kFullMask, incl, 31);
    if (total == 0) return;
    __syncwarp();
    sx[lane] = incl - dd;
    ss[lane] = s;
    sdu[lane] = du;
    __syncwarp();
    constexpr int U = 4;
    for (int base = 0; base < total; base += 32 * U) {
        bool act[U];
        int ee[U];
        typename Op::RV dd2[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = base + 32 * u + lane;
            act[u] = k < total;
            ee[u] = 0;
            dd2[u] = typename Op::RV{};
            if (act[u]) {
                int r = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (sx[r + step] <= k) r += step;
                ee[u] = ss[r] + (k - sx[r]);
                dd2[u] = sdu[r];
            }
        }
        relax_batch<Op, kClassify, CH, U>(P, Q, act, ee, dd2);
    }
    __syncwarp();
}

// One vertex's row expanded by the whole warp (the per-vertex child of the naive variant).
template <class Op, bool kClassify, int CH>
__device__ __forceinline__ void warp_row(const ExpandParams& P, const PushCtx& Q, int s, int d,
                                         typename Op::RV du) {
    const int lane = lane_id();
    constexpr int U = 4;
    for (int base = 0; base < d; base += 32 * U) {
        bool act[U];
        int ee[U];
        typename Op::RV dd[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int t = base + 32 * u + lane;
            act[u] = t < d;
            ee[u] = s + t;
            dd[u] = du;
        }
        relax_batch<Op, kClassify, CH, U>(P, Q, act, ee, dd);
    }
}

// CTAs per SM of the binned SSSP and direction-optimizing BFS kernels on wide graphs (hubs, or more
// than 8 arcs per vertex): 64 registers with small spills, a third more warps to hide the
// relaxations' round trips. R-MAT 24, same box, alternated: SSSP 5.71 / 5.67 -> 5.06 / 4.88 ms,
// BFS 0.95 -> 0.87 ms. On the 4096^2 grid the same kernels were 2-13 % slower (small iterations:
// more CTAs at every barrier, and the spills), so sparse graphs without hubs keep Op::min_blocks.
constexpr int kWideBlocks = 4;

template <class Op, int POL, int CH = kHubChunk, int MINB = 0>
__global__ void __launch_bounds__(kBlock, MINB > 0 ? MINB : Op::min_blocks(CH)) expand_kernel(ExpandParams P) {
    using RV = typename Op::RV;
    constexpr bool kDirOpt = (POL == DPG_SOL_DIROPT);
    constexpr bool kNearFar = (POL == DPG_SOL_NEARFAR);
    constexpr bool kBinned = (POL == DPG_SOL_BINNED || kDirOpt || kNearFar);
    constexpr bool kClassify = (POL == DPG_SOL_GRID || kBinned);
    __shared__ int s_excl[kWarps][32];
    __shared__ int s_start[kWarps][32];
    __shared__ RV s_du[kWarps][32];
    // CTA consolidation buffer (DPG_SOL_BLOCK).
    __shared__ int c_start[kBlock];
    __shared__ int c_deg[kBlock];
    __shared__ RV c_du[kBlock];
    __shared__ int c_excl[kBlock];
    __shared__ int c_wsum[kWarps];
    __shared__ int c_n;
    __shared__ int c_total;
    // Per-warp frontier push buffers (flush_pushes).
    __shared__ int p_v[kWarps][kPushBuf];
    __shared__ int2 p_se[kWarps][kPushBuf];
    __shared__ unsigned p_n[kWarps];
    __shared__ unsigned long long p_mf[kWarps];
    __shared__ unsigned p_nf[kWarps];

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const unsigned gwarp = blockIdx.x * kWarps + warp;
    const unsigned nwarps = gridDim.x * kWarps;
    unsigned long long my_edges = 0, my_pops = 0;
    if (threadIdx.x == 0) c_n = 0;
    if (lane == 0) {
        p_n[warp] = 0u;
        p_mf[warp] = 0ull;
        p_nf[warp] = 0u;
    }
    __syncthreads();

    // Direction-optimizing BFS (Beamer, Asanovic, Patterson, "Direction-Optimizing Breadth-First
    // Search", SC 2012), with the switch rule set for this kernel: a step runs bottom-up when the
    // frontier's out-arcs mf exceed both a quarter of the still unexplored arcs and V. A bottom-up
    // step costs a sweep over all vertices plus in-arc scans, so on GPU it pays only for frontiers
    // far larger than the CPU rule (mf > unexplored / 14) assumes; measured on R-MAT 22 and 24, this
    // picks the faster direction at every level. Every CTA reads the same counters after the
    // barrier, so all make the same choice.
    bool bottom_up = false;
    long long unexplored = kDirOpt ? static_cast<long long>(P.E) : 0;
    // Near-far (Davidson, Baxter, Garland, Owens, "Work-Efficient Parallel GPU Methods for
    // Single-Source Shortest Paths", IPDPS 2014): improvements below the threshold form the next
    // frontier, the others wait in the active far pile. When the frontier runs dry the threshold
    // moves past delta and the pile's minimum, and one split step moves the pile's still-current
    // entries below it into the frontier and the rest into the next pile. Piles rotate over three
    // buffers so the one being reset is never the one being read or written.
    int threshold = kNearFar ? P.delta : 0;
    int pile = 0;
    int j = 0;
    // The iteration's counters. In the 3-CTA builds (sparse graphs, whose thousands of small
    // iterations each pay this) one thread per CTA reads them and shares them: with every warp of
    // 456 CTAs reading the same few words, the L2 served some 15 K requests to one line per
    // iteration. Same box, alternated: 4096^2 grid BFS 51.9 -> 46.6 ms, near-far SSSP 66.1 ->
    // 62.0 ms. The 4-CTA build (R-MAT graphs) reads them per warp: with the shared read its
    // bottom-up BFS steps ran 10-50 % longer, though the frontiers and direction choices were
    // the same.
    constexpr bool kCtaCounters = (MINB == 0);
    __shared__ unsigned s_ctr[3];
    __shared__ int s_far_min;
    __shared__ unsigned long long s_mf;
    for (;; ++j) {
        const int p = j & 1;
        // Counters can pass the capacities only after a push has already raised DPG_ERR_CAPACITY
        // (which stops the loop at the barrier); the clamps keep every read inside its buffer anyway.
        // The previous iteration's grid barrier (which starts and ends with __syncthreads) keeps
        // the shared copies' writes after every thread's reads of the last values.
        auto read_q = [&] { return min(ld_volatile(P.ws.qcount + (j % 3)), static_cast<unsigned>(P.ws.cap_v)); };
        auto read_c = [&] { return min(ld_volatile(P.ws.ccount + (j % 3)), static_cast<unsigned>(P.ws.cap_chunks)); };
        auto read_far_n = [&] {
            return static_cast<unsigned>(min(static_cast<int64_t>(ld_volatile(P.far_count + pile)), P.far_cap));
        };
        auto read_far_min = [&] { return *reinterpret_cast<const volatile int*>(P.far_min + pile); };
        auto read_mf = [&] { return *reinterpret_cast<const volatile unsigned long long*>(P.mf + j % 3); };
        if constexpr (kCtaCounters) {
            if (threadIdx.x == 0) {
                s_ctr[0] = read_q();
                s_ctr[1] = read_c();
                if (kNearFar) {
                    s_ctr[2] = read_far_n();
                    s_far_min = read_far_min();
                }
                if (kDirOpt) s_mf = read_mf();
            }
            __syncthreads();
        }
        const unsigned n = kCtaCounters ? s_ctr[0] : read_q();
        const unsigned nch = kCtaCounters ? s_ctr[1] : read_c();
        bool split = false;
        unsigned far_n = 0;
        if (kNearFar && n == 0 && nch == 0) {
            far_n = kCtaCounters ? s_ctr[2] : read_far_n();
            if (far_n == 0) break;
            split = true;
            const int fmin = kCtaCounters ? s_far_min : read_far_min();
            const long long t = max(static_cast<long long>(threshold) + P.delta, static_cast<long long>(fmin) + 1);
            threshold = static_cast<int>(min(t, static_cast<long long>(0x7FFFFFFF)));
        }
        if (!split && n == 0 && nch == 0) break;
        if (j >= P.max_iter) {
            if (blockIdx.x == 0 && threadIdx.x == 0) raise_error(P.st, DPG_ERR_CAPACITY, 2);
            break;
        }
        if (kDirOpt) {
            const unsigned long long mf = kCtaCounters ? s_mf : read_mf();
            bottom_up = static_cast<long long>(mf) * 4 > unexplored && static_cast<long long>(mf) > P.V;
            unexplored -= static_cast<long long>(mf);
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            P.ws.qcount[(j + 2) % 3] = 0u;
            P.ws.ccount[(j + 2) % 3] = 0u;
            if (kDirOpt) {
                P.mf[(j + 2) % 3] = 0ull;
                P.nf[(j + 2) % 3] = 0u;
            }
            if (kNearFar && split) {  // the pile read by the previous split is free again
                P.far_count[(pile + 2) % 3] = 0u;
                P.far_min[(pile + 2) % 3] = 0x7FFFFFFF;
            }
            if (P.trace && j < P.trace_cap) {
                P.trace[4 * j + 0] = global_timer_ns();
                P.trace[4 * j + 1] = n;
                P.trace[4 * j + 2] = nch;
                P.trace[4 * j + 3] = bottom_up ? 2ull : 0ull;
            }
        }
        // Push buffering pays only when an iteration's pushes are many (the global counter is then
        // contended); with the few pushes of a high-diameter graph's iterations its flush is one more
        // round trip per iteration. The arcs to relax (vertices plus 256-arc chunks) decide, the
        // same for every CTA. On R-MAT 24 it cut SSSP from 7.6 to 5.6 ms and BFS from 1.70 to 1.16
        // ms; on the 4096^2 grid, buffering every iteration cost near-far SSSP 11 %.
        const unsigned long long work = static_cast<unsigned long long>(n) + 256ull * nch + (split ? far_n : 0u);
        const bool buffered = work >= kPushBufferWork || (kDirOpt && bottom_up);
        // Parity selects are written as ternaries so the pointer pairs stay in registers.
        const PushCtx Q = {p ? P.ws.qv[0] : P.ws.qv[1], p ? P.ws.qse[0] : P.ws.qse[1],
                           P.ws.qcount + (j + 1) % 3, p ? P.ws.bmp[0] : P.ws.bmp[1],
                           p ? P.ws.chunks[0] : P.ws.chunks[1], P.ws.ccount + (j + 1) % 3,
                           p ? P.dirty[0] : P.dirty[1], static_cast<unsigned>(j + 1),
                           kDirOpt ? P.mf + (j + 1) % 3 : nullptr, kDirOpt ? P.nf + (j + 1) % 3 : nullptr,
                           kNearFar ? P.far[split ? (pile + 1) % 3 : pile] : nullptr,
                           kNearFar ? P.far_count + (split ? (pile + 1) % 3 : pile) : nullptr,
                           kNearFar ? P.far_min + (split ? (pile + 1) % 3 : pile) : nullptr, threshold,
                           !buffered, buffered ? p_v[warp] : nullptr, buffered ? p_se[warp] : nullptr,
                           buffered ? &p_n[warp] : nullptr, &p_mf[warp], &p_nf[warp]};
        const int32_t* qv_cur = p ? P.ws.qv[1] : P.ws.qv[0];
        const int2* qse_cur = p ? P.ws.qse[1] : P.ws.qse[0];
        uint32_t* bmp_cur = p ? P.ws.bmp[1] : P.ws.bmp[0];
        const int4* chunks_cur = p ? P.ws.chunks[1] : P.ws.chunks[0];
        const unsigned fchunks = (n + 31u) / 32u;

        if (kNearFar && split) {
            // Split: still-current entries below the new threshold join the frontier (de-duplicated
            // by the bitmap), the rest move to the next pile; stale entries are dropped.
            const int2* src = P.far[pile];
            for (int64_t base = static_cast<int64_t>(gwarp) * 32; base < far_n; base += static_cast<int64_t>(nwarps) * 32) {
                const int64_t i = base + lane;
                int2 F = make_int2(0, 0);
                bool cur = false;
                if (i < far_n) {
                    F = __ldcg(src + i);
                    cur = __ldcg(P.label + F.x) == F.y;
                }
                bool keep[1] = {cur && F.y >= threshold};
                const int fv[1] = {F.x};
                const int fc[1] = {F.y};
                far_push<1>(P, Q, keep, fv, fc);
                push_converged<Op, kClassify, CH>(P, Q, cur && F.y < threshold, cur ? F.x : 0);
            }
        } else if (kDirOpt && bottom_up) {
            // Bottom-up: every unvisited vertex looks for an in-neighbour on the frontier's level j.
            // A lane takes kBu vertices at a time and issues their loads together (level, in-arc
            // range, first in-arc and its level; the out-row range a push needs comes with the in-row
            // range), so the common cases (a parent at the first in-arc, no in-arcs) cost one chain of
            // round trips for all of them; the others go on arc by arc.
            // The parent test and the arcs counted are those of a one-vertex-at-a-time scan.
            // R-MAT 24, 8 sources, same box: 9.12 ms in all at 4 vertices per lane, 7.64 at 2, 8.17
            // at 1 (4 ran the vertices that scan many in-arcs one after another in the lane).
            constexpr int kBu = 2;
            const int64_t stride = static_cast<int64_t>(nwarps) * 32 * kBu;
            for (int64_t base = static_cast<int64_t>(gwarp) * 32 * kBu; base < P.V; base += stride) {
                int vv[kBu], b[kBu], e[kBu], t0[kBu];
                bool unv[kBu], found[kBu];
#pragma unroll
                for (int r = 0; r < kBu; ++r) {
                    const int64_t x = base + 32 * r + lane;
                    vv[r] = x < P.V ? static_cast<int>(x) : 0;
                    unv[r] = x < P.V && __ldcg(P.label + vv[r]) == DPG_UNDEFINED_LEVEL;
                }
                int2 ose[kBu];  // out-row ranges for the push, fetched with the in-row ranges
#pragma unroll
                for (int r = 0; r < kBu; ++r) {
                    b[r] = unv[r] ? __ldg(P.t_off + vv[r]) : 0;
                    e[r] = unv[r] ? __ldg(P.t_off + vv[r] + 1) : 0;
                    ose[r] = unv[r] ? make_int2(__ldg(P.off + vv[r]), __ldg(P.off + vv[r] + 1)) : make_int2(0, 0);
                }
#pragma unroll
                for (int r = 0; r < kBu; ++r) t0[r] = b[r] < e[r] ? __ldg(P.t_col + b[r]) : -1;
#pragma unroll
                for (int r = 0; r < kBu; ++r) found[r] = t0[r] >= 0 && __ldcg(P.label + t0[r]) == j;
#pragma unroll
                for (int r = 0; r < kBu; ++r) {
                    if (!unv[r]) continue;
                    int k = b[r];
                    if (!found[r]) {
                        // The rest of the in-arcs kBuArcs at a time: their tails, then the tails'
                        // levels, loaded together; the first parent among them ends the scan, so
                        // the count is that of an arc-by-arc scan (a few loads past it are spare).
                        // R-MAT 24, 8 sources, same box: 7.63 ms in all arc by arc, 6.42 two at a
                        // time, 6.08 four at a time; a uniform random graph (16 M vertices, 8 arcs
                        // each) 2.05 -> 1.25 ms; the grid unchanged.
                        constexpr int kBuArcs = 4;
                        for (k = b[r] + 1; k < e[r]; k += kBuArcs) {
                            int c[kBuArcs], l[kBuArcs];
#pragma unroll
                            for (int q = 0; q < kBuArcs; ++q) c[q] = k + q < e[r] ? __ldg(P.t_col + k + q) : -1;
#pragma unroll
                            for (int q = 0; q < kBuArcs; ++q) l[q] = c[q] >= 0 ? __ldcg(P.label + c[q]) : -1;
                            int hit = -1;
#pragma unroll
                            for (int q = kBuArcs - 1; q >= 0; --q)
                                if (l[q] == j) hit = q;
                            if (hit >= 0) {
                                k += hit;
                                found[r] = true;
                                break;
                            }
                        }
                    }
                    my_edges += static_cast<unsigned long long>((found[r] ? k + 1 : e[r]) - b[r]);
                    if (found[r]) {
                        P.label[vv[r]] = j + 1;
                        my_pops += 1;
                    }
                }
#pragma unroll
                for (int r = 0; r < kBu; ++r)
                    push_converged<Op, kClassify, CH>(P, Q, found[r], found[r] ? vv[r] : 0, &ose[r]);
            }
        } else if (POL == DPG_SOL_BLOCK) {
            const unsigned per_round = gridDim.x * kWarps;
            const unsigned rounds = (fchunks + per_round - 1) / per_round;
            for (unsigned r = 0; r < rounds; ++r) {
                const unsigned chunk = r * per_round + blockIdx.x * kWarps + warp;
                const unsigned i = chunk * 32u + lane;
                int u = 0, s = 0, d = 0;
                RV du{};
                const bool has = chunk < fchunks && i < n;
                if (has) {
                    u = __ldcg(qv_cur + i);
                    const int2 se = __ldcg(qse_cur + i);
                    s = se.x;
                    d = se.y - se.x;
                    du = Op::row_value(P, u, j);
                    if (Op::kDedup) __stcg(bmp_cur + (u >> 5), 0u);
                    my_pops += 1;
                    my_edges += static_cast<unsigned long long>(d);
                }
                const bool big = has && d >= P.threshold;
                serial_rows<Op, false, CH>(P, Q, has && !big, s, d, du);
                if (big) {
                    const int slot = atomicAdd(&c_n, 1);
                    c_start[slot] = s;
                    c_deg[slot] = d;
                    c_du[slot] = du;
                }
                __syncthreads();
                const int cn = c_n;
                if (cn > 0) {
                    // CTA-wide exclusive scan of the consolidated degrees.
                    const int dg = threadIdx.x < cn ? c_deg[threadIdx.x] : 0;
                    const int incl = warp_inclusive_scan(dg);
                    if (lane == 31) c_wsum[warp] = incl;
                    __syncthreads();
                    if (warp == 0) {
                        const int w = lane < kWarps ? c_wsum[lane] : 0;
                        const int wi = warp_inclusive_scan(w);
                        if (lane < kWarps) c_wsum[lane] = wi - w;
                        if (lane == kWarps - 1) c_total = wi;
                    }
                    __syncthreads();
                    c_excl[threadIdx.x] = incl - dg + c_wsum[warp];
                    __syncthreads();
                    const int total = c_total;
                    for (int base = 0; base < total; base += kBlock) {
                        const int k = base + static_cast<int>(threadIdx.x);
                        int ee = 0;
                        RV dd{};
                        if (k < total) {
                            int rr = 0;
#pragma unroll
                            for (int step = kBlock / 2; step > 0; step >>= 1)
                                if (rr + step < kBlock && c_excl[rr + step] <= k) rr += step;
                            ee = c_start[rr] + (k - c_excl[rr]);
                            dd = c_du[rr];
                        }
                        relax_one<Op, false, CH>(P, Q, k < total, ee, dd);
                    }
                    __syncthreads();
                    if (threadIdx.x == 0) c_n = 0;
                }
                __syncthreads();
            }
        } else {
            const unsigned hub_items = kClassify ? nch : 0u;
            const unsigned total_items = hub_items + fchunks;
            for (unsigned item = gwarp; item < total_items; item += nwarps) {
                if (kClassify && item < hub_items) {
                    // Grid-wide consolidation: one chunk (<= 256 arcs) of a chunked vertex.
                    const int4 C = __ldcg(chunks_cur + item);
                    const int v0 = C.x, k0 = C.y, k1 = C.z;
                    const RV du = Op::row_value(P, v0, j);
                    if (C.w && lane == 0) {
                        if (Op::kDedup) __stcg(bmp_cur + (v0 >> 5), 0u);
                        my_pops += 1;
                    }
                    if (lane == 0) my_edges += static_cast<unsigned long long>(k1 - k0);
                    {
                        constexpr int U = CH / 32;  // the whole chunk in one batch
                        bool act[U];
                        int ee[U];
                        RV dd[U];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            ee[u] = k0 + 32 * u + lane;
                            act[u] = ee[u] < k1;
                            dd[u] = du;
                        }
                        relax_batch<Op, kClassify, CH, U>(P, Q, act, ee, dd);
                    }
                    continue;
                }
                const unsigned chunk = item - hub_items;
                const unsigned i = chunk * 32u + lane;
                int u = 0, s = 0, d = 0;
                RV du{};
                const bool has = i < n;
                if (has) {
                    u = __ldcg(qv_cur + i);
                    const int2 se = __ldcg(qse_cur + i);
                    s = se.x;
                    d = se.y - se.x;
                    du = Op::row_value(P, u, j);
                    if (Op::kDedup) __stcg(bmp_cur + (u >> 5), 0u);
                    my_pops += 1;
                    my_edges += static_cast<unsigned long long>(d);
                }
                if (POL == DPG_SOL_THREAD || POL == DPG_SOL_GRID) {
                    serial_rows<Op, kClassify, CH>(P, Q, has, s, d, du);
                } else if (kBinned) {
                    warp_gather<Op, kClassify, CH>(P, Q, has, s, d, du, s_excl[warp], s_start[warp], s_du[warp]);
                } else {
                    const bool big = has && d >= P.threshold;
                    serial_rows<Op, kClassify, CH>(P, Q, has && !big, s, d, du);
                    if (POL == DPG_SOL_WARP) {
                        warp_gather<Op, kClassify, CH>(P, Q, big, s, d, du, s_excl[warp], s_start[warp], s_du[warp]);
                    } else {  // DPG_SOL_NAIVE
                        unsigned bigmask = __ballot_sync(kFullMask, big);
                        while (bigmask) {
                            const int src = __ffs(bigmask) - 1;
                            bigmask &= bigmask - 1u;
                            const int bs = __shfl_sync(kFullMask, s, src);
                            const int bd = __shfl_sync(kFullMask, d, src);
                            const RV bdu = shfl_rv(du, src);
                            warp_row<Op, kClassify, CH>(P, Q, bs, bd, bdu);
                        }
                    }
                }
            }
        }
        flush_pushes(P, Q);
        if (!grid_barrier(P.st, gridDim.x, P.timeout_ns)) break;
        if (kNearFar && split) pile = (pile + 1) % 3;
    }

    my_edges = warp_sum_u64(my_edges);
    my_pops = warp_sum_u64(my_pops);
    if (lane == 0) {
        if (my_edges) atomicAdd(&P.st->edges, my_edges);
        if (my_pops) atomicAdd(&P.st->pops, my_pops);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.st->iterations = static_cast<unsigned long long>(j);
        if (P.trace && j < P.trace_cap) {  // end marker: time the last barrier was passed
            P.trace[4 * j + 0] = global_timer_ns();
            P.trace[4 * j + 1] = 0ull;
            P.trace[4 * j + 2] = 0ull;
            P.trace[4 * j + 3] = 1ull;
        }
    }
}

__global__ void expand_init_kernel(ExpandParams P, int32_t source, int32_t init_label, int classify) {
    const int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = tid; i < P.V; i += stride) P.label[i] = (i == source) ? 0 : init_label;
    for (int64_t w = tid; w < P.ws.bmp_words; w += stride) {
        P.ws.bmp[0][w] = 0u;
        P.ws.bmp[1][w] = 0u;
    }
    // The source enters the first frontier: chunked when its degree calls for it.
    const int s = P.off[source];
    const int e = P.off[source + 1];
    const bool chunked = classify && e > s && e - s >= P.hub_threshold;
    const int nch = chunked ? (e - s + kHubChunk - 1) / kHubChunk : 0;
    for (int64_t c = tid; c < nch; c += stride) {
        const int k0 = s + static_cast<int>(c) * kHubChunk;
        P.ws.chunks[0][c] = make_int4(source, k0, min(e, k0 + kHubChunk), c == 0 ? 1 : 0);
    }
    if (tid == 0) {
        for (int k = 0; k < 3; ++k) {
            P.ws.qcount[k] = 0u;
            P.ws.ccount[k] = 0u;
        }
        P.st->bar_count = 0u;
        P.st->iterations = 0ull;
        P.st->edges = 0ull;
        P.st->pops = 0ull;
        if (P.far_count) {
            for (int k = 0; k < 3; ++k) {
                P.far_count[k] = 0u;
                P.far_min[k] = 0x7FFFFFFF;
            }
        }
        if (P.mf) {
            for (int k = 0; k < 3; ++k) {
                P.mf[k] = 0ull;
                P.nf[k] = 0u;
            }
            P.mf[0] = static_cast<unsigned long long>(e - s);
            P.nf[0] = e > s ? 1u : 0u;
        }
        if (chunked) {
            P.ws.ccount[0] = static_cast<unsigned>(nch);
        } else if (e > s) {
            P.ws.qv[0][0] = source;
            P.ws.qse[0][0] = make_int2(s, e);
            P.ws.qcount[0] = 1u;
        }
    }
}

// Multi-source start, part 1: every label to infinity, marks, bitmaps and counters cleared. A
// launch that continues a solve (another group of graphs, nlabels = nmarks = 0) clears only the
// queue counters, so the arcs and pops statistics add up over the solve's launches.
__global__ void multi_fill_kernel(ExpandParams P, int64_t nlabels, int64_t nmarks) {
    const int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = tid; i < nlabels; i += stride) P.label[i] = DPG_INF_COST;
    for (int64_t v = tid; v < nmarks; v += stride) {
        P.dirty[0][v] = 0ull;
        P.dirty[1][v] = 0ull;
    }
    if (tid == 0) {
        for (int k = 0; k < 3; ++k) {
            P.ws.qcount[k] = 0u;
            P.ws.ccount[k] = 0u;
        }
        P.st->bar_count = 0u;
        if (nmarks > 0) {
            P.st->iterations = 0ull;
            P.st->edges = 0ull;
            P.st->pops = 0ull;
        }
    }
}

// Part 2: sources[i] = v * nsrc + k (source k at vertex v) gets distance 0 and its bit in v's mark
// for iteration 0; the first bit to arrive pushes v, cut into CH-arc chunks when its degree reaches
// hub_threshold.
template <int CH>
__global__ void multi_seed_kernel(ExpandParams P, const int32_t* __restrict__ sources, int32_t nsources) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nsources; i += gridDim.x * blockDim.x) {
        const int x = sources[i];
        const int v = x / P.nsrc, k = x - v * P.nsrc;
        P.label[x] = 0;
        const unsigned long long old = atomicOr(P.dirty[0] + v, 1ull << k);  // tag 0 in the high word
        if (old != 0ull) continue;
        const int s = P.off[v], e = P.off[v + 1];
        if (e <= s) continue;
        if (e - s >= P.hub_threshold) {
            const int nch = (e - s + CH - 1) / CH;
            const unsigned first = atomicAdd(P.ws.ccount, static_cast<unsigned>(nch));
            if (static_cast<int64_t>(first) + nch > P.ws.cap_chunks) {
                raise_error(P.st, DPG_ERR_CAPACITY, 12);
                continue;
            }
            for (int c = 0; c < nch; ++c) {
                const int k0 = s + c * CH;
                P.ws.chunks[0][first + c] = make_int4(v, k0, min(e, k0 + CH), c == 0 ? 1 : 0);
            }
        } else {
            const unsigned pos = atomicAdd(P.ws.qcount, 1u);
            if (static_cast<int64_t>(pos) >= P.ws.cap_v) {
                raise_error(P.st, DPG_ERR_CAPACITY, 13);
                continue;
            }
            P.ws.qv[0][pos] = v;
            P.ws.qse[0][pos] = make_int2(s, e);
        }
    }
}

// Colouring start: pending[v] = out-neighbours u < v (with multiplicity); vertices with none take
// colour 1 and form the first frontier over the transposed graph (P.off / P.col).
__global__ void color_init_kernel(ExpandParams P, const int32_t* __restrict__ out_off,
                                  const int32_t* __restrict__ out_col) {
    const int lane = lane_id();
    const int64_t wid = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const PushCtx Q = {P.ws.qv[0], P.ws.qse[0], P.ws.qcount, P.ws.bmp[0], P.ws.chunks[0], P.ws.ccount, nullptr, 0u};
    for (int64_t base = wid * 32; base < P.V; base += nw * 32) {  // warp-uniform trip count
        const int v = static_cast<int>(base) + lane;
        bool ready = false;
        if (v < P.V) {
            int pending = 0;
            for (int e = out_off[v]; e < out_off[v + 1]; ++e) pending += __ldg(out_col + e) < v;
            P.aux[v] = pending;
            P.label[v] = pending == 0 ? 1 : 0;
            ready = pending == 0;
        }
        push_converged<ColorOp, true, kHubChunk>(P, Q, ready, v < P.V ? v : 0);
    }
}

__global__ void barrier_timeout_kernel(DevStatus* st, unsigned long long timeout_ns) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st->bar_count = 0u;
    // Only gridDim.x CTAs exist but the barrier waits for one more: every wait must time out.
    // (CTA 0 resets the counter before arriving; a late reset can only make the wait longer.)
    grid_barrier(st, gridDim.x + 1, timeout_ns);
}

// The kernel of a solution id; `wide` selects the kWideBlocks build of the binned and
// direction-optimizing kernels.
template <class Op>
const void* pick_kernel(int solution, bool wide) {
    const void* binned = wide ? reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_BINNED, kHubChunk, kWideBlocks>)
                              : reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_BINNED>);
    const void* diropt = wide ? reinterpret_cast<const void*>(expand_kernel<BfsOp, DPG_SOL_DIROPT, kHubChunk, kWideBlocks>)
                              : reinterpret_cast<const void*>(expand_kernel<BfsOp, DPG_SOL_DIROPT>);
    switch (solution) {
        case DPG_SOL_THREAD: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_THREAD>);
        case DPG_SOL_NAIVE: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_NAIVE>);
        case DPG_SOL_WARP: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_WARP>);
        case DPG_SOL_BLOCK: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_BLOCK>);
        case DPG_SOL_GRID: return reinterpret_cast<const void*>(expand_kernel<Op, DPG_SOL_GRID>);
        case DPG_SOL_BINNED: return binned;
        case DPG_SOL_NEARFAR:  // a distance threshold: SSSP only, BFS runs direction-optimizing
            if constexpr (std::is_same<Op, SsspOp>::value)
                return reinterpret_cast<const void*>(expand_kernel<SsspOp, DPG_SOL_NEARFAR>);
            else
                return diropt;
        case DPG_SOL_DIROPT:  // bottom-up steps need a level rule: BFS only, SSSP runs binned
            if constexpr (std::is_same<Op, BfsOp>::value)
                return diropt;
            else
                return binned;
        default: return nullptr;
    }
}

}  // namespace

int64_t expand_chunk_capacity(int32_t V, int64_t E, int32_t min_chunked_degree, int32_t chunk) {
    const int64_t d = min_chunked_degree < 1 ? 1 : min_chunked_degree;
    int64_t vertices = E / d + 1;
    if (vertices > static_cast<int64_t>(V) + 1) vertices = static_cast<int64_t>(V) + 1;
    return E / (chunk < 1 ? kHubChunk : chunk) + vertices + 1;
}

namespace {
template <int CH>
cudaError_t run_multi(const MultiExpandLaunch& L, const ExpandWorkspace& ws, DevStatus* st, cudaStream_t stream,
                      int sm_count, int* grid_out, LaunchHook* hook) {
    const void* fn = reinterpret_cast<const void*>(expand_kernel<MaskSsspOp, DPG_SOL_BINNED, CH>);
    int per_sm = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBlock, 0);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int grid = per_sm * sm_count;
    ExpandParams P;
    memset(&P, 0, sizeof(P));
    P.off = L.off;
    P.adj = L.adj;
    P.label = L.label;
    P.V = L.V;
    P.threshold = L.hub_threshold;
    P.hub_threshold = L.hub_threshold;
    P.max_iter = L.max_iter;
    P.timeout_ns = L.timeout_ns;
    P.ws = ws;
    P.st = st;
    P.nsrc = L.nsrc;
    P.dirty[0] = L.dirty[0];
    P.dirty[1] = L.dirty[1];
    P.label_vec4 = (L.nsrc % 4 == 0 && (reinterpret_cast<uintptr_t>(L.label) & 15u) == 0) ? 1 : 0;
    const int64_t nlabels = static_cast<int64_t>(L.V) * L.nsrc;
    {
        HookScope hs(hook, DPG_KERNEL_INIT, stream);
        multi_fill_kernel<<<sm_count * 8, kBlock, 0, stream>>>(P, L.skip_fill ? 0 : nlabels,
                                                                L.skip_fill ? 0 : static_cast<int64_t>(L.V));
        if (L.nsources > 0)
            multi_seed_kernel<CH><<<(L.nsources + kBlock - 1) / kBlock, kBlock, 0, stream>>>(P, L.sources, L.nsources);
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    void* args[] = {&P};
    {
        HookScope hs(hook, DPG_KERNEL_EXPAND, stream);
        err = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kBlock), args, 0, stream);
    }
    if (grid_out) *grid_out = grid;
    return err;
}
}  // namespace

cudaError_t launch_expand_multi(const MultiExpandLaunch& L, const ExpandWorkspace& ws, DevStatus* st,
                                cudaStream_t stream, int sm_count, int* grid_out, LaunchHook* hook) {
    if (L.V < 1 || L.nsrc < 1 || L.nsrc > 32 || static_cast<int64_t>(L.V) * L.nsrc > INT32_MAX)
        return cudaErrorInvalidValue;
    switch (L.chunk) {
        case 128: return run_multi<128>(L, ws, st, stream, sm_count, grid_out, hook);
        case 256: return run_multi<256>(L, ws, st, stream, sm_count, grid_out, hook);
        case 512: return run_multi<512>(L, ws, st, stream, sm_count, grid_out, hook);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_expand(const ExpandLaunch& L, const ExpandWorkspace& ws, DevStatus* st,
                          cudaStream_t stream, int sm_count, int* grid_out, int* block_out,
                          LaunchHook* hook) {
    const void* fn = L.bfs ? pick_kernel<BfsOp>(L.solution, L.wide) : pick_kernel<SsspOp>(L.solution, L.wide);
    if (!fn) return cudaErrorInvalidValue;
    int per_sm = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBlock, 0);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int grid = per_sm * sm_count;
    ExpandParams P;
    P.off = L.off;
    P.col = L.col;
    P.adj = L.adj;
    P.label = L.label;
    P.V = L.V;
    P.threshold = L.threshold;
    P.hub_threshold = L.hub_threshold;
    P.max_iter = L.max_iter;
    P.timeout_ns = L.timeout_ns;
    P.ws = ws;
    P.st = st;
    P.trace = L.trace;
    P.trace_cap = L.trace_cap;
    P.aux = nullptr;
    P.nsrc = 0;
    P.dirty[0] = P.dirty[1] = nullptr;
    const bool diropt = L.bfs && (L.solution == DPG_SOL_DIROPT || L.solution == DPG_SOL_NEARFAR);
    const bool nearfar = !L.bfs && L.solution == DPG_SOL_NEARFAR;
    for (int k = 0; k < 3; ++k) P.far[k] = nearfar ? L.far[k] : nullptr;
    P.far_count = nearfar ? L.far_count : nullptr;
    P.far_min = nearfar ? L.far_min : nullptr;
    P.far_cap = L.far_cap;
    P.delta = L.delta > 0 ? L.delta : 1;
    P.t_off = diropt ? L.t_off : nullptr;
    P.t_col = diropt ? L.t_col : nullptr;
    P.mf = diropt ? L.do_mf : nullptr;
    P.nf = diropt ? L.do_nf : nullptr;
    P.E = L.E;
    const int classify =
        (L.solution == DPG_SOL_GRID || L.solution == DPG_SOL_BINNED || L.solution == DPG_SOL_DIROPT ||
         L.solution == DPG_SOL_NEARFAR) ? 1 : 0;
    const int32_t init_label = L.bfs ? DPG_UNDEFINED_LEVEL : DPG_INF_COST;
    int init_blocks = static_cast<int>((static_cast<int64_t>(L.V) + kBlock - 1) / kBlock);
    if (init_blocks > sm_count * 8) init_blocks = sm_count * 8;
    if (init_blocks < 1) init_blocks = 1;
    {
        HookScope hs(hook, DPG_KERNEL_INIT, stream);
        expand_init_kernel<<<init_blocks, kBlock, 0, stream>>>(P, L.source, init_label, classify);
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    void* args[] = {&P};
    {
        HookScope hs(hook, DPG_KERNEL_EXPAND, stream);
        err = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kBlock), args, 0, stream);
    }
    if (grid_out) *grid_out = grid;
    if (block_out) *block_out = kBlock;
    return err;
}

cudaError_t launch_color(const ExpandLaunch& L, const int32_t* out_off, const int32_t* out_col, int32_t* pending,
                         const ExpandWorkspace& ws, DevStatus* st, cudaStream_t stream, int sm_count, int* grid_out,
                         int* block_out, LaunchHook* hook) {
    const void* fn = reinterpret_cast<const void*>(expand_kernel<ColorOp, DPG_SOL_BINNED>);
    int per_sm = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBlock, 0);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int grid = per_sm * sm_count;
    ExpandParams P;
    memset(&P, 0, sizeof(P));
    P.off = L.off;
    P.col = L.col;
    P.adj = nullptr;
    P.label = L.label;
    P.V = L.V;
    P.threshold = L.threshold;
    P.hub_threshold = L.hub_threshold;
    P.max_iter = L.max_iter;
    P.timeout_ns = L.timeout_ns;
    P.ws = ws;
    P.st = st;
    P.trace = L.trace;
    P.trace_cap = L.trace_cap;
    P.aux = pending;
    err = cudaMemsetAsync(ws.qcount, 0, sizeof(uint32_t) * 3, stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(ws.ccount, 0, sizeof(uint32_t) * 3, stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(&st->bar_count, 0, sizeof(unsigned), stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(&st->iterations, 0, sizeof(unsigned long long) * 3, stream);
    if (err != cudaSuccess) return err;
    int init_blocks = static_cast<int>((static_cast<int64_t>(L.V) + kBlock - 1) / kBlock);
    if (init_blocks > sm_count * 8) init_blocks = sm_count * 8;
    if (init_blocks < 1) init_blocks = 1;
    {
        HookScope hs(hook, DPG_KERNEL_INIT, stream);
        color_init_kernel<<<init_blocks, kBlock, 0, stream>>>(P, out_off, out_col);
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    void* args[] = {&P};
    {
        HookScope hs(hook, DPG_KERNEL_EXPAND, stream);
        err = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kBlock), args, 0, stream);
    }
    if (grid_out) *grid_out = grid;
    if (block_out) *block_out = kBlock;
    return err;
}

cudaError_t launch_barrier_timeout_test(DevStatus* st, unsigned long long timeout_ns, cudaStream_t stream) {
    void* args[] = {&st, &timeout_ns};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(barrier_timeout_kernel), dim3(2),
                                       dim3(32), args, 0, stream);
}

}  // namespace dpg
