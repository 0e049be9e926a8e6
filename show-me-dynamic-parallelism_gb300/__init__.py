"""dpg: GB300-native irregular CSR neighbour expansion (SSSP, BFS, SpMV, PageRank).

Python binding of the C ABI declared in include/dpg.h (libdpg.so, built in-tree by build.py).
The reference apps (show-me-dynamic-parallelism) call zero-argument wrappers over globals:
SSSP_GPU (apps/sssp/src/sssp.h:32), BFS_REC_GPU (apps/bfs-rec/src/bfs_rec.h:34), SpMV_GPU
(apps/SpMV/src/SpMV.h:38) and PAGERANK_GPU (apps/pagerank/src/pagerank.h:36). Here the same
operations take explicit arrays:

    ctx = Context(0)
    g = Graph(ctx, offsets, col, weights)           # prepare_gpu's H2D half
    dist = sssp(ctx, g, source, solution=4)         # SSSP_GPU with -s 4
    level = bfs(ctx, g, source)                     # BFS_REC_GPU
    y = spmv(ctx, g_vals, vals, x)                  # SpMV_GPU
    rank = pagerank(ctx, g_in, outdeg)              # PAGERANK_GPU (pull over the transposed CSR)

There is no CPU fallback: every solver runs the CUDA kernels of libdpg.so, and importing this
module fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_char_p, c_double, c_int, c_int32, c_int64, c_uint64, c_void_p
from pathlib import Path
from typing import NamedTuple

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libdpg.so"

INF_COST = 1073741824  # apps/sssp/src/sssp_wrapper.cu:5
UNDEFINED_LEVEL = 0x7FFFFFFF  # apps/bfs-rec/src/bfs_rec.h:13
REF_THRESHOLD = 64  # apps/sssp/src/sssp_kernel.cu:7

SOL_THREAD, SOL_NAIVE, SOL_WARP, SOL_BLOCK, SOL_GRID, SOL_BINNED, SOL_DIROPT, SOL_NEARFAR = range(8)
KERNEL_EXPAND, KERNEL_ROWGATHER, KERNEL_FIXUP, KERNEL_INIT = range(4)
SOLUTION_NAMES = {
    SOL_THREAD: "thread",
    SOL_NAIVE: "naive",
    SOL_WARP: "warp",
    SOL_BLOCK: "block",
    SOL_GRID: "grid",
    SOL_BINNED: "binned",
    SOL_DIROPT: "direction-optimizing (BFS)",
    SOL_NEARFAR: "near-far (SSSP)",
}

STATUS = {
    0: "DPG_OK",
    1: "DPG_ERR_INVALID_ARG",
    2: "DPG_ERR_CAPACITY",
    3: "DPG_ERR_TIMEOUT",
    4: "DPG_ERR_CUDA",
    5: "DPG_ERR_NO_DEVICE",
    6: "DPG_ERR_IO",
    7: "DPG_ERR_FORMAT",
    8: "DPG_ERR_UNSUPPORTED",
}
ERR_INVALID_ARG, ERR_CAPACITY, ERR_TIMEOUT, ERR_CUDA, ERR_NO_DEVICE, ERR_IO, ERR_FORMAT = 1, 2, 3, 4, 5, 6, 7


class DpgError(RuntimeError):
    """A dpg_status other than DPG_OK, with the library's thread-local message."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class ExpandOpts(ctypes.Structure):
    _fields_ = [
        ("solution", c_int32),
        ("threshold", c_int32),
        ("hub_threshold", c_int32),
        ("max_iterations", c_int32),
        ("timeout_seconds", c_double),
        ("delta", c_int32),
    ]


class PrOpts(ctypes.Structure):
    _fields_ = [
        ("damping", c_double),
        ("total_rank", c_double),
        ("init_zero", c_int32),
        ("iterations", c_int32),
        ("epsilon", c_double),
    ]


class BatchTuning(ctypes.Structure):
    _fields_ = [("hub_threshold", c_int32), ("chunk", c_int32), ("pr_hot", c_int32)]

    def as_dict(self) -> dict:
        return {"hub_threshold": self.hub_threshold, "chunk": self.chunk, "pr_hot": self.pr_hot}


class CdpStats(ctypes.Structure):
    _fields_ = [("launches", c_int64), ("failed_launches", c_int64), ("buffer_entries", c_int64)]


class RunStats(ctypes.Structure):
    _fields_ = [
        ("iterations", c_int64),
        ("edges_scanned", c_int64),
        ("vertices_popped", c_int64),
        ("grid_blocks", c_int32),
        ("block_threads", c_int32),
    ]


class _HostGraph(ctypes.Structure):
    _fields_ = [
        ("V", c_int32),
        ("E", c_int64),
        ("source", c_int32),
        ("offsets", POINTER(c_int32)),
        ("col", POINTER(c_int32)),
        ("weights", POINTER(c_int32)),
    ]


_P = c_void_p  # opaque handles and raw pointers
# name -> argtypes (all return dpg_status = int unless listed in _RESTYPES)
_SIGS = {
    "dpg_status_string": [c_int],
    "dpg_last_error": [],
    "dpg_version": [],
    "dpg_ctx_create": [c_int, POINTER(_P)],
    "dpg_ctx_destroy": [_P],
    "dpg_ctx_set_stream": [_P, _P],
    "dpg_ctx_synchronize": [_P],
    "dpg_ctx_last_stats": [_P, POINTER(RunStats)],
    "dpg_ctx_sm_count": [_P, POINTER(c_int32)],
    "dpg_ctx_profile_enable": [_P, c_int32],
    "dpg_ctx_profile_reset": [_P],
    "dpg_ctx_profile_read": [_P, c_int32, POINTER(c_int64), POINTER(c_double)],
    "dpg_ctx_trace_enable": [_P, c_int32],
    "dpg_ctx_trace_read": [_P, _P, c_int32, POINTER(c_int32)],
    "dpg_graph_create": [_P, c_int32, c_int64, _P, _P, _P, POINTER(_P)],
    "dpg_graph_create_device": [_P, c_int32, c_int64, _P, _P, _P, POINTER(_P)],
    "dpg_graph_destroy": [_P],
    "dpg_graph_relabel": [_P, c_int32],
    "dpg_graph_info": [_P, POINTER(c_int32), POINTER(c_int64), POINTER(c_int32)],
    "dpg_graph_plan_info": [_P, POINTER(c_int32), POINTER(c_int32), POINTER(c_int32), POINTER(c_int32)],
    "dpg_sssp": [_P, _P, c_int32, POINTER(ExpandOpts), _P],
    "dpg_sssp_dev": [_P, _P, c_int32, POINTER(ExpandOpts), _P],
    "dpg_bfs": [_P, _P, c_int32, POINTER(ExpandOpts), _P],
    "dpg_bfs_dev": [_P, _P, c_int32, POINTER(ExpandOpts), _P],
    "dpg_color": [_P, _P, POINTER(ExpandOpts), _P],
    "dpg_color_dev": [_P, _P, POINTER(ExpandOpts), _P],
    "dpg_spmv_f32": [_P, _P, _P, _P, _P],
    "dpg_spmv_f32_dev": [_P, _P, _P, _P, _P],
    "dpg_pagerank_f32": [_P, _P, _P, POINTER(PrOpts), _P],
    "dpg_pagerank_f32_dev": [_P, _P, _P, POINTER(PrOpts), _P],
    "dpg_sssp_host": [_P, c_int32, c_int64, _P, _P, _P, c_int32, POINTER(ExpandOpts), _P],
    "dpg_pagerank_f32_host": [_P, c_int32, c_int64, _P, _P, _P, POINTER(PrOpts), _P],
    "dpg_selftest_barrier_timeout": [_P, c_double],
    "dpg_sssp_noalloc_dev": [c_int32, c_int64, _P, _P, c_int32, _P, _P],
    "dpg_read_graph": [c_char_p, c_int32, POINTER(_HostGraph)],
    "dpg_read_graph_ex": [c_char_p, c_int32, c_int32, POINTER(_HostGraph)],
    "dpg_write_graph_cache": [c_char_p, POINTER(_HostGraph)],
    "dpg_read_graph_cache": [c_char_p, POINTER(_HostGraph)],
    "dpg_host_graph_free": [POINTER(_HostGraph)],
    "dpg_csr_from_arcs": [c_int32, c_int64, _P, _P, _P, _P, _P, _P],
    "dpg_csr_transpose": [c_int32, c_int64, _P, _P, _P, _P],
    "dpg_csr_transpose_perm": [c_int32, c_int64, _P, _P, _P, _P, _P],
    "dpg_spmm_f32_dev": [_P, _P, _P, c_int32, _P, _P],
    "dpg_spmv_bwd_f32_dev": [_P, _P, _P, c_int32, _P, _P, _P, _P],
    "dpg_pagerank_grad_f32_dev": [_P, _P, _P, _P, _P, c_double, _P, _P],
    "dpg_batch_create": [_P, c_int32, _P, c_int64, _P, _P, _P, _P],
    "dpg_batch_destroy": [_P],
    "dpg_batch_info": [_P, POINTER(c_int32), POINTER(c_int32), POINTER(c_int64)],
    "dpg_batch_set_tuning": [_P, _P],
    "dpg_batch_get_tuning": [_P, _P],
    "dpg_batch_sssp_dev": [_P, _P, c_int32, _P, _P, _P],
    "dpg_batch_pagerank_dev": [_P, _P, _P, _P],
    "dpg_batch_run": [_P, _P, c_int32, _P, _P, _P, _P, _P],
    "dpg_batch_launches": [_P, POINTER(c_int64)],
    "dpg_batch_autotune": [_P, _P, c_int32, _P, _P],
    "dpg_calibrate_random_reads": [_P, c_int64, c_int32, POINTER(c_double)],
    "dpg_graph_hot_cache": [_P, POINTER(c_int32), POINTER(c_int64)],
    "dpg_batch_set_graph_tuning": [_P, _P, _P],
    "dpg_batch_get_graph_tuning": [_P, _P, _P],
    "dpg_partition_lpt": [c_int32, _P, c_int32, _P, _P],
    "dpg_bfs_cdp_dev": [_P, _P, c_int32, c_int32, c_int32, _P, _P],
    "dpg_csr_transpose_dev": [_P, c_int32, c_int64, _P, _P, _P, _P, _P],
    "dpg_ctx_grad_sweeps": [_P, POINTER(c_int64), POINTER(c_int64)],
    "dpg_write_dimacs9": [c_char_p, c_int32, c_int64, _P, _P, _P, c_int32],
    "dpg_write_cost": [c_char_p, c_int32, c_int32, _P],
    "dpg_write_level": [c_char_p, c_int32, _P],
    "dpg_write_rank": [c_char_p, c_int32, _P],
    "dpg_write_color": [c_char_p, c_int32, _P],
    "dpg_rmat_arcs": [c_int32, c_int32, c_int64, c_uint64, c_double, c_double, c_double, c_int32, c_int32, c_int32,
                      _P, _P, _P],
    "dpg_grid_arcs": [c_int32, c_int32, c_uint64, c_int32, c_int32, _P, _P, _P],
}
_RESTYPES = {"dpg_status_string": c_char_p, "dpg_last_error": c_char_p, "dpg_version": c_int,
             "dpg_host_graph_free": None}

_lib = None


def load_library(path: Path | str | None = None) -> ctypes.CDLL:
    """Loads libdpg.so and declares every entry point; raises if the library was not built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with show-me-dynamic-parallelism_gb300/build.py "
                          "(or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(str(p))
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, c_int)
    if path is None:
        _lib = lib
    return lib


def lib() -> ctypes.CDLL:
    return load_library()


def exported_symbols() -> list[str]:
    return list(_SIGS)


def _check(status: int) -> None:
    if status != 0:
        msg = lib().dpg_last_error()
        raise DpgError(status, msg.decode() if msg else "")


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(c_void_p)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


# ----------------------------------------------------------------------------- host-side helpers --
class CSR(NamedTuple):
    V: int
    E: int
    source: int
    offsets: np.ndarray
    col: np.ndarray
    weights: np.ndarray | None


def _host_to_csr(hg) -> CSR:
    try:
        V, E = hg.V, hg.E
        off = np.ctypeslib.as_array(hg.offsets, shape=(V + 1,)).copy()
        col = np.ctypeslib.as_array(hg.col, shape=(max(E, 1),))[:E].copy()
        w = np.ctypeslib.as_array(hg.weights, shape=(max(E, 1),))[:E].copy()
        return CSR(V, E, hg.source, off, col, w)
    finally:
        lib().dpg_host_graph_free(byref(hg))


def read_graph(path: str | Path, fmt: int = 0, threads: int = 0) -> CSR:
    """readInputDIMACS9/10/SLNDC + convertCSR (common/global.cpp:29-235); fmt is the apps' -f flag.
    DIMACS9 is parsed in parallel unless threads == 1 (identical results)."""
    hg = _HostGraph()
    _check(lib().dpg_read_graph_ex(str(path).encode(), fmt, threads, byref(hg)))
    return _host_to_csr(hg)


def write_graph_cache(path: str | Path, g: CSR) -> None:
    """Binary CSR cache of g (offsets, columns, weights, source)."""
    off, col = _i32(g.offsets), _i32(g.col)
    w = _i32(g.weights) if g.weights is not None else None
    hg = _HostGraph()
    hg.V, hg.E, hg.source = g.V, g.E, g.source
    hg.offsets = off.ctypes.data_as(POINTER(c_int32))
    hg.col = col.ctypes.data_as(POINTER(c_int32))
    hg.weights = w.ctypes.data_as(POINTER(c_int32)) if w is not None else None
    _check(lib().dpg_write_graph_cache(str(path).encode(), byref(hg)))


def read_graph_cache(path: str | Path) -> CSR:
    hg = _HostGraph()
    _check(lib().dpg_read_graph_cache(str(path).encode(), byref(hg)))
    return _host_to_csr(hg)


def csr_from_arcs(V: int, src, dst, w=None) -> CSR:
    """convertCSR on arcs in file order: each row lists its arcs in reverse (global.cpp:192-235)."""
    src, dst = _i32(src), _i32(dst)
    E = int(src.shape[0])
    w = None if w is None else _i32(w)
    off = np.empty(V + 1, np.int32)
    col = np.empty(max(E, 1), np.int32)
    wo = None if w is None else np.empty(max(E, 1), np.int32)
    _check(lib().dpg_csr_from_arcs(V, E, _ptr(src), _ptr(dst), _ptr(w), _ptr(off), _ptr(col), _ptr(wo)))
    return CSR(V, E, 0, off, col[:E], None if wo is None else wo[:E])


def csr_transpose(V: int, offsets, col) -> tuple[np.ndarray, np.ndarray]:
    """invertGraph (global.cpp:237-277): in-edge CSR in the reference's neighbour order."""
    offsets, col = _i32(offsets), _i32(col)
    E = int(col.shape[0])
    in_off = np.empty(V + 1, np.int32)
    in_col = np.empty(max(E, 1), np.int32)
    _check(lib().dpg_csr_transpose(V, E, _ptr(offsets), _ptr(col), _ptr(in_off), _ptr(in_col)))
    return in_off, in_col[:E]


def out_degrees(offsets) -> np.ndarray:
    """outdegreeArray (apps/pagerank/src/pagerank.cpp:108-113)."""
    o = _i32(offsets)
    return (o[1:] - o[:-1]).astype(np.int32)


def write_dimacs9(path, V, src, dst, w, source=-1) -> None:
    src, dst, w = _i32(src), _i32(dst), _i32(w)
    _check(lib().dpg_write_dimacs9(str(path).encode(), V, int(src.shape[0]), _ptr(src), _ptr(dst), _ptr(w), source))


def write_cost(path, source, dist) -> None:
    d = _i32(dist)
    _check(lib().dpg_write_cost(str(path).encode(), int(d.shape[0]), source, _ptr(d)))


def write_level(path, level) -> None:
    d = _i32(level)
    _check(lib().dpg_write_level(str(path).encode(), int(d.shape[0]), _ptr(d)))


def write_rank(path, rank) -> None:
    r = np.ascontiguousarray(rank, dtype=np.float32)
    _check(lib().dpg_write_rank(str(path).encode(), int(r.shape[0]), _ptr(r)))


def write_color(path, color) -> None:
    c = _i32(color)
    _check(lib().dpg_write_color(str(path).encode(), int(c.shape[0]), _ptr(c)))


def rmat_arcs(scale: int, E: int, seed: int, a=0.57, b=0.19, c=0.19, wmin=1, wmax=100, permute=True,
              V: int | None = None, weights=True):
    """Seeded R-MAT arc list (src, dst, w); V defaults to 2**scale."""
    V = (1 << scale) if V is None else V
    src = np.empty(max(E, 1), np.int32)
    dst = np.empty(max(E, 1), np.int32)
    w = np.empty(max(E, 1), np.int32) if weights else None
    _check(lib().dpg_rmat_arcs(scale, V, E, seed & (2**64 - 1), a, b, c, wmin, wmax, 1 if permute else 0, _ptr(src),
                               _ptr(dst), _ptr(w)))
    return src[:E], dst[:E], (None if w is None else w[:E])


def grid_arcs(rows: int, cols: int, seed: int, wmin=1, wmax=1000):
    E = 2 * (rows * (cols - 1) + cols * (rows - 1))
    src = np.empty(max(E, 1), np.int32)
    dst = np.empty(max(E, 1), np.int32)
    w = np.empty(max(E, 1), np.int32)
    _check(lib().dpg_grid_arcs(rows, cols, seed & (2**64 - 1), wmin, wmax, _ptr(src), _ptr(dst), _ptr(w)))
    return src[:E], dst[:E], w[:E]


def rmat_csr(scale: int, edge_factor: int, seed: int, wmin=1, wmax=100, permute=True, weights=True) -> CSR:
    """R-MAT(0.57,0.19,0.19,0.05) graph as the reference loader would build it from a .gr file."""
    V = 1 << scale
    src, dst, w = rmat_arcs(scale, edge_factor * V, seed, wmin=wmin, wmax=wmax, permute=permute, weights=weights)
    return csr_from_arcs(V, src, dst, w)


def grid_csr(rows: int, cols: int, seed: int, wmin=1, wmax=1000) -> CSR:
    src, dst, w = grid_arcs(rows, cols, seed, wmin, wmax)
    return csr_from_arcs(rows * cols, src, dst, w)


# -------------------------------------------------------------------------------- device side ----
class Context:
    """dpg_ctx: one device, one stream, a status word and a scratch arena."""

    def __init__(self, device: int = 0):
        h = c_void_p()
        _check(lib().dpg_ctx_create(device, byref(h)))
        self.handle = h
        self.device = device

    def close(self) -> None:
        if self.handle:
            lib().dpg_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None) -> None:
        """Runs later calls on a cudaStream_t handle. None restores the context's own stream; 0 (what
        torch reports for the default stream) selects the legacy default stream (cudaStreamLegacy)."""
        if stream_handle is None:
            h = None
        elif stream_handle == 0:
            h = c_void_p(1)  # cudaStreamLegacy
        else:
            h = c_void_p(stream_handle)
        _check(lib().dpg_ctx_set_stream(self.handle, h))

    def synchronize(self) -> None:
        _check(lib().dpg_ctx_synchronize(self.handle))

    def last_stats(self) -> RunStats:
        s = RunStats()
        _check(lib().dpg_ctx_last_stats(self.handle, byref(s)))
        return s

    def profile(self, enable: bool = True) -> None:
        """Brackets every later kernel launch with CUDA events (launch counts are always kept)."""
        _check(lib().dpg_ctx_profile_enable(self.handle, 1 if enable else 0))

    def profile_reset(self) -> None:
        _check(lib().dpg_ctx_profile_reset(self.handle))

    def profile_read(self, kind: int) -> tuple[int, float]:
        """(launches, summed device ms) of one kernel kind since the last reset."""
        n, ms = c_int64(), c_double()
        _check(lib().dpg_ctx_profile_read(self.handle, kind, byref(n), byref(ms)))
        return n.value, ms.value

    def trace(self, max_iterations: int) -> None:
        """Records a per-iteration trace of later SSSP/BFS solves (0 turns it off)."""
        _check(lib().dpg_ctx_trace_enable(self.handle, max_iterations))

    def trace_read(self, capacity: int = 100000) -> np.ndarray:
        """[k, 4] int64 rows {ns at iteration start, small frontier, chunks, end flag} of the last solve."""
        buf = np.zeros((capacity, 4), np.int64)
        n = c_int32()
        _check(lib().dpg_ctx_trace_read(self.handle, _ptr(buf), capacity, byref(n)))
        rows = buf[: n.value]
        end = np.flatnonzero(rows[:, 3] == 1)
        return rows[: end[0] + 1] if end.size else rows[(rows[:, 0] != 0)]

    @property
    def sm_count(self) -> int:
        n = c_int32()
        _check(lib().dpg_ctx_sm_count(self.handle, byref(n)))
        return n.value


class Graph:
    """dpg_graph: a CSR resident on the context's device (weights optional)."""

    def __init__(self, ctx: Context, offsets, col, weights=None, *, _handle=None, _V=0, _E=0):
        self.ctx = ctx
        if _handle is not None:
            self.handle, self.V, self.E = _handle, _V, _E
            return
        off = _i32(offsets)
        col = _i32(col)
        w = None if weights is None else _i32(weights)
        self.V = int(off.shape[0]) - 1
        self.E = int(col.shape[0])
        h = c_void_p()
        _check(lib().dpg_graph_create(ctx.handle, self.V, self.E, _ptr(off), _ptr(col), _ptr(w), byref(h)))
        self.handle = h

    @classmethod
    def from_device(cls, ctx: Context, V: int, E: int, d_offsets: int, d_col: int, d_weights: int | None = None):
        h = c_void_p()
        _check(lib().dpg_graph_create_device(ctx.handle, V, E, c_void_p(d_offsets), c_void_p(d_col),
                                             c_void_p(d_weights) if d_weights else None, byref(h)))
        return cls(ctx, None, None, _handle=h, _V=V, _E=E)

    def plan_info(self) -> dict:
        """Row-gather plan counts: tiles (normal tiles and hub segments), small and big hubs, segments."""
        t, hs, hb, sg = c_int32(), c_int32(), c_int32(), c_int32()
        _check(lib().dpg_graph_plan_info(self.handle, byref(t), byref(hs), byref(hb), byref(sg)))
        return {"tiles": t.value, "hubs_small": hs.value, "hubs_big": hb.value, "segments": sg.value}

    def hot_cache(self) -> dict:
        """Shared-memory hot cache of the row gathers: entries kept per CTA and arcs served by them."""
        n, a = c_int32(), c_int64()
        _check(lib().dpg_graph_hot_cache(self.handle, byref(n), byref(a)))
        return {"hot_entries": n.value, "hot_arcs": a.value}

    def set_relabel(self, enable: bool) -> None:
        """Column renaming by frequency for SpMV/PageRank (on by default; results are identical)."""
        _check(lib().dpg_graph_relabel(self.handle, 1 if enable else 0))

    def close(self) -> None:
        if self.handle:
            lib().dpg_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """dpg_batch: many graphs packed as one union CSR on the context's device.

    graphs: weighted CSRs (local vertex ids). vstart[g] is graph g's first union vertex."""

    def __init__(self, ctx: Context, graphs):
        self.ctx = ctx
        self.n = len(graphs)
        Vs = np.array([g.V for g in graphs], np.int64)
        Es = np.array([g.E for g in graphs], np.int64)
        self.vstart = np.zeros(self.n + 1, np.int64)
        np.cumsum(Vs, out=self.vstart[1:])
        estart = np.zeros(self.n + 1, np.int64)
        np.cumsum(Es, out=estart[1:])
        self.V, self.E = int(self.vstart[-1]), int(estart[-1])
        if self.V >= 2**31 or self.E >= 2**31:
            raise ValueError("a batch holds fewer than 2^31 vertices and arcs")
        off = np.empty(self.V + 1, np.int32)
        col = np.empty(max(self.E, 1), np.int32)
        w = np.empty(max(self.E, 1), np.int32)
        for k, g in enumerate(graphs):
            v0, v1, e0, e1 = int(self.vstart[k]), int(self.vstart[k + 1]), int(estart[k]), int(estart[k + 1])
            off[v0:v1] = np.asarray(g.offsets[:-1], np.int64) + e0
            col[e0:e1] = np.asarray(g.col, np.int64) + v0
            w[e0:e1] = g.weights
        off[self.V] = self.E
        self.vstart = self.vstart.astype(np.int32)
        h = c_void_p()
        _check(lib().dpg_batch_create(ctx.handle, self.n, _ptr(self.vstart), self.E, _ptr(off), _ptr(col), _ptr(w),
                                      byref(h)))
        self.handle = h

    def sources_array(self, sources) -> np.ndarray:
        src = _i32(sources)
        if src.ndim != 2 or src.shape[0] != self.n:
            raise ValueError("sources must be [ngraphs, nsrc]")
        return np.ascontiguousarray(src)

    def sssp_dev(self, sources, d_dist: int, **opts) -> None:
        src = self.sources_array(sources)
        o = expand_opts(**opts)
        _check(lib().dpg_batch_sssp_dev(self.ctx.handle, self.handle, src.shape[1], _ptr(src), byref(o),
                                        c_void_p(d_dist)))

    def pagerank_dev(self, d_rank: int, **opts) -> None:
        o = pr_opts(**opts)
        _check(lib().dpg_batch_pagerank_dev(self.ctx.handle, self.handle, byref(o), c_void_p(d_rank)))

    def run(self, sources, d_dist: int, d_rank: int, sssp_opts: dict | None = None,
            pr_opts_: dict | None = None) -> None:
        """Both solves as one CUDA-graph launch (captured on first use, replayed after)."""
        src = self.sources_array(sources)
        so = expand_opts(**(sssp_opts or {}))
        po = pr_opts(**(pr_opts_ or {}))
        _check(lib().dpg_batch_run(self.ctx.handle, self.handle, src.shape[1], _ptr(src), byref(so), c_void_p(d_dist),
                                   byref(po), c_void_p(d_rank)))

    def launches(self) -> int:
        n = c_int64(0)
        _check(lib().dpg_batch_launches(self.handle, byref(n)))
        return int(n.value)

    def autotune(self, sources) -> dict:
        src = self.sources_array(sources)
        t = BatchTuning()
        _check(lib().dpg_batch_autotune(self.ctx.handle, self.handle, src.shape[1], _ptr(src), byref(t)))
        return t.as_dict()

    @property
    def tuning(self) -> dict:
        t = BatchTuning()
        _check(lib().dpg_batch_get_tuning(self.handle, byref(t)))
        return t.as_dict()

    @tuning.setter
    def tuning(self, d: dict) -> None:
        t = BatchTuning(d["hub_threshold"], d["chunk"], d["pr_hot"])
        _check(lib().dpg_batch_set_tuning(self.handle, byref(t)))

    def graph_tuning(self) -> dict:
        """The SSSP setting each graph runs with: {"hub_threshold": [n], "chunk": [n]}."""
        hub = np.empty(self.n, np.int32)
        chunk = np.empty(self.n, np.int32)
        _check(lib().dpg_batch_get_graph_tuning(self.handle, _ptr(hub), _ptr(chunk)))
        return {"hub_threshold": hub, "chunk": chunk}

    def set_graph_tuning(self, hub_threshold=None, chunk=None) -> None:
        """Per-graph SSSP settings (both None: back to the batch-wide one)."""
        if hub_threshold is None and chunk is None:
            _check(lib().dpg_batch_set_graph_tuning(self.handle, None, None))
            return
        hub, ch = _i32(hub_threshold), _i32(chunk)
        if hub.shape != (self.n,) or ch.shape != (self.n,):
            raise ValueError("one hub_threshold and one chunk per graph")
        _check(lib().dpg_batch_set_graph_tuning(self.handle, _ptr(hub), _ptr(ch)))

    def close(self) -> None:
        if self.handle:
            lib().dpg_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def calibrate_random_reads(ctx: Context, n_floats: int, iters: int = 400) -> float:
    """Random 4-byte reads per second from an array of n_floats floats (see include/dpg.h)."""
    r = c_double(0.0)
    _check(lib().dpg_calibrate_random_reads(ctx.handle, n_floats, iters, byref(r)))
    return float(r.value)


CDP_NAIVE, CDP_WARP, CDP_BLOCK, CDP_GRID = 1, 2, 3, 4


def bfs_cdp_dev(ctx: Context, g: Graph, source: int, variant: int, d_level: int, pending_limit: int = 0) -> dict:
    """Recursive BFS with device-side child launches (measured comparison); returns launch counts.
    Raises DpgError (DPG_ERR_CAPACITY) when a child launch failed or was skipped."""
    st = CdpStats()
    _check(lib().dpg_bfs_cdp_dev(ctx.handle, g.handle, source, variant, pending_limit, c_void_p(d_level), byref(st)))
    return {"launches": int(st.launches), "failed_launches": int(st.failed_launches),
            "buffer_entries": int(st.buffer_entries)}


def partition_lpt(costs, parts: int) -> tuple[np.ndarray, np.ndarray]:
    """Owner rank of each unit (longest processing time first) and each rank's total cost."""
    c = np.ascontiguousarray(costs, dtype=np.int64)
    owner = np.empty(max(c.shape[0], 1), np.int32)
    load = np.empty(parts, np.int64)
    _check(lib().dpg_partition_lpt(int(c.shape[0]), _ptr(c), parts, _ptr(owner), _ptr(load)))
    return owner[:c.shape[0]], load


def rmat_batch_specs(n: int, seed: int, vmin=1024, vmax=1 << 20, edge_factors=(8, 16, 32)):
    """Vertex counts log-uniform in [vmin, vmax] and edge factors uniform over edge_factors."""
    rng = np.random.default_rng(seed)
    V = np.exp(rng.uniform(np.log(vmin), np.log(vmax), n)).astype(np.int64)
    V = np.clip(V, vmin, vmax)
    ef = rng.choice(np.asarray(edge_factors), n)
    return [(int(v), int(e)) for v, e in zip(V, ef)]


def rmat_batch(specs, seed: int, wmin=1, wmax=100):
    """One seeded R-MAT(0.57,0.19,0.19,0.05) CSR per (V, edge factor); graph k uses seed + k."""
    out = []
    for k, (V, ef) in enumerate(specs):
        scale = max(1, int(np.ceil(np.log2(V))))
        src, dst, w = rmat_arcs(scale, V * ef, seed + k, wmin=wmin, wmax=wmax, V=V)
        out.append(csr_from_arcs(V, src, dst, w))
    return out


def expand_opts(solution=SOL_DIROPT, threshold=0, hub_threshold=0, max_iterations=0, timeout=0.0,
                delta=0) -> ExpandOpts:
    return ExpandOpts(solution, threshold, hub_threshold, max_iterations, timeout, delta)


def sssp(ctx: Context, g: Graph, source: int, **opts) -> np.ndarray:
    """SSSP_GPU: int32 distances, INF_COST (2^30) when unreachable."""
    out = np.empty(max(g.V, 1), np.int32)
    o = expand_opts(**opts)
    _check(lib().dpg_sssp(ctx.handle, g.handle, source, byref(o), _ptr(out)))
    return out[:g.V]


def sssp_dev(ctx: Context, g: Graph, source: int, d_dist: int, **opts) -> None:
    o = expand_opts(**opts)
    _check(lib().dpg_sssp_dev(ctx.handle, g.handle, source, byref(o), c_void_p(d_dist)))


def bfs(ctx: Context, g: Graph, source: int, **opts) -> np.ndarray:
    """BFS_REC_GPU: int32 levels, UNDEFINED_LEVEL when unreachable."""
    out = np.empty(max(g.V, 1), np.int32)
    o = expand_opts(**opts)
    _check(lib().dpg_bfs(ctx.handle, g.handle, source, byref(o), _ptr(out)))
    return out[:g.V]


def bfs_dev(ctx: Context, g: Graph, source: int, d_level: int, **opts) -> None:
    o = expand_opts(**opts)
    _check(lib().dpg_bfs_dev(ctx.handle, g.handle, source, byref(o), c_void_p(d_level)))


def color(ctx: Context, g: Graph, **opts) -> np.ndarray:
    """GRAPH_COLOR_GPU: colour of each vertex under the reference's round rule (1-based)."""
    out = np.empty(max(g.V, 1), np.int32)
    o = expand_opts(**opts)
    _check(lib().dpg_color(ctx.handle, g.handle, byref(o), _ptr(out)))
    return out[:g.V]


def color_dev(ctx: Context, g: Graph, d_color: int, **opts) -> None:
    o = expand_opts(**opts)
    _check(lib().dpg_color_dev(ctx.handle, g.handle, byref(o), c_void_p(d_color)))


def spmv(ctx: Context, g: Graph, vals, x) -> np.ndarray:
    """SpMV_GPU in FP32: y = A x with A's nonzeros in CSR order."""
    v = np.ascontiguousarray(vals, dtype=np.float32)
    xx = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(max(g.V, 1), np.float32)
    _check(lib().dpg_spmv_f32(ctx.handle, g.handle, _ptr(v), _ptr(xx), _ptr(y)))
    return y[:g.V]


def spmm_dev(ctx: Context, g: Graph, d_vals: int, nrhs: int, d_X: int, d_Y: int) -> None:
    """Y = A X for nrhs row-major columns (device pointers)."""
    _check(lib().dpg_spmm_f32_dev(ctx.handle, g.handle, c_void_p(d_vals), nrhs, c_void_p(d_X), c_void_p(d_Y)))


def spmv_bwd_dev(ctx: Context, g: Graph, d_vals: int, nrhs: int, d_X: int | None, d_G: int, d_dX: int | None,
                 d_dA: int | None) -> None:
    """dX = A^T G and dA[e] = <G[row(e)], X[col(e)]> (device pointers; None skips an output)."""
    _check(lib().dpg_spmv_bwd_f32_dev(ctx.handle, g.handle, c_void_p(d_vals), nrhs,
                                      c_void_p(d_X) if d_X else None, c_void_p(d_G),
                                      c_void_p(d_dX) if d_dX else None, c_void_p(d_dA) if d_dA else None))


def pagerank_grad_dev(ctx: Context, g: Graph, d_weights: int, d_seed: int, d_rank: int, d_grad: int,
                      adjoint_epsilon: float = 0.0, **opts) -> tuple[int, int]:
    """Weighted PageRank r on the out-adjacency g and dL/dw for the seed dL/dr (device pointers).
    Returns (forward sweeps, adjoint sweeps)."""
    o = pr_opts(**opts)
    _check(lib().dpg_pagerank_grad_f32_dev(ctx.handle, g.handle, c_void_p(d_weights), c_void_p(d_seed), byref(o),
                                           float(adjoint_epsilon), c_void_p(d_rank), c_void_p(d_grad)))
    f, a = c_int64(0), c_int64(0)
    _check(lib().dpg_ctx_grad_sweeps(ctx.handle, byref(f), byref(a)))
    return int(f.value), int(a.value)


def csr_transpose_dev(ctx: Context, V: int, E: int, d_offsets: int, d_col: int, d_in_offsets: int, d_in_col: int,
                      d_in_arc: int | None = None) -> None:
    """invertGraph on the device (device pointers; stream-ordered)."""
    _check(lib().dpg_csr_transpose_dev(ctx.handle, V, E, c_void_p(d_offsets), c_void_p(d_col), c_void_p(d_in_offsets),
                                       c_void_p(d_in_col), c_void_p(d_in_arc) if d_in_arc else None))


def csr_transpose_perm(V: int, offsets, col):
    """invertGraph order plus in_arc[p] = index of the arc that transposed slot p came from."""
    offsets, col = _i32(offsets), _i32(col)
    E = int(col.shape[0])
    in_off = np.empty(V + 1, np.int32)
    in_col = np.empty(max(E, 1), np.int32)
    in_arc = np.empty(max(E, 1), np.int32)
    _check(lib().dpg_csr_transpose_perm(V, E, _ptr(offsets), _ptr(col), _ptr(in_off), _ptr(in_col), _ptr(in_arc)))
    return in_off, in_col[:E], in_arc[:E]


def spmv_dev(ctx: Context, g: Graph, d_vals: int, d_x: int, d_y: int) -> None:
    _check(lib().dpg_spmv_f32_dev(ctx.handle, g.handle, c_void_p(d_vals), c_void_p(d_x), c_void_p(d_y)))


def pr_opts(damping=0.85, total_rank=1.0, init_zero=False, iterations=20, epsilon=0.0) -> PrOpts:
    return PrOpts(damping, total_rank, 1 if init_zero else 0, iterations, epsilon)


def pagerank(ctx: Context, g_in: Graph, outdeg, **opts) -> np.ndarray:
    """PAGERANK_GPU (pull): g_in is the transposed CSR, outdeg the original out-degrees."""
    od = _i32(outdeg)
    r = np.empty(max(g_in.V, 1), np.float32)
    o = pr_opts(**opts)
    _check(lib().dpg_pagerank_f32(ctx.handle, g_in.handle, _ptr(od), byref(o), _ptr(r)))
    return r[:g_in.V]


def pagerank_dev(ctx: Context, g_in: Graph, d_outdeg: int, d_rank: int, **opts) -> None:
    o = pr_opts(**opts)
    _check(lib().dpg_pagerank_f32_dev(ctx.handle, g_in.handle, c_void_p(d_outdeg), byref(o), c_void_p(d_rank)))


def sssp_host(ctx: Context, offsets, col, weights, source: int, **opts) -> np.ndarray:
    """One call with host buffers: upload, solve, download (the whole SSSP_GPU)."""
    off, c, w = _i32(offsets), _i32(col), _i32(weights)
    V = int(off.shape[0]) - 1
    out = np.empty(max(V, 1), np.int32)
    o = expand_opts(**opts)
    _check(lib().dpg_sssp_host(ctx.handle, V, int(c.shape[0]), _ptr(off), _ptr(c), _ptr(w), source, byref(o),
                               _ptr(out)))
    return out[:V]


def pagerank_host(ctx: Context, in_offsets, in_col, outdeg, out=None, **opts) -> np.ndarray:
    """One call with host buffers: upload the transposed CSR, run the sweeps, download ranks."""
    io, ic, od = _i32(in_offsets), _i32(in_col), _i32(outdeg)
    V = int(io.shape[0]) - 1
    r = np.empty(max(V, 1), np.float32) if out is None else out
    o = pr_opts(**opts)
    _check(lib().dpg_pagerank_f32_host(ctx.handle, V, int(ic.shape[0]), _ptr(io), _ptr(ic), _ptr(od), byref(o),
                                       _ptr(r)))
    return r[:V]


NOALLOC_MAX_VERTICES = 1 << 18
NOALLOC_MAX_ARCS = 1 << 22


def sssp_noalloc_dev(V: int, E: int, d_offsets: int, d_adj_pairs: int, source: int, d_dist: int,
                     stream: int = 0) -> None:
    """SSSP that allocates nothing (see include/dpg.h): device pointers in and out, workspace in a
    fixed array inside the library; synchronises `stream`."""
    _check(lib().dpg_sssp_noalloc_dev(V, E, c_void_p(d_offsets), c_void_p(d_adj_pairs), source, c_void_p(d_dist),
                                      c_void_p(stream) if stream else None))


def selftest_barrier_timeout(ctx: Context, seconds: float = 0.5) -> int:
    """Runs a grid barrier that can never complete; returns the status (DPG_ERR_TIMEOUT expected)."""
    return int(lib().dpg_selftest_barrier_timeout(ctx.handle, seconds))
