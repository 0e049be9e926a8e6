"""CPU oracle bindings — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import this module, and only
as the checker or as the timed CPU baseline. The product library (libdpg.so) never calls it.

Libraries:
  * oracle/_build/liboracle.so — our C restatement of the reference algorithms (dpg_oracle.c),
    plus the benchmark graph generator and CSR/transpose builders the CPU arms use;
  * oracle/_ref/libref.so      — the reference's own host code (common/global.cpp loader + CSR +
    invertGraph, apps/bfs-rec/src/bfs_rec.cpp bfs_cpu), compiled from the reference tree by
    oracle/Makefile when that tree is present. It does not exist where the reference is absent;
  * oracle/_ref/ref_*.cubin     — the reference's own kernels as device modules (ref_kernels.cu),
    run by oracle/_build/librefgpu.so (ref_gpu_driver.cpp) only to generate tests/golden/refgpu.npz.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_longlong, c_void_p, POINTER
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "liboracle.so"
REF_SO = HERE / "_ref" / "libref.so"


def _find_reference_tree():
    """The reference source tree: $DPG_REFERENCE_TREE, else a checkout named `reference` beside this
    repository; None when neither holds the reference's common/global.cpp."""
    cands = [Path(os.environ["DPG_REFERENCE_TREE"])] if os.environ.get("DPG_REFERENCE_TREE") else []
    cands.append(HERE.parents[1] / "reference")
    for c in cands:
        if (c / "common" / "global.cpp").exists():
            return c
    return None


REFERENCE_TREE = _find_reference_tree()

INF = 1073741824
UNDEFINED = 0x7FFFFFFF

_P = c_void_p
_ORACLE_SIGS = {
    "oracle_num_threads": ([], c_int),
    "oracle_sssp_dijkstra": ([c_int32, _P, _P, _P, c_int32, _P], c_int),
    "oracle_sssp_worklist": ([c_int32, _P, _P, _P, c_int32, _P], c_int64),
    "oracle_sssp_bf_omp": ([c_int32, _P, _P, _P, c_int32, _P, c_int32], c_int),
    "oracle_bfs": ([c_int32, _P, _P, c_int32, _P], c_int64),
    "oracle_bfs_omp": ([c_int32, _P, _P, c_int32, _P, c_int32], c_int),
    "oracle_spmv_f64": ([c_int32, _P, _P, _P, _P, _P], None),
    "oracle_spmv_f32in": ([c_int32, _P, _P, _P, _P, _P, _P, c_int32], None),
    "oracle_spmv_omp_f32": ([c_int32, _P, _P, _P, _P, _P, c_int32], None),
    "oracle_pagerank_f64": ([c_int32, _P, _P, _P, c_double, c_double, c_int32, c_int32, c_double, _P, c_int32],
                            c_int64),
    "oracle_pagerank_ref_f32": ([c_int32, _P, _P, _P, c_float, c_double, c_int32, c_int32, c_double, _P], c_int64),
    "oracle_pagerank_omp_f32": ([c_int32, _P, _P, _P, c_float, c_float, c_int32, _P, c_int32], c_int64),
    "oracle_color": ([c_int32, _P, _P, _P], c_int64),
    "oracle_rmat_arcs": ([c_int32, c_int32, c_int64, ctypes.c_uint64, c_double, c_double, c_double, c_int32, c_int32,
                          c_int32, _P, _P, _P], c_int),
    "oracle_csr_from_arcs": ([c_int32, c_int64, _P, _P, _P, _P, _P, _P], c_int),
    "oracle_csr_transpose": ([c_int32, _P, _P, _P, _P], c_int),
}
_REF_SIGS = {
    "ref_load": ([c_char_p, c_int, POINTER(c_int), POINTER(c_longlong), POINTER(c_int)], c_int),
    "ref_get_csr": ([_P, _P, _P], None),
    "ref_get_transpose": ([_P, _P], None),
    "ref_bfs_cpu": ([c_int, _P], None),
    "ref_output_cost": ([c_char_p, c_int, _P], c_int),
    "ref_output_rank": ([c_char_p, _P], c_int),
    "ref_output_color": ([c_char_p, _P], c_int),
}

_oracle = None
_ref = None


def build(with_reference: bool | None = None) -> None:
    """Compiles liboracle.so; where the reference tree is present, also libref.so (its host code) and
    the device modules of its kernels (oracle/_ref/ref_*.cubin, for tests/golden/make_golden_gpu.py)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if with_reference is None:
        with_reference = REFERENCE_TREE is not None
    if with_reference:
        if REFERENCE_TREE is None:
            raise FileNotFoundError("set DPG_REFERENCE_TREE to the reference source tree")
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", "refgpu", f"REF={REFERENCE_TREE}"], check=True)


def _load(path: Path, sigs):
    lib = ctypes.CDLL(str(path))
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


def oracle_lib():
    global _oracle
    if _oracle is None:
        if not ORACLE_SO.exists():
            build(with_reference=False)
        _oracle = _load(ORACLE_SO, _ORACLE_SIGS)
    return _oracle


def ref_available() -> bool:
    return REF_SO.exists()


def ref_lib():
    global _ref
    if _ref is None:
        if not REF_SO.exists():
            raise FileNotFoundError("oracle/_ref/libref.so is not built (the reference tree is absent here)")
        _ref = _load(REF_SO, _REF_SIGS)
    return _ref


def _p(a):
    return a.ctypes.data_as(c_void_p)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def num_threads() -> int:
    return int(oracle_lib().oracle_num_threads())


def sssp_dijkstra(off, col, w, src) -> np.ndarray:
    off, col, w = _i32(off), _i32(col), _i32(w)
    V = off.shape[0] - 1
    d = np.empty(max(V, 1), np.int32)
    rc = oracle_lib().oracle_sssp_dijkstra(V, _p(off), _p(col), _p(w), src, _p(d))
    if rc != 0:
        raise RuntimeError(f"oracle_sssp_dijkstra failed ({rc})")
    return d[:V]


def sssp_worklist(off, col, w, src) -> tuple[np.ndarray, int]:
    off, col, w = _i32(off), _i32(col), _i32(w)
    V = off.shape[0] - 1
    d = np.empty(max(V, 1), np.int32)
    passes = oracle_lib().oracle_sssp_worklist(V, _p(off), _p(col), _p(w), src, _p(d))
    return d[:V], int(passes)


def sssp_bf_omp(off, col, w, src, threads=0) -> np.ndarray:
    off, col, w = _i32(off), _i32(col), _i32(w)
    V = off.shape[0] - 1
    d = np.empty(max(V, 1), np.int32)
    if oracle_lib().oracle_sssp_bf_omp(V, _p(off), _p(col), _p(w), src, _p(d), threads) != 0:
        raise RuntimeError("oracle_sssp_bf_omp failed")
    return d[:V]


def bfs(off, col, src) -> np.ndarray:
    off, col = _i32(off), _i32(col)
    V = off.shape[0] - 1
    lv = np.empty(max(V, 1), np.int32)
    if oracle_lib().oracle_bfs(V, _p(off), _p(col), src, _p(lv)) < 0:
        raise RuntimeError("oracle_bfs failed")
    return lv[:V]


def bfs_omp(off, col, src, threads=0) -> np.ndarray:
    off, col = _i32(off), _i32(col)
    V = off.shape[0] - 1
    lv = np.empty(max(V, 1), np.int32)
    if oracle_lib().oracle_bfs_omp(V, _p(off), _p(col), src, _p(lv), threads) != 0:
        raise RuntimeError("oracle_bfs_omp failed")
    return lv[:V]


def spmv_f64(off, col, data, x) -> np.ndarray:
    off, col = _i32(off), _i32(col)
    data = np.ascontiguousarray(data, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    V = off.shape[0] - 1
    y = np.empty(max(V, 1), np.float64)
    oracle_lib().oracle_spmv_f64(V, _p(off), _p(col), _p(data), _p(x), _p(y))
    return y[:V]


def spmv_f32in(off, col, data, x, threads=0) -> tuple[np.ndarray, np.ndarray]:
    """FP64 accumulation of FP32 products; returns (y, sum |a_ij x_j| per row)."""
    off, col = _i32(off), _i32(col)
    data = np.ascontiguousarray(data, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    V = off.shape[0] - 1
    y = np.empty(max(V, 1), np.float64)
    a = np.empty(max(V, 1), np.float64)
    oracle_lib().oracle_spmv_f32in(V, _p(off), _p(col), _p(data), _p(x), _p(y), _p(a), threads)
    return y[:V], a[:V]


def spmv_omp_f32(off, col, data, x, threads=0) -> np.ndarray:
    off, col = _i32(off), _i32(col)
    data = np.ascontiguousarray(data, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    V = off.shape[0] - 1
    y = np.empty(max(V, 1), np.float32)
    oracle_lib().oracle_spmv_omp_f32(V, _p(off), _p(col), _p(data), _p(x), _p(y), threads)
    return y[:V]


def pagerank_f64(in_off, in_col, outdeg, damping=0.85, total=1.0, init_zero=False, iterations=20, epsilon=0.0,
                 threads=0) -> tuple[np.ndarray, int]:
    in_off, in_col, outdeg = _i32(in_off), _i32(in_col), _i32(outdeg)
    V = in_off.shape[0] - 1
    r = np.empty(max(V, 1), np.float64)
    n = oracle_lib().oracle_pagerank_f64(V, _p(in_off), _p(in_col), _p(outdeg), damping, total, 1 if init_zero else 0,
                                         iterations, epsilon, _p(r), threads)
    return r[:V], int(n)


def pagerank_ref_f32(in_off, in_col, outdeg, damping=0.5, total=1000.0, init_zero=True, max_iterations=10000,
                     epsilon=1e-13) -> tuple[np.ndarray, int]:
    """The reference's FP32 PageRank loop (defaults: its own parameters). epsilon < 0: exactly
    max_iterations sweeps."""
    in_off, in_col, outdeg = _i32(in_off), _i32(in_col), _i32(outdeg)
    V = in_off.shape[0] - 1
    r = np.empty(max(V, 1), np.float32)
    n = oracle_lib().oracle_pagerank_ref_f32(V, _p(in_off), _p(in_col), _p(outdeg), damping, total,
                                             1 if init_zero else 0, max_iterations, epsilon, _p(r))
    return r[:V], int(n)


def pagerank_omp_f32(in_off, in_col, outdeg, damping=0.85, total=1.0, iterations=20, threads=0) -> np.ndarray:
    in_off, in_col, outdeg = _i32(in_off), _i32(in_col), _i32(outdeg)
    V = in_off.shape[0] - 1
    r = np.empty(max(V, 1), np.float32)
    oracle_lib().oracle_pagerank_omp_f32(V, _p(in_off), _p(in_col), _p(outdeg), damping, total, iterations, _p(r),
                                         threads)
    return r[:V]


def rmat_arcs(scale, E, seed, wmin=1, wmax=100, permute=True, weights=True, V=None, a=0.57, b=0.19, c=0.19):
    """The benchmark's seeded R-MAT arc list (src, dst, w or None), generated on the CPU."""
    V = (1 << scale) if V is None else V
    src = np.empty(max(E, 1), np.int32)
    dst = np.empty(max(E, 1), np.int32)
    w = np.empty(max(E, 1), np.int32) if weights else None
    rc = oracle_lib().oracle_rmat_arcs(scale, V, E, seed, a, b, c, wmin, wmax, 1 if permute else 0, _p(src), _p(dst),
                                       _p(w) if weights else None)
    if rc != 0:
        raise RuntimeError(f"oracle_rmat_arcs failed ({rc})")
    return src[:E], dst[:E], (w[:E] if weights else None)


def csr_from_arcs(V, src, dst, w=None):
    """convertCSR's arrays (off, col, w or None) from an arc list in input order."""
    src, dst = _i32(src), _i32(dst)
    E = src.shape[0]
    off = np.empty(V + 1, np.int32)
    col = np.empty(max(E, 1), np.int32)
    wo = np.empty(max(E, 1), np.int32) if w is not None else None
    wi = _i32(w) if w is not None else None
    rc = oracle_lib().oracle_csr_from_arcs(V, E, _p(src), _p(dst), _p(wi) if wi is not None else None, _p(off), _p(col),
                                           _p(wo) if wo is not None else None)
    if rc != 0:
        raise RuntimeError(f"oracle_csr_from_arcs failed ({rc})")
    return off, col[:E], (wo[:E] if wo is not None else None)


def rmat_csr(scale, edge_factor, seed, wmin=1, wmax=100, permute=True, weights=True):
    """(off, col, w or None) of the benchmark's R-MAT graph as the reference loader would build it."""
    V = 1 << scale
    src, dst, w = rmat_arcs(scale, edge_factor * V, seed, wmin, wmax, permute, weights)
    return csr_from_arcs(V, src, dst, w)


def csr_transpose(off, col):
    """invertGraph's arrays (in_off, in_col)."""
    off, col = _i32(off), _i32(col)
    V = off.shape[0] - 1
    in_off = np.empty(V + 1, np.int32)
    in_col = np.empty(max(col.shape[0], 1), np.int32)
    rc = oracle_lib().oracle_csr_transpose(V, _p(off), _p(col), _p(in_off), _p(in_col))
    if rc != 0:
        raise RuntimeError(f"oracle_csr_transpose failed ({rc})")
    return in_off, in_col[:col.shape[0]]


def color(off, col) -> tuple[np.ndarray, int]:
    off, col = _i32(off), _i32(col)
    V = off.shape[0] - 1
    c = np.empty(max(V, 1), np.int32)
    n = oracle_lib().oracle_color(V, _p(off), _p(col), _p(c))
    return c[:V], int(n)


# ------------------------------------------- weighted PageRank and its edge-weight gradient (FP64) --
# No counterpart in the reference; restated from the fixed-point equations that
# dpg_pagerank_grad_f32_dev documents, and checked against central differences of the forward map.
def _weighted_operator(off, col, w):
    import scipy.sparse as sp

    off = np.asarray(off, np.int64)
    V = off.shape[0] - 1
    # Copies: scipy may canonicalise (sum duplicate arcs) in place on the arrays it is given.
    A = sp.csr_matrix((np.asarray(w, np.float64).copy(), np.asarray(col, np.int64).copy(), off.copy()), shape=(V, V))
    W = np.zeros(V)
    np.add.at(W, np.repeat(np.arange(V), np.diff(off)), np.asarray(w, np.float64))
    return A, W


def pagerank_weighted_f64(off, col, w, damping=0.85, total=1.0, init_zero=False, iterations=5000, epsilon=1e-15):
    """r[v] = (1-d)T/V + d D/V + d sum_{u->v} w r[u]/W[u]; sweeps until every |change| <= epsilon * |r|.
    Returns (r, sweeps)."""
    A, W = _weighted_operator(off, col, w)
    V = W.shape[0]
    AT = A.T.tocsr()
    dang = W == 0
    Wn = np.where(dang, 1.0, W)
    r = np.zeros(V) if init_zero else np.full(V, total / V)
    sweeps = 0
    for _ in range(iterations):
        contrib = np.where(dang, 0.0, r / Wn)
        rn = (1 - damping) * total / V + damping * r[dang].sum() / V + damping * (AT @ contrib)
        sweeps += 1
        done = bool(np.all(np.abs(rn - r) <= epsilon * np.abs(rn)))
        r = rn
        if epsilon > 0 and done:
            break
    return r, sweeps


def pagerank_weighted_grad_f64(off, col, w, seed, damping=0.85, total=1.0, iterations=5000, epsilon=1e-15):
    """(r, lambda, dL/dw) for seed = dL/dr, by the adjoint fixed point
    lambda[u] = s[u] + d/W[u] sum_{u->t} w lambda[t] (dangling: s[u] + d/V sum lambda)."""
    off = np.asarray(off, np.int64)
    col = np.asarray(col, np.int64)
    r, _ = pagerank_weighted_f64(off, col, w, damping, total, False, iterations, epsilon)
    A, W = _weighted_operator(off, col, w)
    V = W.shape[0]
    dang = W == 0
    Wn = np.where(dang, 1.0, W)
    s = np.asarray(seed, np.float64)
    lam = s.copy()
    for _ in range(iterations):
        y = A @ lam
        ln = s + np.where(dang, damping / V * lam.sum(), damping * y / Wn)
        done = bool(np.all(np.abs(ln - lam) <= epsilon * np.abs(ln)))
        lam = ln
        if epsilon > 0 and done:
            break
    q = np.where(dang, 0.0, (A @ lam) / Wn)
    rows = np.repeat(np.arange(V), np.diff(off))
    c = np.where(dang, 0.0, damping * r / Wn)
    grad = c[rows] * (lam[col] - q[rows])
    return r, lam, grad


# ----------------------------------------------------------------- the reference's own host code --
def ref_load(path, fmt=0):
    """The reference loader itself: returns (V, E, source, off, col, w, in_off, in_col)."""
    lib = ref_lib()
    V, E, s = c_int(), c_longlong(), c_int()
    rc = lib.ref_load(str(path).encode(), fmt, ctypes.byref(V), ctypes.byref(E), ctypes.byref(s))
    if rc != 0:
        raise RuntimeError(f"ref_load failed ({rc})")
    n, m = V.value, E.value
    off = np.empty(n + 1, np.int32)
    col = np.empty(max(m, 1), np.int32)
    w = np.empty(max(m, 1), np.int32)
    lib.ref_get_csr(_p(off), _p(col), _p(w))
    in_off = np.empty(n + 1, np.int32)
    in_col = np.empty(max(m, 1), np.int32)
    lib.ref_get_transpose(_p(in_off), _p(in_col))
    return n, m, s.value, off, col[:m], w[:m], in_off, in_col[:m]


def ref_bfs_cpu(src, V) -> np.ndarray:
    """bfs_cpu of the reference on the graph loaded last by ref_load."""
    lv = np.empty(max(V, 1), np.int32)
    ref_lib().ref_bfs_cpu(src, _p(lv))
    return lv[:V]
