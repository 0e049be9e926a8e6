"""Golden vectors from the reference's own kernels, run on a GPU: tests/golden/refgpu.npz.

The reference has no CPU SSSP, colouring, SpMV or PageRank; its kernels are the only reference
implementation of them. This script runs those kernels, compiled from the reference tree into
device modules by oracle/Makefile (`refgpu`, see oracle/ref_kernels.cu), through the driver in
oracle/ref_gpu_driver.cpp, and records their outputs:

    # where the reference tree is (any machine with nvcc):
    make -C oracle refgpu REF=<reference tree>
    # on a machine with a GB300 (the modules travel in oracle/_ref/):
    make -C oracle all refgpu-driver && python tests/golden/make_golden_gpu.py --out tests/golden/refgpu.npz

Inputs (no file from the reference tree is read here):
  * data_test: the CSR and transposed CSR that the reference loader builds from its
    datasets/data_test.gr, as recorded in tests/golden/data_test.json by make_golden.py;
  * rmat14: the R-MAT scale-14, edge-factor-16 graph with weights uniform in [1, 100] (seed 1),
    built by the oracle's generator and convertCSR restatement, which the CPU tests pin to the
    reference loader; SSSP sources 0 (the stated source), the vertex of largest out-degree and two
    seeded random vertices with out-arcs;
  * rmat12: R-MAT scale 12, edge factor 16, seed 3 (unweighted), for SpMV and PageRank; its FP32
    values come from `hash_uniform`, a counter hash that needs no random-number library.
Runs per graph: SSSP (solution 0: unorder_generateQueue_kernel + unorder_threadQueue_kernel),
colouring (gclr_bitmap_kernel rounds), SpMV in FP64 (csr_spmv_kernel) with the reference's own
values (data[e] = e%13+0.5, x[i] = i%17+0.5) and with FP32-representable random values (values in
(0, 1], x in [-1, 1]), and PageRank (pagerank_thread_pull_kernel with the dangling and delta
kernels) in the reference's mode (d = 0.5, total 1000, ranks from 0, until no change exceeds
1e-13) and with d = 0.85, total 1, ranks from 1/V and exactly 20 sweeps.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import sys
from ctypes import c_char_p, c_double, c_float, c_int, c_longlong, c_void_p
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
GOLDEN = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "oracle"))

RMAT14 = dict(scale=14, edge_factor=16, seed=1, wmin=1, wmax=100)
RMAT12 = dict(scale=12, edge_factor=16, seed=3)
SPMV_SEED = 12
PR_SWEEPS = 20


def hash_uniform(n: int, seed: int) -> np.ndarray:
    """n FP32 values k / 2^24 (k in [0, 2^24)) from splitmix64 of (seed, index): exact in FP32 and
    the same on every machine and numpy version."""
    with np.errstate(over="ignore"):
        x = np.arange(n, dtype=np.uint64) + np.uint64(seed) * np.uint64(0xD1B54A32D192ED03)
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return ((x >> np.uint64(40)).astype(np.float64) / float(1 << 24)).astype(np.float32)


def spmv_random_inputs(E: int, V: int):
    """FP32 values in (0, 1] and x in [-1, 1), the distributions of the SpMV benchmark."""
    vals = (np.float32(1.0) - hash_uniform(E, SPMV_SEED)).astype(np.float32)
    x = (np.float32(2.0) * hash_uniform(V, SPMV_SEED + 1) - np.float32(1.0)).astype(np.float32)
    return vals, x


def spmv_reference_inputs(E: int, V: int):
    """The SpMV app's own values (SpMV_wrapper.cu:105-110)."""
    return np.arange(E) % 13 + 0.5, np.arange(V) % 17 + 0.5


def graphs():
    """name -> (off, col, w, in_off, in_col) for every input graph."""
    import oracle

    dt = json.loads((GOLDEN / "data_test.json").read_text())
    i32 = lambda a: np.asarray(a, np.int32)  # noqa: E731
    out = {"data_test": (i32(dt["offsets"]), i32(dt["col"]), i32(dt["weights"]), i32(dt["in_offsets"]),
                         i32(dt["in_col"]))}
    off, col, w = oracle.rmat_csr(RMAT14["scale"], RMAT14["edge_factor"], RMAT14["seed"], RMAT14["wmin"],
                                  RMAT14["wmax"])
    out["rmat14"] = (off, col, w) + oracle.csr_transpose(off, col)
    off, col, _ = oracle.rmat_csr(RMAT12["scale"], RMAT12["edge_factor"], RMAT12["seed"], weights=False)
    out["rmat12"] = (off, col, None) + oracle.csr_transpose(off, col)
    return out, int(dt["source"])


def rmat14_sources(off) -> list[int]:
    deg = np.diff(off)
    rnd = np.random.default_rng(14).choice(np.flatnonzero(deg > 0), 2, replace=False)
    return [0, int(np.argmax(deg))] + [int(s) for s in rnd]


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(GOLDEN / "refgpu.npz"))
    args = ap.parse_args()
    mods = {a: ROOT / "oracle" / "_ref" / f"ref_{a}.cubin" for a in ("sssp", "color", "spmv", "pagerank")}
    for a, m in mods.items():
        if not m.exists():
            raise SystemExit(f"{m} is missing: run `make -C oracle refgpu REF=<reference tree>` first")
    lib = ctypes.CDLL(str(ROOT / "oracle" / "_build" / "librefgpu.so"))
    P = c_void_p
    lib.refgpu_sssp.argtypes = [c_char_p, c_int, c_longlong, P, P, P, c_int, P]
    lib.refgpu_color.argtypes = [c_char_p, c_int, c_longlong, P, P, P]
    lib.refgpu_spmv_f64.argtypes = [c_char_p, c_int, c_longlong, P, P, P, P, P]
    lib.refgpu_pagerank.argtypes = [c_char_p, c_int, c_longlong, P, P, P, c_float, c_double, c_int, c_int, c_int, P]
    for f in (lib.refgpu_sssp, lib.refgpu_color, lib.refgpu_spmv_f64, lib.refgpu_pagerank):
        f.restype = c_int
    p = lambda a: a.ctypes.data_as(c_void_p)  # noqa: E731
    m = lambda a: str(mods[a]).encode()  # noqa: E731

    def check(rc, what):
        if rc < 0:
            raise SystemExit(f"{what} failed ({rc})")
        return rc

    gs, dt_source = graphs()
    rec: dict[str, np.ndarray] = {}
    for name, (off, col, w, in_off, in_col) in gs.items():
        V, E = off.shape[0] - 1, col.shape[0]
        if w is not None:
            sources = [dt_source] if name == "data_test" else rmat14_sources(off)
            rec[f"{name}/sssp_sources"] = np.asarray(sources, np.int32)
            dists, iters = [], []
            for s in sources:
                d = np.empty(V, np.int32)
                iters.append(check(lib.refgpu_sssp(m("sssp"), V, E, p(off), p(col), p(w), s, p(d)), f"{name} sssp"))
                dists.append(d)
            rec[f"{name}/sssp_dist"] = np.stack(dists)
            rec[f"{name}/sssp_iterations"] = np.asarray(iters, np.int32)
            c = np.empty(V, np.int32)
            rec[f"{name}/color_rounds"] = np.int32(check(lib.refgpu_color(m("color"), V, E, p(off), p(col), p(c)),
                                                         f"{name} color"))
            rec[f"{name}/color"] = c
        if name == "rmat14":
            continue  # SpMV and PageRank run on data_test and rmat12
        for mode, (data, x) in (("refvals", spmv_reference_inputs(E, V)), ("f32vals", spmv_random_inputs(E, V))):
            d64 = np.ascontiguousarray(data, np.float64)
            x64 = np.ascontiguousarray(x, np.float64)
            y = np.empty(V, np.float64)
            check(lib.refgpu_spmv_f64(m("spmv"), V, E, p(off), p(col), p(d64), p(x64), p(y)), f"{name} spmv")
            rec[f"{name}/spmv_{mode}_y"] = y
        od = np.diff(off).astype(np.int32)
        r = np.empty(V, np.float32)
        n = check(lib.refgpu_pagerank(m("pagerank"), V, E, p(in_off), p(in_col), p(od), 0.5, 1000.0, 0, 100000, 0,
                                      p(r)), f"{name} pagerank (reference mode)")
        rec[f"{name}/pagerank_refmode_rank"] = r.copy()
        rec[f"{name}/pagerank_refmode_sweeps"] = np.int32(n)
        n = check(lib.refgpu_pagerank(m("pagerank"), V, E, p(in_off), p(in_col), p(od), 0.85, 1.0, 1, PR_SWEEPS, 1,
                                      p(r)), f"{name} pagerank (d=0.85)")
        rec[f"{name}/pagerank_d085_rank"] = r.copy()
        rec[f"{name}/pagerank_d085_sweeps"] = np.int32(n)
    out = Path(args.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(out, **rec)
    print(f"wrote {out}: " + ", ".join(f"{k}{list(v.shape)}" for k, v in rec.items()))
    return 0


if __name__ == "__main__":
    sys.exit(main())
