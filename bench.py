#!/usr/bin/env python3
"""Benchmark of the irregular CSR neighbour-expansion path on GB300.

Headline workload (one "step"): a 20-sweep pull PageRank (damping 0.85, out-degree normalised,
dangling mass spread uniformly) over a seeded R-MAT graph of scale 22 and edge factor 16
(4,194,304 vertices, 67,108,864 arcs). Metric: GTEPS = arcs x sweeps / second, whole job.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl dpg|reference] [--no-extra]

* value: device-resident inputs, CUDA events around K steps on the launching stream.
* e2e: the one-shot C-ABI call with host buffers (pinned), H2D of the transposed CSR and
  out-degrees and D2H of the ranks inside the timed region.
* roofline: the row-gather kernel's algorithmic bytes per sweep / its average launch time from
  CUDA events recorded around every launch inside the timed region.
* cpu_baseline / --impl reference: the CPU restatement of the reference's PageRank (the reference
  has no CPU PageRank), all host threads, timed on a bounded sample.
* extra: SpMV on the same graph; SSSP, BFS and PageRank on R-MAT scale 24 (268,435,456 arcs); the
  adjoint, gradient, batch, grid and CDP2 legs.
Multi-GPU (torchrun): replicas only, one independent copy of the workload per rank; time = max over
ranks; value = all ranks' arcs x sweeps / that time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GTEPS (SSSP/PageRank) on 1 GB300, % of HBM roofline; batched+adjoint vs plain"
SCALE, EDGE_FACTOR, SWEEPS, DAMPING, GRAPH_SEED = 22, 16, 20, 0.85, 22
WORKLOAD = (f"pagerank-pull rmat(0.57,0.19,0.19,0.05) scale {SCALE} edge-factor {EDGE_FACTOR}, "
            f"{SWEEPS} sweeps, d={DAMPING}")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["dpg", "reference"], default="dpg")
    ap.add_argument("--no-extra", action="store_true", help="skip the SpMV / SSSP / BFS side measurements")
    ap.add_argument("--workload", choices=["pagerank", "pagerank-large", "spmv", "sssp", "bfs", "adjoint", "prgrad",
                                           "batch", "cdp", "grid"],
                    default="pagerank",
                    help="pagerank is the headline; the others print their own line (used for profiling)")
    ap.add_argument("--scale", type=int, default=0, help="R-MAT scale for --workload spmv/sssp/bfs")
    ap.add_argument("--batch-graphs", type=int, default=512, help="graphs in --workload batch")
    ap.add_argument("--solution", type=int, default=-1, help="dpg.SOL_* id for --workload sssp/bfs (-1: default)")
    ap.add_argument("--no-relabel", action="store_true", help="turn off the column renaming of SpMV/PageRank")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer (e2e) leg and the CPU baseline")
    ap.add_argument("--ingest-traffic", metavar="CSV", help="write profiles/" + TRAFFIC_FILE + " from the ncu CSV "
                    "of the traffic capture command, then exit")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# The sources of the headline kernel (row gather + its plan) whose DRAM traffic an ncu capture records.
GATHER_SOURCES = ["show-me-dynamic-parallelism_gb300/csrc/dpg_rowgather.cu",
                  "show-me-dynamic-parallelism_gb300/csrc/dpg_layout.cu",
                  "show-me-dynamic-parallelism_gb300/csrc/dpg_kernels.h"]
TRAFFIC_FILE = "traffic_rowgather_pagerank_rmat22.txt"
TRAFFIC_KERNEL = "rowgather_kernel"
# The command whose ncu output --ingest-traffic turns into profiles/<TRAFFIC_FILE> (one launch,
# one pass: DRAM bytes only, on the headline workload after 40 gather launches of warm-up).
TRAFFIC_COMMAND = ("ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum --clock-control none "
                   "-k regex:rowgather_kernel -s 40 -c 1 --csv --page raw --log-file traffic.csv "
                   "python bench.py --steps 3 --warmup 3 --no-extra --no-e2e")


def sources_fingerprint(paths=GATHER_SOURCES) -> str:
    import hashlib

    h = hashlib.sha256()
    for rel in paths:
        h.update(rel.encode())
        h.update((ROOT / rel).read_bytes())
    return h.hexdigest()[:16]


def ingest_traffic(csv_path: str) -> int:
    """Turns the raw-page CSV of TRAFFIC_COMMAND into profiles/<TRAFFIC_FILE>, stamped with the
    fingerprint of the kernel sources it was captured from."""
    import csv

    rows = [r for r in csv.reader(open(csv_path)) if r]
    hdr = next(i for i, r in enumerate(rows) if "Kernel Name" in r)
    names = rows[hdr]
    data = [r for r in rows[hdr + 1:] if len(r) == len(names) and TRAFFIC_KERNEL in r[names.index("Kernel Name")]]
    if not data:
        print(f"no {TRAFFIC_KERNEL} launch in {csv_path}", file=sys.stderr)
        return 1
    r = data[0]
    val = {m: float(r[names.index(m)].replace(",", "")) for m in ("dram__bytes_read.sum", "dram__bytes_write.sum")}
    units = rows[hdr + 1][names.index("dram__bytes_read.sum")] if len(rows) > hdr + 1 else ""
    scale = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "KB": 1e3, "MB": 1e6, "GB": 1e9}.get(units.strip(), 1)
    out = ROOT / "profiles" / TRAFFIC_FILE
    out.write_text(
        f"# DRAM bytes of one {TRAFFIC_KERNEL} launch (PageRank sweep, R-MAT scale 22), from ncu.\n"
        f"# command: {TRAFFIC_COMMAND}\n"
        f"# ingested by: python bench.py --ingest-traffic traffic.csv\n"
        f"sources_fingerprint = {sources_fingerprint()}\n"
        f"kernel = {r[names.index('Kernel Name')]}\n"
        f"dram__bytes_read.sum = {val['dram__bytes_read.sum'] * scale:.0f}\n"
        f"dram__bytes_write.sum = {val['dram__bytes_write.sum'] * scale:.0f}\n")
    print(out.read_text())
    return 0


def capture_traffic():
    """(DRAM bytes per gather launch, note) from profiles/<TRAFFIC_FILE>; None when the file is
    absent or was captured from other kernel sources than the ones built now."""
    p = ROOT / "profiles" / TRAFFIC_FILE
    if not p.exists():
        return None, "no capture"
    kv = {}
    for line in p.read_text().splitlines():
        if "=" in line and not line.startswith("#"):
            k, v = line.split("=", 1)
            kv[k.strip()] = v.strip()
    if kv.get("sources_fingerprint") != sources_fingerprint():
        return None, "capture is of other kernel sources (stale)"
    try:
        return float(kv["dram__bytes_read.sum"]) + float(kv["dram__bytes_write.sum"]), "ncu capture of these sources"
    except (KeyError, ValueError):
        return None, "unreadable capture"


def bench_config(world: int, V: int, E: int) -> dict:
    """The workload's config, printed identically by both arms."""
    return {"workload": WORKLOAD, "vertices": V, "arcs": E, "graph_seed": GRAPH_SEED,
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "l2": "inputs larger than L2 (in-arcs 268 MB > 129 MB), no flush"}


def build_workload(dpg):
    g = dpg.rmat_csr(SCALE, EDGE_FACTOR, seed=GRAPH_SEED, weights=False)
    in_off, in_col = dpg.csr_transpose(g.V, g.offsets, g.col)
    od = dpg.out_degrees(g.offsets)
    return g, in_off, in_col, od


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.proc = None
        self.lines: list[str] = []
        cmd = ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "50"]
        if gpu_id:
            cmd += ["-i", gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.12)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def cpu_pagerank_sample(orc, in_off, in_col, od, E, target_s=10.0):
    """Times the CPU restatement (all host threads) on whole 20-sweep solves, repeated to ~target_s."""
    threads = orc.num_threads()
    t0 = time.perf_counter()
    orc.pagerank_omp_f32(in_off, in_col, od, damping=DAMPING, total=1.0, iterations=1)
    one = time.perf_counter() - t0
    sweeps = SWEEPS if one * SWEEPS <= target_s else max(1, int(target_s / max(one, 1e-9)))
    reps = max(1, int(target_s / max(one * sweeps, 1e-9)))
    t0 = time.perf_counter()
    for _ in range(reps):
        orc.pagerank_omp_f32(in_off, in_col, od, damping=DAMPING, total=1.0, iterations=sweeps)
    dt = time.perf_counter() - t0
    return {"value": E * sweeps * reps / dt / 1e9, "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": f"{reps} x {sweeps}-sweep pull PageRank on the full scale-{SCALE} graph ({dt:.1f} s, "
                      f"CPU restatement: the reference has no CPU PageRank)"}


def run_reference(args, world, rank):
    """The reference's PageRank on the host cores. The reference has no CPU PageRank (its only CPU
    algorithm is bfs_cpu), so this times the oracle's restatement of pagerank_thread_pull_kernel and
    its host loop (apps/pagerank/src/pagerank_kernel.cu:95-120, pagerank_wrapper.cu:147-241) on all
    host threads. The graph is generated and transposed by the oracle as well: this arm loads no
    library of the GPU implementation."""
    if rank != 0:
        return 0
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc

    off, col, _ = orc.rmat_csr(SCALE, EDGE_FACTOR, GRAPH_SEED, weights=False)
    in_off, in_col = orc.csr_transpose(off, col)
    od = np.diff(off).astype(np.int32)
    V, E = off.shape[0] - 1, col.shape[0]
    del off, col
    threads = orc.num_threads()
    t0 = time.perf_counter()
    orc.pagerank_omp_f32(in_off, in_col, od, damping=DAMPING, total=1.0, iterations=1)
    one = time.perf_counter() - t0
    sweeps = SWEEPS if one * SWEEPS <= 3.0 else max(1, int(3.0 / max(one, 1e-9)))
    for _ in range(args.warmup):
        orc.pagerank_omp_f32(in_off, in_col, od, damping=DAMPING, total=1.0, iterations=sweeps)
    steps = min(args.steps, 20)
    t0 = time.perf_counter()
    for _ in range(steps):
        orc.pagerank_omp_f32(in_off, in_col, od, damping=DAMPING, total=1.0, iterations=sweeps)
    dt = time.perf_counter() - t0
    value = E * sweeps * steps / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": dt / steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": bench_config(world, V, E),
        "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": f"{steps} steps x {sweeps} sweeps of the pull PageRank restatement on the "
                                   f"full scale-{SCALE} graph, all host threads (the reference has no CPU PageRank)"},
        "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def measure_spmv(dpg, ctx, torch, g, peak, steps, relabel=True):
    """SpMV over the out-edge CSR with FP32 values in (0,1] and x in [-1,1]; CUDA events."""
    dev = torch.device("cuda", torch.cuda.current_device())
    V, E = g.V, g.E
    rng = np.random.default_rng(22)
    vals = torch.from_numpy((1.0 - rng.random(E, dtype=np.float32)).astype(np.float32)).to(dev)
    x = torch.from_numpy(rng.uniform(-1, 1, V).astype(np.float32)).to(dev)
    y = torch.empty(V, dtype=torch.float32, device=dev)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    dg.set_relabel(relabel)
    ctx.profile(True)
    for _ in range(3):
        dpg.spmv_dev(ctx, dg, vals.data_ptr(), x.data_ptr(), y.data_ptr())
    ctx.profile_reset()
    n = max(20, steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(n):
        dpg.spmv_dev(ctx, dg, vals.data_ptr(), x.data_ptr(), y.data_ptr())
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / n
    lg, msg = ctx.profile_read(dpg.KERNEL_ROWGATHER)
    gather_ms = msg / max(lg, 1)
    bytes_spmv = 4 * (V + 1) + 8 * E + 8 * V
    return {"gteps": E / (t / 1e3) / 1e9, "ms": t, "gather_ms": gather_ms,
            "roofline_frac": bytes_spmv / (gather_ms / 1e3) / 1e9 / peak, "bytes_per_launch": bytes_spmv}


def measure_expand(dpg, ctx, torch, g, peak, kind, nsrc=8, seed=24, solution=None):
    """SSSP or BFS from seeded random sources with out-degree > 0; CUDA events around each solve.
    solution: a dpg.SOL_* id (None: the library default)."""
    dev = torch.device("cuda", torch.cuda.current_device())
    V, E = g.V, g.E
    dg = dpg.Graph(ctx, g.offsets, g.col, g.weights)
    deg = np.diff(g.offsets)
    srcs = [int(s) for s in np.random.default_rng(seed).choice(np.flatnonzero(deg > 0), nsrc, replace=False)]
    label = torch.empty(V, dtype=torch.int32, device=dev)
    fn0 = dpg.sssp_dev if kind == "sssp" else dpg.bfs_dev
    opts = {} if solution is None else {"solution": solution}

    def fn(c, graph, s, ptr):
        fn0(c, graph, s, ptr, **opts)
    bytes_pass = 4 * (V + 1) + (8 if kind == "sssp" else 4) * E + 8 * V
    ctx.profile(True)
    fn(ctx, dg, srcs[0], label.data_ptr())
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times, kms, scanned, iters = [], [], [], []
    for s in srcs:
        ctx.profile_reset()
        e0.record()
        fn(ctx, dg, s, label.data_ptr())
        e1.record()
        torch.cuda.synchronize()
        ctx.synchronize()
        times.append(e0.elapsed_time(e1))
        _, km = ctx.profile_read(dpg.KERNEL_EXPAND)
        kms.append(km)
        st = ctx.last_stats()
        scanned.append(st.edges_scanned / E)
        iters.append(st.iterations)
    ctx.trace(100000)
    fn(ctx, dg, srcs[0], label.data_ptr())
    tr = ctx.trace_read()
    ctx.trace(0)
    trace = [[round((tr[i + 1, 0] - tr[i, 0]) / 1e3, 1), int(tr[i, 1]), int(tr[i, 2])] for i in range(len(tr) - 1)]
    if len(trace) > 64:  # high-diameter graphs: the first 64 iterations only
        trace = trace[:64]
    t = statistics.median(times)
    km = statistics.median(kms)
    return {"gteps": E / (t / 1e3) / 1e9, "ms": t, "ms_min": min(times), "ms_max": max(times),
            "ms_per_source": [round(x, 4) for x in times],
            "iterations_per_source": [int(x) for x in iters], "kernel_ms": km, "trace_us_small_chunks": trace,
            "roofline_frac": bytes_pass / (km / 1e3) / 1e9 / peak, "bytes_per_solve": bytes_pass,
            "edges_scanned_over_E": statistics.median(scanned), "iterations": statistics.median(iters),
            "sources": srcs}


def measure_mapping(dpg, ctx, torch, g, nsrc=2, seed=22):
    """SSSP under each work mapping: the reference's solutions 0-4 (thread per vertex; rows of degree
    >= 64 per warp, consolidated per warp, per CTA or grid-wide) and the binned default (warp
    scan-gather, grid-wide chunks from degree 128). Median ms over nsrc sources; distances must agree
    across every mapping."""
    dev = torch.device("cuda", torch.cuda.current_device())
    dg = dpg.Graph(ctx, g.offsets, g.col, g.weights)
    deg = np.diff(g.offsets)
    srcs = [int(s) for s in np.random.default_rng(seed).choice(np.flatnonzero(deg > 0), nsrc, replace=False)]
    label = torch.empty(g.V, dtype=torch.int32, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    runs = [(dpg.SOLUTION_NAMES[s], {"solution": s}) for s in (dpg.SOL_THREAD, dpg.SOL_NAIVE, dpg.SOL_WARP,
                                                              dpg.SOL_BLOCK, dpg.SOL_GRID, dpg.SOL_BINNED)]
    out, ref = {}, [None] * nsrc
    for name, opts in runs:
        times, same = [], True
        for k, s in enumerate(srcs):
            dpg.sssp_dev(ctx, dg, s, label.data_ptr(), **opts)  # warm-up
            ctx.synchronize()
            e0.record()
            dpg.sssp_dev(ctx, dg, s, label.data_ptr(), **opts)
            e1.record()
            torch.cuda.synchronize()
            ctx.synchronize()
            times.append(e0.elapsed_time(e1))
            if ref[k] is None:
                ref[k] = label.clone()
            same = same and bool(torch.equal(ref[k], label))
        out[name] = {"ms": statistics.median(times), "distances_equal": same}
    dg.close()
    return {"sources": srcs, "mappings": out}


def measure_adjoint(dpg, ctx, torch, g, peak, nrhs=64, reps=5):
    """SpMV backward on g with lognormal(0,1) FP32 values and nrhs right-hand sides: the batched call
    (dX = A^T G and dA together) against looping the plain single-vector kernels once per column."""
    dev = torch.device("cuda", torch.cuda.current_device())
    ctx.profile(False)  # no per-launch events in either arm
    V, E = g.V, g.E
    gen = torch.Generator(device=dev)
    gen.manual_seed(5)
    vals = torch.exp(torch.randn(E, device=dev, generator=gen))
    X = torch.rand((V, nrhs), device=dev, generator=gen) * 2 - 1
    G = torch.rand((V, nrhs), device=dev, generator=gen) * 2 - 1
    dX = torch.empty((V, nrhs), device=dev)
    dA = torch.empty(E, device=dev)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def batched():
        dpg.spmv_bwd_dev(ctx, dg, vals.data_ptr(), nrhs, X.data_ptr(), G.data_ptr(), dX.data_ptr(), dA.data_ptr())

    # Plain kernels per column: dX[:, j] = A^T G[:, j] by the row-gather SpMV on the transposed graph
    # (values permuted once, outside the loop), dA += G[row, j] * X[col, j] by the arc kernel.
    t_off, t_col, t_arc = dpg.csr_transpose_perm(V, g.offsets, g.col)
    gT = dpg.Graph(ctx, t_off, t_col)
    vals_t = vals[torch.from_numpy(t_arc.astype(np.int64)).to(dev)].contiguous()
    Xc, Gc = X.t().contiguous(), G.t().contiguous()
    dXc = torch.empty((nrhs, V), device=dev)
    dA1 = torch.empty(E, device=dev)
    dA_loop = torch.empty(E, device=dev)

    def looped():
        dA_loop.zero_()
        for j in range(nrhs):
            dpg.spmv_dev(ctx, gT, vals_t.data_ptr(), Gc[j].data_ptr(), dXc[j].data_ptr())
            dpg.spmv_bwd_dev(ctx, dg, vals.data_ptr(), 1, Xc[j].data_ptr(), Gc[j].data_ptr(), None, dA1.data_ptr())
            dA_loop.add_(dA1)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    t_b = timed(batched)
    t_l = timed(looped)
    # Agreement is judged against the magnitude bound |A|^T |G| (and |G[row]|.|X[col]| for dA): the two
    # arms sum in different orders, and hub columns of the transpose cancel heavily.
    dX_b, dA_b = dX.clone(), dA.clone()
    Xa, Ga, va = X.abs(), G.abs(), vals.abs()
    dpg.spmv_bwd_dev(ctx, dg, va.data_ptr(), nrhs, Xa.data_ptr(), Ga.data_ptr(), dX.data_ptr(), dA.data_ptr())
    torch.cuda.synchronize()
    err_x = float(((dX_b.t() - dXc).abs() / (dX.t() + 1e-30)).max())
    err_a = float(((dA_b - dA_loop).abs() / (dA + 1e-30)).max())
    ok = err_x < 1e-5 and err_a < 1e-5
    bytes_bwd = 4 * (V + 1) + 8 * E + 4 * nrhs * V * 3 + 4 * E
    return {"nrhs": nrhs, "batched_ms": t_b, "looped_ms": t_l, "speedup": t_l / t_b,
            "batched_gteps": E * nrhs / (t_b / 1e3) / 1e9, "roofline_frac": bytes_bwd / (t_b / 1e3) / 1e9 / peak,
            "bytes_per_call": bytes_bwd, "results_agree": ok, "max_err_dx_over_bound": err_x,
            "max_err_da_over_bound": err_a}


def measure_prgrad(dpg, ctx, torch, g, peak, reps=3):
    """Weighted PageRank gradient on g (out-adjacency) with lognormal(0,1) FP32 weights and the loss
    sum of r over a seeded random 1% vertex subset: forward to a relative change of 3e-7, the
    adjoint fixed point to the same tolerance, and the per-arc gradient, against the forward alone."""
    dev = torch.device("cuda", torch.cuda.current_device())
    V, E = g.V, g.E
    rng = np.random.default_rng(20)
    w = torch.from_numpy(np.exp(rng.standard_normal(E)).astype(np.float32)).to(dev)
    seed_np = np.zeros(V, np.float32)
    seed_np[rng.choice(V, max(1, V // 100), replace=False)] = 1.0
    seed = torch.from_numpy(seed_np).to(dev)
    zero = torch.zeros(V, device=dev)
    r = torch.empty(V, device=dev)
    gr = torch.empty(E, device=dev)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    opts = dict(damping=0.85, total_rank=1.0, iterations=2000, epsilon=3e-7, adjoint_epsilon=3e-7)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(sd):
        dpg.pagerank_grad_dev(ctx, dg, w.data_ptr(), sd.data_ptr(), r.data_ptr(), gr.data_ptr(), **opts)
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0.record()
            sw = dpg.pagerank_grad_dev(ctx, dg, w.data_ptr(), sd.data_ptr(), r.data_ptr(), gr.data_ptr(), **opts)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return min(ts), sw

    t_fwd, (nf, _) = timed(zero)   # zero seed: the adjoint loop stops after one sweep
    t_all, (nf2, na) = timed(seed)
    sweeps = nf2 + na + 2
    # The loop the batched seed replaces: one gradient call per seed vertex (the loss is a sum over
    # the subset, so the gradients add up). Timed on 4 of the seed vertices, scaled to all of them.
    seeds = np.flatnonzero(seed_np)
    one = torch.zeros(V, device=dev)
    t_one = []
    for v in seeds[:4]:
        one.zero_()
        one[int(v)] = 1.0
        t_one.append(timed(one)[0])
    loop_ms = statistics.mean(t_one) * len(seeds)
    return {"ms_total": t_all, "ms_forward_only": t_fwd, "forward_sweeps": nf2, "adjoint_sweeps": na,
            "ms_per_sweep": t_all / sweeps, "gteps_sweeps": sweeps * E / (t_all / 1e3) / 1e9,
            "grad_over_forward": t_all / t_fwd, "rank_sum": float(r.double().sum()),
            "seed_vertices": int(len(seeds)), "ms_one_seed_vertex": statistics.mean(t_one),
            "ms_loop_over_seed_vertices": loop_ms, "speedup_vs_loop": loop_ms / t_all}


def measure_batch(dpg, ctx, torch, peak, ngraphs=512, nsrc=8, sweeps=20, seed=512, reps=3, rank=0, world=1):
    """Batched workload: ngraphs seeded R-MAT graphs (V log-uniform in [1K, 1M], edge factor uniform
    in {8, 16, 32}, weights uniform in [1, 100]), nsrc random SSSP sources and one sweeps-sweep
    PageRank per graph. The batch (one CUDA-graph launch, autotuned) against looping the plain
    single-graph kernels per source and per graph; results compared between the two.
    Under torchrun the graphs are sharded over the ranks by LPT on arcs x tasks (no exchange);
    times are the maximum over ranks."""
    dev = torch.device("cuda", torch.cuda.current_device())
    ctx.profile(False)  # no per-launch events: they would slow the 4,608-call plain loop
    t0 = time.perf_counter()
    specs = dpg.rmat_batch_specs(ngraphs, seed=seed)
    owner, load = dpg.partition_lpt([v * ef * (nsrc + sweeps) for v, ef in specs], world)
    mine = [k for k in range(ngraphs) if owner[k] == rank]
    graphs = [dpg.rmat_batch([specs[k]], seed=seed * 1000 + k)[0] for k in mine]
    t_gen = time.perf_counter() - t0
    src_all = np.random.default_rng(seed)
    src_rows = [src_all.integers(0, v, nsrc) for v, _ in specs]
    src = np.stack([src_rows[k] for k in mine]).astype(np.int32)
    if world > 1:
        import torch.distributed as tdist

    def max_over_ranks(x):
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        return float(t.item())

    def sync_all():
        torch.cuda.synchronize()
        if world > 1:
            tdist.barrier()
    t0 = time.perf_counter()
    b = dpg.Batch(ctx, graphs)
    t_pack = time.perf_counter() - t0
    V, E = b.V, b.E
    dist = torch.empty(nsrc * V, dtype=torch.int32, device=dev)
    rank_v = torch.empty(V, dtype=torch.float32, device=dev)
    t0 = time.perf_counter()
    tuning = b.autotune(src)
    t_tune = time.perf_counter() - t0
    gt = b.graph_tuning()
    settings: dict[str, int] = {}
    for h, c in zip(gt["hub_threshold"].tolist(), gt["chunk"].tolist()):
        settings[f"hub{h}_chunk{c}"] = settings.get(f"hub{h}_chunk{c}", 0) + 1
    pr = {"iterations": sweeps, "damping": DAMPING, "total_rank": 1.0}
    b.run(src, dist.data_ptr(), rank_v.data_ptr(), pr_opts_=pr)  # capture
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ts = []
    for _ in range(reps):
        sync_all()
        e0.record()
        b.run(src, dist.data_ptr(), rank_v.data_ptr(), pr_opts_=pr)
        e1.record()
        torch.cuda.synchronize()
        ts.append(max_over_ranks(e0.elapsed_time(e1)))
    ctx.synchronize()
    t_batch = min(ts)
    # Plain kernels, one call per graph and source (graphs resident before the timed loop).
    plain = []
    for g in graphs:
        in_off, in_col = dpg.csr_transpose(g.V, g.offsets, g.col)
        od = torch.from_numpy(np.diff(g.offsets).astype(np.int32)).to(dev)
        plain.append((dpg.Graph(ctx, g.offsets, g.col, g.weights), dpg.Graph(ctx, in_off, in_col), od))
    pdist = torch.empty(nsrc * V, dtype=torch.int32, device=dev)
    prank = torch.empty(V, dtype=torch.float32, device=dev)

    def loop():
        for k, (go, gi, od) in enumerate(plain):
            v0 = int(b.vstart[k])
            for c in range(nsrc):
                dpg.sssp_dev(ctx, go, int(src[k, c]), pdist[c * V + v0:].data_ptr())
            dpg.pagerank_dev(ctx, gi, od.data_ptr(), prank[v0:].data_ptr(), damping=DAMPING, total_rank=1.0,
                             iterations=sweeps)

    loop()
    ctx.synchronize()
    tl = []
    for _ in range(max(1, reps - 1)):
        sync_all()
        e0.record()
        loop()
        e1.record()
        torch.cuda.synchronize()
        tl.append(max_over_ranks(e0.elapsed_time(e1)))
    ctx.synchronize()
    t_loop = min(tl)
    # Split of both arms into their SSSP and PageRank parts (direct calls, not the captured graph).
    def timed(fn):
        fn()
        ctx.synchronize()
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ctx.synchronize()
        return e0.elapsed_time(e1)

    split = {
        "ms_batch_sssp": timed(lambda: b.sssp_dev(src, dist.data_ptr())),
        "ms_batch_pagerank": timed(lambda: b.pagerank_dev(rank_v.data_ptr(), **pr)),
        "ms_loop_sssp": timed(lambda: [dpg.sssp_dev(ctx, go, int(src[k, c]), pdist[c * V + int(b.vstart[k]):].data_ptr())
                                       for k, (go, _, _) in enumerate(plain) for c in range(nsrc)]),
        "ms_loop_pagerank": timed(lambda: [dpg.pagerank_dev(ctx, gi, od.data_ptr(), prank[int(b.vstart[k]):].data_ptr(),
                                                            damping=DAMPING, total_rank=1.0, iterations=sweeps)
                                           for k, (_, gi, od) in enumerate(plain)]),
    }
    ctx.profile(True)
    ctx.profile_reset()
    b.sssp_dev(src, dist.data_ptr())
    ctx.synchronize()
    st = ctx.last_stats()
    split["batch_sssp_iterations"] = int(st.iterations)
    split["batch_sssp_arcs_scanned_over_E"] = st.edges_scanned / E
    # The batch writes distances vertex-major (dist[v * nsrc + k]), the plain loop source-major.
    sssp_equal = bool(torch.equal(dist.view(V, nsrc), pdist.view(nsrc, V).t()))
    rmax = float(prank.max())
    pr_err = float((rank_v - prank).abs().max()) / rmax
    arcs = (nsrc + sweeps) * E
    if world > 1:
        t = torch.tensor([arcs], dtype=torch.float64, device=dev)
        tdist.all_reduce(t)
        arcs = float(t.item())
    return {"ranks": world, "lpt_loads": [int(x) for x in load], "graphs_this_rank": len(mine), "graphs": ngraphs,
            "sources_per_graph": nsrc, "pagerank_sweeps": sweeps, "vertices": V, "arcs": E,
            "ms_batch": t_batch, "ms_loop": t_loop, "speedup": t_loop / t_batch,
            "gteps_batch": arcs / (t_batch / 1e3) / 1e9, "gteps_loop": arcs / (t_loop / 1e3) / 1e9,
            "tuning": tuning, "graphs_per_sssp_setting": settings, "kernels_per_batch": b.launches(), "plain_calls": len(mine) * (nsrc + 1),
            "sssp_bit_exact_vs_plain": sssp_equal, "pagerank_max_err_over_max_rank": pr_err,
            "s_generate": t_gen, "s_pack": t_pack, "s_autotune": t_tune, **split}


def measure_cdp(dpg, ctx, torch, g, nsrc=3, seed=16):
    """The reference's recursive BFS variants as CDP2 child launches against the persistent BFS, on
    the same graph and sources (CUDA events around each synchronous solve)."""
    dev = torch.device("cuda", torch.cuda.current_device())
    ctx.profile(False)
    dg = dpg.Graph(ctx, g.offsets, g.col)
    deg = np.diff(g.offsets)
    srcs = [int(s) for s in np.random.default_rng(seed).choice(np.flatnonzero(deg > 0), nsrc, replace=False)]
    lv = torch.empty(g.V, dtype=torch.int32, device=dev)
    ref = torch.empty(g.V, dtype=torch.int32, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    names = {0: "persistent", dpg.CDP_NAIVE: "cdp_naive", dpg.CDP_WARP: "cdp_warp", dpg.CDP_BLOCK: "cdp_block",
             dpg.CDP_GRID: "cdp_grid"}
    for variant, name in names.items():
        ts, launches, failed, agree = [], 0, 0, True
        for s in srcs:
            dpg.bfs_dev(ctx, dg, s, ref.data_ptr())
            ctx.synchronize()
            e0.record()
            try:
                if variant == 0:
                    dpg.bfs_dev(ctx, dg, s, lv.data_ptr())
                    ctx.synchronize()
                    st = {"launches": 1, "failed_launches": 0}
                else:
                    st = dpg.bfs_cdp_dev(ctx, dg, s, variant, lv.data_ptr(), pending_limit=1 << 18)
            except dpg.DpgError as err:
                st = {"launches": -1, "failed_launches": -1, "error": str(err)[:120]}
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
            launches += st["launches"]
            failed += st["failed_launches"]
            agree = agree and st["failed_launches"] == 0 and bool(torch.equal(lv, ref))
            if "error" in st:
                out.setdefault(name + "_error", st["error"])
        out[name] = {"ms": statistics.median(ts), "launches_per_solve": launches / len(srcs),
                     "failed_launches": failed, "levels_equal_persistent": agree}
    base = out["persistent"]["ms"]
    for name in names.values():
        out[name]["x_slower_than_persistent"] = out[name]["ms"] / base
    return out


def measure_grid(dpg, ctx, torch, peak, n=4096, nsrc=2):
    """The high-diameter graph: an n x n 4-neighbour grid, weights uniform in [1, 1000]. SSSP with the
    binned and the near-far expansion, and BFS (direction-optimizing)."""
    g = dpg.grid_csr(n, n, seed=n, wmin=1, wmax=1000)
    return {f"sssp_grid{n}_binned": measure_expand(dpg, ctx, torch, g, peak, "sssp", nsrc=nsrc, solution=dpg.SOL_BINNED),
            f"sssp_grid{n}_nearfar": measure_expand(dpg, ctx, torch, g, peak, "sssp", nsrc=nsrc,
                                                    solution=dpg.SOL_NEARFAR),
            f"bfs_grid{n}": measure_expand(dpg, ctx, torch, g, peak, "bfs", nsrc=nsrc)}


def measure_pagerank_large(dpg, ctx, torch, g, peak, steps=5):
    """20-sweep pull PageRank (d = 0.85) on a large graph, device-resident: the in-edge CSR is built
    on the device (invertGraph order), the sweeps are timed with CUDA events, and the gather kernel's
    average launch gives the roofline fraction. rank_sum (1 up to rounding) is a size-independent
    check of the result."""
    dev = torch.device("cuda", torch.cuda.current_device())
    V, E = g.V, g.E
    off = torch.from_numpy(g.offsets).to(dev)
    col = torch.from_numpy(g.col).to(dev)
    in_off = torch.empty(V + 1, dtype=torch.int32, device=dev)
    in_col = torch.empty(E, dtype=torch.int32, device=dev)
    dpg.csr_transpose_dev(ctx, V, E, off.data_ptr(), col.data_ptr(), in_off.data_ptr(), in_col.data_ptr())
    od = (off[1:] - off[:-1]).to(torch.int32).contiguous()
    ctx.synchronize()
    del col
    gi = dpg.Graph.from_device(ctx, V, E, in_off.data_ptr(), in_col.data_ptr())
    del in_col
    rank = torch.empty(V, dtype=torch.float32, device=dev)
    for _ in range(2):
        dpg.pagerank_dev(ctx, gi, od.data_ptr(), rank.data_ptr(), damping=DAMPING, iterations=SWEEPS)
    ctx.synchronize()
    ctx.profile(True)
    ctx.profile_reset()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        dpg.pagerank_dev(ctx, gi, od.data_ptr(), rank.data_ptr(), damping=DAMPING, iterations=SWEEPS)
    e1.record()
    torch.cuda.synchronize()
    ctx.synchronize()
    n_g, ms_g = ctx.profile_read(dpg.KERNEL_ROWGATHER)
    ctx.profile(False)
    t_ms = e0.elapsed_time(e1) / steps
    gather_ms = ms_g / max(n_g, 1)
    bytes_sweep = 4 * (V + 1) + 4 * E + 12 * V
    achieved = bytes_sweep / (gather_ms / 1e3) / 1e9
    out = {"gteps": E * SWEEPS / (t_ms / 1e3) / 1e9, "ms_per_solve": t_ms, "sweeps": SWEEPS,
           "gather_ms_per_sweep": gather_ms, "roofline_frac": achieved / peak, "bytes_per_sweep": bytes_sweep,
           "rank_sum": float(rank.double().sum().item())}
    del gi
    return out


def host_cpu() -> dict:
    model = ""
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")) or line.startswith("CPU part"):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    import platform

    return {"cores": os.cpu_count(), "machine": platform.machine(), "model": model}


def cpu_baselines(dpg, g22, in_off, in_col, od, g24) -> dict:
    """The CPU restatements, one thread and all threads, timed once each on the GPU host (the
    reference's only CPU algorithm is bfs_cpu, restated as oracle.bfs; it has no CPU SSSP, SpMV or
    PageRank). Bounded samples: one SpMV, one PageRank sweep, one BFS and one Dijkstra solve."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as orc

    nall = orc.num_threads()  # read before any call sets a thread count (the setting persists)
    out = {"host": host_cpu(), "threads_all": nall}

    def timed(fn):
        t0 = time.perf_counter()
        fn()
        return time.perf_counter() - t0

    rng = np.random.default_rng(22)
    vals = (1.0 - rng.random(g22.E, dtype=np.float32)).astype(np.float32)
    x = rng.uniform(-1, 1, g22.V).astype(np.float32)
    for th, tag in ((1, "1_thread"), (nall, "all_threads")):
        t = timed(lambda: orc.spmv_omp_f32(g22.offsets, g22.col, vals, x, threads=th))
        out[f"spmv_rmat22_{tag}"] = {"gteps": g22.E / t / 1e9, "s": t}
        t = timed(lambda: orc.pagerank_omp_f32(in_off, in_col, od, iterations=1, threads=th))
        out[f"pagerank_sweep_rmat22_{tag}"] = {"gteps": g22.E / t / 1e9, "s": t}
    deg = np.diff(g24.offsets)
    s24 = int(np.random.default_rng(24).choice(np.flatnonzero(deg > 0)))
    t = timed(lambda: orc.bfs(g24.offsets, g24.col, s24))
    out["bfs_rmat24_1_thread_bfs_cpu_restated"] = {"gteps": g24.E / t / 1e9, "s": t}
    t = timed(lambda: orc.bfs_omp(g24.offsets, g24.col, s24, threads=nall))
    out["bfs_rmat24_all_threads"] = {"gteps": g24.E / t / 1e9, "s": t}
    gw = dpg.rmat_csr(22, 16, seed=22, wmin=1, wmax=255)
    s22 = int(np.random.default_rng(22).choice(np.flatnonzero(np.diff(gw.offsets) > 0)))
    t = timed(lambda: orc.sssp_dijkstra(gw.offsets, gw.col, gw.weights, s22))
    out["sssp_rmat22_1_thread_dijkstra"] = {"gteps": gw.E / t / 1e9, "s": t}
    t = timed(lambda: orc.sssp_bf_omp(gw.offsets, gw.col, gw.weights, s22, threads=nall))
    out["sssp_rmat22_all_threads_frontier_bf"] = {"gteps": gw.E / t / 1e9, "s": t}
    return out


def extra_measurements(dpg, ctx, torch, g, peak, steps, pr_inputs=None):
    """SpMV and the SpMV adjoint on the scale-22 graph; SSSP, BFS and PageRank on R-MAT scale 24; the
    PageRank edge-weight gradient on scale 20; the 512-graph batch; the recursive CDP2 BFS variants against
    the persistent BFS on scale 16 (device-resident, CUDA events)."""
    out = {"random_read_ceiling": {
        "l2_resident_16MB_gloads_per_s": dpg.calibrate_random_reads(ctx, 4 << 20) / 1e9,
        "hbm_resident_4GB_gloads_per_s": dpg.calibrate_random_reads(ctx, 1 << 30, iters=100) / 1e9,
        "note": "random 4-byte reads, 2 x 1024-thread CTAs per SM, 8 loads in flight per thread"}}
    out["spmv_rmat22"] = measure_spmv(dpg, ctx, torch, g, peak, steps)
    out["spmv_bwd_rmat22_64rhs"] = measure_adjoint(dpg, ctx, torch, g, peak)
    out["sssp_mapping_rmat22"] = measure_mapping(dpg, ctx, torch, dpg.rmat_csr(22, 16, seed=22, wmin=1, wmax=255))
    g24 = dpg.rmat_csr(24, 16, seed=24, wmin=1, wmax=255)
    out["sssp_rmat24"] = measure_expand(dpg, ctx, torch, g24, peak, "sssp")
    # SSSP against the random-read ceiling of its label array (16 M int32, 64 MB): every scanned
    # arc peeks its head's label at a random address.
    ceiling = dpg.calibrate_random_reads(ctx, g24.V)
    r = out["sssp_rmat24"]
    relax = r["edges_scanned_over_E"] * g24.E / (r["kernel_ms"] / 1e3)
    r["random_read"] = {"label_array_mb": 4 * g24.V / 2**20, "ceiling_gloads_per_s": ceiling / 1e9,
                        "scanned_arcs_per_s_g": relax / 1e9, "frac": relax / ceiling,
                        "ceiling_source": "dpg_calibrate_random_reads on an array the size of the labels, this run"}
    out["bfs_rmat24"] = measure_expand(dpg, ctx, torch, g24, peak, "bfs")
    out["pagerank_rmat24"] = measure_pagerank_large(dpg, ctx, torch, g24, peak)
    if pr_inputs is not None:
        out["cpu_baselines"] = cpu_baselines(dpg, g, *pr_inputs, g24)
    out.update(measure_grid(dpg, ctx, torch, peak))
    del g24
    g20 = dpg.rmat_csr(20, 16, seed=20, weights=False)
    out["pagerank_grad_rmat20"] = measure_prgrad(dpg, ctx, torch, g20, peak)
    del g20
    out["batch_512_graphs"] = measure_batch(dpg, ctx, torch, peak)
    out["cdp_bfs_rmat16"] = measure_cdp(dpg, ctx, torch, dpg.rmat_csr(16, 16, seed=16, weights=False))
    return out


def run_single_workload(args, world=1, rank=0, local=0):
    """--workload spmv|sssp|bfs|adjoint|prgrad|batch: one measurement, one JSON line. Under torchrun
    only the batch shards (LPT over ranks); the other workloads run on rank 0 alone."""
    import torch

    import __graft_entry__

    dpg = __graft_entry__.load_package()
    if world > 1 and args.workload != "batch" and rank != 0:
        return 0
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1 and args.workload == "batch":
        import torch.distributed as tdist

        tdist.init_process_group("nccl", device_id=dev)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    peak, peak_kind = measured_peaks()
    ctx = dpg.Context(0)
    ctx.set_stream(stream.cuda_stream)
    if args.workload == "batch":
        bw = world if world > 1 else 1
        res = measure_batch(dpg, ctx, torch, peak, ngraphs=args.batch_graphs, rank=rank if bw > 1 else 0, world=bw)
        res["gteps"] = res["gteps_batch"]
        if bw > 1:
            import torch.distributed as tdist

            tdist.barrier()
            tdist.destroy_process_group()
            if rank != 0:
                return 0
        scale = 0
        g = None
    elif args.workload == "grid":
        scale = 0
        g = dpg.grid_csr(4096, 4096, seed=4096, wmin=1, wmax=1000)
        res = measure_grid(dpg, ctx, torch, peak)
        res["gteps"] = res["sssp_grid4096_binned"]["gteps"]
    elif args.workload == "cdp":
        scale = args.scale or 16
        g = dpg.rmat_csr(scale, 16, seed=scale, weights=False)
        res = measure_cdp(dpg, ctx, torch, g)
        res["gteps"] = g.E / (res["persistent"]["ms"] / 1e3) / 1e9
    elif args.workload == "pagerank-large":
        scale = args.scale or 24
        g = dpg.rmat_csr(scale, 16, seed=scale, wmin=1, wmax=255)
        res = measure_pagerank_large(dpg, ctx, torch, g, peak, steps=max(1, min(args.steps, 5)))
    elif args.workload == "prgrad":
        scale = args.scale or 20
        g = dpg.rmat_csr(scale, 16, seed=scale, weights=False)
        res = measure_prgrad(dpg, ctx, torch, g, peak)
        res["gteps"] = res["gteps_sweeps"]
    elif args.workload in ("spmv", "adjoint"):
        scale = args.scale or 22
        g = dpg.rmat_csr(scale, 16, seed=scale, weights=False)
        if args.workload == "spmv":
            res = measure_spmv(dpg, ctx, torch, g, peak, args.steps, relabel=not args.no_relabel)
        else:
            res = measure_adjoint(dpg, ctx, torch, g, peak)
            res["gteps"] = res["batched_gteps"]
    else:
        scale = args.scale or 24
        g = dpg.rmat_csr(scale, 16, seed=scale, wmin=1, wmax=255)
        res = measure_expand(dpg, ctx, torch, g, peak, args.workload,
                             solution=None if args.solution < 0 else args.solution)
    if g is None:
        cfg = {"workload": f"batch of {res['graphs']} rmat graphs, V log-uniform [1K, 1M], edge factor "
                           f"{{8, 16, 32}}, {res['sources_per_graph']} SSSP sources + {res['pagerank_sweeps']}-sweep "
                           "PageRank each", "vertices": res["vertices"], "arcs": res["arcs"]}
    else:
        cfg = {"workload": f"{args.workload} rmat scale {scale} edge-factor 16", "vertices": g.V, "arcs": g.E}
    line = {"metric": f"GTEPS ({args.workload})", "value": res["gteps"], "unit": "GTEPS",
            "n_gpus": world if args.workload == "batch" else 1,
            "config": cfg, "peak_source": peak_kind, **res}
    print(json.dumps(line), flush=True)
    return 0


def run_dpg(args, world, rank, local):
    import torch

    import __graft_entry__

    dpg = __graft_entry__.load_package()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    # One dedicated stream for the library launches and the timing events.
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    if world > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl", device_id=dev)
    peak, peak_kind = measured_peaks()

    g, in_off, in_col, od = build_workload(dpg)
    V, E = g.V, g.E
    ctx = dpg.Context(local)
    ctx.set_stream(stream.cuda_stream)
    gi = dpg.Graph(ctx, in_off, in_col)
    gi.set_relabel(not args.no_relabel)
    od_t = torch.from_numpy(od).to(dev)
    rank_t = torch.empty(V, dtype=torch.float32, device=dev)
    for _ in range(max(args.warmup, 3)):
        dpg.pagerank_dev(ctx, gi, od_t.data_ptr(), rank_t.data_ptr(), damping=DAMPING, iterations=SWEEPS)
    ctx.synchronize()

    gpu_id = None
    try:
        gpu_id = str(torch.cuda.get_device_properties(dev).uuid)
        gpu_id = gpu_id if gpu_id.startswith("GPU-") else f"GPU-{gpu_id}"
    except Exception:
        gpu_id = None
    ctx.profile(True)
    ctx.profile_reset()
    sampler = ClockSampler(gpu_id) if rank == 0 else None
    time.sleep(0.1)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        dpg.pagerank_dev(ctx, gi, od_t.data_ptr(), rank_t.data_ptr(), damping=DAMPING, iterations=SWEEPS)
    e1.record()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop() if sampler else None
    ctx.synchronize()
    t_ms = e0.elapsed_time(e1)
    t_max = t_ms
    if world > 1:
        tt = torch.tensor([t_ms], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_max = float(tt.item())
    n_g, ms_g = ctx.profile_read(dpg.KERNEL_ROWGATHER)
    n_f, ms_f = ctx.profile_read(dpg.KERNEL_FIXUP)
    n_i, ms_i = ctx.profile_read(dpg.KERNEL_INIT)
    ctx.profile(False)
    value = E * SWEEPS * args.steps * world / (t_max / 1e3) / 1e9
    gather_avg_ms = ms_g / max(n_g, 1)
    bytes_sweep = 4 * (V + 1) + 4 * E + 12 * V  # in-offsets, in-arcs, contrib read, contrib write, outdeg read
    achieved = bytes_sweep / (gather_avg_ms / 1e3) / 1e9
    traffic, traffic_note = capture_traffic()
    # The second ceiling: the sweep's gathers that miss the shared-memory hot cache are random 4-byte
    # reads of the 16.8 MB contribution vector, which stays in L2; measured against the random-read
    # rate of an L2-resident array on this GPU.
    hc = gi.hot_cache()
    cold = E - hc["hot_arcs"]
    ceiling = dpg.calibrate_random_reads(ctx, 4 << 20)
    random_read = {"reads_per_launch": cold, "hot_cache_entries": hc["hot_entries"],
                   "achieved_gloads_per_s": cold / (gather_avg_ms / 1e3) / 1e9,
                   "ceiling_gloads_per_s": ceiling / 1e9,
                   "frac": cold / (gather_avg_ms / 1e3) / ceiling,
                   "ceiling_source": "dpg_calibrate_random_reads, 16 MB array, measured in this run"}

    # e2e: one-shot C-ABI call with pinned host buffers (upload, solve, download inside the region).
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
        h_off, h_col, h_od = pin(in_off), pin(in_col), pin(od)
        h_rank = torch.empty(V, dtype=torch.float32).pin_memory().numpy()
        dpg.pagerank_host(ctx, h_off, h_col, h_od, out=h_rank, damping=DAMPING, iterations=SWEEPS)
        e2e_steps = max(3, min(args.steps, 10))
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            dpg.pagerank_host(ctx, h_off, h_col, h_od, out=h_rank, damping=DAMPING, iterations=SWEEPS)
        t_e2e = time.perf_counter() - t0
        if world > 1:
            tt = torch.tensor([t_e2e], dtype=torch.float64, device=dev)
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t_e2e = float(tt.item())
        e2e = {"value": E * SWEEPS * e2e_steps * world / t_e2e / 1e9, "unit": "GTEPS", "steps": e2e_steps,
               "h2d_bytes_per_step": int(h_off.nbytes + h_col.nbytes + h_od.nbytes),
               "d2h_bytes_per_step": int(h_rank.nbytes)}

    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
            torch.distributed.destroy_process_group()
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(world, V, E),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": traffic_note, "kernel": "rowgather_kernel<PageRank>",
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": bytes_sweep, "avg_launch_ms": gather_avg_ms,
                     "random_read": random_read},
        "e2e": e2e,
        "gpu_launches": int(n_g + n_f + n_i),
        "kernel_ms": {"rowgather": ms_g, "fixup": ms_f, "init": ms_i},
    }
    if clocks:
        line["clocks"] = clocks
    if world == 1:
        if not args.no_e2e:
            sys.path.insert(0, str(ROOT / "oracle"))
            import oracle as orc

            line["cpu_baseline"] = cpu_pagerank_sample(orc, in_off, in_col, od, E)
        if not args.no_extra:
            del gi
            line["extra"] = extra_measurements(dpg, ctx, torch, g, peak, args.steps, (in_off, in_col, od))
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


def main() -> int:
    args = parse_args()
    if args.ingest_traffic:
        return ingest_traffic(args.ingest_traffic)
    world, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if args.workload != "pagerank":
        return run_single_workload(args, world, rank, local)
    return run_dpg(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
