"""Builds libdpg.so (the C-ABI library) and the command-line apps for sm_103a.

Every translation unit is compiled in parallel with one -gencode (compute_103a -> sm_103a); a unit is
recompiled only when it or a header it may include is newer than its object file.

    python show-me-dynamic-parallelism_gb300/build.py [--force] [--verbose]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
APPS = PKG / "apps"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libdpg.so"
BIN = PKG / "bin"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp", "--expt-relaxed-constexpr"]
# Extra nvcc flags for tuning builds, e.g. DPG_NVCC_EXTRA="-DDPG_GATHER_TILES=1" (use with --force).
NVCC_FLAGS += os.environ.get("DPG_NVCC_EXTRA", "").split()
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wextra", "-Wno-unused-parameter"]

LIB_CU = ["dpg_api.cu", "dpg_expand.cu", "dpg_rowgather.cu", "dpg_noalloc.cu", "dpg_layout.cu", "dpg_adjoint.cu", "dpg_prgrad.cu", "dpg_batch.cu", "dpg_cdp.cu", "dpg_transpose.cu", "dpg_calib.cu"]
# Translation units with device-side launches (relocatable device code, linked with cudadevrt).
RDC_CU = {"dpg_cdp.cu"}
LIB_CXX = ["dpg_host.cpp"]
# app name -> source file (apps link against libdpg.so)
APP_SOURCES = {
    "gpu-sssp": "app_sssp.cpp",
    "gpu-bfs-rec": "app_bfs_rec.cpp",
    "gpu-SpMV": "app_spmv.cpp",
    "gpu-pg": "app_pagerank.cpp",
    "gpu-graph-color": "app_graph_color.cpp",
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def cuda_home() -> Path:
    return Path(nvcc()).resolve().parent.parent


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")) + list(APPS.glob("*.h"))


def _stale(out: Path, srcs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}):\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)


def build(force: bool = False, verbose: bool = False, apps: bool = True) -> Path:
    BUILD.mkdir(exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for name in LIB_CU:
        src = CSRC / name
        obj = BUILD / (name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            rdc = ["-rdc=true"] if name in RDC_CU else []
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, *rdc, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)])
    for name in LIB_CXX:
        src = CSRC / name
        obj = BUILD / (name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["g++", *CXX_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", f"-I{cuda_home() / 'include'}", "-c", str(src),
                         "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        # -rdc=true links the relocatable device code of RDC_CU against the device runtime.
        _run([nvcc(), *ARCH, "-shared", "-rdc=true", "-o", str(tmp), *map(str, objs), "-lcudadevrt", "-Xcompiler",
              "-fopenmp", "-lgomp"], verbose)
        os.replace(tmp, LIB)
    if apps and APPS.exists():
        BIN.mkdir(exist_ok=True)
        app_jobs = []
        for app, srcname in APP_SOURCES.items():
            src = APPS / srcname
            if not src.exists():
                continue
            out = BIN / app
            if force or _stale(out, [src, LIB] + hdrs):
                app_jobs.append(["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", f"-I{APPS}", str(src), "-o", str(out),
                                 f"-L{PKG}", "-ldpg", f"-Wl,-rpath,{PKG}"])
        with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
            list(ex.map(lambda c: _run(c, verbose), app_jobs))
    return LIB


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    args = ap.parse_args()
    print(build(force=args.force, verbose=args.verbose))
    return 0


if __name__ == "__main__":
    sys.exit(main())
