"""Generates the golden fixtures in tests/golden/ from the reference's own host code.

Run here (where the reference tree exists), never on the GPU machine:

    make -C oracle all ref && python tests/golden/make_golden.py

What it records, all produced by the reference's code compiled by oracle/Makefile into
oracle/_ref/libref.so (common/global.cpp, apps/bfs-rec/src/bfs_rec.cpp):
  * data_test.json: the reference's only dataset (datasets/data_test.gr, 20 vertices, 40 arcs,
    source `s 8`) as an arc list in file order, the CSR and transposed CSR that readInputDIMACS9 +
    convertCSR + invertGraph build from it, bfs_cpu levels from its source, and the text that
    outputCost / outputRank / outputColor print for given vectors;
  * loaders.json: small DIMACS9 / DIMACS10 / SLNDC files (content written by this script) with the
    CSR the reference loader builds from each, including the srand(7)/rand() weights of the
    DIMACS10 and SLNDC readers;
  * rmat_s8.json: a seeded R-MAT scale-8 arc list written as .gr and loaded back by the reference
    loader (self-loops and duplicate arcs included), with bfs_cpu levels from vertex 0.
"""
from __future__ import annotations

import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle  # noqa: E402

REF = oracle.REFERENCE_TREE
GOLDEN = Path(__file__).resolve().parent


def parse_gr_arcs(text: str):
    src, dst, w = [], [], []
    for line in text.splitlines():
        if line.startswith("a"):
            _, t, h, wt = line.split()[:4]
            src.append(int(t) - 1)
            dst.append(int(h) - 1)
            w.append(int(wt))
    return src, dst, w


def ref_outputs(tmp: Path, V: int, source: int):
    lib = oracle.ref_lib()
    dist = np.arange(V, dtype=np.int32) * 7 + 3
    rank = (np.arange(V, dtype=np.float32) + 0.5) / 3.0
    color = (np.arange(V, dtype=np.int32) % 5) + 1
    p = tmp / "out.txt"
    lib.ref_output_cost(str(p).encode(), source, oracle._p(dist))
    cost_txt = p.read_text()
    lib.ref_output_rank(str(p).encode(), oracle._p(rank))
    rank_txt = p.read_text()
    lib.ref_output_color(str(p).encode(), oracle._p(color))
    color_txt = p.read_text()
    return {
        "cost_input": dist.tolist(), "cost_text": cost_txt,
        "rank_input": rank.tolist(), "rank_text": rank_txt,
        "color_input": color.tolist(), "color_text": color_txt,
    }


def load_record(path: Path, fmt: int):
    V, E, s, off, col, w, in_off, in_col = oracle.ref_load(path, fmt)
    return {"V": V, "E": E, "source": s, "offsets": off.tolist(), "col": col.tolist(), "weights": w.tolist(),
            "in_offsets": in_off.tolist(), "in_col": in_col.tolist()}


def main() -> int:
    oracle.build(with_reference=True)
    data_test = REF / "datasets" / "data_test.gr"
    text = data_test.read_text()
    src, dst, w = parse_gr_arcs(text)
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        rec = load_record(data_test, 0)
        rec["arcs"] = {"src": src, "dst": dst, "w": w}
        rec["bfs_levels"] = oracle.ref_bfs_cpu(rec["source"], rec["V"]).tolist()
        rec["outputs"] = ref_outputs(tmp, rec["V"], rec["source"])
        rec["origin"] = "datasets/data_test.gr loaded by the reference (common/global.cpp) ; bfs_cpu (bfs_rec.cpp:102)"
        (GOLDEN / "data_test.json").write_text(json.dumps(rec, separators=(",", ":")))

        loaders = {}
        # DIMACS9 with duplicate arcs, a self-loop, a vertex without arcs and an 's' line.
        gr = "c tiny\np sp 6 9\ns 2\na 1 2 5\na 1 3 2\na 2 3 1\na 1 2 7\na 3 3 4\na 3 5 9\na 5 1 1\na 2 5 3\na 5 6 2\n"
        (tmp / "t.gr").write_text(gr)
        loaders["dimacs9"] = {"text": gr, "format": 0, **load_record(tmp / "t.gr", 0)}
        # DIMACS10 (METIS-like) adjacency lists: header "V E", then one line per vertex.
        g10 = "% tiny undirected graph\n5 6\n2 3\n1 3 4\n1 2 5\n2 5\n3 4\n"
        (tmp / "t.graph").write_text(g10)
        loaders["dimacs10"] = {"text": g10, "format": 1, **load_record(tmp / "t.graph", 1)}
        # SLNDC (SNAP) edge list with sparse ids that the reader compacts.
        sl = ("# Directed graph: tiny\n# comment\n# Nodes: 6 Edges: 8\n# FromNodeId\tToNodeId\n"
              "0\t4\n4\t7\n7\t0\n0\t7\n9\t4\n4\t9\n7\t11\n11\t0\n")
        (tmp / "t.txt").write_text(sl)
        loaders["slndc"] = {"text": sl, "format": 2, **load_record(tmp / "t.txt", 2)}
        (GOLDEN / "loaders.json").write_text(json.dumps(loaders, separators=(",", ":")))

        # R-MAT scale 8 through the product writer, then the reference loader.
        import importlib.util
        spec = importlib.util.spec_from_file_location(
            "smdp_gb300", ROOT / "show-me-dynamic-parallelism_gb300" / "__init__.py",
            submodule_search_locations=[str(ROOT / "show-me-dynamic-parallelism_gb300")])
        dpg = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(dpg)
        s8, d8, w8 = dpg.rmat_arcs(8, 8 * 256, seed=1234, wmin=1, wmax=100)
        dpg.write_dimacs9(tmp / "r.gr", 256, s8, d8, w8, source=0)
        r = load_record(tmp / "r.gr", 0)
        r["arcs"] = {"src": s8.tolist(), "dst": d8.tolist(), "w": w8.tolist()}
        r["generator"] = {"scale": 8, "E": 8 * 256, "seed": 1234, "wmin": 1, "wmax": 100, "permute": True}
        r["bfs_levels"] = oracle.ref_bfs_cpu(0, r["V"]).tolist()
        (GOLDEN / "rmat_s8.json").write_text(json.dumps(r, separators=(",", ":")))
    print("wrote", sorted(p.name for p in GOLDEN.glob("*.json")))
    return 0


if __name__ == "__main__":
    sys.exit(main())
