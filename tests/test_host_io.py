"""The library's host-side graph path against the reference loader's recorded output: DIMACS9,
DIMACS10 and SLNDC readers (global.cpp:29-190), convertCSR's reversed neighbour order
(global.cpp:192-235), invertGraph (global.cpp:237-277), the output writers (global.cpp:361-399),
and the seeded generators. No GPU needed."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import dpg, load_golden


@pytest.mark.parametrize("name", ["dimacs9", "dimacs10", "slndc"])
def test_readers_match_reference_loader(tmp_path, name):
    rec = load_golden("loaders.json")[name]
    p = tmp_path / f"g.{name}"
    p.write_text(rec["text"])
    g = dpg.read_graph(p, rec["format"])
    assert (g.V, g.E, g.source) == (rec["V"], rec["E"], rec["source"])
    assert g.offsets.tolist() == rec["offsets"]
    assert g.col.tolist() == rec["col"]
    assert g.weights.tolist() == rec["weights"]
    in_off, in_col = dpg.csr_transpose(g.V, g.offsets, g.col)
    assert in_off.tolist() == rec["in_offsets"] and in_col.tolist() == rec["in_col"]


def test_data_test_arcs_to_reference_csr():
    rec = load_golden("data_test.json")
    a = rec["arcs"]
    g = dpg.csr_from_arcs(rec["V"], a["src"], a["dst"], a["w"])
    assert g.offsets.tolist() == rec["offsets"]
    assert g.col.tolist() == rec["col"] and g.weights.tolist() == rec["weights"]
    in_off, in_col = dpg.csr_transpose(rec["V"], g.offsets, g.col)
    assert in_off.tolist() == rec["in_offsets"] and in_col.tolist() == rec["in_col"]


def test_data_test_roundtrip_through_gr_file(tmp_path):
    rec = load_golden("data_test.json")
    a = rec["arcs"]
    p = tmp_path / "d.gr"
    dpg.write_dimacs9(p, rec["V"], a["src"], a["dst"], a["w"], source=rec["source"])
    g = dpg.read_graph(p, 0)
    assert g.source == rec["source"] and g.offsets.tolist() == rec["offsets"] and g.col.tolist() == rec["col"]


def test_rmat_fixture_regenerates_and_matches_reference_csr():
    rec = load_golden("rmat_s8.json")
    gen = rec["generator"]
    s, d, w = dpg.rmat_arcs(gen["scale"], gen["E"], seed=gen["seed"], wmin=gen["wmin"], wmax=gen["wmax"],
                            permute=gen["permute"])
    assert s.tolist() == rec["arcs"]["src"] and d.tolist() == rec["arcs"]["dst"] and w.tolist() == rec["arcs"]["w"]
    g = dpg.csr_from_arcs(rec["V"], s, d, w)
    assert g.offsets.tolist() == rec["offsets"] and g.col.tolist() == rec["col"]
    assert g.weights.tolist() == rec["weights"]
    in_off, in_col = dpg.csr_transpose(rec["V"], g.offsets, g.col)
    assert in_col.tolist() == rec["in_col"]


def test_writers_byte_identical_to_reference(tmp_path):
    out = load_golden("data_test.json")["outputs"]
    src = load_golden("data_test.json")["source"]
    p = tmp_path / "o.txt"
    dpg.write_cost(p, src, out["cost_input"])
    assert p.read_text() == out["cost_text"]
    dpg.write_rank(p, np.array(out["rank_input"], np.float32))
    assert p.read_text() == out["rank_text"]
    dpg.write_color(p, out["color_input"])
    assert p.read_text() == out["color_text"]


def test_write_level_format(tmp_path):
    p = tmp_path / "l.txt"
    dpg.write_level(p, [0, 3, dpg.UNDEFINED_LEVEL])
    assert p.read_text() == "Node 1 is in level 0\nNode 2 is in level 3\nNode 3 is in level 2147483647\n"


def test_glibc_rand_stream_matches_libc(tmp_path):
    # The DIMACS10/SLNDC readers draw weights as rand()%1000+1 after srand(7) (global.cpp:84-98).
    libc = ctypes.CDLL(None)
    libc.srand(7)
    expect = [libc.rand() % 1000 + 1 for _ in range(40)]
    # A 41-vertex star in DIMACS10: the hub row lists 40 neighbours; the other rows list the hub.
    lines = ["41 40", " ".join(str(i) for i in range(2, 42))] + ["1"] * 40
    p = tmp_path / "star.graph"
    p.write_text("\n".join(lines) + "\n")
    g = dpg.read_graph(p, 1)
    assert g.E == 80
    # Weights are drawn in read order: the hub's 40 first; convertCSR reverses the hub's row.
    assert g.weights[: 40].tolist() == expect[::-1]


def test_rmat_properties():
    s, d, w = dpg.rmat_arcs(12, 16 * 4096, seed=5, wmin=1, wmax=255)
    assert s.min() >= 0 and s.max() < 4096 and d.min() >= 0 and d.max() < 4096
    assert w.min() >= 1 and w.max() <= 255
    s2, d2, w2 = dpg.rmat_arcs(12, 16 * 4096, seed=5, wmin=1, wmax=255)
    assert np.array_equal(s, s2) and np.array_equal(d, d2) and np.array_equal(w, w2)
    s3, _, _ = dpg.rmat_arcs(12, 16 * 4096, seed=6, wmin=1, wmax=255)
    assert not np.array_equal(s, s3)
    deg = np.bincount(s, minlength=4096)
    assert deg.max() > 20 * deg.mean()  # skewed (power-law-like) out-degrees


def test_rmat_non_power_of_two_vertex_count():
    s, d, _ = dpg.rmat_arcs(10, 5000, seed=9, V=700)
    assert s.max() < 700 and d.max() < 700


def test_grid_arcs_shape():
    s, d, w = dpg.grid_arcs(4, 5, seed=1, wmin=1, wmax=1000)
    assert s.shape[0] == 2 * (4 * 4 + 5 * 3)
    g = dpg.csr_from_arcs(20, s, d, w)
    deg = np.diff(g.offsets)
    assert deg.min() == 2 and deg.max() == 4  # corners 2, interior 4
    pairs = {(a, b): c for a, b, c in zip(s.tolist(), d.tolist(), w.tolist())}
    assert all(pairs[(b, a)] == c for (a, b), c in pairs.items())  # symmetric weights


@pytest.mark.parametrize("text,fmt", [
    ("p sp 3 2\na 1 2 5\n", 0),              # fewer arcs than declared
    ("a 1 2 5\np sp 3 1\n", 0),              # arc before the problem line
    ("p sp 3 1\na 1 9 5\n", 0),              # endpoint out of range
    ("p sp 3 1\na 1 2\n", 0),                # missing weight
    ("4 2\n2\n1\n", 1),                      # missing adjacency lines
    ("# a\n# b\n# Nodes: 2 Edges: 1\n# x\n0 x\n", 2),  # malformed edge line
])
def test_malformed_files_report_format_errors(tmp_path, text, fmt):
    p = tmp_path / "bad.txt"
    p.write_text(text)
    with pytest.raises(dpg.DpgError) as e:
        dpg.read_graph(p, fmt)
    assert e.value.status == dpg.ERR_FORMAT


def test_missing_file_and_bad_format_code(tmp_path):
    with pytest.raises(dpg.DpgError) as e:
        dpg.read_graph(tmp_path / "nope.gr", 0)
    assert e.value.status == dpg.ERR_IO
    p = tmp_path / "x.gr"
    p.write_text("p sp 1 0\n")
    with pytest.raises(dpg.DpgError) as e:
        dpg.read_graph(p, 7)
    assert e.value.status == dpg.ERR_INVALID_ARG


def test_csr_builder_rejects_bad_arcs():
    with pytest.raises(dpg.DpgError):
        dpg.csr_from_arcs(3, [0, 5], [1, 2], [1, 1])
    with pytest.raises(dpg.DpgError):
        dpg.csr_transpose(2, np.array([0, 1, 3], np.int32), np.array([1, 0], np.int32))


def test_empty_graph_roundtrip():
    g = dpg.csr_from_arcs(5, [], [], [])
    assert g.offsets.tolist() == [0] * 6 and g.E == 0
    in_off, in_col = dpg.csr_transpose(5, g.offsets, g.col)
    assert in_off.tolist() == [0] * 6 and in_col.size == 0
