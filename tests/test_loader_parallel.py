"""The parallel DIMACS9 reader against the serial one (the reference's readInputDIMACS9 semantics,
common/global.cpp:29-61): identical arrays, source and first error on every file; and the binary
CSR cache round trip."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dpg


def _write(path, lines, newline="\n", trailing=True):
    text = newline.join(lines) + (newline if trailing else "")
    path.write_bytes(text.encode())
    return path


def _random_gr(rng, V, E, with_s=True):
    lines = ["c generated", f"p sp {V} {E}"]
    if with_s:
        lines.append(f"s {int(rng.integers(1, V + 1))}")
    for k in range(E):
        u, v, w = int(rng.integers(1, V + 1)), int(rng.integers(1, V + 1)), int(rng.integers(-5, 1000))
        sep = " " if k % 7 else "  "
        tail = " " if k % 11 == 0 else ""
        lines.append(f"a{sep}{u}{sep}{v} {w}{tail}")
        if k % 5000 == 0:
            lines.append("c interleaved comment")
    return lines


def _same(path):
    a = dpg.read_graph(path, 0, threads=1)
    for t in (2, 3, 8):
        b = dpg.read_graph(path, 0, threads=t)
        assert (a.V, a.E, a.source) == (b.V, b.E, b.source)
        assert np.array_equal(a.offsets, b.offsets) and np.array_equal(a.col, b.col)
        assert np.array_equal(a.weights, b.weights)
    return a


@pytest.mark.parametrize("newline,trailing", [("\n", True), ("\r\n", True), ("\n", False)])
def test_parallel_equals_serial(tmp_path, newline, trailing):
    rng = np.random.default_rng(5)
    g = _same(_write(tmp_path / "g.gr", _random_gr(rng, 3000, 60000), newline, trailing))
    assert g.E == 60000


def _error(path, threads):
    with pytest.raises(dpg.DpgError) as ei:
        dpg.read_graph(path, 0, threads=threads)
    return str(ei.value)


@pytest.mark.parametrize("case", ["a_before_p", "bad_a", "range_first", "count", "source", "short_p", "two_p"])
def test_errors_match_serial(tmp_path, case):
    rng = np.random.default_rng(6)
    lines = _random_gr(rng, 500, 20000)
    if case == "a_before_p":
        lines.insert(1, "a 1 2 3")
    elif case == "bad_a":
        lines[9000] = "a 1 x 3"
    elif case == "range_first":
        lines[15000] = "a 1 501 3"   # later out-of-range arc
        lines[7000] = "a 600 1 3"    # the first one in file order
    elif case == "count":
        lines[1] = "p sp 500 19999"
    elif case == "source":
        lines[2] = "s 900"
    elif case == "short_p":
        lines[1] = "p"
    elif case == "two_p":
        lines.insert(5000, "p sp 500 20000")
        path = _write(tmp_path / "g.gr", lines)
        _same(path)  # several 'p' lines: the parallel reader defers to the serial one
        return
    path = _write(tmp_path / "g.gr", lines)
    serial = _error(path, 1)
    for t in (2, 4, 8):
        assert _error(path, t) == serial


def test_reference_fixture_through_parallel_reader(tmp_path):
    from conftest import load_golden

    rec = load_golden("data_test.json")
    a = rec["arcs"]
    p = tmp_path / "d.gr"
    dpg.write_dimacs9(p, rec["V"], a["src"], a["dst"], a["w"], source=rec["source"])
    for t in (1, 4):
        g = dpg.read_graph(p, 0, threads=t)
        assert g.source == rec["source"] and g.offsets.tolist() == rec["offsets"]
        assert g.col.tolist() == rec["col"] and g.weights.tolist() == rec["weights"]


def test_cache_round_trip(tmp_path):
    rng = np.random.default_rng(7)
    g = _same(_write(tmp_path / "g.gr", _random_gr(rng, 1000, 10000)))
    dpg.write_graph_cache(tmp_path / "g.dpgcsr", g)
    h = dpg.read_graph_cache(tmp_path / "g.dpgcsr")
    assert (g.V, g.E, g.source) == (h.V, h.E, h.source)
    assert np.array_equal(g.offsets, h.offsets) and np.array_equal(g.col, h.col)
    assert np.array_equal(g.weights, h.weights)
    (tmp_path / "bad.dpgcsr").write_bytes(b"DPGCSR01" + b"\x00" * 10)
    with pytest.raises(dpg.DpgError):
        dpg.read_graph_cache(tmp_path / "bad.dpgcsr")
    (tmp_path / "junk.dpgcsr").write_bytes(b"not a cache at all")
    with pytest.raises(dpg.DpgError):
        dpg.read_graph_cache(tmp_path / "junk.dpgcsr")
