"""bench.py's DRAM-traffic bookkeeping on the CPU: an ncu raw-page CSV is turned into the profile
file with the fingerprint of the gather's sources, read back as read + write bytes, and reported
as stale once a source changes (no GPU; the sources are copied into a scratch tree)."""
from __future__ import annotations

import shutil
import sys

import pytest

from conftest import ROOT


@pytest.fixture()
def bench_in_tmp(tmp_path, monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    for rel in bench.GATHER_SOURCES:
        (tmp_path / rel).parent.mkdir(parents=True, exist_ok=True)
        shutil.copy(ROOT / rel, tmp_path / rel)
    (tmp_path / "profiles").mkdir()
    monkeypatch.setattr(bench, "ROOT", tmp_path)
    return bench, tmp_path


def _csv(path, kernel, read, write, unit="byte"):
    rows = ['"ID","Kernel Name","dram__bytes_read.sum","dram__bytes_write.sum"',
            f'"","","{unit}","{unit}"',
            f'"0","{kernel}","{read}","{write}"']
    path.write_text("==PROF== some log line\n" + "\n".join(rows) + "\n")
    return str(path)


def test_ingest_then_read_back(bench_in_tmp, tmp_path):
    bench, root = bench_in_tmp
    csv = _csv(tmp_path / "t.csv", "void rowgather_kernel<1, 2>(RowGatherLaunch)", "1,234,000", "5,000")
    assert bench.ingest_traffic(csv) == 0
    text = (root / "profiles" / bench.TRAFFIC_FILE).read_text()
    assert bench.TRAFFIC_COMMAND in text and f"sources_fingerprint = {bench.sources_fingerprint()}" in text
    assert bench.capture_traffic() == (1239000.0, "ncu capture of these sources")


def test_units_are_scaled(bench_in_tmp, tmp_path):
    bench, _ = bench_in_tmp
    assert bench.ingest_traffic(_csv(tmp_path / "t.csv", "rowgather_kernel", "336.61", "4.03", "Mbyte")) == 0
    value, note = bench.capture_traffic()
    assert value == pytest.approx(340.64e6) and note == "ncu capture of these sources"


def test_changed_source_makes_the_capture_stale(bench_in_tmp, tmp_path):
    bench, root = bench_in_tmp
    assert bench.ingest_traffic(_csv(tmp_path / "t.csv", "rowgather_kernel", "10", "2")) == 0
    src = root / bench.GATHER_SOURCES[0]
    src.write_text(src.read_text() + "\n// edited\n")
    assert bench.capture_traffic() == (None, "capture is of other kernel sources (stale)")


def test_missing_kernel_or_file(bench_in_tmp, tmp_path):
    bench, _ = bench_in_tmp
    assert bench.capture_traffic() == (None, "no capture")
    assert bench.ingest_traffic(_csv(tmp_path / "t.csv", "expand_kernel", "10", "2")) == 1
