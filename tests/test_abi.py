"""The C-ABI library loads and exports every entry point declared in include/dpg.h (no GPU calls
beyond context creation's device probe)."""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT, dpg

HEADER = ROOT / "include" / "dpg.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]*?\b(dpg_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_solvers():
    names = declared_functions()
    for must in ["dpg_ctx_create", "dpg_graph_create", "dpg_sssp", "dpg_bfs", "dpg_spmv_f32", "dpg_pagerank_f32",
                 "dpg_read_graph", "dpg_csr_from_arcs", "dpg_csr_transpose"]:
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(dpg.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\s[TW]\s(dpg_\w+)$", out, flags=re.M))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared in include/dpg.h but not exported: {missing}"


def test_binding_covers_every_declared_symbol():
    assert sorted(dpg.exported_symbols()) == declared_functions()


def test_status_strings_and_version(lib):
    assert lib.dpg_version() == 1
    assert lib.dpg_status_string(0) == b"DPG_OK"
    assert lib.dpg_status_string(3) == b"DPG_ERR_TIMEOUT"


def test_null_arguments_are_errors_not_crashes(lib):
    assert lib.dpg_ctx_create(0, None) == dpg.ERR_INVALID_ARG
    assert lib.dpg_read_graph(None, 0, None) == dpg.ERR_INVALID_ARG
    assert lib.dpg_csr_from_arcs(-1, 0, None, None, None, None, None, None) == dpg.ERR_INVALID_ARG


def test_no_device_reports_status():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(dpg.DpgError) as e:
        dpg.Context(0)
    assert e.value.status == dpg.ERR_NO_DEVICE


def test_no_reference_or_oracle_in_product_library():
    out = subprocess.run(["nm", "-D", str(dpg.LIB_PATH)], capture_output=True, text=True, check=True).stdout
    assert "oracle_" not in out and "ref_load" not in out
    deps = subprocess.run(["ldd", str(dpg.LIB_PATH)], capture_output=True, text=True).stdout
    assert "liboracle" not in deps and "libref" not in deps


STRUCTS = {"dpg_expand_opts": "ExpandOpts", "dpg_pr_opts": "PrOpts", "dpg_run_stats": "RunStats",
           "dpg_batch_tuning": "BatchTuning", "dpg_cdp_stats": "CdpStats", "dpg_host_graph": "_HostGraph"}


def test_binding_structs_match_the_header(tmp_path):
    """Size and every field offset of the option and result structs, from a C program compiled
    against include/dpg.h, equal those of the Python binding's ctypes structures."""
    import ctypes

    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "dpg.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        cls = getattr(dpg, pyname)
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    want = []
    for cname, pyname in STRUCTS.items():
        cls = getattr(dpg, pyname)
        want.append(f"{cname} size {ctypes.sizeof(cls)}")
        want += [f"{cname} {fname} {getattr(cls, fname).offset}" for fname, _ in cls._fields_]
    assert got[:-1] == want
