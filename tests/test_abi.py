"""CPU checks of the C ABI: libgbvdb.so builds for sm_103a, loads, and exports
every entry point include/gbvdb.h declares.  No kernel is launched here."""
import ctypes
import os
import re
import subprocess

import pytest

import build_lib
import gbvdb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbvdb.h")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"GBVDB_API\s+[\w\s\*]+?\b(gbvdb_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib_path():
    try:
        return build_lib.build()
    except RuntimeError as e:  # nvcc missing is a hard failure: there is no fallback
        pytest.fail(str(e))


def test_header_matches_binding():
    assert declared() == sorted(gbvdb.EXPORTS)


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True).stdout
    syms = set(re.findall(r"\bT (gbvdb_\w+)", out))
    missing = [s for s in declared() if s not in syms]
    assert not missing, missing
    lib = ctypes.CDLL(lib_path)
    for s in declared():
        assert hasattr(lib, s)


def test_build_targets_sm103a_only():
    assert build_lib.GENCODE == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_node_record_layout():
    assert gbvdb.NODE_DTYPE.itemsize == 64
    off = {k: v[1] for k, v in gbvdb.NODE_DTYPE.fields.items()}
    assert (off["pos"], off["value"], off["vrange"], off["parent"], off["childlist"], off["mask"]) == \
        (4, 16, 28, 40, 48, 56)


def test_create_without_device_fails_cleanly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = gbvdb.load()
    h = ctypes.c_void_p()
    st = L.gbvdb_create(0, ctypes.byref(h))
    assert st == gbvdb.CUDA_ERROR and not h.value


def test_tuning_table_is_read(tmp_path):
    """the library reads the tuning table beside it (or $GBVDB_TUNE_TABLE) at first use"""
    import json
    import subprocess
    import sys

    table = os.path.join(ROOT, "gvdb-voxels_gb300", "tune_table.json")
    assert os.path.exists(table)
    d = json.load(open(table))
    assert d["buckets"] and all({"max_points", "dense_min", "gather_blocks", "bin_unroll", "scatter_unroll"}
                                <= set(b) for b in d["buckets"])
    L = gbvdb.load()
    assert L.gbvdb_tune_table_source().decode() == os.path.realpath(table) or \
        os.path.samefile(L.gbvdb_tune_table_source().decode(), table)
    # an explicit table through the environment (a fresh process: the table is read once)
    alt = tmp_path / "t.json"
    alt.write_text(json.dumps({"buckets": [{"max_points": 5, "dense_min": 1, "gather_blocks": 8,
                                            "bin_unroll": 4, "scatter_unroll": 8}]}))
    code = ("import sys; sys.path.insert(0, %r); import gbvdb; "
            "print(gbvdb.load().gbvdb_tune_table_source().decode())" % os.path.join(ROOT, "gvdb-voxels_gb300"))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         env=dict(os.environ, GBVDB_TUNE_TABLE=str(alt))).stdout.strip()
    assert out == str(alt)
