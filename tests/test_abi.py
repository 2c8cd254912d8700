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
