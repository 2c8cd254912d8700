"""The apron record index math (apron_index, its inverse apron_shell_pos and the
edge/corner table of the fused apron) checked on the host: a small program built
with nvcc from csrc/common.cuh (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "apron_index_check.cu")


def test_apron_index_inverse_and_edge_table(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "apron_index_check")
    cmd = [nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "gvdb-voxels_gb300", "csrc"), "-I", os.path.join(ROOT, "include"), SRC, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
