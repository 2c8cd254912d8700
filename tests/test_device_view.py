"""The device-side view for user kernels (include/gbvdb_device.cuh): a kernel
written against the reference's VDBInfo layout (tests/cpp/device_view_sample.cu)
walks this library's node pools from top_lev and reads the atlas at the
reference's atlas coordinates (getAtlasPos), and sees the same voxels as
gbvdb_export_atlas_bricks and the same leaves as the atlas map."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import build_lib
import datasets

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "device_view_sample.cu")


def build_sample(tmp_path):
    out = str(tmp_path / "libdevice_view.so")
    cmd = ["nvcc", "-shared", "-Xcompiler", "-fPIC", "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(ROOT, "include"), SRC, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_device_view_sample_compiles(tmp_path):
    assert os.path.exists(build_sample(tmp_path))


def test_vdb_info_size_matches_header(tmp_path):
    import gbvdb

    src = tmp_path / "sz.cu"
    src.write_text('#include "gbvdb_device.cuh"\n#include <cstdio>\nint main(){printf("%zu", sizeof(gbvdb_vdb_info));}\n')
    exe = str(tmp_path / "sz")
    r = subprocess.run(["nvcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert int(subprocess.run([exe], capture_output=True, text=True).stdout) == gbvdb.VDB_INFO_BYTES


@pytest.mark.gpu
@pytest.mark.parametrize("log2dims", [(3, 3, 3, 4), (4, 4, 3, 4)])
def test_consumer_kernel_reads_the_exported_atlas(tmp_path, gpu_lib, log2dims):
    import torch

    import gbvdb

    build_lib.build()
    lib = ctypes.CDLL(build_sample(tmp_path))
    lib.dv_read_bricks.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p]
    lib.dv_find_leaves.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p]
    if log2dims == (3, 3, 3, 4):
        pts = datasets.shell(60_000, seed=7)
    else:
        pts = datasets.sphere_surface(80_000, seed=7, domain=3000.0)
        pts = pts[np.all(pts > 1.0, axis=1)]
    g = gbvdb.Grid(0, log2dims)
    g.add_channel(0)
    n = g.set_points(torch.from_numpy(np.ascontiguousarray(pts)).cuda())
    g.rebuild_topology(n, 1.0)
    g.update_atlas()
    _, ln = g.insert_points_subcell(4, n, 1.0)
    g.gather_density(4, n, 1.0, (0, 0, 0), ln)
    g.update_apron(0, 0.0)
    info = g.vdb_info()
    torch.cuda.synchronize()
    ref = g.atlas_bricks(0)
    used = ref.shape[0]
    assert used > 0
    got = np.zeros(used * 5832 + 1, dtype=np.float32)
    assert lib.dv_read_bricks(info, used, got.ctypes.data) == 0
    assert np.array_equal(got[:used * 5832].reshape(used, 18, 18, 18), ref)
    leaves = np.zeros(2 * used + 2, dtype=np.int32)
    assert lib.dv_find_leaves(info, used, leaves.ctypes.data) == 0
    amap = g.atlas_map()
    assert np.array_equal(leaves[0:2 * used:2], amap["leaf"][:used])
    assert leaves[1:2 * used:2].all()
