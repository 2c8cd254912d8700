"""The VolumeGVDB facade (include/gbvdb_volume.hpp) compiles and links against
libgbvdb.so (CPU), and on a GPU a reference-style C++ frame gives the same
topology, list length and checksum as the Python binding."""
import os
import subprocess

import numpy as np
import pytest

import build_lib
import datasets

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_sample.cpp")
CUDA = "/usr/local/cuda"


def build_sample(tmp_path):
    lib = build_lib.build()
    exe = str(tmp_path / "facade_sample")
    cmd = ["g++", "-std=c++17", "-O1", SRC, "-o", exe, "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(CUDA, "include"), "-L", os.path.dirname(lib), "-lgbvdb",
           "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_compiles_and_links(tmp_path):
    assert os.path.exists(build_sample(tmp_path))


@pytest.mark.gpu
def test_facade_frame_matches_python(tmp_path, gpu_lib):
    import torch

    import gbvdb

    exe = build_sample(tmp_path)
    pts = datasets.shell(40_000, seed=12)
    f = tmp_path / "pts.f32"
    pts.astype(np.float32).tofile(str(f))
    r = subprocess.run([exe, str(f), "1.0", "density"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    tot, used, ln, cs = r.stdout.split()
    g = gbvdb.Grid(0, (3, 3, 3, 3, 4))
    g.add_channel(0)
    n = g.set_points(torch.from_numpy(pts).cuda())
    g.rebuild_topology(n, 1.0)
    g.update_atlas()
    _, ln2 = g.insert_points_subcell(4, n, 1.0)
    g.gather_density(4, n, 1.0, (0, 0, 0), ln2)
    g.update_apron(0, 0.0)
    t2, u2 = g.node_counts()
    assert (int(tot), int(used), int(ln)) == (t2[0], u2[0], ln2)
    cs2 = g.checksum(0)
    assert abs(float(cs) - cs2) <= 1e-9 * max(1.0, abs(cs2))
