"""VBX save / load (SaveVBX / LoadVBX, gvdb_volume_gvdb.cpp:1626-1767, 507-683).

CPU: the oracle's restatement of SaveVBX, read back by an independent reader
written from the format description, holds the oracle's pools and atlas.
GPU: the CUDA path writes the same header and topology bytes as the oracle
(bit-exact) and atlas values within the gather tolerance; a file loaded into a
new grid gives back every pool, the atlas map and every brick bit-exactly, and
the loaded grid keeps working (UpdateApron, a new frame).
"""
import os

import numpy as np
import pytest

import _helpers as H
import datasets
from vbx_reader import atlas_bricks, read_vbx


def _oracle_grid(pts, rho=1.0, radius=1.0):
    import oracle

    g = oracle.OracleGrid((3, 3, 3, 4))
    g.add_channel(0, 3, 1, (0, 0, 0))
    assert g.rebuild_topology(pts, radius) == 0
    g.update_atlas()
    g.insert_points_subcell(pts, radius)
    g.gather_density(rho)
    g.update_apron(0, 0.0)
    return g


def test_oracle_vbx_layout(tmp_path):
    pts = datasets.shell(6000, seed=61, rmin=30.0, rmax=40.0)
    g = _oracle_grid(pts)
    path = str(tmp_path / "o.vbx")
    g.save_vbx(path)
    v = read_vbx(path)
    assert (v["major"], v["minor"], v["num_grids"]) == (1, 11, 1)
    assert list(v["scale"]) == [1, 1, 1] and not np.any(v["pretrans"]) and not np.any(v["trans"])
    assert v["grid_offsets"][0] == v["grid_header_offset"] == 2 + 48 + 4 + 8
    assert (v["dtype"], v["components"], v["compression"], v["topology_type"], v["layout"]) == ("f", 1, 0, 2, 0)
    assert list(v["brick_dims"]) == [16, 16, 16] and v["apron"] == 1 and v["num_channels"] == 1
    ax, ay, az, used = g.atlas_dims()
    assert list(v["axiscnt"]) == [ax, ay, az] and list(v["axisres"]) == [ax * 18, ay * 18, az * 18]
    assert v["atlas_size"] == 4 * ax * ay * az * 18 ** 3
    assert v["levels"] == 4 and v["root"] == g.depth << 8
    assert v["brick_count"] == g.node_count(0)
    for lev, d in enumerate(v["level_info"]):
        assert (d["log2dim"], d["res"]) == ((4, 3, 3, 3)[lev], 1 << (4, 3, 3, 3)[lev])
        assert d["cnt0"] == g.node_count(lev) and d["width0"] == 64
        assert v["nodes"][lev].tobytes() == g.nodes(lev).tobytes()
        if lev >= 1:
            assert d["cnt1"] == g.node_count(lev) and d["width1"] == 8 * 512
            assert np.array_equal(v["childlists"][lev], g.childlist(lev))
        else:
            assert d["cnt1"] * d["width1"] == 0
    ch = v["channels"][0]
    assert (ch["type"], ch["stride"]) == (3, 4)
    b = atlas_bricks(ch["volume"], v["axiscnt"], ax * ay * az)
    assert np.array_equal(b[:used], g.atlas_bricks(0).astype(np.float32))
    assert not np.any(b[used:])
    assert v["end"] == v["size"]


@pytest.mark.gpu
def test_vbx_save_matches_oracle_and_loads_back(gpu_lib, tmp_path):
    import torch

    import gbvdb

    pts = datasets.shell(40_000, seed=62)
    og = _oracle_grid(pts)
    opath = str(tmp_path / "o.vbx")
    og.save_vbx(opath)
    ov = read_vbx(opath)

    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0, gbvdb.T_FLOAT)
    d = torch.from_numpy(pts).cuda()
    n = g.set_points(d)
    g.rebuild_topology(n, 1.0)
    g.update_atlas()
    _, ln = g.insert_points_subcell(4, n, 1.0)
    g.gather_density(4, n, 1.0, (0, 0, 0), ln)
    g.update_apron(0, 0.0)
    gpath = str(tmp_path / "g.vbx")
    g.save_vbx(gpath)
    gv = read_vbx(gpath)

    # header and topology sections byte for byte; atlas within the gather tolerance
    with open(opath, "rb") as f:
        ob = f.read()
    with open(gpath, "rb") as f:
        gb = f.read()
    assert ov["atlas_offset"] == gv["atlas_offset"] and len(ob) == len(gb)
    assert ob[:gv["atlas_offset"]] == gb[:gv["atlas_offset"]]
    ovol, gvol = ov["channels"][0]["volume"].astype(np.float64), gv["channels"][0]["volume"].astype(np.float64)
    assert np.all(np.abs(ovol - gvol) <= H.ATOL + H.RTOL * np.abs(ovol))

    # the file's atlas holds the grid's bricks
    info = g.atlas_info(0)
    bricks = g.atlas_bricks(0)
    vb = atlas_bricks(gv["channels"][0]["volume"], gv["axiscnt"], info["used"])
    assert vb.tobytes() == bricks.tobytes()

    # load into a new grid: pools, atlas map, bricks and checksum come back bit-exactly
    g2 = gbvdb.Grid(0, (3, 3, 3, 4))
    g2.load_vbx(gpath)
    for lev in range(4):
        assert g2.nodes(lev).tobytes() == g.nodes(lev).tobytes()
        assert np.array_equal(g2.childlist(lev), g.childlist(lev))
    assert g2.atlas_map().tobytes() == g.atlas_map().tobytes()
    assert g2.atlas_info(0) == info
    assert g2.atlas_bricks(0).tobytes() == bricks.tobytes()
    assert g2.checksum(0) == g.checksum(0)
    # the loaded grid keeps working: apron again, then a new frame (a full rebuild)
    g2.update_apron(0, 0.0)
    assert g2.atlas_bricks(0).tobytes() == bricks.tobytes()
    n2 = g2.set_points(d)
    g2.rebuild_topology(n2, 1.0)
    g2.update_atlas()
    _, ln2 = g2.insert_points_subcell(4, n2, 1.0)
    g2.gather_density(4, n2, 1.0, (0, 0, 0), ln2)
    g2.update_apron(0, 0.0)
    assert ln2 == ln
    assert g2.checksum(0) == g.checksum(0)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["half", "bf16"])
def test_vbx_reduced_precision_roundtrip(gpu_lib, tmp_path, dtype):
    import torch

    import gbvdb

    dt = gbvdb.T_HALF if dtype == "half" else gbvdb.T_BFLOAT16
    pts = datasets.shell(20_000, seed=63)
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0, dt)
    n = g.set_points(torch.from_numpy(pts).cuda())
    g.rebuild_topology(n, 1.0)
    g.update_atlas()
    _, ln = g.insert_points_subcell(4, n, 1.0)
    g.gather_density(4, n, 1.0, (0, 0, 0), ln)
    g.update_apron(0, 0.0)
    path = str(tmp_path / "h.vbx")
    g.save_vbx(path)
    v = read_vbx(path)
    assert (v["channels"][0]["type"], v["channels"][0]["stride"]) == (dt, 2)
    g2 = gbvdb.Grid(0, (3, 3, 3, 4))
    g2.load_vbx(path)
    assert g2.atlas_info(0)["dtype"] == dt
    assert g2.atlas_bricks(0).tobytes() == g.atlas_bricks(0).tobytes()
    assert os.path.getsize(path) == v["end"]
