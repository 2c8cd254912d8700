"""The host topology path (ActivateSpace / RebuildTopologyCPU, gvdb_volume_gvdb.cpp
:1220-1227, 2707-2875) through the C ABI against the oracle's restatement of it
(og_rebuild_topology_cpu, itself cross-checked in tests/test_oracle_cpu_path.py):
node pools (every field) and the child lists in use bit-exact, the root grown to the
same level; then the device path (UpdateAtlas, InsertPointsSubcell, GatherDensity,
UpdateApron) on that topology against the oracle."""
import numpy as np
import pytest

import datasets
from _helpers import check_apron_self, compare_values

pytestmark = pytest.mark.gpu
UNDEFL = 0xFFFFFFFF


def lists_in_use(nodes):
    cl = nodes["childlist"]
    live = cl[cl != np.uint64(UNDEFL)]
    return int((live >> np.uint64(16)).max()) + 1 if live.size else 0


def compare_pools(og, g, levs):
    for lev in range(levs):
        a, b = og.nodes(lev), g.nodes(lev)
        assert a.shape == b.shape, (lev, a.shape, b.shape)
        for f in ("lev", "flags", "pos", "value", "parent", "childlist"):
            assert np.array_equal(a[f], b[f]), (lev, f)
        if lev > 0:
            k = lists_in_use(a)
            assert np.array_equal(og.childlist(lev)[:k], g.childlist(lev)[:k]), lev
            assert np.all(g.childlist(lev)[k:] == np.uint64(0xFFFFFFFFFFFFFFFF)), lev


@pytest.mark.parametrize("which", ["shell", "fluid_crop", "two_clusters"])
def test_rebuild_topology_cpu_matches_oracle(gpu_lib, which):
    import torch

    import gbvdb
    import oracle

    if which == "shell":
        pts = datasets.shell(200_000, seed=0)
    elif which == "fluid_crop":
        pos, vel = datasets.fluid(n=300_000, seed=3, box=(64, 96, 64), domain=160)
        pts = (pos + 0.5 * vel).astype(np.float32)
        pts = pts[np.all(pts > 0, axis=1)]
    else:  # far apart: the root grows by Reparent through several levels
        a = datasets.shell(20_000, seed=9, center=(40.0, 40.0, 40.0), rmin=10.0, rmax=14.0)
        b = datasets.shell(20_000, seed=10, center=(1500.0, 700.0, 900.0), rmin=10.0, rmax=14.0)
        pts = np.concatenate([a, b]).astype(np.float32)
    og = oracle.OracleGrid((3, 3, 3, 4))
    og.add_channel(0)
    og.rebuild_topology_cpu(pts)
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0)
    g.rebuild_topology_cpu(pts)
    g.finish_topology(True, True)
    compare_pools(og, g, 4)
    assert g.depth()[0] == og.cpu_root_level()
    assert np.array_equal(og.compute_bounds(), g.vol_bounds())
    # the device path on the host-built topology
    og.update_atlas()
    _, ln_o = og.insert_points_subcell(pts, 1.0)
    og.gather_density(1.0)
    og.update_apron(0, 0.0)
    d = torch.from_numpy(pts).cuda()
    n = g.set_points(d)
    g.update_atlas()
    _, ln = g.insert_points_subcell(4, n, 1.0)
    g.gather_density(4, n, 1.0, (0, 0, 0), ln)
    g.update_apron(0, 0.0)
    torch.cuda.synchronize()
    assert ln == ln_o
    info = g.atlas_info(0)
    o = {"bricks": og.atlas_bricks(0)}
    s = {"bricks": g.atlas_bricks(0), "dtype": info["dtype"], "amap": g.atlas_map()}
    compare_values(o, s)
    check_apron_self(s, np.float32(0.0))


def test_activate_space_per_point(gpu_lib):
    import gbvdb
    import oracle

    pts = datasets.shell(3000, seed=2, center=(300.0, 300.0, 300.0), rmin=40.0, rmax=50.0)
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0)
    first = [g.activate_space(p) for p in pts]
    again = [g.activate_space(p) for p in pts]
    # the first activation of a leaf reports a new leaf; a second one returns the leaf
    assert all(v != UNDEFL for v in again)
    assert all((v >> 8) & 0xFF == 0 for v in again)
    leaves = g.nodes(0)  # commits
    for p, v in zip(pts[:200], again[:200]):
        lp = leaves["pos"][v >> 16]
        assert np.all(lp <= p.astype(np.int32)) and np.all(p.astype(np.int32) < lp + 16)
    # every leaf but the first (created as the root) was reported new once
    assert sum(v == UNDEFL for v in first) == leaves.shape[0] - 1
    og = oracle.OracleGrid((3, 3, 3, 4))
    og.rebuild_topology_cpu(pts)
    compare_pools(og, g, 4)
