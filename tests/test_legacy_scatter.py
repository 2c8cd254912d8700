"""Legacy InsertPoints + ScatterDensity (gvdb_volume_gvdb.cpp:5219-5267, 5624-5660;
cuda_gvdb_particles.cuh:19-68, 516-571) against the oracle's restatement: the leaf
of every point and the per-leaf groups exactly, the splatted channel (interior and
the apron voxels that `expand` reaches) within the gather tolerance."""
import numpy as np
import pytest

import _helpers as H
import datasets

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("expand", [False, True])
def test_insert_points_and_scatter_density(gpu_lib, expand):
    import torch

    import gbvdb
    import oracle

    pts = datasets.shell(80_000, seed=81)
    og = oracle.OracleGrid((3, 3, 3, 4))
    og.add_channel(0, 3, 1, (0, 0, 0))
    assert og.rebuild_topology(pts, 1.0) == 0
    og.update_atlas()
    o_pnode, o_counts = og.insert_points(pts)
    og.scatter_density(pts, 1.5, expand=expand)
    o_bricks = og.atlas_bricks(0)

    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0, gbvdb.T_FLOAT)
    d = torch.from_numpy(pts).cuda()
    n = g.set_points(d)
    g.rebuild_topology(n, 1.0)
    g.update_atlas()
    g.insert_points(n)
    pnode, off, grouped = g.point_leaves(n)
    assert np.array_equal(pnode, o_pnode)
    assert np.array_equal(np.diff(off), o_counts)
    # groups hold each leaf's points (order inside a group unspecified)
    order = np.argsort(pnode, kind="stable")
    valid = pnode[order] >= 0
    ref = pts[order][valid]
    leaf_of = np.repeat(np.arange(len(o_counts)), o_counts)
    for lf in np.unique(leaf_of)[:200]:
        a = grouped[off[lf]:off[lf + 1]]
        b = ref[leaf_of == lf]
        assert np.array_equal(a[np.lexsort(a.T)], b[np.lexsort(b.T)])
    g.scatter_density(n, 1.5, expand=expand)
    b = g.atlas_bricks(0).astype(np.float64)
    assert b.shape == o_bricks.shape
    err = np.abs(b - o_bricks)
    assert np.all(err <= 1e-6 + 1e-5 * np.abs(o_bricks)), err.max()
    assert np.abs(o_bricks).sum() > 0
    if expand:  # apron voxels next to points were reached
        assert np.abs(o_bricks[:, 0, 1:17, 1:17]).sum() > 0
