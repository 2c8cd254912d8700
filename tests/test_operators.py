"""UpdateNeighbors, UpdateApronFaces and Compute(FUNC_SMOOTH) on the CUDA path
against the oracle's restatements, bit-exact on the same FP32 atlas input
(gvdb_volume_gvdb.cpp:2527-2556, 4461-4496, 4532-4558;
cuda_gvdb_operators.cuh:27-61, 383-400)."""
import numpy as np
import pytest

import datasets

pytestmark = pytest.mark.gpu


def _grids(pts, radius=1.0, rho=1.0):
    import torch

    import gbvdb
    import oracle

    og = oracle.OracleGrid((3, 3, 3, 4))
    og.add_channel(0, 3, 1, (0, 0, 0))
    assert og.rebuild_topology(pts, radius) == 0
    og.update_atlas()
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0, gbvdb.T_FLOAT)
    d = torch.from_numpy(pts).cuda()
    n = g.set_points(d)
    g.rebuild_topology(n, radius)
    g.update_atlas()
    _, ln = g.insert_points_subcell(4, n, radius)
    g.gather_density(4, n, rho, (0, 0, 0), ln)
    g._keep = d
    return og, g


def test_neighbors_faces_smooth(gpu_lib):
    import gbvdb

    pts = datasets.shell(60_000, seed=71)
    og, g = _grids(pts)
    for lev in range(4):  # same topology, so the oracle's tables and slots apply
        assert g.nodes(lev).tobytes() == og.nodes(lev).tobytes()

    g.update_neighbors()
    table = g.neighbors()
    assert np.array_equal(table, og.neighbors())
    assert (table >= 0).any() and (table < 0).any()

    b0 = np.ascontiguousarray(g.atlas_bricks(0))  # gathered interiors, aprons as cleared
    g.update_apron_faces(0)
    b1 = g.atlas_bricks(0)
    ref = b0.copy()
    og.apron_faces_f32(ref, table)
    assert ref.tobytes() == b1.tobytes()
    # faces only: edges and corners untouched
    assert np.array_equal(b1[:, 0, 0, :], b0[:, 0, 0, :]) and np.array_equal(b1[:, 17, 17, 17], b0[:, 17, 17, 17])

    g.update_apron(0, 0.0)
    b2 = g.atlas_bricks(0)
    ref = np.ascontiguousarray(b1.copy())
    og.apron_full_f32(ref, 0.0)
    assert ref.tobytes() == b2.tobytes()

    p1, p2 = 2.0, 0.05
    g.compute(gbvdb.FUNC_SMOOTH, 0, 3, (p1, p2, 0.0), update_apron=True, boundval=0.0)
    b3 = g.atlas_bricks(0)
    ref = np.ascontiguousarray(b2.copy())
    for _ in range(3):
        og.smooth_f32(ref, p1, p2)
        og.apron_full_f32(ref, 0.0)
    assert ref.tobytes() == b3.tobytes()
    assert not np.array_equal(b3, b2)


def test_operator_call_order_and_types(gpu_lib):
    import torch

    import gbvdb

    pts = datasets.shell(20_000, seed=72)
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0, gbvdb.T_HALF)
    n = g.set_points(torch.from_numpy(pts).cuda())
    g.rebuild_topology(n, 1.0)
    g.update_atlas()
    with pytest.raises(gbvdb.GbvdbError) as e:  # no neighbour table for this topology yet
        g.update_apron_faces(0)
    assert e.value.status == gbvdb.INVALID_ARG
    g.update_neighbors()
    g.update_apron_faces(0)  # FP16 faces are copies, supported
    with pytest.raises(gbvdb.GbvdbError) as e:  # the smoothing kernel is FP32 only, as in the reference
        g.compute(gbvdb.FUNC_SMOOTH, 0, 1, (1.0, 0.0, 0.0))
    assert e.value.status == gbvdb.NOT_SUPPORTED
    g.rebuild_topology(n, 1.0)  # a new topology invalidates the table
    with pytest.raises(gbvdb.GbvdbError):
        g.update_apron_faces(0)
