"""gbvdb_checksum_noalloc: the FP64 atlas checksum for callers that may not
allocate device memory (a host application that owns every device allocation,
or a serving loop working inside a fixed memory budget).

Checked through the C ABI on two calls in a row that share its static scratch
array: each result equals gbvdb_checksum's bit for bit (both run the same
kernels in the same fixed order) and the oracle's FP64 sum within the parity
tolerance; the grid's device byte total is unchanged by the calls and torch's
allocator holds no more than before them; a grid with more atlas slots than the static array holds is refused
with GBVDB_CAPACITY.  This file sorts last so that a run stopping at the first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest

import datasets

pytestmark = pytest.mark.gpu


def _grids(points, radius, mode):
    import torch

    import gbvdb
    import oracle

    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0)
    d = torch.from_numpy(np.ascontiguousarray(points, dtype=np.float32)).cuda()
    n = g.set_points(d)
    g.rebuild_topology(n, radius)
    g.update_atlas()
    _, ln = g.insert_points_subcell(4, n, radius)
    og = oracle.OracleGrid((3, 3, 3, 4))
    og.add_channel(0)
    og.rebuild_topology(points, radius)
    og.update_atlas()
    og.insert_points_subcell(points, radius)
    if mode == "density":
        g.gather_density(4, n, radius, (0, 0, 0), ln)
        og.gather_density(radius)
    else:
        g.gather_levelset(4, n, radius, (0, 0, 0), ln)
        og.gather_levelset(radius)
    g.update_apron(0, 0.0)
    torch.cuda.synchronize()
    return g, og, d


def _noalloc(g, out):
    import torch

    import gbvdb

    st = g.L.gbvdb_checksum_noalloc(g._h, 0, ctypes.c_void_p(out.data_ptr()))
    torch.cuda.synchronize()
    return st, float(out.item())


def test_checksum_noalloc_matches_checksum_twice(gpu_lib):
    import torch

    import gbvdb

    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    for pts, radius, mode in ((datasets.shell(120_000, seed=4), 1.0, "levelset"),
                              (datasets.shell(15_000, seed=8, rmin=30.0, rmax=40.0), 1.5, "density")):
        g, og, _ = _grids(pts, radius, mode)
        ref = g.checksum(0)
        bytes_before = g.device_bytes()
        torch_before = torch.cuda.memory_allocated()
        st, got = _noalloc(g, out)
        assert st == gbvdb.OK, g.L.gbvdb_last_error(g._h)
        assert g.device_bytes() == bytes_before
        assert torch.cuda.memory_allocated() <= torch_before
        assert got == ref, (got, ref)
        exact = og.checksum(0)
        assert abs(got - exact) <= 1e-6 + 1e-5 * abs(exact), (got, exact)
        g.close()


def test_checksum_noalloc_refuses_grids_beyond_its_scratch(gpu_lib):
    import torch

    import gbvdb

    # one point at the centre of each brick of a 48 x 48 x 32 brick block: 73,728 leaves,
    # more than the 65,536 slots of the static scratch
    ix, iy, iz = np.meshgrid(np.arange(48), np.arange(48), np.arange(32), indexing="ij")
    pts = (np.stack([ix, iy, iz], axis=-1).reshape(-1, 3) * 16 + 8).astype(np.float32)
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0)
    d = torch.from_numpy(pts).cuda()
    n = g.set_points(d)
    g.rebuild_topology(n, 0.0)
    g.update_atlas()
    assert g.atlas_info(0)["used"] == pts.shape[0]
    out = torch.zeros((1,), dtype=torch.float64, device="cuda")
    st, _ = _noalloc(g, out)
    assert st == gbvdb.CAPACITY
    assert b"static scratch" in g.L.gbvdb_last_error(g._h)
    g.close()
