"""GPU parity tests: the CUDA path (through the C ABI of libgbvdb.so) against the
CPU oracle on the same seeded inputs.

Rules (see tests/_helpers.py): node pools, child lists, atlas map and subcell
membership bit-exact; gathered values within 1e-5 relative + 1e-6 absolute of
the FP64 oracle; apron voxels bit-exact copies of the neighbour interior (or
the boundary value) and within the same tolerance of the oracle.
"""
import numpy as np
import pytest

import _helpers as H
import datasets

pytestmark = pytest.mark.gpu


def _mini_fluid(n=60000, seed=11):
    pos, vel = datasets.fluid(n=n, seed=seed, box=(32, 64, 32), domain=128)
    return pos, vel


def _full_check(o, g, boundval, tol=None):
    H.compare_topology(o, g)
    H.compare_subcells(o, g)
    err = H.compare_values(o, g) if tol is None else H.compare_values(o, g, *tol)
    H.check_apron_self(g, boundval)
    return err


def test_shell_200k_density(gpu_lib):
    """Plain path, small: the 200,000-point shell, grid (3,3,3,4), r = R = rho = 1."""
    pts = datasets.shell(200_000, seed=0)
    _, o = H.run_oracle(pts, radius=1.0, R=1.0, rho=1.0, mode="density", boundval=0.0)
    _, g = H.run_gpu(pts, radius=1.0, R=1.0, rho=1.0, mode="density", boundval=0.0)
    _full_check(o[0], g[0], 0.0)
    assert abs(o[0]["checksum"] - g[0]["checksum"]) <= 1e-6 * max(1.0, abs(o[0]["checksum"]))


@pytest.mark.parametrize("touch_dirs", [1, 0])
def test_fluid_frames_levelset(gpu_lib, touch_dirs):
    """Dam-break frames: RebuildTopology(r=4), InsertPointsSubcell(R=4), GatherLevelSet(rho=2),
    UpdateApron(3.0); frame 2 is a full rebuild (mCurrDepth quirk), frames 3+ incremental.
    Both forms of the box passes (direction sets per home leaf, per-point walk)."""
    pos, vel = _mini_fluid()
    frames = []
    p = pos.copy()
    for f in range(4):
        p = (p + 0.5 * vel).astype(np.float32)
        frames.append(p.copy())
    _, o = H.run_oracle(None, frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0)
    _, g = H.run_gpu(None, frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0,
                     touch_dirs=touch_dirs)
    for k in range(len(frames)):
        _full_check(o[k], g[k], 3.0)


@pytest.mark.parametrize("unroll", [(1, 2), (2, 8), (4, 4)])
def test_binning_variants(gpu_lib, unroll):
    """every points-per-thread form of the binning passes (the tuning table's choices),
    on a point count that is not a multiple of four (the four-point forms' tail)"""
    pos, vel = _mini_fluid(n=40003, seed=71)
    frames = [(pos + 0.5 * (k + 1) * vel).astype(np.float32) for k in range(3)]
    _, o = H.run_oracle(None, frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0)
    _, g = H.run_gpu(None, frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0, unroll=unroll)
    for k in range(len(frames)):
        _full_check(o[k], g[k], 3.0)


@pytest.mark.parametrize("dense_min", [0, 2**31 - 1])
@pytest.mark.parametrize("mode,rho", [("levelset", 2.0), ("density", 1.0), ("density", 2.5)])
def test_gather_forms(gpu_lib, dense_min, mode, rho):
    """Both gather forms on every brick (the form is chosen per brick by point count):
    the dam (dense: unit-box pass, then the search for voxels left at >= 1) and the
    scattered particles around it, level set and density, cutoffs below and above 1."""
    pos, vel = _mini_fluid(n=40000, seed=21)
    p = np.maximum(pos + 1.5 * vel, 0.0).astype(np.float32)
    _, o = H.run_oracle(p, radius=4.0, R=4.0, rho=rho, mode=mode, boundval=0.0)
    _, g = H.run_gpu(p, radius=4.0, R=4.0, rho=rho, mode=mode, boundval=0.0, dense_min=dense_min)
    _full_check(o[0], g[0], 0.0)


@pytest.mark.parametrize("case", ["fluid_levelset", "shell_density_half", "surface_bf16", "accumulate"])
def test_fused_apron_matches_full_apron(gpu_lib, case):
    """The fused apron (each gather brick writes its boundary voxels into its
    neighbours' apron records; UpdateApron then only writes the faces of missing
    neighbours) leaves every padded brick bit-identical to the full UpdateApron
    pass, frame after frame (full, full, incremental rebuilds) and for 16-bit storage."""
    import gbvdb

    kw = {}
    if case == "fluid_levelset":
        pos, vel = _mini_fluid(n=40000, seed=31)
        frames = [(pos + 0.5 * k * vel).astype(np.float32) for k in range(1, 5)]
        kw = dict(frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0)
    elif case == "shell_density_half":
        kw = dict(points=datasets.shell(50_000, seed=32), radius=1.0, R=1.0, rho=1.0, mode="density",
                  boundval=0.5, dtype=gbvdb.T_HALF)
    elif case == "surface_bf16":
        kw = dict(points=datasets.sphere_surface(60_000, seed=33), radius=1.5, R=1.5, rho=1.5, mode="density",
                  boundval=0.0, dtype=gbvdb.T_BFLOAT16)
    else:
        pos, vel = _mini_fluid(n=20000, seed=34)
        frames = [np.maximum(f, 0.0).astype(np.float32)
                  for f in (pos, pos + 3.0 * vel, pos - 3.0 * vel)]
        kw = dict(frames=frames, radius=2.0, R=2.0, rho=1.5, accumulate=True)
    pts = kw.pop("points", None)
    _, a = H.run_gpu(pts, fused_apron=1, export_subcells=False, **kw)
    _, b = H.run_gpu(pts, fused_apron=0, export_subcells=False, **kw)
    assert len(a) == len(b)
    for sa, sb in zip(a, b):
        assert np.array_equal(sa["amap"], sb["amap"])
        assert sa["bricks"].dtype == sb["bricks"].dtype
        assert np.array_equal(sa["bricks"].view(np.uint8), sb["bricks"].view(np.uint8))
        H.check_apron_self(sa, kw["boundval"] if "boundval" in kw else 0.0)


def test_fused_apron_falls_back_when_the_grid_is_not_in_frame_state(gpu_lib):
    """When the grid is not in the state a frame of the path leaves (here: a second
    rebuild added leaves and UpdateAtlas was not called, so new leaves have no slot
    and slots no longer equal linked ranks), the gather's push check fails, nothing
    is pushed and UpdateApron copies every apron voxel: the atlas is bit-identical to
    the one the full apron pass leaves."""
    import torch

    import gbvdb

    pos, vel = _mini_fluid(n=30000, seed=51)
    f1 = np.maximum(pos, 0.0).astype(np.float32)
    f2 = np.maximum(pos + 3.0 * vel, 0.0).astype(np.float32)
    snaps = []
    for fused in (1, 0):
        g = gbvdb.Grid(0, (3, 3, 3, 4))
        g.set_tuning(gbvdb.TUNE_FUSED_APRON, fused)
        g.add_channel(0)
        for k, f in enumerate((f1, f1, f2)):
            n = g.set_points(torch.from_numpy(f).cuda())
            g.rebuild_topology(n, 2.0)
            if k < 2:
                g.update_atlas()
            _, ln = g.insert_points_subcell(4, n, 2.0)
            g.gather_levelset(4, n, 1.5, (0, 0, 0), ln)
            g.update_apron(0, 3.0)
        torch.cuda.synchronize()
        snaps.append((g.atlas_map(), g.atlas_bricks(0)))
    assert np.array_equal(snaps[0][0], snaps[1][0])
    assert np.array_equal(snaps[0][1].view(np.uint8), snaps[1][1].view(np.uint8))


def test_autotuned_threshold_gives_the_same_atlas(gpu_lib):
    """The dense-form threshold autotuner only changes which gather form a brick takes;
    both forms give the same bits, so frames with the autotuner (measuring its
    candidates, then keeping one) equal frames at each fixed threshold bit for bit."""
    import gbvdb

    pos, vel = _mini_fluid(n=40000, seed=61)
    frames = [(pos + 0.5 * k * vel).astype(np.float32) for k in range(1, 6)]
    kw = dict(frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0, export_subcells=False)
    _, auto = H.run_gpu(None, **kw)
    for dm in (2048, 4096):
        _, fixed = H.run_gpu(None, dense_min=dm, **kw)
        for a, b in zip(auto, fixed):
            assert np.array_equal(a["bricks"].view(np.uint8), b["bricks"].view(np.uint8))
            assert a["checksum"] == b["checksum"]


@pytest.mark.parametrize("dense_min", [None, 0])
def test_gather_launch_order_gives_the_same_atlas(gpu_lib, dense_min):
    """The gather's launch order (linked, or the bricks with many candidate points first,
    each group in an order that varies from run to run) changes no bit of the atlas,
    apron included: every brick writes its own slot and the apron voxels it alone
    sources.  dense_min 0 puts every brick in the gather form, so every brick is long."""
    pos, vel = _mini_fluid(n=40000, seed=67)
    frames = [(pos + 0.5 * k * vel).astype(np.float32) for k in range(1, 4)]
    kw = dict(frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0, export_subcells=False,
              dense_min=dense_min)
    _, linked = H.run_gpu(None, long_min=-1, **kw)
    for lm in (1, 200, 2048):
        _, other = H.run_gpu(None, long_min=lm, **kw)
        for a, b in zip(linked, other):
            # padded bricks: interiors and aprons
            assert np.array_equal(a["bricks"].view(np.uint8), b["bricks"].view(np.uint8))
            assert a["checksum"] == b["checksum"]


def test_accumulate_topology(gpu_lib):
    pos, vel = _mini_fluid(n=20000, seed=5)
    frames = [pos, (pos + 3.0 * vel).astype(np.float32), (pos - 3.0 * vel).astype(np.float32)]
    frames = [np.maximum(f, 0.0).astype(np.float32) for f in frames]
    _, o = H.run_oracle(None, frames=frames, radius=2.0, R=2.0, rho=1.5, accumulate=True)
    _, g = H.run_gpu(None, frames=frames, radius=2.0, R=2.0, rho=1.5, accumulate=True)
    for k in range(len(frames)):
        _full_check(o[k], g[k], 0.0)


@pytest.mark.parametrize("dtype,rtol", [("half", 1e-3), ("bf16", 8e-3)])
def test_reduced_precision_storage(gpu_lib, dtype, rtol):
    import gbvdb

    dt = gbvdb.T_HALF if dtype == "half" else gbvdb.T_BFLOAT16
    pts = datasets.shell(50_000, seed=7)
    _, o = H.run_oracle(pts, radius=1.5, R=1.5, rho=1.5)
    _, g = H.run_gpu(pts, radius=1.5, R=1.5, rho=1.5, dtype=dt)
    H.compare_topology(o[0], g[0])
    H.compare_subcells(o[0], g[0])
    err = H.compare_values(o[0], g[0], rtol, 1e-3, dtype=dt)
    assert err < 0.05


def test_surface_depth3(gpu_lib):
    """Sphere-surface points in a 4096^3 domain with grid (4,4,3,4): depth 3, default atlas."""
    pts = datasets.sphere_surface(40_000, seed=21, domain=4096.0, nspheres=6)
    pts = pts[np.all(pts >= 0, axis=1)]
    _, o = H.run_oracle(pts, log2dims=(4, 4, 3, 4), radius=1.5, R=1.5, rho=1.5)
    _, g = H.run_gpu(pts, log2dims=(4, 4, 3, 4), radius=1.5, R=1.5, rho=1.5)
    assert o[0]["depth"] == 3
    _full_check(o[0], g[0], 0.0)


def test_strided_input_and_translation(gpu_lib):
    """Positions read at pos + i*stride + off (DataPtr), with orig / trans offsets."""
    import torch

    import gbvdb

    pts = datasets.shell(30_000, seed=3)
    orig = (5.25, -3.5, 7.0)
    _, o = H.run_oracle(pts, radius=1.0, R=1.0, rho=1.0, orig=orig)
    # oracle insert/gather used trans = 0 on the raw points; run the same on the GPU
    wide = np.zeros((pts.shape[0], 5), dtype=np.float32)
    wide[:, :3] = pts
    wide[:, 3:] = 123.0
    d = torch.from_numpy(wide).cuda()
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0)
    n = g.set_points(d)
    g.rebuild_topology(n, 1.0, orig)
    g.update_atlas()
    st, ln = g.insert_points_subcell(4, n, 1.0)
    g.gather_density(4, n, 1.0, (0, 0, 0), ln)
    g.update_apron(0, 0.0)
    s = H.snapshot_gpu(g, ln)
    _full_check(o[0], s, 0.0)


def test_orphan_points_use_the_list_path(gpu_lib):
    """InsertPointsSubcell with points whose home brick is not in the topology: the
    reference still lists them in neighbouring subcells; the result must match."""
    import oracle
    import torch

    import gbvdb

    base = datasets.shell(20_000, seed=1)
    moved = (base + np.array([6.0, 0.0, 0.0], dtype=np.float32)).astype(np.float32)
    og = oracle.OracleGrid((3, 3, 3, 4))
    og.add_channel(0)
    assert og.rebuild_topology(base, 1.0) == 0
    og.update_atlas()
    rc, ln_o = og.insert_points_subcell(moved, 2.0)
    og.gather_density(2.0)
    og.update_apron(0, 0.0)
    o = H.snapshot_oracle(og, ln_o)

    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0)
    db = torch.from_numpy(base).cuda()
    dm = torch.from_numpy(moved).cuda()
    n = g.set_points(db)
    g.rebuild_topology(n, 1.0)
    g.update_atlas()
    g.set_points(dm)
    st, ln = g.insert_points_subcell(4, n, 2.0)
    g.gather_density(4, n, 2.0, (0, 0, 0), ln)
    g.update_apron(0, 0.0)
    s = H.snapshot_gpu(g, ln)
    _full_check(o, s, 0.0)


def test_edge_cases(gpu_lib):
    import torch

    import gbvdb

    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0)
    # empty input: nothing to do
    d = torch.zeros((0, 3), dtype=torch.float32, device="cuda")
    g.set_points(d)
    assert g.rebuild_topology(0, 1.0) == gbvdb.NOOP
    # all points in one brick: depth 0 is an error (VG.cpp:1187-1190)
    one = torch.tensor([[20.5, 20.5, 20.5]], dtype=torch.float32, device="cuda")
    n = g.set_points(one)
    with pytest.raises(gbvdb.GbvdbError) as e:
        g.rebuild_topology(n, 1.0)
    assert e.value.status == gbvdb.DEPTH_UNSUPPORTED
    # extents beyond the configured levels
    far = torch.tensor([[1.0, 1.0, 1.0], [60000.0, 1.0, 1.0]], dtype=torch.float32, device="cuda")
    n = g.set_points(far)
    with pytest.raises(gbvdb.GbvdbError) as e:
        g.rebuild_topology(n, 1.0)
    assert e.value.status == gbvdb.DEPTH_UNSUPPORTED
    # all points negative except bbox-defining ones: negative points make no keys
    pts = np.array([[-5.0, 10.0, 10.0], [30.5, 30.5, 30.5], [40.5, 40.5, 40.5], [-1.0, -1.0, -1.0]],
                   dtype=np.float32)
    _, o = H.run_oracle(pts, radius=1.0, R=1.0, rho=1.0)
    _, s = H.run_gpu(pts, radius=1.0, R=1.0, rho=1.0)
    _full_check(o[0], s[0], 0.0)
    # NOHIT points are skipped by InsertPointsSubcell but still bound the box (PT.cuh:282)
    # a single point per brick corner, ragged counts per brick
    rng = np.random.default_rng(9)
    ragged = np.concatenate([rng.uniform(0, 64, size=(500, 3)), rng.uniform(200, 203, size=(7, 3))]).astype(np.float32)
    _, o = H.run_oracle(ragged, radius=2.0, R=3.0, rho=2.5, mode="levelset", boundval=3.0)
    _, s = H.run_gpu(ragged, radius=2.0, R=3.0, rho=2.5, mode="levelset", boundval=3.0)
    _full_check(o[0], s[0], 3.0)


def test_insert_before_topology_is_noop(gpu_lib):
    import torch

    import gbvdb

    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0)
    d = torch.from_numpy(datasets.shell(1000, seed=2)).cuda()
    n = g.set_points(d)
    st, ln = g.insert_points_subcell(4, n, 1.0)
    assert st == gbvdb.NOOP and ln == -1


def _surface_crop():
    """The surface-fusion workload (16,777,216 points, seed 2, grid (4,4,3,4)) cropped to
    x, y in [1792, 2304) and z < 600: part of the z = 0 plane patch and the spheres there,
    across the x = y = 2048 level-2 node boundary (depth 3)."""
    pts = datasets.surface(16_777_216, seed=2)
    m = (pts[:, 0] >= 1792) & (pts[:, 0] < 2304) & (pts[:, 1] >= 1792) & (pts[:, 1] < 2304) & (pts[:, 2] < 600)
    return np.ascontiguousarray(pts[m])


@pytest.mark.parametrize("dtype,rtol,atol", [("f32", 1e-5, 1e-6), ("half", 1e-3, 1e-3), ("bf16", 8e-3, 8e-3)])
def test_surface_config_storage_types(gpu_lib, dtype, rtol, atol):
    """Density (rho = r = R = 1.5) of the surface workload stored as FP32, FP16 and BF16
    (FP32 accumulation in all three) against the FP64 oracle: topology and subcells
    exact, values within the storage type's tolerance (max errors printed)."""
    import gbvdb

    dt = {"f32": gbvdb.T_FLOAT, "half": gbvdb.T_HALF, "bf16": gbvdb.T_BFLOAT16}[dtype]
    pts = _surface_crop()
    assert pts.shape[0] > 100_000
    _, o = H.run_oracle(pts, log2dims=(4, 4, 3, 4), radius=1.5, R=1.5, rho=1.5)
    _, g = H.run_gpu(pts, log2dims=(4, 4, 3, 4), radius=1.5, R=1.5, rho=1.5, dtype=dt)
    assert o[0]["depth"] == 3
    H.compare_topology(o[0], g[0])
    H.compare_subcells(o[0], g[0])
    err = H.compare_values(o[0], g[0], rtol, atol, dtype=dt)
    print("surface crop %s: %d points, max abs error vs FP64 %.3g" % (dtype, pts.shape[0], err))


def test_fp16_subcells_levelset(gpu_lib):
    """InsertPointsSubcell_FP16 + GatherLevelSet_FP16 (the point-cloud sample's path): lists
    hold 16-bit-quantised positions over the point bounds; membership, lists, values and
    apron match the oracle's restatement, and quantisation changes some values."""
    pos, vel = _mini_fluid()
    frames = [(pos + 0.5 * (k + 1) * vel).astype(np.float32) for k in range(3)]
    kw = dict(frames=frames, radius=2.0, R=2.0, rho=1.0, mode="levelset", boundval=3.0)
    _, o = H.run_oracle(None, fp16_subcells=True, **kw)
    _, g = H.run_gpu(None, fp16_subcells=True, **kw)
    for k in range(3):
        _full_check(o[k], g[k], 3.0)
    _, g32 = H.run_gpu(None, **kw)
    assert not np.array_equal(g32[-1]["bricks"], g[-1]["bricks"])
    assert np.abs(g32[-1]["bricks"].astype(np.float64) - g[-1]["bricks"]).max() < 0.05


def test_apron_after_other_interior_writers(gpu_lib):
    """UpdateApron copies the interiors as they are now, whoever wrote them last: after a
    gather (whose fused apron already wrote the neighbours' boundary voxels), after
    FillChannel, and after the caller wrote the interior through gbvdb_get_atlas_device
    (which turns the fused apron off for the grid)."""
    import ctypes

    import torch

    import gbvdb

    pts = datasets.shell(30_000, seed=91)
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0, gbvdb.T_FLOAT)
    n = g.set_points(torch.from_numpy(pts).cuda())
    g.rebuild_topology(n, 1.0)
    g.update_atlas()
    _, ln = g.insert_points_subcell(4, n, 1.0)
    g.gather_density(4, n, 1.0, (0, 0, 0), ln)
    g.update_apron(0, 0.0)
    snap = {"bricks": g.atlas_bricks(0), "amap": g.atlas_map()}
    H.check_apron_self(snap, 0.0)
    g.fill_channel(0, 0.75)
    g.update_apron(0, 0.25)
    snap = {"bricks": g.atlas_bricks(0), "amap": g.atlas_map()}
    H.check_apron_self(snap, 0.25)
    assert np.all(snap["bricks"][:, 1:17, 1:17, 1:17] == 0.75)
    # the caller writes the interior of every slot: voxel value = slot + x / 16
    ip, ap = ctypes.c_void_p(), ctypes.c_void_p()
    assert g.L.gbvdb_get_atlas_device(g._h, 0, ctypes.byref(ip), ctypes.byref(ap)) == gbvdb.OK
    used = g.atlas_info(0)["used"]
    vals = (torch.arange(used, dtype=torch.float32, device="cuda")[:, None]
            + (torch.arange(4096, device="cuda") % 16).float()[None, :] / 16.0).contiguous()


    class _Dev:  # a zero-copy torch view of the channel's interior storage
        __cuda_array_interface__ = {"shape": (used, 4096), "typestr": "<f4", "data": (ip.value, False),
                                    "version": 3}

    interior = torch.as_tensor(_Dev(), device="cuda")
    torch.cuda.synchronize()
    interior.copy_(vals)
    torch.cuda.synchronize()
    g.gather_density(4, n, 1.0, (0, 0, 0), ln)  # overwritten by a gather, then written again below
    torch.cuda.synchronize()
    interior.copy_(vals)
    torch.cuda.synchronize()
    g.update_apron(0, -1.0)
    snap = {"bricks": g.atlas_bricks(0), "amap": g.atlas_map()}
    H.check_apron_self(snap, -1.0)
    assert np.array_equal(snap["bricks"][:, 1:17, 1:17, 1:17].reshape(used, -1), vals.cpu().numpy())


def test_checksum_device_matches_checksum(gpu_lib):
    import torch

    import gbvdb

    pts = datasets.shell(20_000, seed=93)
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0, gbvdb.T_FLOAT)
    n = g.set_points(torch.from_numpy(pts).cuda())
    g.rebuild_topology(n, 1.0)
    g.update_atlas()
    _, ln = g.insert_points_subcell(4, n, 1.0)
    g.gather_density(4, n, 1.0, (0, 0, 0), ln)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    g.checksum_device(out[1])
    torch.cuda.synchronize()
    assert out[1].item() == g.checksum(0) and out[0].item() == 0 and out[2].item() == 0


def test_checksum_overlap_is_ordered_before_the_next_gather(gpu_lib):
    """gbvdb_checksum_overlap runs on the grid's side stream while the next frame's
    topology and binning go on; the next gather waits for it, so each frame's overlapped
    sum equals that frame's gbvdb_checksum (taken on a second grid fed the same frames)"""
    import torch

    import gbvdb

    pos, vel = _mini_fluid(n=60000, seed=95)
    frames = [torch.from_numpy((pos + 0.5 * (k + 1) * vel).astype(np.float32)).cuda() for k in range(5)]
    stream = torch.cuda.Stream()
    g = gbvdb.Grid(0, (3, 3, 3, 4), stream=stream)
    ref = gbvdb.Grid(0, (3, 3, 3, 4))
    for x in (g, ref):
        x.add_channel(0)
    dev = torch.zeros(len(frames), dtype=torch.float64, device="cuda")
    host = torch.zeros(len(frames), dtype=torch.float64).pin_memory()
    expect = []
    with torch.cuda.stream(stream):
        for k, f in enumerate(frames):
            for x in (g, ref):
                n = x.set_points(f)
                x.rebuild_topology(n, 4.0)
                x.update_atlas()
                _, ln = x.insert_points_subcell(4, n, 4.0)
                x.gather_levelset(4, n, 2.0, (0, 0, 0), ln)
                x.update_apron(0, 3.0)
            g.checksum_overlap(dev[k], host[k])
            expect.append(ref.checksum(0))
        g.join()
    torch.cuda.synchronize()
    assert host.tolist() == expect
    assert dev.cpu().tolist() == expect


def test_incremental_frames_after_a_jump(gpu_lib):
    """Incremental frames run their key pass on the last pass's key domains, widened by a
    node, and read the frame's bounds back with the key counts; a frame whose keys leave
    those domains (here all points jump 40 voxels in x) is redone on its exact domains.
    Every frame against the oracle."""
    pos, vel = _mini_fluid(n=30000, seed=17)
    f1 = pos
    f2 = (pos + 0.5 * vel).astype(np.float32)
    f3 = (f2 + 0.5 * vel).astype(np.float32)
    f4 = (f3 + np.array([40.0, 0.0, 0.0], np.float32)).astype(np.float32)
    f5 = (f4 + 0.5 * vel).astype(np.float32)
    frames = [np.maximum(f, 0.0).astype(np.float32) for f in (f1, f2, f3, f4, f5)]
    _, o = H.run_oracle(None, frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0)
    _, g = H.run_gpu(None, frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0)
    for k in range(len(frames)):
        _full_check(o[k], g[k], 3.0)
