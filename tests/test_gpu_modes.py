"""GPU parity of the gather modes the reference's samples use beyond plain
frames, each against the CPU oracle on the same call sequence:

  accumulating gathers (bAccumulate): GatherLevelSet after FillChannel(0, 3)
    with AccumulateTopology (source/gPointFusion/main_point_fusion.cpp:576-590)
    and GatherDensity on a fixed topology (source/gSprayDeposit/main_spray_deposit.cpp:290-298);
  colour gathers into a T_UCHAR4 channel (the points' RGBA8 colours averaged per
    subcell, cuda_gvdb_particles.cuh:717-731, 757-771), with and without accumulation,
    through the binned form and the materialized-list form;
  FinishTopology(false, true) bounds (ComputeBounds, gvdb_volume_gvdb.cpp:1792-1816);
  FillChannel / ClearChannel.

Rules: topology and atlas map bit-exact; gathered values within 1e-5 relative /
1e-6 absolute of the FP64 oracle; colour bytes bit-exact against the oracle (both
sum the member bytes exactly and then take the same FP32 steps); apron voxels bit-
exact copies.  The inputs include the golden fixtures' inputs, whose outputs from
the reference's own kernels pin the oracle (tests/test_oracle_golden.py).
"""
import glob
import os

import numpy as np
import pytest

import datasets
from _helpers import check_apron_self, compare_topology, compare_values

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
UNDEF64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def colours_for(rng, n):
    c = rng.integers(0, 256, size=(n, 4), dtype=np.uint32)
    c[: n // 3, 3] = 255
    return (c[:, 0] | (c[:, 1] << 8) | (c[:, 2] << 16) | (c[:, 3] << 24)).astype(np.uint32)


def run_oracle_seq(case):
    import oracle

    g = oracle.OracleGrid(case["log2dims"])
    g.add_channel(0)
    colour = case.get("colours") is not None
    if colour:
        g.add_channel(1, dtype=2)  # frames whose colours are None gather no colour
    if case.get("fill") is not None:
        g.fill_channel(0, case["fill"])
    outs = []
    for k, pts in enumerate(case["frames"]):
        clr = case["colours"][k] if colour else None
        topo = case.get("topology", "rebuild")
        if topo == "accumulate":
            assert g.accumulate_topology(pts, case["radius"]) == 0
        elif topo == "rebuild" or k == 0:
            assert g.rebuild_topology(pts, case["radius"]) == 0
        bounds = g.compute_bounds()
        if topo != "fixed" or k == 0:
            g.update_atlas()
        _, ln = g.insert_points_subcell(pts, case["R"], colours=clr)
        cc = 1 if colour else -1
        if case["mode"] == "density":
            g.gather_density(case["rho"], accum=case.get("accum", False), clr_chan=cc)
        else:
            g.gather_levelset(case["rho"], accum=case.get("accum", False), clr_chan=cc)
        g.update_apron(0, case["boundval"])
        if colour:
            g.update_apron(1, 0.0)
        snap = {"len": ln, "depth": g.depth, "top": g.top_lev, "used": g.used_count(0),
                "nodes": [g.nodes(l) for l in range(g.levs)], "clist": [g.childlist(l) for l in range(g.levs)],
                "atlas_dims": g.atlas_dims(), "amap": g.atlas_map(), "bricks": g.atlas_bricks(0), "bounds": bounds}
        if colour:
            snap["colour"] = g.atlas_bricks(1).astype(np.uint32)
        outs.append(snap)
    return outs


def run_gpu_seq(case, dense_min=None, fused_apron=None):
    import torch

    import gbvdb

    g = gbvdb.Grid(0, case["log2dims"])
    if dense_min is not None:
        g.set_tuning(gbvdb.TUNE_DENSE_MIN, dense_min)
    if fused_apron is not None:
        g.set_tuning(gbvdb.TUNE_FUSED_APRON, fused_apron)
    g.add_channel(0)
    colour = case.get("colours") is not None
    if colour:
        g.add_channel(1, gbvdb.T_UCHAR4)
    if case.get("fill") is not None:
        g.fill_channel(0, case["fill"])
    outs = []
    for k, pts in enumerate(case["frames"]):
        d = torch.from_numpy(np.ascontiguousarray(pts, dtype=np.float32)).cuda()
        clr = case["colours"][k] if colour else None
        c = torch.from_numpy(clr.view(np.int32)).cuda() if clr is not None else None
        n = g.set_points(d, colours=c)
        topo = case.get("topology", "rebuild")
        if topo == "accumulate":
            g.accumulate_topology(n, case["radius"])
        elif topo == "rebuild" or k == 0:
            g.rebuild_topology(n, case["radius"])
        g.finish_topology(False, True)
        bounds = g.vol_bounds()
        if topo != "fixed" or k == 0:
            g.update_atlas()
        _, ln = g.insert_points_subcell(4, n, case["R"])
        cc = 1 if colour else -1
        if case["mode"] == "density":
            g.gather_density(4, n, case["rho"], (0, 0, 0), ln, 0, cc, case.get("accum", False))
        else:
            g.gather_levelset(4, n, case["rho"], (0, 0, 0), ln, 0, cc, case.get("accum", False))
        g.update_apron(0, case["boundval"])
        if colour:
            g.update_apron(1, 0.0)
        torch.cuda.synchronize()
        tot, used = g.node_counts()
        info = g.atlas_info(0)
        snap = {"len": ln, "used": used[0], "nodes": [g.nodes(l) for l in range(g.levs)],
                "clist": [g.childlist(l) for l in range(g.levs)],
                "atlas_dims": (info["ax"], info["ay"], info["az"], info["used"]), "amap": g.atlas_map(),
                "bricks": g.atlas_bricks(0), "dtype": info["dtype"], "bounds": bounds}
        snap["depth"], snap["top"] = g.depth()
        if colour:
            snap["colour"] = g.atlas_bricks(1)
        outs.append(snap)
    g.close()
    return outs


def compare_seq(oo, gg, boundval):
    for k, (o, g) in enumerate(zip(oo, gg)):
        compare_topology(o, g)
        assert o["len"] == g["len"], (k, o["len"], g["len"])
        compare_values(o, g)
        check_apron_self(g, np.float32(boundval))
        ob, gb = o["bounds"], g["bounds"]
        assert (ob is None) == (gb is None), k
        if ob is not None:
            assert np.array_equal(ob, gb), (k, ob, gb)
        if "colour" in o:
            oc, gc = o["colour"], g["colour"]
            assert oc.shape == gc.shape, (k, oc.shape, gc.shape)
            if not np.array_equal(oc, gc):
                bad = np.argwhere(oc != gc)
                i = tuple(bad[0])
                raise AssertionError("frame %d: %d colour voxels differ, first %s: oracle %08x gpu %08x"
                                     % (k, len(bad), i, int(oc[i]), int(gc[i])))
            check_apron_self({"amap": g["amap"], "bricks": gc}, np.uint32(0))


def golden_cases():
    out = []
    for p in sorted(glob.glob(os.path.join(HERE, "golden", "*.npz"))):
        if os.path.basename(p).startswith("op_"):  # operator fixtures (test_oracle_golden.py)
            continue
        fx = np.load(p)
        nf = int(fx["nframes"])
        case = {"name": os.path.basename(p), "log2dims": tuple(int(v) for v in fx["log2dims"]),
                "radius": float(fx["radius"]), "R": float(fx["R"]), "rho": float(fx["rho"]),
                "mode": str(fx["mode"]), "boundval": float(fx["boundval"]),
                "frames": [fx["f%d_points" % k] for k in range(nf)],
                "topology": str(fx["topology"]) if "topology" in fx.files else "rebuild",
                "accum": bool(fx["accum"]) if "accum" in fx.files else False,
                "fill": float(fx["fill"]) if "fill" in fx.files else None}
        if "colour" in fx.files and bool(fx["colour"]):
            # frames without colours in the fixture (its topology frame) gather no colour
            case["colours"] = [fx["f%d_colours" % k] if ("f%d_colours" % k) in fx.files else None
                               for k in range(nf)]
        out.append(case)
    return out


GOLDEN = golden_cases()


@pytest.mark.parametrize("case", [c for c in GOLDEN if "colours" not in c], ids=lambda c: c["name"])
def test_golden_inputs_match_oracle(gpu_lib, case):
    """the call sequences of the golden fixtures, GPU against the oracle"""
    compare_seq(run_oracle_seq(case), run_gpu_seq(case), case["boundval"])


def _fluid_frames(n, seed, shift, steps, scale):
    pos, vel = datasets.fluid(n=n, seed=seed, box=(48, 64, 48), domain=96)
    pos = pos + np.asarray(shift, dtype=np.float32)
    return [(pos + scale * (k + 1) * vel).astype(np.float32) for k in range(steps)]


@pytest.mark.parametrize("mode", ["density", "levelset"])
def test_accumulating_gathers(gpu_lib, mode):
    """FillChannel then AccumulateTopology + accumulating gathers over four frames: every
    frame reads the values the previous one left in the (re-assigned) atlas slots"""
    frames = _fluid_frames(60_000, 11, (100.0, 80.0, 60.0), 4, 2.0)
    case = {"log2dims": (3, 3, 3, 4), "radius": 2.0, "R": 2.0, "rho": 1.0 if mode == "density" else 1.5,
            "mode": mode, "boundval": 0.0 if mode == "density" else 3.0, "frames": frames,
            "topology": "accumulate", "accum": True, "fill": 0.25 if mode == "density" else 3.0}
    oo = run_oracle_seq(case)
    for dense_min in (None, 0):  # autotuned forms, then the dense form on every brick
        compare_seq(oo, run_gpu_seq(case, dense_min=dense_min), case["boundval"])


def test_accumulating_density_on_fixed_topology(gpu_lib):
    """gSprayDeposit's sequence: one topology, then batches of points gathered with
    accumulation (points off the topology take the materialized-list form)"""
    rng = np.random.default_rng(21)
    base = datasets.shell(40_000, seed=21, center=(300.0, 300.0, 300.0), rmin=60.0, rmax=70.0)
    frames = [base]
    for _ in range(3):
        sub = base[rng.choice(base.shape[0], 9000, replace=False)]
        frames.append((sub + rng.normal(0.0, 0.5, size=sub.shape)).astype(np.float32))
    case = {"log2dims": (3, 3, 3, 4), "radius": 1.0, "R": 1.0, "rho": 1.0, "mode": "density", "boundval": 0.0,
            "frames": frames, "topology": "fixed", "accum": True}
    compare_seq(run_oracle_seq(case), run_gpu_seq(case), 0.0)


@pytest.mark.parametrize("accum", [False, True])
@pytest.mark.parametrize("mode", ["density", "levelset"])
def test_colour_gathers(gpu_lib, mode, accum):
    """colour averages into a T_UCHAR4 channel, full then incremental frames (level set
    as gFluidSurface with m_use_color; density with accumulation as gSprayDeposit)"""
    rng = np.random.default_rng(31)
    frames = _fluid_frames(50_000, 12, (60.0, 70.0, 80.0), 3, 0.5)
    case = {"log2dims": (3, 3, 3, 4), "radius": 4.0 if mode == "levelset" else 1.0,
            "R": 4.0 if mode == "levelset" else 1.0, "rho": 2.0 if mode == "levelset" else 1.0, "mode": mode,
            "boundval": 3.0 if mode == "levelset" else 0.0, "frames": frames, "accum": accum,
            "colours": [colours_for(rng, f.shape[0]) for f in frames]}
    oo = run_oracle_seq(case)
    for dense_min in (None, 0):
        compare_seq(oo, run_gpu_seq(case, dense_min=dense_min), case["boundval"])


def test_colour_gathers_list_form(gpu_lib):
    """points whose home brick is not linked force the materialized-list gather; colours
    follow the same lists"""
    rng = np.random.default_rng(41)
    base = datasets.shell(30_000, seed=41, center=(200.0, 200.0, 200.0), rmin=50.0, rmax=58.0)
    moved = (base + rng.normal(0.0, 1.5, size=base.shape)).astype(np.float32)
    case = {"log2dims": (3, 3, 3, 4), "radius": 1.0, "R": 1.0, "rho": 1.0, "mode": "density", "boundval": 0.0,
            "frames": [base, moved], "topology": "fixed", "accum": False,
            "colours": [colours_for(rng, base.shape[0]), colours_for(rng, moved.shape[0])]}
    compare_seq(run_oracle_seq(case), run_gpu_seq(case), 0.0)


@pytest.mark.parametrize("case", [c for c in GOLDEN if "colours" in c], ids=lambda c: c["name"])
def test_golden_colour_inputs_match_oracle(gpu_lib, case):
    """the golden colour cases, GPU against the oracle"""
    compare_seq(run_oracle_seq(case), run_gpu_seq(case), case["boundval"])


def test_fill_and_clear_channel(gpu_lib):
    import torch

    import gbvdb
    import oracle

    pts = datasets.shell(20_000, seed=5)
    og = oracle.OracleGrid((3, 3, 3, 4))
    og.add_channel(0)
    og.add_channel(1, dtype=2)
    og.rebuild_topology(pts, 1.0)
    og.update_atlas()
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0)
    g.add_channel(1, gbvdb.T_UCHAR4)
    n = g.set_points(torch.from_numpy(pts).cuda())
    g.rebuild_topology(n, 1.0)
    g.update_atlas()
    for v in ((0.7, 0.2, 0.9, 0.0), (0.0, 0.0, 0.0, 0.0)):
        og.fill_channel(0, v)
        og.fill_channel(1, v)
        g.fill_channel(0, v)
        g.fill_channel(1, v)
        torch.cuda.synchronize()
        assert np.array_equal(g.atlas_bricks(0).astype(np.float64), og.atlas_bricks(0))
        assert np.array_equal(g.atlas_bricks(1), og.atlas_bricks(1).astype(np.uint32))
    g.fill_channel(0, 5.0)
    g.clear_channel(0)
    og.clear_channel(0)
    torch.cuda.synchronize()
    assert not g.atlas_bricks(0).any() and not og.atlas_bricks(0).any()


def test_finish_topology_bounds_with_inactive_leaf0(gpu_lib):
    """ComputeBounds starts from leaf 0 even when an incremental frame deactivated it"""
    import torch

    import gbvdb
    import oracle

    a = datasets.shell(20_000, seed=6, center=(300.0, 300.0, 300.0), rmin=15.0, rmax=20.0)
    # the cloud moves along x inside the same level-1 node (no depth change): the third call
    # is incremental and delinks the lowest leaves, leaf 0 among them
    b = (a + np.array([40.0, 0.0, 0.0], dtype=np.float32)).astype(np.float32)
    og = oracle.OracleGrid((3, 3, 3, 4))
    og.add_channel(0)
    g = gbvdb.Grid(0, (3, 3, 3, 4))
    g.add_channel(0)
    seen_inactive = False
    for pts in (a, a, b):
        og.rebuild_topology(pts, 1.0)
        n = g.set_points(torch.from_numpy(pts).cuda())
        g.rebuild_topology(n, 1.0)
        g.finish_topology(False, True)
        assert np.array_equal(og.compute_bounds(), g.vol_bounds())
        seen_inactive |= og.nodes(0)["flags"][0] == 0
    assert seen_inactive
