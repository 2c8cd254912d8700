"""The CPU oracle against golden fixtures produced by the reference's own CUDA
kernels (tests/golden/make_golden.py: PTX compiled from the reference's
kernels/cuda_gvdb_module.cu, run under a restatement of its host code).

Pinned bit-exactly: node pools (lev, flags, pos, value, parent, childlist),
child lists, top level, used leaf count, atlas dimensions and map, subcell list
lengths and per-subcell membership hashes.  Gathered values: every voxel of
every padded brick (interior and apron) within 1e-5 relative / 1e-6 absolute
(the reference computes sqrtf under --use_fast_math).  Colours (T_UCHAR4): every
byte within 1 of the reference's, which adds its FP32 terms c/255 in the
arbitrary order of its atomically filled lists.

Call sequences: RebuildTopology frames (full, then incremental);
AccumulateTopology with accumulating gathers after FillChannel; a fixed
topology with accumulating, coloured density gathers; coloured level sets.

Operator fixtures (op_*.npz), each on one full rebuild: UpdateApronFaces from the
reference's own gathered bricks (faces bit-exact); one Compute(FUNC_SMOOTH) pass
on a field whose block-face voxels stay zero (so the reference's unordered
blocks give one answer), within 1e-6 absolute / 1e-5 relative; the FP16 subcell
pair (list lengths exact; values within the tolerance plus one 16-bit
quantisation step, since the reference quantises with approximate division);
legacy InsertPoints + ScatterDensity on points whose splats never share a voxel
(the reference kernel's updates are unsynchronised), within 1e-5 relative.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from golden.make_golden import membership_hash

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                  if not os.path.basename(p).startswith("op_"))
OP_FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "op_*.npz")))


def run_oracle(fx):
    g = oracle.OracleGrid(tuple(int(v) for v in fx["log2dims"]))
    g.add_channel(0)
    mode = str(fx["mode"])
    topo = str(fx["topology"]) if "topology" in fx.files else "rebuild"
    accum = bool(fx["accum"]) if "accum" in fx.files else False
    colour = bool(fx["colour"]) if "colour" in fx.files else False
    if colour:
        g.add_channel(1, dtype=2)
    if "fill" in fx.files:
        g.fill_channel(0, float(fx["fill"]))
    for k in range(int(fx["nframes"])):
        pts = fx["f%d_points" % k]
        clr = fx["f%d_colours" % k] if ("f%d_colours" % k) in fx.files else None
        if topo == "accumulate":
            assert g.accumulate_topology(pts, float(fx["radius"])) == 0
        elif topo == "rebuild" or k == 0:
            assert g.rebuild_topology(pts, float(fx["radius"])) == 0
        if topo != "fixed" or k == 0:
            g.update_atlas()
        rc, ln = g.insert_points_subcell(pts, float(fx["R"]), colours=clr)
        cc = 1 if colour else -1
        if mode == "density":
            g.gather_density(float(fx["rho"]), accum=accum, clr_chan=cc)
        else:
            g.gather_levelset(float(fx["rho"]), accum=accum, clr_chan=cc)
        g.update_apron(0, float(fx["boundval"]))
        if colour:
            g.update_apron(1, 0.0)
        yield k, g, ln


def rgba_bytes(u32):
    return np.asarray(u32, dtype=np.uint32).view(np.uint8).astype(np.int16)


@pytest.mark.skipif(not FIXTURES, reason="no golden fixtures")
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_matches_reference_kernels(path):
    fx = np.load(path)
    for k, g, ln in run_oracle(fx):
        p = "f%d_" % k
        assert g.top_lev == int(fx[p + "top_lev"])
        assert g.used_count(0) == int(fx[p + "used"])
        for lev in range(g.levs):
            n = g.nodes(lev)
            for f in ("lev", "flags", "pos", "value", "parent", "childlist"):
                assert np.array_equal(n[f], fx[p + "L%d_%s" % (lev, f)]), (k, lev, f)
            if lev > 0:
                assert np.array_equal(g.childlist(lev), fx[p + "L%d_clist" % lev]), (k, lev)
        assert tuple(g.atlas_dims()) == tuple(int(v) for v in fx[p + "atlas_dims"])
        assert np.array_equal(g.atlas_map().view(np.int32), fx[p + "amap"])
        assert ln == int(fx[p + "len"])
        off, pts = g.subcells()
        cnt = np.diff(off)
        ref_cnt = fx[p + "sc_cnt"]
        assert np.array_equal(cnt, ref_cnt[:len(cnt)]) and not ref_cnt[len(cnt):].any()
        h = membership_hash(off[:-1], cnt, pts)
        assert np.array_equal(h, fx[p + "sc_hash"][:len(h)])
        ref_b = fx[p + "bricks"].astype(np.float64)
        mine = g.atlas_bricks(0)
        assert mine.shape == ref_b.shape, k
        err = np.abs(mine - ref_b)
        assert np.all(err <= 1e-6 + 1e-5 * np.abs(ref_b)), (k, float(err.max()))
        if (p + "colour") in fx.files:
            ref_c = rgba_bytes(fx[p + "colour"])
            mine_c = rgba_bytes(g.atlas_bricks(1).astype(np.uint32))
            d = np.abs(mine_c - ref_c)
            assert d.max() <= 1, (k, int(d.max()), int((d > 0).sum()))


def topology_matches(g, fx):
    assert g.top_lev == int(fx["top_lev"])
    assert g.used_count(0) == int(fx["used"])
    for lev in range(g.levs):
        n = g.nodes(lev)
        for f in ("lev", "flags", "pos", "value", "parent", "childlist"):
            assert np.array_equal(n[f], fx["L%d_%s" % (lev, f)]), (lev, f)
        if lev > 0:
            assert np.array_equal(g.childlist(lev), fx["L%d_clist" % lev]), lev
    assert tuple(g.atlas_dims()) == tuple(int(v) for v in fx["atlas_dims"])
    assert np.array_equal(g.atlas_map().view(np.int32), fx["amap"])


@pytest.mark.skipif(not OP_FIXTURES, reason="no operator fixtures")
@pytest.mark.parametrize("path", OP_FIXTURES, ids=[os.path.basename(p) for p in OP_FIXTURES])
def test_oracle_matches_reference_operators(path):
    fx = np.load(path)
    kind = str(fx["kind"])
    pts = fx["points"]
    g = oracle.OracleGrid(tuple(int(v) for v in fx["log2dims"]))
    g.add_channel(0)
    assert g.rebuild_topology(pts, float(fx["radius"])) == 0
    g.update_atlas()
    topology_matches(g, fx)
    if kind == "faces_smooth":
        b = np.ascontiguousarray(fx["gathered"], dtype=np.float32).copy()
        g.apron_faces_f32(b, g.neighbors())
        assert np.array_equal(b, fx["faces"])
        p1, p2 = (float(v) for v in fx["smooth_params"])
        b = np.ascontiguousarray(fx["smooth_in"], dtype=np.float32).copy()
        g.smooth_f32(b, p1, p2)
        ref = fx["smooth_out"].astype(np.float64)
        inner = (slice(None), slice(1, 17), slice(1, 17), slice(1, 17))
        err = np.abs(b[inner].astype(np.float64) - ref[inner])
        assert np.all(err <= 1e-6 + 1e-5 * np.abs(ref[inner])), float(err.max())
    elif kind == "fp16":
        rc, ln = g.insert_points_subcell_fp16(pts, float(fx["R"]))
        assert ln == int(fx["len"])
        off, _ = g.subcells()
        cnt = np.diff(off)
        ref_cnt = fx["sc_cnt"]
        assert np.array_equal(cnt, ref_cnt[:len(cnt)]) and not ref_cnt[len(cnt):].any()
        g.gather_levelset(float(fx["rho"]))
        g.update_apron(0, 3.0)
        b, ref = g.atlas_bricks(0), fx["bricks"].astype(np.float64)
        lo, hi = pts.min(axis=0) - 1.0, pts.max(axis=0) + 2.0
        step = float(np.sqrt(3.0) * np.max(hi - np.maximum(lo, 0.0)) / 65535.0) * 1.01
        err = np.abs(b - ref)
        assert np.all(err <= 1e-6 + 1e-5 * np.abs(ref) + step), float(err.max())
    else:
        g.insert_points(pts)
        g.scatter_density(pts, float(fx["sradius"]), expand=True)
        b, ref = g.atlas_bricks(0), fx["bricks"].astype(np.float64)
        err = np.abs(b - ref)
        assert np.all(err <= 1e-6 + 1e-5 * np.abs(ref)), float(err.max())
