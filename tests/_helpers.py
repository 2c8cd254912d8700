"""Shared test helpers: run the oracle and the CUDA path on the same seeded
inputs and compare their results under the parity rules:

  topology     node pools (every field), child lists and atlas map: bit-exact
  subcells     per-subcell point multisets: exact
  gather       interior voxels within 1e-5 relative + 1e-6 absolute of FP64
  apron        apron voxels copy the neighbour's interior bit-exactly (GPU
               self-consistency) and match the oracle within the same tolerance
"""
import numpy as np

RTOL = 1e-5
ATOL = 1e-6


def run_oracle(points, log2dims=(3, 3, 3, 4), frames=None, radius=1.0, R=1.0, rho=1.0, mode="density",
               boundval=0.0, orig=(0, 0, 0), axiscnt=(0, 0, 0), accumulate=False, threads=0, fp16_subcells=False):
    import oracle

    g = oracle.OracleGrid(log2dims, threads=threads)
    g.add_channel(0, 3, 1, axiscnt)
    seq = frames if frames is not None else [points]
    outs = []
    for pts in seq:
        if accumulate and outs:
            rc = g.accumulate_topology(pts, radius, orig)
        else:
            rc = g.rebuild_topology(pts, radius, orig)
        assert rc == 0, rc
        g.update_atlas()
        rc, ln = (g.insert_points_subcell_fp16 if fp16_subcells else g.insert_points_subcell)(pts, R)
        if mode == "density":
            g.gather_density(rho)
        else:
            g.gather_levelset(rho)
        g.update_apron(0, boundval)
        outs.append(snapshot_oracle(g, ln))
    return g, outs


def snapshot_oracle(g, ln):
    levs = g.levs
    snap = {"len": ln, "depth": g.depth, "top": g.top_lev}
    snap["nodes"] = [g.nodes(l) for l in range(levs)]
    snap["clist"] = [g.childlist(l) for l in range(levs)]
    snap["used"] = g.used_count(0)
    snap["atlas_dims"] = g.atlas_dims()
    snap["amap"] = g.atlas_map()
    snap["bricks"] = g.atlas_bricks(0)
    off, pts = g.subcells()
    snap["sc_off"], snap["sc_pts"] = off, pts
    snap["checksum"] = g.checksum(0)
    return snap


def run_gpu(points, log2dims=(3, 3, 3, 4), frames=None, radius=1.0, R=1.0, rho=1.0, mode="density",
            boundval=0.0, orig=(0, 0, 0), axiscnt=(0, 0, 0), dtype=None, accumulate=False, export_subcells=True,
            fp16_subcells=False, dense_min=None, fused_apron=None, touch_dirs=None, unroll=None, keyset=None,
            long_min=None):
    import torch

    import gbvdb

    dtype = gbvdb.T_FLOAT if dtype is None else dtype
    g = gbvdb.Grid(0, log2dims)
    if dense_min is not None:  # force one gather form: 0 = gather form everywhere, 2**31-1 = scatter form
        g.set_tuning(gbvdb.TUNE_DENSE_MIN, dense_min)
    if fused_apron is not None:  # 0: every UpdateApron copies all apron voxels
        g.set_tuning(gbvdb.TUNE_FUSED_APRON, fused_apron)
    if touch_dirs is not None:  # 0: the box passes walk every point's box positions
        g.set_tuning(gbvdb.TUNE_TOUCH_DIRS, touch_dirs)
    if keyset is not None:  # 2: RebuildTopology's key sets as hash tables (the sparse form)
        g.set_tuning(gbvdb.TUNE_KEYSET, keyset)
    if long_min is not None:  # the gather's launch order: -1 linked, k: bricks over k candidates first
        g.set_tuning(gbvdb.TUNE_GATHER_LONG_MIN, long_min)
    if unroll is not None:  # (points per thread of the count pass, of the scatter pass)
        g.set_tuning(gbvdb.TUNE_BIN_UNROLL, unroll[0])
        g.set_tuning(gbvdb.TUNE_SCATTER_UNROLL, unroll[1])
    g.add_channel(0, dtype, 1, axiscnt)
    seq = frames if frames is not None else [points]
    outs = []
    for k, pts in enumerate(seq):
        d = torch.from_numpy(np.ascontiguousarray(pts, dtype=np.float32)).cuda()
        n = g.set_points(d)
        if accumulate and k > 0:
            g.accumulate_topology(n, radius, orig)
        else:
            g.rebuild_topology(n, radius, orig)
        g.update_atlas()
        st, ln = (g.insert_points_subcell_fp16 if fp16_subcells else g.insert_points_subcell)(4, n, R)
        if mode == "density":
            g.gather_density(4, n, rho, (0, 0, 0), ln)
        elif fp16_subcells:
            g.gather_levelset_fp16(4, n, rho, (0, 0, 0), ln)
        else:
            g.gather_levelset(4, n, rho, (0, 0, 0), ln)
        g.update_apron(0, boundval)
        outs.append(snapshot_gpu(g, ln, export_subcells))
        torch.cuda.synchronize()
    return g, outs


def snapshot_gpu(g, ln, export_subcells=True):
    tot, used = g.node_counts()
    snap = {"len": ln}
    snap["depth"], snap["top"] = g.depth()
    snap["nodes"] = [g.nodes(l) for l in range(g.levs)]
    snap["clist"] = [g.childlist(l) for l in range(g.levs)]
    snap["used"] = used[0]
    info = g.atlas_info(0)
    snap["atlas_dims"] = (info["ax"], info["ay"], info["az"], info["used"])
    snap["amap"] = g.atlas_map()
    snap["bricks"] = g.atlas_bricks(0)
    snap["dtype"] = info["dtype"]
    if export_subcells and ln >= 0:
        nsub = 64 * int((snap["nodes"][0]["parent"] != np.uint64(0xFFFFFFFFFFFFFFFF)).sum())
        snap["sc_off"], snap["sc_pts"] = g.subcells(ln, nsub)
    snap["checksum"] = g.checksum(0)
    return snap


def compare_topology(o, g):
    assert o["depth"] == g["depth"], (o["depth"], g["depth"])
    assert o["top"] == g["top"], (o["top"], g["top"])
    assert len(o["nodes"]) == len(g["nodes"])
    for lev, (a, b) in enumerate(zip(o["nodes"], g["nodes"])):
        assert a.shape == b.shape, "level %d node count %d vs %d" % (lev, a.shape[0], b.shape[0])
        for f in ("lev", "flags", "pos", "value", "parent", "childlist"):
            if not np.array_equal(a[f], b[f]):
                bad = np.nonzero(np.any((a[f] != b[f]).reshape(a.shape[0], -1), axis=1))[0]
                raise AssertionError("level %d field %s differs at %d nodes, first %s: %s vs %s"
                                     % (lev, f, bad.size, bad[:5], a[bad[0]], b[bad[0]]))
    for lev, (a, b) in enumerate(zip(o["clist"], g["clist"])):
        if lev == 0:
            continue
        assert np.array_equal(a, b), "child list of level %d differs" % lev
    assert o["used"] == g["used"], (o["used"], g["used"])
    assert tuple(o["atlas_dims"]) == tuple(g["atlas_dims"]), (o["atlas_dims"], g["atlas_dims"])
    assert np.array_equal(o["amap"], g["amap"]), "atlas map differs"


def compare_subcells(o, g):
    assert o["len"] == g["len"], ("subcell list length", o["len"], g["len"])
    oo, op = o["sc_off"], o["sc_pts"]
    go, gp = g["sc_off"], g["sc_pts"]
    assert np.array_equal(oo, go), "subcell counts differ"
    # same multiset per subcell: sort each list by (x, y, z)
    seg = np.repeat(np.arange(len(oo) - 1), np.diff(oo))
    for pts, name in ((op, "o"), (gp, "g")):
        pass
    ko = np.lexsort((op[:, 2], op[:, 1], op[:, 0], seg))
    kg = np.lexsort((gp[:, 2], gp[:, 1], gp[:, 0], seg))
    assert np.array_equal(op[ko], gp[kg]), "subcell membership differs"


def to_f32(bricks, dtype):
    import gbvdb

    if dtype == gbvdb.T_BFLOAT16:
        return gbvdb.bf16_to_f32(bricks)
    return bricks.astype(np.float32)


def interior(b):
    return b[:, 1:17, 1:17, 1:17]


def apron_mask():
    m = np.ones((18, 18, 18), dtype=bool)
    m[1:17, 1:17, 1:17] = False
    return m


def compare_values(o, g, rtol=RTOL, atol=ATOL, dtype=None):
    ob = o["bricks"]
    gb = to_f32(g["bricks"], g.get("dtype", 3) if dtype is None else dtype).astype(np.float64)
    assert ob.shape == gb.shape, (ob.shape, gb.shape)
    err = np.abs(gb - ob)
    lim = atol + rtol * np.abs(ob)
    bad = err > lim
    if bad.any():
        idx = np.argwhere(bad)[0]
        raise AssertionError("%d voxels outside tolerance; first %s: gpu %r oracle %r (max err %g)"
                             % (bad.sum(), idx, gb[tuple(idx)], ob[tuple(idx)], err.max()))
    return float(err.max())


def _key(p):
    p = np.asarray(p, dtype=np.int64)
    return ((p[..., 0] + (1 << 20)) << 42) | ((p[..., 1] + (1 << 20)) << 21) | (p[..., 2] + (1 << 20))


def check_apron_self(g, boundval):
    """every GPU apron voxel equals the interior voxel of the neighbouring brick at the same
    index-space position (bit-exact), or boundval where no active brick exists"""
    amap = g["amap"]
    b = g["bricks"]
    used = b.shape[0]
    if used == 0:
        return
    pos = amap["pos"][:used].astype(np.int64)
    keys = _key(pos)
    order = np.argsort(keys)
    skeys = keys[order]
    zz, yy, xx = np.nonzero(apron_mask())
    raw = b.reshape(used, -1).view(np.uint8).reshape(used, 5832, -1)
    bv = np.asarray(boundval, dtype=b.dtype).tobytes()
    for z, y, x in zip(zz, yy, xx):
        w = pos + np.array([x - 1, y - 1, z - 1])
        nb = (w // 16) * 16
        k = _key(nb)
        i = np.searchsorted(skeys, k)
        i = np.minimum(i, used - 1)
        hit = skeys[i] == k
        ns = order[i]
        l = w - nb
        got = raw[:, (z * 18 + y) * 18 + x]
        exp_idx = ((l[:, 2] + 1) * 18 + (l[:, 1] + 1)) * 18 + (l[:, 0] + 1)
        exp = raw[ns, exp_idx]
        exp = np.where(hit[:, None], exp, np.frombuffer(bv, dtype=np.uint8)[None, :])
        if not np.array_equal(got, exp):
            s_bad = int(np.nonzero(np.any(got != exp, axis=1))[0][0])
            raise AssertionError("apron slot %d voxel %s differs (neighbour present: %s)"
                                 % (s_bad, (x, y, z), bool(hit[s_bad])))
