"""The CPU oracle against golden fixtures produced by the reference's own CUDA
kernels (tests/golden/make_golden.py: PTX compiled from the reference's
kernels/cuda_gvdb_module.cu, run under a restatement of its host code).

Pinned bit-exactly: node pools (lev, flags, pos, value, parent, childlist),
child lists, top level, used leaf count, atlas dimensions and map, subcell list
lengths and per-subcell membership hashes.  Gathered values: per-slot sums of
the interior and apron voxels and four full bricks within 1e-5 relative /
1e-6 absolute per voxel (the reference computes sqrtf under --use_fast_math).
"""
import glob
import os

import numpy as np
import pytest

import oracle
from golden.make_golden import membership_hash

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def run_oracle(fx):
    g = oracle.OracleGrid(tuple(int(v) for v in fx["log2dims"]))
    g.add_channel(0)
    mode = str(fx["mode"])
    for k in range(int(fx["nframes"])):
        pts = fx["f%d_points" % k]
        assert g.rebuild_topology(pts, float(fx["radius"])) == 0
        g.update_atlas()
        rc, ln = g.insert_points_subcell(pts, float(fx["R"]))
        if mode == "density":
            g.gather_density(float(fx["rho"]))
        else:
            g.gather_levelset(float(fx["rho"]))
        g.update_apron(0, float(fx["boundval"]))
        yield k, g, ln


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
        b = g.atlas_bricks(0)
        inner = b[:, 1:17, 1:17, 1:17].reshape(b.shape[0], -1)
        m = np.ones((18, 18, 18), bool)
        m[1:17, 1:17, 1:17] = False
        lim = 1e-6 * 4096 + 1e-5 * np.abs(inner).sum(axis=1)
        assert np.all(np.abs(inner.sum(axis=1) - fx[p + "slot_sum"]) <= lim), k
        alim = 1e-6 * 1736 + 1e-5 * np.abs(b[:, m]).sum(axis=1)
        assert np.all(np.abs(b[:, m].sum(axis=1) - fx[p + "apron_sum"]) <= alim), k
        ref_b = fx[p + "bricks"].astype(np.float64)
        mine = b[:ref_b.shape[0]]
        assert np.all(np.abs(mine - ref_b) <= 1e-6 + 1e-5 * np.abs(ref_b)), k
