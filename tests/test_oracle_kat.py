"""Known-answer tests of the CPU oracle, hand-computed from the reference's
kernel and host code (no GPU).  Each case cites the rule it pins:

  key per level, covering node       PT.cuh:352-382 (gvdbCalcBrickId), PT.cuh:74-100
  extra-brick box [int(p)-r, int(p)+2r]            PT.cuh:467-512
  incremental box [int(p)-r, int(p)+r], markers    PT.cuh:420-465
  early return keeps stale leaf flags              VG.cpp:1066
  second call is a full rebuild (mCurrDepth = -1)  VG.cpp:1195-1205, 2356
  link slot b = (z*r+y)*r+x, mParent = Elem(0,L+1,p)  ND.cuh:470-505
  top_lev = lowest level with one node             VG.cpp:3957-3968
  subcell range int(w-R)/4*4 .. int(w+1+R)/4*4     PT.cuh:286-291
  density max(0, rho-d), level set min(3, d-rho)   PT.cuh:696-773
  apron = neighbour interior or boundval           OP.cuh:72-131
"""
import numpy as np
import pytest

import oracle

UNDEF64 = np.uint64(0xFFFFFFFFFFFFFFFF)
A = (30.5, 30.5, 30.5)
B = (40.5, 40.5, 40.5)


def grid(points, radius=1.0, log2dims=(3, 3, 3, 4)):
    g = oracle.OracleGrid(log2dims)
    g.add_channel(0)
    rc = g.rebuild_topology(np.array(points, dtype=np.float32), radius)
    return g, rc


def leaf_positions(g):
    return [tuple(int(v) for v in p) for p in g.nodes(0)["pos"]]


def test_depth_too_small_is_an_error():
    g, rc = grid([(20.5, 20.5, 20.5)])
    assert rc == oracle.DEPTH_UNSUPPORTED
    assert g.node_count(0) == 0


def test_pass1_keys_and_links():
    g, rc = grid([(20.5, 20.5, 20.5), (40.5, 40.5, 40.5)], radius=0.0)
    assert rc == 0
    assert g.depth == 1 and g.top_lev == 1
    assert leaf_positions(g) == [(16, 16, 16), (32, 32, 32)]
    root = g.nodes(1)
    assert root.shape[0] == 1 and tuple(root["pos"][0]) == (0, 0, 0)
    assert root["childlist"][0] == (1 | (1 << 8))  # Elem(1, 1, 0)
    cl = g.childlist(1)[0]
    b0 = (1 * 8 + 1) * 8 + 1
    b1 = (2 * 8 + 2) * 8 + 2
    assert cl[b0] == 0 and cl[b1] == (1 << 16)
    assert np.count_nonzero(cl != UNDEF64) == 2
    n0 = g.nodes(0)
    assert list(n0["parent"]) == [256, 256]  # Elem(0, 1, 0)
    assert list(n0["childlist"]) == [0xFFFFFFFF, 0xFFFFFFFF]  # ID_UNDEFL
    assert all(tuple(v) == (-1, -1, -1) for v in n0["value"])


def test_extra_bricks_box_and_append_order():
    g, rc = grid([A, B], radius=1.0)
    assert rc == 0
    assert leaf_positions(g) == [(16, 16, 16), (32, 32, 32),
                                 (16, 16, 32), (16, 32, 16), (16, 32, 32),
                                 (32, 16, 16), (32, 16, 32), (32, 32, 16)]
    assert g.used_count(0) == 8


def test_negative_points_are_dropped():
    g, rc = grid([A, B, (-1.0, 35.0, 35.0)], radius=1.0)
    assert rc == 0
    assert g.node_count(0) == 8
    assert tuple(g.bbox()[:3]) == (0.0, 29.5, 29.5)


def test_subcell_membership_and_length():
    g, rc = grid([A, B], radius=1.0)
    g.update_atlas()
    rc, ln = g.insert_points_subcell(np.array([A, B], dtype=np.float32), 1.0)
    assert rc == 0 and ln == 16
    off, pts = g.subcells()
    nodes = g.nodes(0)
    lists = {}
    for i, nd in enumerate(nodes):
        for s in range(64):
            k = i * 64 + s
            if off[k + 1] > off[k]:
                org = nd["pos"] + 4 * np.array([s % 4, (s // 4) % 4, s // 16])
                lists[tuple(int(v) for v in org)] = pts[off[k]:off[k + 1]].tolist()
    expect = {}
    for p, lo, hi in ((A, 28, 32), (B, 36, 40)):
        for x in (lo, hi):
            for y in (lo, hi):
                for z in (lo, hi):
                    expect.setdefault((x, y, z), []).append(list(p))
    assert lists == expect


def test_gather_density_and_levelset_values():
    pts = np.array([A, B], dtype=np.float32)
    for mode in ("density", "levelset"):
        g, rc = grid(pts, radius=1.0)
        g.update_atlas()
        g.insert_points_subcell(pts, 1.0)
        if mode == "density":
            g.gather_density(1.0)
        else:
            g.gather_levelset(1.0)
        bricks = g.atlas_bricks(0)
        slot = leaf_positions(g).index((16, 16, 16))
        b = bricks[slot]
        d = np.sqrt(0.75)
        # voxel (30,30,30) is local (14,14,14), padded (15,15,15)
        v = b[15, 15, 15]
        far = b[1, 1, 1]  # voxel (16,16,16): A is not in that subcell's list
        if mode == "density":
            assert v == pytest.approx(1.0 - d, abs=1e-12)
            assert far == 0.0
            assert b[15, 15, 14] == 0.0  # voxel (29,30,30): d > 1
        else:
            assert v == pytest.approx(d - 1.0, abs=1e-12)
            assert far == 3.0


def test_apron_copies_neighbour_or_boundval():
    pts = np.array([A, B], dtype=np.float32)
    g, rc = grid(pts, radius=1.0)
    g.update_atlas()
    g.insert_points_subcell(pts, 1.0)
    g.gather_density(1.0)
    g.update_apron(0, -7.0)
    bricks = g.atlas_bricks(0)
    pos = leaf_positions(g)
    s0 = pos.index((16, 16, 16))
    s1 = pos.index((32, 16, 16))
    # padded x = 17 of brick (16,16,16) is world x = 32 -> brick (32,16,16), local x = 0
    assert np.array_equal(bricks[s0, 1:17, 1:17, 17], bricks[s1, 1:17, 1:17, 1])
    # padded x = 0 is world x = 15 -> brick (0,16,16) does not exist
    assert np.all(bricks[s0, :, :, 0] == -7.0)


def test_second_call_is_a_full_rebuild():
    f1 = np.array([A, B], dtype=np.float32)
    f2 = np.array([(50.5, 30.5, 30.5), B], dtype=np.float32)
    g = oracle.OracleGrid((3, 3, 3, 4))
    g.add_channel(0)
    assert g.rebuild_topology(f1, 1.0) == 0
    assert g.rebuild_topology(f2, 1.0) == 0  # depth "changes" from -1: full rebuild
    fresh, _ = grid(f2, radius=1.0)
    assert leaf_positions(g) == leaf_positions(fresh)
    n_before = g.node_count(0)
    assert g.rebuild_topology(f1, 1.0) == 0  # third call: incremental, appends
    pos = leaf_positions(g)
    assert pos[:n_before] == leaf_positions(fresh)
    assert len(pos) > n_before


def test_incremental_early_return_keeps_stale_flags():
    f1 = np.array([A, B], dtype=np.float32)
    g = oracle.OracleGrid((3, 3, 3, 4))
    g.add_channel(0)
    g.rebuild_topology(f1, 0.0)
    g.rebuild_topology(f1, 0.0)
    assert g.node_count(0) == 2
    # only A: nothing missing -> return before the markers are applied
    assert g.rebuild_topology(np.array([A, B], dtype=np.float32)[:1].copy(), 0.0) == 0
    assert list(g.nodes(0)["flags"]) == [1, 1]
    assert g.used_count(0) == 2
    # A and a point in a new brick: markers applied, B's leaf deactivated and delinked
    assert g.rebuild_topology(np.array([A, (40.5, 20.5, 20.5)], dtype=np.float32), 0.0) == 0
    n0 = g.nodes(0)
    assert [tuple(p) for p in n0["pos"]] == [(16, 16, 16), (32, 32, 32), (32, 16, 16)]
    assert list(n0["flags"]) == [1, 0, 1]
    assert n0["parent"][1] == UNDEF64
    assert g.used_count(0) == 2
    cl = g.childlist(1)[0]
    assert cl[(2 * 8 + 2) * 8 + 2] == UNDEF64


def test_top_level_is_lowest_single_node_level():
    # D = 2 (points span two level-1 nodes? no: one level-1 node, two leaves)
    pts = np.array([(200.5, 200.5, 200.5), (230.5, 230.5, 230.5)], dtype=np.float32)
    g, rc = grid(pts, radius=0.0)
    # posmin 199.5, posmax 232.5: level 1 (128): 1 vs 1 -> D = 1 with root at level 1
    assert g.depth == 1 and g.top_lev == 1
    pts = np.array([(100.5, 100.5, 100.5), (140.5, 100.5, 100.5)], dtype=np.float32)
    g, rc = grid(pts, radius=0.0)
    # level 1: 99/128 = 0 vs 142/128 = 1 -> D = 2; level 1 has 2 nodes, level 2 one
    assert g.depth == 2 and g.top_lev == 2
    assert g.node_count(1) == 2


def test_accumulate_keeps_old_flags():
    f1 = np.array([A, B], dtype=np.float32)
    g = oracle.OracleGrid((3, 3, 3, 4))
    g.add_channel(0)
    g.rebuild_topology(f1, 0.0)
    g.rebuild_topology(f1, 0.0)
    assert g.accumulate_topology(np.array([A, (40.5, 20.5, 20.5)], dtype=np.float32), 0.0) == 0
    assert list(g.nodes(0)["flags"]) == [1, 1, 1]
    assert g.used_count(0) == 3
