"""The reference's host topology path (RebuildTopologyCPU -> ActivateSpace, the CPU
path the reference offers besides its GPU topology pass), restated in the oracle:
every point activates the leaf containing it, the root grows upwards from the first
point's leaf (Reparent).  Checked against the oracle's restatement of the GPU path
with radius 0 (pass 1 only: the leaves containing the points), and for the links it
builds.  CPU only."""
import numpy as np
import pytest

import datasets
import oracle


def _sets(g, lev):
    return {tuple(int(v) for v in x) for x in g.nodes(lev)["pos"]}


def _check_links(g, levs):
    """every node below the root hangs from its parent's child slot at its own position"""
    for lev in range(levs - 1):
        nd = g.nodes(lev)
        up = g.nodes(lev + 1)
        cl = g.childlist(lev + 1)
        res = 1 << (4 if lev == 0 else 3)
        rng = 16 if lev == 0 else 16 * 8 ** lev
        for i in range(nd.shape[0]):
            par = int(nd["parent"][i])
            if par == 0xFFFFFFFF:
                continue
            assert (par >> 8) & 0xFF == lev + 1
            p = up[par >> 16]
            local = (nd["pos"][i] - p["pos"]) // rng
            assert np.all(local >= 0) and np.all(local < 8)
            b = (int(local[2]) * 8 + int(local[1])) * 8 + int(local[0])
            k = int(p["childlist"]) >> 16
            assert int(cl[k][b]) == ((lev << 8) | (i << 16))


@pytest.mark.parametrize("case", ["shell", "fluid_crop", "far_first"])
def test_cpu_path_matches_pass1_leaves(case):
    if case == "shell":
        pts = datasets.shell(30_000, seed=7)
    elif case == "fluid_crop":
        pos, vel = datasets.fluid(n=50_000, seed=9, box=(32, 64, 32), domain=128)
        pts = np.maximum(pos, 0.0).astype(np.float32)
    else:  # the first point far from the rest: the root starts there and must grow
        p = datasets.shell(10_000, seed=11)
        pts = np.concatenate([np.array([[900.0, 5.0, 700.0]], dtype=np.float32), p]).astype(np.float32)
    cpu = oracle.OracleGrid((3, 3, 3, 4))
    assert cpu.rebuild_topology_cpu(pts) == pts.shape[0]
    gpu = oracle.OracleGrid((3, 3, 3, 4))
    gpu.add_channel(0)
    assert gpu.rebuild_topology(pts, 0.0) == 0
    assert _sets(cpu, 0) == _sets(gpu, 0)
    # upper levels: the ancestors of those leaves, up to the lower of the two roots
    top = min(cpu.cpu_root_level(), gpu.depth)
    for lev in range(1, top):
        assert _sets(cpu, lev) == _sets(gpu, lev)
    # each point lies in an activated leaf, and the links are consistent
    leaves = _sets(cpu, 0)
    for q in pts[::97]:
        key = tuple(int(v) // 16 * 16 for v in q)
        assert key in leaves
    _check_links(cpu, cpu.cpu_root_level() + 1)
    # one root: the only node of its level, with no parent
    rl = cpu.cpu_root_level()
    assert cpu.node_count(rl) == 1 and int(cpu.nodes(rl)["parent"][0]) == 0xFFFFFFFF
