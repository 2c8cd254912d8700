"""Generate the golden fixtures that pin the CPU oracle to the reference itself.

Runs on a GPU: the reference's own kernels (oracle/_ref/cuda_gvdb_module.ptx,
compiled from the reference's kernels/cuda_gvdb_module.cu) are driven by
oracle/ref_harness.cu, a restatement of VolumeGVDB's host code for the path,
on small seeded inputs.  Each fixture stores the inputs and the reference's
outputs: node pools, child lists, atlas map, subcell counts and per-subcell
membership hashes and every padded brick of the gathered channel (and of the
colour channel where the case has one).

Cases cover the call sequences of the reference's samples: RebuildTopology
frames (full, then incremental), GatherDensity and GatherLevelSet, the
accumulating gathers after FillChannel with AccumulateTopology
(gPointFusion's sequence), GatherDensity with accumulation and point colours
into a T_UCHAR4 channel on a fixed topology (gSprayDeposit's), and
GatherLevelSet with colours (gFluidSurface's with m_use_color).

    python tests/golden/make_golden.py [out_dir]      (default: tests/golden)

Inputs keep every box and subcell position inside the root and >= 0 and span
two level-1 nodes, so the reference kernels never index outside their buffers.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "gvdb-voxels_gb300")):
    sys.path.insert(0, p)

import datasets  # noqa: E402

UNDEF64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def cases():
    out = []
    pts = datasets.shell(3000, seed=100)
    out.append(dict(name="shell_density", log2dims=(3, 3, 3, 4), radius=1.0, R=1.0, rho=1.0, mode="density",
                    boundval=0.0, frames=[pts]))
    pos, vel = datasets.fluid(n=6000, seed=101, box=(16, 32, 16), domain=32)
    pos = pos + np.array([120.0, 40.0, 40.0], dtype=np.float32)
    frames = [(pos + 0.5 * (k + 1) * vel).astype(np.float32) for k in range(4)]
    out.append(dict(name="fluid_levelset_frames", log2dims=(3, 3, 3, 4), radius=2.0, R=2.0, rho=1.5,
                    mode="levelset", boundval=3.0, frames=frames))
    pts = datasets.shell(2000, seed=102, rmin=30.0, rmax=40.0)
    out.append(dict(name="shell_levelset_r4", log2dims=(3, 3, 3, 4), radius=4.0, R=4.0, rho=2.0, mode="levelset",
                    boundval=3.0, frames=[pts]))
    # AccumulateTopology + accumulating GatherLevelSet after FillChannel(0, 3)
    pos, vel = datasets.fluid(n=5000, seed=103, box=(16, 24, 16), domain=32)
    pos = pos + np.array([100.0, 60.0, 30.0], dtype=np.float32)
    frames = [(pos + 1.5 * (k + 1) * vel).astype(np.float32) for k in range(3)]
    out.append(dict(name="accum_levelset", log2dims=(3, 3, 3, 4), radius=2.0, R=2.0, rho=1.0, mode="levelset",
                    boundval=3.0, frames=frames, topology="accumulate", fill=3.0, accum=True))
    # fixed topology from a shell, then three batches of coloured points gathered with
    # accumulation (density) into channel 0 and colours into channel 1
    rng = np.random.default_rng(104)
    base = datasets.shell(3000, seed=104, center=(200.0, 200.0, 200.0), rmin=40.0, rmax=50.0)
    frames, colours = [base], [None]
    for k in range(3):
        sub = base[rng.choice(base.shape[0], 700, replace=False)]
        sub = (sub + rng.normal(0.0, 0.7, size=sub.shape)).astype(np.float32)
        frames.append(sub)
        colours.append(_colours(rng, sub.shape[0]))
    out.append(dict(name="accum_density_colour", log2dims=(3, 3, 3, 4), radius=1.0, R=1.0, rho=1.0, mode="density",
                    boundval=0.0, frames=frames, colours=colours, topology="fixed", accum=True))
    # GatherLevelSet with colours, full then incremental frame, on a depth-1 tree (root at
    # level 1, [0, 128)^3; every box position stays inside it)
    pos, vel = datasets.fluid(n=4000, seed=105, box=(16, 16, 16), domain=32)
    pos = pos + np.array([24.0, 30.0, 20.0], dtype=np.float32)
    frames = [(pos + 0.5 * (k + 1) * vel).astype(np.float32) for k in range(3)]
    colours = [_colours(rng, f.shape[0]) for f in frames]
    out.append(dict(name="colour_levelset", log2dims=(3, 3, 3, 4), radius=4.0, R=4.0, rho=2.0, mode="levelset",
                    boundval=3.0, frames=frames, colours=colours))
    return out


def fcases():
    """fixtures of the operators after the gather (UpdateApronFaces, Compute(FUNC_SMOOTH)),
    the FP16 subcell pair and the legacy InsertPoints + ScatterDensity; each runs on one
    fresh full rebuild, so every leaf holds an assigned atlas slot"""
    out = []
    pts = datasets.shell(4000, seed=110, center=(180.0, 180.0, 180.0), rmin=30.0, rmax=38.0)
    out.append(dict(name="faces_smooth", kind="faces_smooth", log2dims=(3, 3, 3, 4), radius=1.0, R=1.0, rho=1.0,
                    points=pts, smooth=(1.5, 0.0)))
    pos, vel = datasets.fluid(n=6000, seed=111, box=(16, 32, 16), domain=32)
    pts = (pos + np.array([150.0, 60.0, 60.0], dtype=np.float32)).astype(np.float32)
    out.append(dict(name="fp16_levelset", kind="fp16", log2dims=(3, 3, 3, 4), radius=2.0, R=2.0, rho=1.5,
                    points=pts))
    # one point per 5-voxel lattice cell, jittered inside it: no two points' seven-voxel
    # splats touch one voxel, so the reference kernel's unsynchronised updates do not race
    rng = np.random.default_rng(112)
    g = np.stack(np.meshgrid(np.arange(14), np.arange(14), np.arange(14), indexing="ij"), axis=-1).reshape(-1, 3)
    pts = (200.0 + 5.0 * g + rng.uniform(1.6, 3.4, size=g.shape)).astype(np.float32)
    out.append(dict(name="scatter_density", kind="scatter", log2dims=(3, 3, 3, 4), radius=1.0, points=pts,
                    sradius=1.5, amp=1.0))
    return out


def smooth_field(rng, n):
    """random values on the voxels 2..5 of every 8^3 block of each 16^3 interior, zero
    elsewhere: after one smoothing pass the voxels on the blocks' faces are still zero, so
    the reference's blocks (which read each other's voxels as halo with no ordering) see
    the same values whether a neighbour block has written already or not"""
    b = np.zeros((n, 18, 18, 18), dtype=np.float32)
    loc = (np.arange(16) % 8 >= 2) & (np.arange(16) % 8 <= 5)
    m = loc[:, None, None] & loc[None, :, None] & loc[None, None, :]
    inner = b[:, 1:17, 1:17, 1:17]
    inner[:, m] = rng.uniform(-2.0, 2.0, size=(n, int(m.sum()))).astype(np.float32)
    return b


def topology(g, store):
    store["top_lev"] = g.top_lev
    store["used"] = g.used_count(0)
    for lev in range(g.levs):
        n = g.nodes(lev)
        for f in ("lev", "flags", "pos", "value", "parent", "childlist"):
            store["L%d_%s" % (lev, f)] = n[f]
        if lev > 0:
            store["L%d_clist" % lev] = g.childlist(lev)
    store["atlas_dims"] = np.array(g.atlas_dims())
    store["amap"] = g.atlas_map().view(np.int32)


def run_fcase(c, store):
    import ref_harness

    g = ref_harness.RefGrid(c["log2dims"])
    pts = c["points"]
    store.update({"kind": c["kind"], "log2dims": np.array(c["log2dims"]), "radius": c["radius"], "points": pts})
    g.set_points(pts)
    g.rebuild_topology(c["radius"])
    g.update_atlas()
    if c["kind"] == "faces_smooth":
        store.update({"R": c["R"], "rho": c["rho"]})
        g.insert_points_subcell(c["R"])
        g.gather_density(c["rho"])
        g.sync()
        store["gathered"] = g.atlas_bricks(0)
        g.update_apron_faces()
        g.sync()
        store["faces"] = g.atlas_bricks(0)
        field = smooth_field(np.random.default_rng(113), store["faces"].shape[0])
        g.write_bricks(field)
        g.smooth(*c["smooth"])
        g.sync()
        store["smooth_in"] = field
        store["smooth_params"] = np.array(c["smooth"], dtype=np.float32)
        store["smooth_out"] = g.atlas_bricks(0)
    elif c["kind"] == "fp16":
        store.update({"R": c["R"], "rho": c["rho"]})
        _, ln = g.insert_points_subcell_fp16(c["R"])
        g.gather_levelset_fp16(c["rho"])
        g.update_apron(3.0, 0)
        g.sync()
        store["len"] = ln
        store["sc_cnt"] = g.subcell_counts()[0]
        store["bricks"] = g.atlas_bricks(0)
    else:
        store.update({"sradius": c["sradius"], "amp": c["amp"]})
        g.insert_points()
        g.scatter_density(c["sradius"], c["amp"])
        g.sync()
        store["bricks"] = g.atlas_bricks(0)
    topology(g, store)


def _colours(rng, n):
    """RGBA8 per point as uint32 (R in the low byte); a third opaque, a third with
    random alpha, a third all-random"""
    c = rng.integers(0, 256, size=(n, 4), dtype=np.uint32)
    c[: n // 3, 3] = 255
    return (c[:, 0] | (c[:, 1] << 8) | (c[:, 2] << 16) | (c[:, 3] << 24)).astype(np.uint32)


def membership_hash(off, cnt, pts):
    """per subcell: xor over its points of a 64-bit mix of the float bits (order-free)"""
    b = pts.view(np.uint32).astype(np.uint64)
    key = b[:, 0] ^ (b[:, 1] << np.uint64(21)) ^ (b[:, 2] << np.uint64(42)) ^ (b[:, 2] >> np.uint64(22))
    h = np.zeros(len(cnt), dtype=np.uint64)
    seg = np.repeat(np.arange(len(cnt)), cnt)
    order = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)]) if len(cnt) else np.zeros(0, np.int64)
    if len(order):
        np.bitwise_xor.at(h, seg, key[order])
    return h


def snapshot(prefix, g, store, colour=False):
    store[prefix + "top_lev"] = g.top_lev
    store[prefix + "used"] = g.used_count(0)
    for lev in range(g.levs):
        n = g.nodes(lev)
        for f in ("lev", "flags", "pos", "value", "parent", "childlist"):
            store[prefix + "L%d_%s" % (lev, f)] = n[f]
        if lev > 0:
            store[prefix + "L%d_clist" % lev] = g.childlist(lev)
    store[prefix + "atlas_dims"] = np.array(g.atlas_dims())
    store[prefix + "amap"] = g.atlas_map().view(np.int32)
    cnt, off, pts = g.subcells()
    store[prefix + "sc_cnt"] = cnt
    store[prefix + "sc_hash"] = membership_hash(off, cnt, pts)
    store[prefix + "len"] = g.len
    store[prefix + "bricks"] = g.atlas_bricks(0)
    if colour:
        store[prefix + "colour"] = g.atlas_bricks(1)


def main(out_dir):
    import ref_harness

    os.makedirs(out_dir, exist_ok=True)
    for c in cases():
        g = ref_harness.RefGrid(c["log2dims"])
        topo = c.get("topology", "rebuild")
        accum = bool(c.get("accum", False))
        colours = c.get("colours")
        store = {"log2dims": np.array(c["log2dims"]), "radius": c["radius"], "R": c["R"], "rho": c["rho"],
                 "mode": c["mode"], "boundval": c["boundval"], "nframes": len(c["frames"]), "topology": topo,
                 "accum": accum, "colour": colours is not None}
        if colours is not None:
            g.add_colour_channel()
        if c.get("fill") is not None:
            store["fill"] = c["fill"]
            g.fill(0, c["fill"])
        for k, pts in enumerate(c["frames"]):
            store["f%d_points" % k] = pts
            clr = colours[k] if colours is not None else None
            if clr is not None:
                store["f%d_colours" % k] = clr
            g.set_points(pts)
            g.set_colors(clr)
            if topo == "accumulate":
                g.accumulate_topology(c["radius"])
            elif topo == "rebuild" or k == 0:
                g.rebuild_topology(c["radius"])
            if topo != "fixed" or k == 0:
                g.update_atlas()
            g.insert_points_subcell(c["R"])
            if c["mode"] == "density":
                g.gather_density(c["rho"], accum)
            else:
                g.gather_levelset(c["rho"], accum)
            g.update_apron(c["boundval"], 0)
            if colours is not None:
                g.update_apron(0.0, 1)
            g.sync()
            snapshot("f%d_" % k, g, store, colours is not None)
        path = os.path.join(out_dir, c["name"] + ".npz")
        np.savez_compressed(path, **store)
        print(path, os.path.getsize(path))
    for c in fcases():
        store = {}
        run_fcase(c, store)
        path = os.path.join(out_dir, "op_" + c["name"] + ".npz")
        np.savez_compressed(path, **store)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
