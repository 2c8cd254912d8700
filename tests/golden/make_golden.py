"""Generate the golden fixtures that pin the CPU oracle to the reference itself.

Runs on a GPU: the reference's own kernels (oracle/_ref/cuda_gvdb_module.ptx,
compiled from the reference's kernels/cuda_gvdb_module.cu) are driven by
oracle/ref_harness.cu, a restatement of VolumeGVDB's host code for the path,
on small seeded inputs.  Each fixture stores the inputs and the reference's
outputs: node pools, child lists, atlas map, subcell counts and per-subcell
membership hashes, per-slot sums of the gathered channel and a few full bricks.

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
    return out


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


def snapshot(prefix, g, store):
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
    b = g.atlas_bricks().astype(np.float64)
    inner = b[:, 1:17, 1:17, 1:17].reshape(b.shape[0], -1)
    m = np.ones((18, 18, 18), bool)
    m[1:17, 1:17, 1:17] = False
    store[prefix + "slot_sum"] = inner.sum(axis=1)
    store[prefix + "apron_sum"] = b[:, m].sum(axis=1)
    store[prefix + "bricks"] = b[:4].astype(np.float32)


def main(out_dir):
    import ref_harness

    os.makedirs(out_dir, exist_ok=True)
    for c in cases():
        g = ref_harness.RefGrid(c["log2dims"])
        store = {"log2dims": np.array(c["log2dims"]), "radius": c["radius"], "R": c["R"], "rho": c["rho"],
                 "mode": c["mode"], "boundval": c["boundval"], "nframes": len(c["frames"])}
        for k, pts in enumerate(c["frames"]):
            store["f%d_points" % k] = pts
            g.set_points(pts)
            g.rebuild_topology(c["radius"])
            g.update_atlas()
            g.insert_points_subcell(c["R"])
            if c["mode"] == "density":
                g.gather_density(c["rho"])
            else:
                g.gather_levelset(c["rho"])
            g.update_apron(c["boundval"])
            g.sync()
            snapshot("f%d_" % k, g, store)
        path = os.path.join(out_dir, c["name"] + ".npz")
        np.savez_compressed(path, **store)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
