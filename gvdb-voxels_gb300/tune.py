"""Tuning run: writes the per point-count bucket table that libgbvdb.so reads at the
first grid creation (tune_table.json beside the library, or $GBVDB_TUNE_TABLE).

For each bucket a representative size is timed on three seeded workloads (a thick
shell with density r = R = rho = 1; dam-break fluid particles with r = R = 4 and a
level set of rho = 2, on their third frame, an incremental rebuild; sphere surfaces
in 4096^3 with density rho = 1.5 and grid (4,4,3,4)).  The binning settings (points per thread of the count and scatter
passes) are chosen on the InsertPointsSubcell time, the gather settings (dense-form
threshold, resident blocks per SM, the candidate count from which bricks launch first)
on the gather time; each candidate's time is
taken relative to the best candidate of its workload and the lowest mean wins.
Results do not depend on the settings, only times do.

    python gvdb-voxels_gb300/tune.py [--out PATH] [--reps 5]
"""
import argparse
import json
import os
import sys

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, PKG)

# bucket upper bounds (points) and the size each is tuned at
BUCKETS = [(30_000, 10_000), (300_000, 100_000), (1_500_000, 1_000_000), (8_000_000, 4_194_304),
           (1 << 62, 16_777_216)]
BIN = [(u, s) for u in (1, 2, 4) for s in (2, 4, 8)]
# gather: dense-form threshold, resident blocks per SM, long-first launch threshold (-1: linked order)
GATHER = [(d, b, l) for d in (1024, 2048, 4096, 8192, 16384, 32768) for b in (10, 8) for l in (-1, 1024, 2048, 4096)]


def workloads(n, seed):
    import datasets

    shell = datasets.shell(n, seed=seed)
    pos, vel = datasets.fluid(n, seed=seed + 1)
    # the fluid is timed on its third frame (p += 0.5 v per frame): an incremental
    # rebuild, as in a running simulation
    fluid = [(pos + 0.5 * (k + 1) * vel).astype(np.float32) for k in range(3)]
    surf = datasets.surface(n, seed=seed + 2)
    surf = surf[np.all(surf >= 0, axis=1)]
    return [("shell", [shell], (3, 3, 3, 4), 0, 1.0, 1.0, (16, 16, 1)),
            ("fluid", fluid, (3, 3, 3, 4), 1, 4.0, 2.0, (16, 16, 1)),
            ("surface", [surf], (4, 4, 3, 4), 0, 1.5, 1.5, (64, 64, 1))]


def time_calls(torch, stream, fn, reps):
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return float(np.median(ts))


def tune_workload(gbvdb, torch, wl, reps):
    name, frames, dims, mode, r, rho, axis = wl
    stream = torch.cuda.current_stream()
    g = gbvdb.Grid(0, dims, stream=stream)
    g.set_tuning(gbvdb.TUNE_TABLE, 0)
    g.set_channel_default(*axis)
    g.add_channel(0)
    for pts in frames:  # the last frame's topology is the one timed
        d = torch.from_numpy(np.ascontiguousarray(pts, dtype=np.float32)).cuda()
        n = g.set_points(d)
        g.rebuild_topology(n, r)
        g.update_atlas()
    state = {}

    def insert():
        state["ln"] = g.insert_points_subcell(4, n, r)[1]

    def gather():
        if mode == 0:
            g.gather_density(4, n, rho, (0, 0, 0), state["ln"])
        else:
            g.gather_levelset(4, n, rho, (0, 0, 0), state["ln"])

    t_bin = {}
    for u, s in BIN:
        g.set_tuning(gbvdb.TUNE_BIN_UNROLL, u)
        g.set_tuning(gbvdb.TUNE_SCATTER_UNROLL, s)
        insert()  # warm-up
        t_bin[(u, s)] = time_calls(torch, stream, insert, reps)
    insert()
    t_gat = {}
    for dm, b, lm in GATHER:
        g.set_tuning(gbvdb.TUNE_DENSE_MIN, dm)
        g.set_tuning(gbvdb.TUNE_GATHER_BLOCKS, b)
        g.set_tuning(gbvdb.TUNE_GATHER_LONG_MIN, lm)
        gather()
        t_gat[(dm, b, lm)] = time_calls(torch, stream, gather, reps)
    g.close()
    return t_bin, t_gat


def best(tables):
    """candidate with the lowest mean time relative to each workload's best"""
    keys = list(tables[0].keys())
    score = {k: float(np.mean([t[k] / min(t.values()) for t in tables])) for k in keys}
    return min(keys, key=lambda k: score[k]), score


def main():
    import torch

    import build_lib
    import gbvdb

    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(PKG, "tune_table.json"))
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    build_lib.build()
    torch.cuda.set_device(0)
    out = {"device": torch.cuda.get_device_name(0), "buckets": [], "measured": []}
    for k, (hi, n) in enumerate(BUCKETS):
        bins, gats = [], []
        for wl in workloads(n, seed=100 + k):
            tb, tg = tune_workload(gbvdb, torch, wl, args.reps)
            bins.append(tb)
            gats.append(tg)
            out["measured"].append({"points": n, "workload": wl[0],
                                    "insert_ms": {"%d/%d" % kk: v for kk, v in tb.items()},
                                    "gather_ms": {"%d/%d/%d" % kk: v for kk, v in tg.items()}})
        (u, s), _ = best(bins)
        (dm, b, lm), _ = best(gats)
        out["buckets"].append({"max_points": hi, "tuned_at": n, "dense_min": dm, "gather_blocks": b,
                               "gather_long_min": lm, "bin_unroll": u, "scatter_unroll": s})
        print("bucket <= %d (tuned at %d): dense_min %d, gather_blocks %d, gather_long_min %d, bin_unroll %d, "
              "scatter_unroll %d" % (hi, n, dm, b, lm, u, s), flush=True)
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    print(args.out)


if __name__ == "__main__":
    main()
