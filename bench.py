#!/usr/bin/env python
"""Throughput of the point-driven dynamic-topology path on one GB300.

Workload (the particle-fluid frames): 4,194,304 FP32 particles, seed 1, dam-break
layout (0.5-voxel lattice over [0,128)x[0,256)x[0,128), jitter U(+-0.1), 5%
scattered in a 512^3 domain), velocities N(0,1), frames advected by 0.5*v
(10-frame cycle, positions precomputed on the device).  One step = one frame:

  RebuildTopology(r=4) -> UpdateAtlas -> InsertPointsSubcell(4, R=4)
  -> GatherLevelSet(rho=2) into an FP32 channel -> UpdateApron(0, 3.0)

through the C ABI of libgbvdb.so, grid (3,3,3,4).  Metric: points/s
(input particles per frame / frame time).  `e2e` repeats the frame with the
positions copied from pinned host memory each step and the FP64 checksum read
back.  `--impl reference` times the reference algorithm's CPU restatement
(oracle/, all host threads) on a bounded sample of the same frames.

Multi-GPU (torchrun): every rank runs its own independent grid (replicas, weak
scaling); value = all ranks' points / the slowest rank's time.
"""
import argparse
import atexit
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "gvdb-voxels_gb300")
sys.path.insert(0, PKG)

METRIC = "points/s rebuild+gather+apron (fluid frame, 4,194,304 particles)"
N_FLUID = 4_194_304
FRAMES = 10
LOG2DIMS = (3, 3, 3, 4)
R_TOPO, R_INSERT, RHO, BOUND = 4.0, 4.0, 2.0, 3.0
# the gather's dense-form threshold is chosen by the library's autotuner (the warm-up
# frames measure its candidates)
SAMPLE_BOX = ((0.0, 0.0, 0.0), (32.0, 512.0, 512.0))  # CPU sample: the x < 32 slab of each frame


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def slowest_rank_ms(ms, world, device):
    """The timed region's length is the slowest replica's (max over ranks; no data exchange)."""
    if world <= 1:
        return float(ms)
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(points_per_rank, ms, world):
    """Whole-job points/s: every rank processed its own frame of points_per_rank points."""
    return world * points_per_rank / (ms / 1000.0)


def fluid_frames(seed, n=N_FLUID):
    import datasets

    pos, vel = datasets.fluid(n, seed=seed)
    return pos, vel


class ClockSampler:
    """nvidia-smi clock / throttle samples (every 20 ms) while the timed regions run: each
    sample is stamped with the host clock when it arrives, the timed regions are marked
    (mark), and the summary keeps the samples that arrive inside one (or within 25 ms after
    it: a sample covers the interval before it)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []
        self.windows = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def wait_first(self, timeout=5.0):
        """until nvidia-smi has printed its first sample (it takes a while to start)"""
        t_end = time.perf_counter() + timeout
        while self.proc and not self.lines and time.perf_counter() < t_end:
            time.sleep(0.005)

    def mark(self, t0, t1):
        self.windows.append((t0, t1))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.proc = None

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in self.lines:
            if not any(a <= t <= b + 0.025 for a, b in self.windows):
                continue
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if parts[4 + k].lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm), "window": "the device-timed loop and the e2e loops, sampled every 20 ms"}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """dram bytes per gather launch from the committed ncu summary (or None)."""
    p = os.path.join(ROOT, "profiles", "gather_fluid_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


def run_frame(grid, n, before_gather=None):
    grid.rebuild_topology(n, R_TOPO)
    grid.update_atlas()
    _, ln = grid.insert_points_subcell(4, n, R_INSERT)
    if before_gather:  # a streaming caller's hook (the e2e loop issues the next frame's upload here)
        before_gather()
    grid.gather_levelset(4, n, RHO, (0, 0, 0), ln)
    grid.update_apron(0, BOUND)
    return ln


def cpu_sample_points(pos, vel, frame):
    import datasets

    p = (pos + 0.5 * (frame + 1) * vel).astype(np.float32)
    return datasets.crop(p, *SAMPLE_BOX)


def cpu_frame(og, pts):
    og.rebuild_topology(pts, R_TOPO)
    og.update_atlas()
    og.insert_points_subcell(pts, R_INSERT)
    og.gather_levelset(RHO)
    og.update_apron(0, BOUND)


def cpu_baseline(pos, vel, steps=2):
    """the oracle (CPU restatement of the reference path) on the x < 32 slab, all host threads"""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    og = oracle.OracleGrid(LOG2DIMS)
    og.add_channel(0)
    pts0 = cpu_sample_points(pos, vel, 0)
    cpu_frame(og, pts0)  # warm-up (full rebuild)
    tot_pts, tot_t = 0, 0.0
    for k in range(1, steps + 1):
        pts = cpu_sample_points(pos, vel, k)
        t0 = time.perf_counter()
        cpu_frame(og, pts)
        tot_t += time.perf_counter() - t0
        tot_pts += pts.shape[0]
    cores = os.cpu_count()
    # the reference's own host topology path (RebuildTopologyCPU / ActivateSpace, one
    # thread by design) on the whole first frame: topology only, no gather or apron
    full = (pos + 0.5 * vel).astype(np.float32)
    cg = oracle.OracleGrid(LOG2DIMS)
    t0 = time.perf_counter()
    reached = cg.rebuild_topology_cpu(full)
    t_cpu = time.perf_counter() - t0
    return {"value": tot_pts / tot_t, "unit": "points/s", "cores": cores, "kind": "port",
            "sample": "fluid frames 2-%d cropped to x < 32 (%d points/frame, density-preserving), FP64 oracle, "
                      "OpenMP %d threads" % (steps + 1, pts0.shape[0], cores),
            "reference_host_topology": {"value": full.shape[0] / t_cpu, "unit": "points/s", "cores": 1,
                                        "kind": "port", "leaves": cg.node_count(0), "points_reached": reached,
                                        "what": "RebuildTopologyCPU / ActivateSpace restated (each point "
                                                "activates its leaf), frame 1, topology only"}}


def ref_cuda_inputs_safe(frames):
    """The reference's kernels index child lists and subcell counters without
    bounds checks; they stay in bounds when every coordinate is either < 0
    (dropped) or > 0 and every box position lies inside the 1024^3 root."""
    for p in frames:
        if np.any(p == 0.0) or np.any(p >= 1024 - 4 * R_TOPO - 8):
            return False
    return True


def bench_ref_cuda(frames_host, steps=5):
    """The reference's own CUDA kernels (PTX built from its cuda_gvdb_module.cu) under a
    restatement of its host code (oracle/ref_harness.cu), same frames and calls.  Per frame:
    the wall clock (its host pool loops and copies included) and the summed device time of
    its kernels and Thrust calls (an event pair around each)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    try:
        import ref_harness
        import ref_build

        if not ref_build.build_ptx():
            return {"unavailable": "the reference kernels' PTX was not built (needs the reference sources)"}
        if not ref_cuda_inputs_safe(frames_host):
            return {"unavailable": "inputs would make the reference kernels index outside their buffers"}
        g = ref_harness.RefGrid(LOG2DIMS)
    except Exception as e:  # noqa: BLE001 - a missing reference build is reported, not fatal
        return {"unavailable": "reference harness: %s" % e}
    wall, kern = [], []
    for k in range(steps + 2):
        pts = frames_host[k % len(frames_host)]
        g.set_points(pts)
        g.sync()
        g.timing(k >= 2)
        t0 = time.perf_counter()
        g.rebuild_topology(R_TOPO)
        g.update_atlas()
        g.insert_points_subcell(R_INSERT)
        g.gather_levelset(RHO)
        g.update_apron(BOUND)
        g.sync()
        if k >= 2:  # frames 0-1 are the two full rebuilds
            wall.append(time.perf_counter() - t0)
            kern.append(g.kernel_ms())
    g.timing(False)
    ms = 1000.0 * float(np.median(wall))
    kms = float(np.median(kern))
    npts = frames_host[0].shape[0]
    return {"value": npts / (ms / 1000.0), "unit": "points/s", "ms_per_frame": ms, "frames": len(wall),
            "kernel_ms_per_frame": kms, "value_kernels_only": npts / (kms / 1000.0),
            "what": "reference kernels (PTX of cuda_gvdb_module.cu, --use_fast_math) + host orchestration restated "
                    "from VolumeGVDB; incremental frames (median); ms_per_frame = host wall clock incl. its D2H/H2D "
                    "pool copies; kernel_ms_per_frame = summed device time of its kernels and Thrust calls"}


def bench_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return 0
    pos, vel = fluid_frames(1)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    og = oracle.OracleGrid(LOG2DIMS)
    og.add_channel(0)
    frame = 0
    for _ in range(args.warmup):
        cpu_frame(og, cpu_sample_points(pos, vel, frame % FRAMES))
        frame += 1
    tot_pts, tot_t = 0, 0.0
    for _ in range(args.steps):
        pts = cpu_sample_points(pos, vel, frame % FRAMES)
        if frame % FRAMES == 0:
            og.request_full_rebuild(True)
        t0 = time.perf_counter()
        cpu_frame(og, pts)
        tot_t += time.perf_counter() - t0
        tot_pts += pts.shape[0]
        frame += 1
    v = tot_pts / tot_t
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tot_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "fluid frames, 4,194,304 particles, grid (3,3,3,4), r=R=4, rho=2 level set",
                   "sample": "x < 32 slab per frame"},
        "cpu_baseline": {"value": v, "unit": "points/s", "cores": cores, "kind": "port",
                         "sample": "x < 32 slab of each fluid frame (%d points avg), CPU restatement of the "
                                   "reference algorithm, OpenMP %d threads" % (tot_pts // args.steps, cores)},
        "e2e": {"value": v, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- served form
SERVE_KINDS = (  # generator, grid (top -> leaf), mode, r = R, rho, boundval
    ("shell", (3, 3, 3, 4), 0, 1.0, 1.0, 0.0),
    ("fluid", (3, 3, 3, 4), 1, 4.0, 2.0, 3.0),
    ("surface", (4, 4, 3, 4), 0, 1.5, 1.5, 0.0),
)


def serve_pools(nmax, seed):
    """One pinned host pool of nmax points per generator (random order, so that the
    first n points are a uniform subset)."""
    import datasets
    import torch

    rng = np.random.default_rng(seed)
    pools = []
    for kind, *_ in SERVE_KINDS:
        if kind == "shell":
            p = datasets.shell(nmax, seed=int(rng.integers(1 << 30)))
        elif kind == "fluid":
            p, _ = datasets.fluid(nmax, seed=int(rng.integers(1 << 30)))
        else:
            p = datasets.surface(nmax, seed=int(rng.integers(1 << 30)))
        p = p[rng.permutation(p.shape[0])]
        t = torch.from_numpy(np.ascontiguousarray(p, dtype=np.float32)).pin_memory()
        pools.append(t)
    return pools


def serve_requests(count, seed, pools, lo=1e4, hi=4e6, upd_frac=0.3, nres=8, nver=4):
    """The request stream: size log-uniform in [lo, hi], generator uniform, 30% incremental
    updates (5% of a resident grid's points moved by N(0, 2)), FP32 / FP16 storage
    alternating.  Payloads are prepared up front in pinned host memory; each resident
    grid's updates cycle through `nver` prepared versions (version v+1 moves 5% of the
    points of version v), so that 10,000 requests fit in a few GB of pinned memory."""
    import torch

    rng = np.random.default_rng(seed)
    reqs, resident = [], {}
    for i in range(count):
        if resident and rng.random() < upd_frac:
            rid = int(rng.choice(sorted(resident)))
            k, vers, nxt = resident[rid]
            if len(vers) < nver:  # the next version: 5% of the last one's points moved
                q = vers[-1].numpy().copy()
                idx = rng.choice(q.shape[0], max(1, q.shape[0] // 20), replace=False)
                q[idx] += rng.normal(0.0, 2.0, size=(idx.size, 3)).astype(np.float32)
                vers.append(torch.from_numpy(q).pin_memory())
            pts = vers[nxt % len(vers)]
            resident[rid] = (k, vers, nxt + 1)
        else:
            k = int(rng.integers(len(SERVE_KINDS)))
            n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
            pts = pools[k][:n]
            rid = -1
            if len(resident) < nres and rng.random() < 0.25:
                rid = len(resident)
                resident[rid] = (k, [pts], 1)
        reqs.append({"kind": k, "points": pts, "resident_id": rid, "dtype": 3 if i % 2 == 0 else 100})
    return reqs


def serve_run(reqs, rate, workers, seed, cap):
    """Submit the stream with Poisson arrivals at `rate` req/s (rate None: all at once) to
    a server with `workers` workers; returns latency percentiles and throughput."""
    import gbvdb

    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(reqs)) if rate else np.zeros(len(reqs))
    arrive = np.cumsum(gaps)
    srv = gbvdb.Server(0, workers=workers, mem_cap_bytes=cap)
    tickets = []
    t0 = time.perf_counter()
    for r, ta in zip(reqs, arrive):
        d = ta - (time.perf_counter() - t0)
        if d > 0:
            time.sleep(d)
        _, dims, mode, rad, rho, bv = SERVE_KINDS[r["kind"]]
        tickets.append(srv.submit(r["points"].numpy(), log2dims=dims, radius=rad, gather_radius=rho, mode=mode,
                                  dtype=r["dtype"], boundval=bv, resident_id=r["resident_id"]))
    res = [srv.wait(t) for t in tickets]
    srv.close()
    bad = [x["status"] for x in res if x["status"] not in (gbvdb.OK, gbvdb.NOOP, gbvdb.DEPTH_UNSUPPORTED)]
    lat = np.array([x["t_end_ms"] - x["t_submit_ms"] for x in res])
    span_s = (max(x["t_end_ms"] for x in res) - min(x["t_submit_ms"] for x in res)) / 1000.0
    pts = float(sum(int(r["points"].shape[0]) for r in reqs))
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "points_per_s": pts / span_s, "requests_per_s": len(reqs) / span_s, "errors": len(bad),
            "checksums": [x["checksum"] for x in res]}


def bench_served(args):
    """Served form vs the plain per-call loop (the same calls back to back on one
    worker) on the mixed-size stream, per arrival rate and at saturation."""
    pools = serve_pools(int(args.serve_max_points), seed=4)
    reqs = serve_requests(args.serve_requests, seed=4, pools=pools, hi=args.serve_max_points)
    cap = 120 << 30
    out = {"requests": len(reqs), "workers": args.serve_workers, "cap_bytes": cap,
           "stream": "log-uniform [1e4, %.0e] points; shell / fluid / surface generators; 30%% incremental "
                     "updates of resident grids (5%% of points moved by N(0,2); each resident grid cycles through 4 "
                     "prepared versions); FP32 / FP16 alternating; Poisson arrivals; host (pinned) points, H2D "
                     "inside each job; saturation = the whole stream, a paced rate = its first rate * %g s "
                     "requests" % (args.serve_max_points, args.serve_seconds),
           "plain": "one worker: the per-frame calls of each request back to back on one stream",
           "points_total": float(sum(int(r["points"].shape[0]) for r in reqs)), "rates": []}
    # warm-up (library, allocator pools)
    serve_run(reqs[: min(20, len(reqs))], None, args.serve_workers, 0, cap)
    for rate in [None] + list(args.serve_rates):
        # saturation: the whole stream; a paced rate: the stream's first rate * serve_seconds
        # requests (10,000 requests at 100 req/s would take 100 s per run)
        sub = reqs if rate is None else reqs[: max(50, min(len(reqs), int(rate * args.serve_seconds)))]
        srv = serve_run(sub, rate, args.serve_workers, 5, cap)
        pln = serve_run(sub, rate, 1, 5, cap)
        same = srv.pop("checksums") == pln.pop("checksums")
        out["rates"].append({"rate_req_s": rate if rate else "saturation", "requests": len(sub), "served": srv,
                             "plain": pln, "same_results": same})
    sat = out["rates"][0]
    out["speedup_points_per_s_at_saturation"] = sat["served"]["points_per_s"] / sat["plain"]["points_per_s"]
    # the stream with every request stored in FP32, and in FP16, at saturation
    for name, dt in (("fp32_only", 3), ("fp16_only", 100)):
        one = [dict(r, dtype=dt) for r in reqs]
        srv = serve_run(one, None, args.serve_workers, 5, cap)
        pln = serve_run(one, None, 1, 5, cap)
        same = srv.pop("checksums") == pln.pop("checksums")
        out[name] = {"served": srv, "plain": pln, "same_results": same,
                     "speedup_points_per_s": srv["points_per_s"] / pln["points_per_s"]}
    return out


def bench_surface(args, steps=5):
    """Surface-fusion workload (16,777,216 points, seed 2, grid (4,4,3,4), density rho = r = R
    = 1.5): full-rebuild frames per storage type (FP32 accumulation in all three)."""
    import datasets
    import torch

    import gbvdb

    pts = datasets.surface(16_777_216, seed=2)
    d = torch.from_numpy(pts).cuda()
    stream = torch.cuda.current_stream()
    out = {"points": int(pts.shape[0]), "valid_points": int(np.all(pts >= 0, axis=1).sum()),
           "frame": "RequestFullRebuild + RebuildTopology(r=1.5) + UpdateAtlas + InsertPointsSubcell(4, R=1.5) + "
                    "GatherDensity(rho=1.5) + UpdateApron(0, 0.0)", "dtypes": {}}
    for name, dt in (("f32", gbvdb.T_FLOAT), ("f16", gbvdb.T_HALF), ("bf16", gbvdb.T_BFLOAT16)):
        g = gbvdb.Grid(0, (4, 4, 3, 4), stream=stream)
        g.set_channel_default(64, 64, 1)
        g.add_channel(0, dt)
        n = g.set_points(d)

        def frame():
            g.request_full_rebuild(True)
            g.rebuild_topology(n, 1.5)
            g.update_atlas()
            _, ln = g.insert_points_subcell(4, n, 1.5)
            g.gather_density(4, n, 1.5, (0, 0, 0), ln)
            g.update_apron(0, 0.0)

        for _ in range(3):
            frame()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            frame()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        st = g.stats()
        info = g.atlas_info(0)
        out["dtypes"][name] = {"ms_per_frame": ms, "points_per_s": pts.shape[0] / (ms / 1000.0),
                               "linked_bricks": st["bricks"], "subcell_list_len": st["sc_len"],
                               "atlas_slots": info["used"] if isinstance(info, dict) else None}
        g.close()
    del d
    torch.cuda.empty_cache()
    return out


def bench_sparse_jobs(args, reps=20):
    """RebuildTopology cost of sparse jobs, per key-set form (TUNE_KEYSET 0: the default
    choice, 1: level bitmaps over the points' key domain, 2: hash tables of the keys +
    radix sort).  Small job:
    10,000 sphere-surface points in 4096^3 (seed 5, grid (4,4,3,4), r = 1.5), a full
    rebuild per call.  Far clusters: 3 x 100,000 points in 80^3 boxes at far corners of a
    65,536^3 root (grid (3,3,3,3,4), r = 2): beyond the bitmaps' 2^34 positions, so only
    the tables.  Wall time per call (host readbacks included), after 3 warm-up calls."""
    import time

    import datasets
    import torch

    import gbvdb

    def clusters(n_each, seed):
        rng = np.random.default_rng(seed)
        cs = ((60, 70, 80), (65300, 200, 32000), (31000, 65250, 65300))
        return np.concatenate([np.asarray(c, np.float32) + rng.uniform(-40, 40, (n_each, 3)).astype(np.float32)
                               for c in cs]).astype(np.float32)

    surf = datasets.surface(10_000, seed=5)
    surf = surf[np.all(surf >= 0, axis=1)]
    jobs = [("small_job_4096", surf, (4, 4, 3, 4), 1.5, (0, 1, 2)),
            ("far_clusters_65536", clusters(100_000, 6), (3, 3, 3, 3, 4), 2.0, (0,))]
    out = {}
    stream = torch.cuda.current_stream()
    for name, pts, dims, r, modes in jobs:
        d = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
        res = {"points": int(pts.shape[0]), "grid_log2dims": list(dims), "radius": r}
        for m in modes:
            g = gbvdb.Grid(0, dims, stream=stream)
            g.set_tuning(gbvdb.TUNE_KEYSET, m)
            g.add_channel(0)
            n = g.set_points(d)
            ts = []
            for k in range(3 + reps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                g.request_full_rebuild(True)
                g.rebuild_topology(n, r)
                torch.cuda.synchronize()
                if k >= 3:
                    ts.append((time.perf_counter() - t0) * 1000.0)
            tot, used = g.node_counts()
            res[{0: "auto", 1: "bitmaps", 2: "tables"}[m]] = {
                "rebuild_ms_median": float(np.median(ts)), "rebuild_ms_min": float(np.min(ts)),
                "leaves": int(tot[0]), "hashed_key_passes": g.stats()["hashed_key_passes"]}
            g.close()
        out[name] = res
        del d
    torch.cuda.empty_cache()
    return out


def bench_batched(args):
    """Batched uneven grids: `count` clouds (seed 3, sizes log-uniform in [1e4, 2e6], shell or
    sphere-surface generator, grid (3,3,3,4), density rho = r = R = 1, FP32) submitted at once
    to the server vs one by one on one worker."""
    import datasets
    import torch

    clouds = datasets.batched(count=args.batch_grids, seed=3)
    host = [torch.from_numpy(c).pin_memory() for c in clouds]
    reqs = [{"kind": 0, "points": h, "resident_id": -1, "dtype": 3} for h in host]
    cap = 120 << 30
    serve_run(reqs[: min(8, len(reqs))], None, args.serve_workers, 0, cap)  # warm-up
    # each arm a few times, interleaved (one pass is a fraction of a second and its span
    # includes thread start-up); the run with the median throughput of each arm is kept
    runs = {"served": [], "plain": []}
    for _ in range(max(1, args.batch_repeats)):
        runs["served"].append(serve_run(reqs, None, args.serve_workers, 0, cap))
        runs["plain"].append(serve_run(reqs, None, 1, 0, cap))
    ref = runs["plain"][0]["checksums"]
    same = all(r["checksums"] == ref for arm in runs.values() for r in arm)
    med = {}
    for arm, rs in runs.items():
        rs = sorted(rs, key=lambda r: r["points_per_s"])
        med[arm] = rs[len(rs) // 2]
        med[arm].pop("checksums")
        med[arm]["points_per_s_runs"] = [r["points_per_s"] for r in runs[arm]]
    srv, pln = med["served"], med["plain"]
    return {"grids": len(reqs), "points_total": float(sum(int(h.shape[0]) for h in host)),
            "repeats": max(1, args.batch_repeats), "served": srv, "plain": pln, "same_results": same,
            "speedup_points_per_s": srv["points_per_s"] / pln["points_per_s"]}


def bench_ours(args):
    import torch

    import gbvdb

    rank, local, world = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import build_lib

    build_lib.build()
    dev = torch.device("cuda", local)
    npts = args.fluid_points
    pos, vel = fluid_frames(1 + rank, npts)
    dpos = torch.from_numpy(pos).to(dev)
    dvel = torch.from_numpy(vel).to(dev)
    frames = [(dpos + 0.5 * (f + 1) * dvel).contiguous() for f in range(FRAMES)]
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    grid = gbvdb.Grid(local, LOG2DIMS, stream=stream)
    grid.set_tuning(gbvdb.TUNE_FUSED_APRON, args.fused_apron)
    grid.add_channel(0, gbvdb.T_FLOAT)

    state = {"frame": 0}

    def step(src=None, before_gather=None):
        f = state["frame"] % FRAMES
        if f == 0:
            grid.request_full_rebuild(True)
        buf = frames[f] if src is None else src(f)
        n = grid.set_points(buf)
        run_frame(grid, n, before_gather)
        state["frame"] += 1

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    clk = ClockSampler(local).__enter__()  # closed after the e2e loops (at exit if they raise)
    atexit.register(clk.__exit__, None, None, None)
    for _ in range(max(args.warmup, 3)):
        step()
    barrier()
    clk.wait_first()
    l0 = grid.stats()["launches"]
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    t0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    barrier()
    wall = time.perf_counter() - t0
    clk.mark(t0, t0 + wall)
    dev_ms = ev0.elapsed_time(ev1)
    launches = grid.stats()["launches"] - l0
    ms = slowest_rank_ms(dev_ms / args.steps, world, dev)
    value = replica_throughput(npts, ms, world)

    # end to end: host positions -> device, frame, checksum -> host.  Every step copies
    # its frame's positions from pinned host memory; the copy of frame k+1 runs on a copy
    # stream while frame k computes (two device buffers), as a streaming caller would.
    # It is issued once frame k's points are binned, so that it overlaps the gather
    # (issue-bound) rather than the latency-bound topology and binning kernels, which
    # the copy's memory traffic slows most (measured: +13 us per frame instead of +78).
    host = [frames[f].cpu().pin_memory() for f in range(FRAMES)]
    bufs = [torch.empty_like(frames[0]) for _ in range(2)]
    copy_stream = torch.cuda.Stream(device=dev)
    copied = [torch.cuda.Event() for _ in range(2)]
    consumed = [torch.cuda.Event() for _ in range(2)]
    # the step's result (FP64 checksum) is read back every step without stalling the host:
    # computed on the grid's side stream (gbvdb_checksum_overlap), overlapping the next
    # frame's topology and binning, and copied into pinned memory there
    csum_dev = torch.zeros(args.steps + 2, dtype=torch.float64, device=dev)
    csum_host = torch.zeros(args.steps + 2, dtype=torch.float64).pin_memory()
    checks = []

    def issue_copy(k, f, after_stream=False):
        b = k % 2
        with torch.cuda.stream(copy_stream):
            if after_stream:  # starts once the frame's work issued so far is done
                copy_stream.wait_stream(stream)
            copy_stream.wait_event(consumed[b])  # the frame that last read this buffer is done
            bufs[b].copy_(host[f], non_blocking=True)
            copied[b].record(copy_stream)

    def e2e_run(nsteps, t_begin=None):
        copy_stream.wait_stream(stream)  # copies start inside the timed region
        issue_copy(0, state["frame"] % FRAMES)
        for k in range(nsteps):
            nxt = None
            if k + 1 < nsteps:
                nxt = (lambda k=k, f=(state["frame"] + 1) % FRAMES: issue_copy(k + 1, f, after_stream=True))
            stream.wait_event(copied[k % 2])
            step(lambda f, b=k % 2: bufs[b], before_gather=nxt)
            consumed[k % 2].record(stream)
            grid.checksum_overlap(csum_dev[k], csum_host[k])

    # every pinned frame buffer goes through the copy path once before timing (its first
    # transfer pays the mapping of its pages)
    for f in range(FRAMES):
        bufs[0].copy_(host[f], non_blocking=True)
    torch.cuda.synchronize()
    e2e_run(2)
    grid.join()
    barrier()
    # the K-step e2e loop, repeated: value = the median repeat (spread reported beside it)
    reps = []
    for _ in range(max(args.e2e_repeats, 1)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        te = time.perf_counter()
        e0.record(stream)
        e2e_run(args.steps)
        grid.join()  # the last frame's checksum and its copy to the host end the timed region
        e1.record(stream)
        barrier()
        clk.mark(te, time.perf_counter())
        reps.append(e0.elapsed_time(e1) / args.steps)
    clk.__exit__(None, None, None)
    checks = csum_host[:args.steps].tolist()
    e2e_ms = slowest_rank_ms(float(np.median(reps)), world, dev)
    # the parts of an e2e step timed alone: one frame's upload and the checksum
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h0.record(stream)
    for f in range(FRAMES):
        bufs[f % 2].copy_(host[f], non_blocking=True)
    h1.record(stream)
    c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    for _ in range(5):
        grid.checksum_device(csum_dev[0])
    c1.record(stream)
    torch.cuda.synchronize()
    h2d_ms, csum_ms = h0.elapsed_time(h1) / FRAMES, c0.elapsed_time(c1) / 5
    e2e = {"value": replica_throughput(npts, e2e_ms, world), "unit": "points/s",
           "h2d_bytes_per_step": npts * 12, "d2h_bytes_per_step": 8, "ms_per_step": e2e_ms,
           "repeats_ms_per_step": reps, "spread_ms": float(max(reps) - min(reps)),
           "h2d_ms_alone": h2d_ms, "h2d_gb_s": npts * 12 / (h2d_ms / 1000.0) / 1e9, "checksum_ms_alone": csum_ms,
           "result_read_back": "the frame's FP64 checksum of the level-set channel (8 bytes, computed on the grid's "
                               "side stream while the next frame's topology and binning run), not the atlas",
           "upload": "the next frame's positions, pinned host -> device on a copy stream, issued after the "
                     "frame's binning so that it overlaps the gather"}

    # per-stage times and the gather roofline (separate pass: profiling synchronizes per call)
    grid.set_profile(True)
    stage_names = ["rebuild", "atlas", "insert", "gather", "apron"]
    stage_ms = {k: 0.0 for k in stage_names}
    stage_dev_ms = {k: 0.0 for k in stage_names}
    gather_ms, sc_len, bricks = [], [], []
    nprof = FRAMES
    for _ in range(nprof):
        f = state["frame"] % FRAMES
        if f == 0:
            grid.request_full_rebuild(True)
        n = grid.set_points(frames[f])
        for name, fn in (("rebuild", lambda: grid.rebuild_topology(n, R_TOPO)),
                         ("atlas", lambda: grid.update_atlas()),
                         ("insert", lambda: state.__setitem__("ln", grid.insert_points_subcell(4, n, R_INSERT)[1])),
                         ("gather", lambda: grid.gather_levelset(4, n, RHO, (0, 0, 0), state["ln"])),
                         ("apron", lambda: grid.update_apron(0, BOUND))):
            torch.cuda.synchronize()
            a = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            stage_ms[name] += 1000.0 * (time.perf_counter() - a) / nprof
            stage_dev_ms[name] += sum(grid.stage_times()) / nprof
            if name == "gather":
                gather_ms.append(sum(grid.stage_times()))
                st = grid.stats()
                sc_len.append(st["sc_len"])
                bricks.append(st["bricks"])
        state["frame"] += 1
    grid.set_profile(False)
    g_ms = float(np.mean(gather_ms))
    S, B = float(np.mean(sc_len)), float(np.mean(bricks))
    alg_bytes = 12.0 * S + 8.0 * 64.0 * B + 4.0 * 4096.0 * B
    formula = "12*S + 8*64*B + 4*4096*B (S = subcell list length, B = linked bricks)"
    kname = "k_gather<float> (GatherLevelSet)"
    if args.fused_apron:
        # the gather also performs the apron stage (each brick writes its neighbours'
        # apron voxels): that stage's algorithmic bytes, read + write of 1736 voxels
        alg_bytes += 2.0 * 4.0 * 1736.0 * B
        formula = "12*S + 8*64*B + 4*4096*B + 2*4*1736*B (gather + the apron stage it performs; " \
                  "S = subcell list length, B = linked bricks)"
        kname = "k_gather<float> (GatherLevelSet with the fused apron)"
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / (g_ms / 1000.0) / 1e9
    traffic = profile_traffic()
    roofline = {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": traffic.get("bytes_per_launch") if traffic else None,
                "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": g_ms, "bytes_formula": formula}
    if traffic:
        # the DRAM bytes this kernel really moves (ncu, one launch of the same workload) over
        # the same event time: its use of HBM, as opposed to the reference-algorithmic rate
        # above (whose subcell-list term the binned form never writes or reads)
        dram_gbs = traffic["bytes_per_launch"] / (g_ms / 1000.0) / 1e9
        roofline["dram_achieved_gbs"] = dram_gbs
        roofline["dram_frac"] = dram_gbs / peak

    # per-stage roofline: the ideal bytes each stage must move (N points, S subcell-list
    # entries, B linked bricks, n_L nodes at level L, 4-byte voxels) over the stage's
    # device time (events around its kernels, host readback bubbles included)
    tot, _ = grid.node_counts()
    res_l = [1 << d for d in reversed(LOG2DIMS)]
    nodes_b = 64.0 * sum(tot) + sum(8.0 * res_l[l] ** 3 * tot[l] for l in range(1, len(res_l)))
    N = float(npts)
    stage_bytes = {
        "rebuild": 12 * N + 12 * N + nodes_b + 16 * B,          # bbox + topology
        "atlas": 64.0 * tot[0] + 16 * B,                         # flags, slots, atlas map
        "insert": 12 * N + 8 * 64 * B + 8 * 64 * B + 12 * N + 12 * S,  # count, scan, insert
        "gather": 12 * S + 8 * 64 * B + 4 * 4096 * B,
        "apron": 2 * 4 * 1736 * B,
    }
    if args.fused_apron:  # the gather performs the apron stage's copies; UpdateApron fills the rest
        stage_bytes["gather"] += stage_bytes["apron"]
        stage_bytes["apron"] = 0.0
    stage_roofline = {}
    for k in stage_names:
        t = stage_dev_ms[k]
        gbs = stage_bytes[k] / (t / 1000.0) / 1e9 if t > 0 else None
        stage_roofline[k] = {"bytes": stage_bytes[k], "device_ms": t, "achieved_gbs": gbs,
                             "frac": gbs / peak if gbs is not None else None}
    frame_bytes = sum(stage_bytes.values())

    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "fluid frames: 4,194,304 particles seed 1, dam-break 0.5-voxel lattice + 5% "
                               "scattered in 512^3, 10-frame cycle of p += 0.5 v",
                   "grid_log2dims": list(LOG2DIMS), "topology_radius": R_TOPO, "insert_radius": R_INSERT,
                   "gather": "levelset rho=2 FP32", "apron_boundval": BOUND, "parallelism": "replicas",
                   "l2": "inputs larger than L2 (per-frame working set about 1 GB, 10 rotating position buffers)",
                   "subcell_list_len": S, "linked_bricks": B},
        "e2e": e2e, "roofline": roofline, "gpu_launches": launches, "wall_s": wall, "clocks": clk.summary(),
        "stage_ms": stage_ms, "stage_roofline": stage_roofline,
        "frame_roofline": {"bytes": frame_bytes, "achieved_gbs": frame_bytes / (ms / 1000.0) / 1e9,
                           "frac": frame_bytes / (ms / 1000.0) / 1e9 / peak, "peak": peak},
        "checksum_last": checks[-1],
    }
    if npts != N_FLUID:  # a smaller case (profiling): the workload is named by its size
        line["config"]["workload"] = line["config"]["workload"].replace("4,194,304", "{:,}".format(npts))
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(pos, vel)
    if rank == 0 and world == 1 and not args.no_sparse:
        line["sparse_jobs"] = bench_sparse_jobs(args)
    if rank == 0 and world == 1 and not args.no_surface:
        grid.close()
        frames.clear()
        torch.cuda.empty_cache()
        line["surface"] = bench_surface(args)
    if rank == 0 and world == 1 and not args.no_served:
        grid.close()
        frames.clear()
        torch.cuda.empty_cache()
        line["served"] = bench_served(args)
        line["batched"] = bench_batched(args)
    if rank == 0 and world == 1 and not args.no_ref_cuda:
        grid.close()
        frames.clear()
        torch.cuda.empty_cache()
        fh = [(pos + 0.5 * (f + 1) * vel).astype(np.float32) for f in range(7)]
        rc = bench_ref_cuda(fh)
        line["reference_cuda"] = rc
        if "value" in rc:
            # the spec bar: the plain path's points/s over the reference CUDA path's
            line["plain_over_reference_cuda"] = {
                "device_vs_wall": value / rc["value"], "e2e_vs_wall": e2e["value"] / rc["value"],
                "device_vs_kernels_only": value / rc["value_kernels_only"],
                "e2e_vs_kernels_only": e2e["value"] / rc["value_kernels_only"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ref-cuda", action="store_true", help="skip timing the reference's own CUDA kernels")
    ap.add_argument("--e2e-repeats", type=int, default=5, help="repeats of the timed e2e loop (median reported)")
    ap.add_argument("--fluid-points", type=int, default=N_FLUID,
                    help="particles per fluid frame (default: the workload's 4,194,304; smaller for profiling)")
    ap.add_argument("--no-served", action="store_true", help="skip the served-form stream")
    ap.add_argument("--no-surface", action="store_true", help="skip the 16.8M-point surface workload")
    ap.add_argument("--no-sparse", action="store_true", help="skip the sparse-job rebuild timings")
    ap.add_argument("--serve-requests", type=int, default=10_000)
    ap.add_argument("--serve-seconds", type=float, default=8.0,
                    help="paced rates run the stream's first rate * serve_seconds requests")
    ap.add_argument("--batch-grids", type=int, default=256)
    ap.add_argument("--batch-repeats", type=int, default=3, help="runs of each batched arm (median kept)")
    ap.add_argument("--serve-workers", type=int, default=8)
    ap.add_argument("--serve-max-points", type=float, default=4e6)
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[100.0, 500.0, 2000.0])
    ap.add_argument("--fused-apron", type=int, default=1, choices=[0, 1],
                    help="gathers write the neighbours' apron voxels (1) or UpdateApron copies them all (0)")
    ap.add_argument("--surface-only", action="store_true",
                    help="only the surface workload (3 warm-up and --steps timed frames per storage type; "
                         "one JSON line with its times, for profiling that workload alone)")
    args = ap.parse_args()
    if args.impl == "reference":
        return bench_reference(args)
    if args.surface_only:
        import torch

        import build_lib

        torch.cuda.set_device(0)
        build_lib.build()
        print(json.dumps({"surface": bench_surface(args, steps=args.steps)}), flush=True)
        return 0
    return bench_ours(args)


if __name__ == "__main__":
    sys.exit(main())
