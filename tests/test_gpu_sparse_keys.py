"""RebuildTopology's sparse key sets (hash tables of node keys, compacted and
radix-sorted, in place of the per-level bitmaps) against the oracle, whose keys go
through a plain sort and unique as the reference's do (gvdb_cutils.cu:11-16,
VG.cpp:843-928).

The form is forced on the small parity cases (full, extra-brick and incremental
passes, accumulation; key counts on both sides of the one-block sort), and taken
automatically on a domain of more than 2^34 node positions: three far-apart
clusters in a 5-level (3,3,3,3,4) grid, which the bitmaps cannot hold.
"""
import numpy as np
import pytest

import _helpers as H
import datasets

pytestmark = pytest.mark.gpu


def _check(o, g, boundval):
    H.compare_topology(o, g)
    H.compare_subcells(o, g)
    H.compare_values(o, g)
    H.check_apron_self(g, boundval)


def _clusters(n_each=3000, seed=3, centres=((60, 70, 80), (65300, 200, 32000), (31000, 65250, 65300)), size=40.0):
    rng = np.random.default_rng(seed)
    parts = [np.asarray(c, np.float32) + rng.uniform(-size, size, (n_each, 3)).astype(np.float32) for c in centres]
    return np.concatenate(parts).astype(np.float32)


def test_fluid_frames_hashed(gpu_lib):
    """dam-break frames through the hash-table form: full rebuild with extra bricks
    (r = 4), the second full rebuild, then incremental frames; 60,000 points (radix sort)"""
    pos, vel = datasets.fluid(n=60000, seed=11, box=(32, 64, 32), domain=128)
    frames = []
    p = pos.copy()
    for _ in range(4):
        p = (p + 0.5 * vel).astype(np.float32)
        frames.append(p.copy())
    _, o = H.run_oracle(None, frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0)
    g, gs = H.run_gpu(None, frames=frames, radius=4.0, R=4.0, rho=2.0, mode="levelset", boundval=3.0, keyset=2)
    for k in range(len(frames)):
        _check(o[k], gs[k], 3.0)
    # two key passes per full rebuild (frames 1 and 2), one per incremental frame
    assert g.stats()["hashed_key_passes"] == 6


@pytest.mark.parametrize("n", [300, 5000])
def test_shell_hashed_small_sorts(gpu_lib, n):
    """few keys: the one-block sort (300 points) and just past it (5,000 points)"""
    pts = datasets.shell(n, seed=9)
    _, o = H.run_oracle(pts, radius=1.0, R=1.0, rho=1.0, mode="density")
    g, gs = H.run_gpu(pts, radius=1.0, R=1.0, rho=1.0, mode="density", keyset=2)
    _check(o[0], gs[0], 0.0)
    assert g.stats()["hashed_key_passes"] == 2


def test_accumulate_hashed(gpu_lib):
    pos, vel = datasets.fluid(n=20000, seed=5, box=(32, 64, 32), domain=128)
    frames = [pos, (pos + 3.0 * vel).astype(np.float32), (pos - 3.0 * vel).astype(np.float32)]
    frames = [np.maximum(f, 0.0).astype(np.float32) for f in frames]
    _, o = H.run_oracle(None, frames=frames, radius=2.0, R=2.0, rho=1.5, accumulate=True)
    _, gs = H.run_gpu(None, frames=frames, radius=2.0, R=2.0, rho=1.5, accumulate=True, keyset=2)
    for k in range(len(frames)):
        _check(o[k], gs[k], 0.0)


def test_far_clusters_take_the_sparse_form(gpu_lib):
    """three clusters at far corners of a 65,536^3 root (grid (3,3,3,3,4)): the level-0
    key domain alone is about 8,100^3 positions, beyond the bitmaps' 2^34; default
    settings take the hash tables; full, second full and incremental frames"""
    base = _clusters()
    rng = np.random.default_rng(4)
    vel = rng.normal(0.0, 1.5, base.shape).astype(np.float32)
    frames = [(base + k * vel).astype(np.float32) for k in range(3)]
    dims = (3, 3, 3, 3, 4)
    _, o = H.run_oracle(None, frames=frames, log2dims=dims, radius=2.0, R=2.0, rho=1.5, mode="levelset",
                        boundval=2.0)
    g, gs = H.run_gpu(None, frames=frames, log2dims=dims, radius=2.0, R=2.0, rho=1.5, mode="levelset",
                      boundval=2.0)
    assert o[0]["depth"] == 4
    for k in range(len(frames)):
        _check(o[k], gs[k], 2.0)
    assert g.stats()["hashed_key_passes"] == 5


@pytest.mark.parametrize("keyset", [0, 1, 2])
def test_surface_4096_each_form(gpu_lib, keyset):
    """sphere surfaces in 4096^3, grid (4,4,3,4): a key domain of about 4.6 M positions
    for 8,423 points (25,269 point keys), where the default takes the tables; the bitmaps
    forced, the tables forced and the default all match the oracle"""
    pts = datasets.sphere_surface(10_000, seed=21, domain=4096.0, nspheres=6)
    pts = pts[np.all(pts >= 0, axis=1)]
    _, o = H.run_oracle(pts, log2dims=(4, 4, 3, 4), radius=1.5, R=1.5, rho=1.5)
    g, gs = H.run_gpu(pts, log2dims=(4, 4, 3, 4), radius=1.5, R=1.5, rho=1.5, keyset=keyset)
    _check(o[0], gs[0], 0.0)
    assert g.stats()["hashed_key_passes"] == (0 if keyset == 1 else 2)

