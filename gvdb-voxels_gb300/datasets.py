"""Seeded synthetic point clouds with the shapes of the benchmark workloads.

No public dataset is involved: every generator draws from numpy's
default_rng(seed) and returns float32 positions of shape (N, 3) in index space
(voxels).  The layouts follow the workload descriptions:

  shell      200,000 points uniform in a spherical shell, radius 100-120,
             centred at (256, 256, 256)                              (seed 0)
  fluid      4,194,304 particles: 95% on distinct sites of a 0.5-voxel lattice
             over [0,128)x[0,256)x[0,128) with U(+-0.1) jitter, 5% uniform in
             the rest of a 512^3 domain; velocities N(0, 1)            (seed 1)
  surface    16,777,216 points on 64 spheres (radius U(20,200), centre
             U(0,4096)^3) plus the z=0 patch x,y in [1024,3072), uniform by
             area, offset along the normal by N(0, 0.5)                (seed 2)
  batched    256 grids, point counts log-uniform in [1e4, 2e6], shell or
             sphere-surface in a 1024^3 domain                         (seed 3)
"""
import numpy as np


def _unit_vectors(rng, n):
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def shell(n=200_000, seed=0, center=(256.0, 256.0, 256.0), rmin=100.0, rmax=120.0):
    rng = np.random.default_rng(seed)
    u = rng.random(n)
    r = np.cbrt(rmin ** 3 + u * (rmax ** 3 - rmin ** 3))
    d = _unit_vectors(rng, n)
    p = np.asarray(center)[None, :] + d * r[:, None]
    return p.astype(np.float32)


def fluid(n=4_194_304, seed=1, frac_lattice=0.95, spacing=0.5, box=(128, 256, 128), domain=512):
    """Dam-break layout.  Returns (positions, velocities), both float32 (N, 3)."""
    rng = np.random.default_rng(seed)
    n_lat = int(round(frac_lattice * n))
    n_sc = n - n_lat
    dims = [int(b / spacing) for b in box]  # sites per axis
    nsites = dims[0] * dims[1] * dims[2]
    sites = rng.choice(nsites, size=n_lat, replace=False)
    ix = sites // (dims[1] * dims[2])
    iy = (sites // dims[2]) % dims[1]
    iz = sites % dims[2]
    lat = np.stack([ix, iy, iz], axis=1).astype(np.float64) * spacing
    lat += rng.uniform(-0.1, 0.1, size=lat.shape)
    # scattered points: uniform in the domain minus the dam box (rejection)
    out = np.empty((0, 3))
    while out.shape[0] < n_sc:
        c = rng.uniform(0, domain, size=(2 * (n_sc - out.shape[0]) + 64, 3))
        inside = (c[:, 0] < box[0]) & (c[:, 1] < box[1]) & (c[:, 2] < box[2])
        out = np.concatenate([out, c[~inside]], axis=0)
    sc = out[:n_sc]
    pos = np.concatenate([lat, sc], axis=0).astype(np.float32)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    return pos, vel


def surface(n=16_777_216, seed=2, nspheres=64, domain=4096.0, patch=(1024.0, 3072.0), sigma=0.5):
    rng = np.random.default_rng(seed)
    radii = rng.uniform(20.0, 200.0, size=nspheres)
    centres = rng.uniform(0.0, domain, size=(nspheres, 3))
    areas = np.concatenate([4.0 * np.pi * radii ** 2, [(patch[1] - patch[0]) ** 2]])
    counts = rng.multinomial(n, areas / areas.sum())
    parts = []
    for k in range(nspheres):
        m = counts[k]
        d = _unit_vectors(rng, m)
        off = rng.normal(0.0, sigma, size=m)
        parts.append(centres[k][None, :] + d * (radii[k] + off)[:, None])
    m = counts[-1]
    xy = rng.uniform(patch[0], patch[1], size=(m, 2))
    z = rng.normal(0.0, sigma, size=(m, 1))
    parts.append(np.concatenate([xy, z], axis=1))
    p = np.concatenate(parts, axis=0)
    p = p[rng.permutation(p.shape[0])]
    return p.astype(np.float32)


def sphere_surface(n, seed, domain=1024.0, nspheres=8, sigma=0.5):
    rng = np.random.default_rng(seed)
    radii = rng.uniform(20.0, 200.0, size=nspheres)
    centres = rng.uniform(0.0, domain, size=(nspheres, 3))
    areas = 4.0 * np.pi * radii ** 2
    counts = rng.multinomial(n, areas / areas.sum())
    parts = []
    for k in range(nspheres):
        d = _unit_vectors(rng, counts[k])
        off = rng.normal(0.0, sigma, size=counts[k])
        parts.append(centres[k][None, :] + d * (radii[k] + off)[:, None])
    p = np.concatenate(parts, axis=0)
    return p[rng.permutation(p.shape[0])].astype(np.float32)


def batched(count=256, seed=3, lo=1e4, hi=2e6):
    """List of float32 (N_i, 3) clouds for the batched-grids workload."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)
    kinds = rng.integers(0, 2, size=count)
    seeds = rng.integers(0, 2 ** 31 - 1, size=count)
    clouds = []
    for k in range(count):
        if kinds[k] == 0:
            clouds.append(shell(int(sizes[k]), seed=int(seeds[k]), center=(512.0, 512.0, 512.0)))
        else:
            clouds.append(sphere_surface(int(sizes[k]), seed=int(seeds[k])))
    return clouds


def crop(points, lo, hi):
    """Points inside the axis-aligned box [lo, hi): a density-preserving sample."""
    lo = np.asarray(lo, dtype=np.float32)
    hi = np.asarray(hi, dtype=np.float32)
    m = np.all((points >= lo) & (points < hi), axis=1)
    return points[m]
