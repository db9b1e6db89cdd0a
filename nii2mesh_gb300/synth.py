"""Seeded synthetic volumes standing in for the five benchmark workloads.

nii2mesh ships no benchmark dataset; these generators produce volumes with the
shapes, value types and intensity distributions of the named workloads
(seed = workload index, numpy ``default_rng``):

  sphere64   64^3 f32, 8 solid spheres (r 6-14) of 100 on 0, N(0,5) noise; iso 50
  brain      182x218x182 u8, perturbed ellipsoid shell + hollow and solid balls
  ct512      512^3 f32, CT-like: N(-1000,20) background, 300 bright ellipsoids,
             1% salt at +2000; iso 300
  atlas256   256^3 int16 labels: power-law weighted Voronoi partition
  sphere128  128^3 f32, the sphere64 generator scaled 2x (r 12-28)
"""
import numpy as np

CONFIGS = ("sphere64", "brain", "ct512", "atlas256", "sphere128")


def _grid(shape):
    nz, ny, nx = shape
    return np.ogrid[0:nz, 0:ny, 0:nx]


def spheres(n=64, count=8, rmin=6, rmax=14, cmin=12, cmax=52, noise=5.0, seed=0):
    """Solid spheres of intensity 100 on 0 plus N(0, noise) (workload 0)."""
    rng = np.random.default_rng(seed)
    z, y, x = _grid((n, n, n))
    vol = np.zeros((n, n, n), np.float32)
    for _ in range(count):
        c = rng.uniform(cmin, cmax, 3)
        r = rng.uniform(rmin, rmax)
        inside = (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 <= r * r
        vol[inside] = 100.0
    vol += rng.normal(0.0, noise, vol.shape).astype(np.float32)
    return vol


def sphere64(seed=0):
    return spheres(seed=seed)


def sphere128(seed=4):
    return spheres(n=128, rmin=12, rmax=28, cmin=24, cmax=104, seed=seed)


def brain(seed=1, shape=(182, 218, 182)):
    """Perturbed ellipsoid shell (semi-axes 70/85/65, thickness 25) holding a
    hollow ball (r 10) and a solid ball (r 8); tissue N(110,15), background
    N(5,3); uint8 (workload 1).  Array shape is (nz, ny, nx) = (182, 218, 182)."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    z, y, x = _grid(shape)
    cx, cy, cz = (nx - 1) / 2, (ny - 1) / 2, (nz - 1) / 2
    ax, ay, az = 70.0, 85.0, 65.0
    rho = np.sqrt(((x - cx) / ax) ** 2 + ((y - cy) / ay) ** 2 + ((z - cz) / az) ** 2)
    mean_axis = (ax + ay + az) / 3
    d = (rho - 1.0) * mean_axis  # approx. signed distance to the outer surface
    # 32 low-frequency Fourier modes (|k| <= 6), amplitude 4 voxels in total
    pert = np.zeros(shape, np.float32)
    ks = []
    while len(ks) < 32:
        k = rng.integers(-6, 7, 3)
        if 0 < np.linalg.norm(k) <= 6:
            ks.append(k)
    amps = rng.uniform(0.5, 1.0, 32)
    amps *= 4.0 / amps.sum() * 4.0  # typical |sum| of random phases ~ amplitude 4
    for k, a in zip(ks, amps):
        ph = rng.uniform(0, 2 * np.pi)
        pert += (a * np.cos(2 * np.pi * (k[0] * x / nx + k[1] * y / ny + k[2] * z / nz) + ph)).astype(np.float32)
    d = d + pert
    tissue = (d < 0) & (d > -25.0)
    r1 = np.sqrt((x - (cx - 15)) ** 2 + (y - (cy + 10)) ** 2 + (z - cz) ** 2)
    r2 = np.sqrt((x - (cx + 14)) ** 2 + (y - (cy - 12)) ** 2 + (z - (cz + 5)) ** 2)
    tissue |= (r1 <= 10.0) & (r1 >= 6.5)  # hollow ball
    tissue |= r2 <= 8.0  # solid ball
    vol = rng.normal(5.0, 3.0, shape)
    vol[tissue] = rng.normal(110.0, 15.0, int(tissue.sum()))
    return np.clip(np.rint(vol), 0, 255).astype(np.uint8)


def ct512(seed=2, n=512, count=300, salt=0.01):
    """CT-like volume (workload 2): background N(-1000,20), `count` rotated
    ellipsoidal structures (semi-axes U[4,40], intensity U[400,1200]) with
    lobulated, partly hollow walls, 1% salt voxels at +2000."""
    rng = np.random.default_rng(seed)
    vol = rng.normal(-1000.0, 20.0, (n, n, n)).astype(np.float32)
    for _ in range(count):
        ab = rng.uniform(4.0, 40.0, 3)
        c = rng.uniform(0, n, 3)
        q = rng.normal(size=(3, 3))
        rot, _ = np.linalg.qr(q)
        val = np.float32(rng.uniform(400.0, 1200.0))
        hollow = rng.random() < 0.6
        wall = rng.uniform(2.5, 6.0)
        lobes = rng.integers(-3, 4, (4, 3))
        lamp = rng.uniform(0.0, 0.12, 4)
        lph = rng.uniform(0, 2 * np.pi, 4)
        r = int(np.ceil(ab.max() * 1.15)) + 1
        lo = np.maximum(np.floor(c - r).astype(int), 0)
        hi = np.minimum(np.ceil(c + r).astype(int) + 1, n)
        if np.any(hi <= lo):
            continue
        zz, yy, xx = np.meshgrid(np.arange(lo[2], hi[2]), np.arange(lo[1], hi[1]), np.arange(lo[0], hi[0]), indexing="ij")
        p = np.stack([xx - c[0], yy - c[1], zz - c[2]], -1) @ rot
        u = p / ab
        rho = np.sqrt((u ** 2).sum(-1))
        ang = np.zeros_like(rho)
        for k, a, ph in zip(lobes, lamp, lph):
            ang += a * np.cos(u @ k * np.pi + ph)
        rho = rho * (1.0 + ang)
        inside = rho <= 1.0
        if hollow:
            inner = rho <= 1.0 - wall / ab.min()
            inside &= ~inner
        sub = vol[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
        sub[inside] = val
    m = rng.random((n, n, n)) < salt
    vol[m] = 2000.0
    return vol


def atlas256(seed=3, n=256, labels=250, alpha=1.6):
    """Label volume (workload 3): multiplicatively weighted Voronoi partition of
    `labels` seeds inside a head-sized ellipsoid; weights follow a power law
    so label bounding boxes range from a few voxels to ~120 voxels."""
    rng = np.random.default_rng(seed)
    c = (n - 1) / 2
    axes = np.array([0.42, 0.46, 0.40]) * n
    seeds = []
    while len(seeds) < labels:
        p = rng.uniform(-1, 1, 3)
        if (p ** 2).sum() <= 1.0:
            seeds.append(c + p * axes)
    seeds = np.array(seeds, np.float32)
    w = (rng.pareto(alpha, labels) + 1.0).astype(np.float32)
    w = np.minimum(w, 12.0)
    out = np.zeros((n, n, n), np.int16)
    y, x = np.mgrid[0:n, 0:n].astype(np.float32)
    for z in range(n):
        inside = ((x - c) / axes[0]) ** 2 + ((y - c) / axes[1]) ** 2 + ((z - c) / axes[2]) ** 2 <= 1.0
        if not inside.any():
            continue
        best = np.full((n, n), np.inf, np.float32)
        lab = np.zeros((n, n), np.int16)
        for i in range(labels):
            d2 = ((x - seeds[i, 0]) ** 2 + (y - seeds[i, 1]) ** 2 + (z - seeds[i, 2]) ** 2) / (w[i] * w[i])
            m = d2 < best
            best = np.where(m, d2, best)
            lab = np.where(m, np.int16(i + 1), lab)
        out[z] = np.where(inside, lab, 0)
    return out


def generate(name):
    return {"sphere64": sphere64, "brain": brain, "ct512": ct512, "atlas256": atlas256, "sphere128": sphere128}[name]()
