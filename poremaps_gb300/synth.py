"""Seeded synthetic geometries in the reference's voxel convention.

Arrays are (nz, ny, nx) uint8, x fastest when written with ``tofile`` (the
``.raw`` layout of the reference, README.md:155-165): 0 = fluid, 1 = solid.
These stand in for the workload shapes the solver is benchmarked on: a
straight cylindrical pore, periodic overlapping-sphere packs and thresholded
Gaussian random fields, each checked for a fluid path along z.
"""
from __future__ import annotations

import numpy as np
from scipy import ndimage


def cylinder(nx: int = 48, ny: int = 48, nz: int = 64, radius: float = 20.0) -> np.ndarray:
    """Straight pore of the given radius (voxels) around the x-y midpoint
    ((n-1)/2), running the full z length; solid elsewhere."""
    y, x = np.mgrid[0:ny, 0:nx]
    cx, cy = (nx - 1) / 2.0, (ny - 1) / 2.0
    solid2d = ((x - cx) ** 2 + (y - cy) ** 2) > radius ** 2
    return np.broadcast_to(solid2d, (nz, ny, nx)).astype(np.uint8).copy()


def percolates_z(geom: np.ndarray, periodic_xy: bool = True) -> bool:
    """True if one fluid cluster touches both z faces (6-connectivity; x and y
    wrap when periodic)."""
    fluid = geom == 0
    if not fluid[0].any() or not fluid[-1].any():
        return False
    lab, n = ndimage.label(fluid)
    if n == 0:
        return False
    if periodic_xy:
        # merge labels across the periodic x and y faces
        parent = np.arange(n + 1)

        def find(a):
            while parent[a] != a:
                parent[a] = parent[parent[a]]
                a = parent[a]
            return a

        for a_face, b_face in ((lab[:, :, 0], lab[:, :, -1]), (lab[:, 0, :], lab[:, -1, :])):
            m = (a_face > 0) & (b_face > 0)
            for a, b in zip(a_face[m].ravel(), b_face[m].ravel()):
                ra, rb = find(a), find(b)
                if ra != rb:
                    parent[ra] = rb
        roots = np.array([find(i) for i in range(n + 1)])
        lab = roots[lab]
    bottom = set(np.unique(lab[0][lab[0] > 0]))
    top = set(np.unique(lab[-1][lab[-1] > 0]))
    return bool(bottom & top)


def sphere_pack(shape=(128, 128, 128), rmin: float = 4.0, rmax: float = 10.0,
                solid_fraction: float = 0.65, seed: int = 0, max_tries: int = 20) -> np.ndarray:
    """Periodic overlapping solid spheres (centres uniform in the box, radii
    uniform in [rmin, rmax]) added until the solid fraction reaches the target;
    reseeded until the pore space percolates along z."""
    nz, ny, nx = shape
    for attempt in range(max_tries):
        rng = np.random.default_rng(seed + 1000003 * attempt)
        solid = np.zeros(shape, bool)
        count = 0
        target = solid_fraction * solid.size
        while count < target:
            r = rng.uniform(rmin, rmax)
            c = rng.uniform(0, 1, 3) * np.array([nz, ny, nx])
            R = int(np.ceil(r))
            zz = np.arange(int(np.floor(c[0])) - R, int(np.floor(c[0])) + R + 2)
            yy = np.arange(int(np.floor(c[1])) - R, int(np.floor(c[1])) + R + 2)
            xx = np.arange(int(np.floor(c[2])) - R, int(np.floor(c[2])) + R + 2)
            dz = (zz + 0.5 - c[0])[:, None, None]
            dy = (yy + 0.5 - c[1])[None, :, None]
            dx = (xx + 0.5 - c[2])[None, None, :]
            ball = dz ** 2 + dy ** 2 + dx ** 2 <= r * r
            iz, iy, ix = np.nonzero(ball)
            solid[zz[iz] % nz, yy[iy] % ny, xx[ix] % nx] = True
            count = int(solid.sum())
        g = solid.astype(np.uint8)
        if percolates_z(g):
            return g
    raise RuntimeError("sphere_pack: no percolating sample found")


def gaussian_field(shape=(64, 64, 64), sigma: float = 3.0, porosity: float = 0.2, seed: int = 0,
                   keep_largest: bool = True, max_tries: int = 20,
                   relax: float = 0.0) -> np.ndarray:
    """iid N(0,1) -> periodic Gaussian filter (sigma voxels) -> fluid = lowest
    `porosity` quantile; optionally keep only the largest z-percolating fluid
    cluster (other pores become solid).  relax > 0: when max_tries draws do
    not percolate, raise the porosity by relax and draw again (up to 0.6)."""
    if relax > 0.0:
        while True:
            try:
                return gaussian_field(shape, sigma, porosity, seed, keep_largest, max_tries)
            except RuntimeError:
                if porosity + relax > 0.6:
                    raise
                porosity += relax
    for attempt in range(max_tries):
        rng = np.random.default_rng(seed + 7919 * attempt)
        f = ndimage.gaussian_filter(rng.standard_normal(shape), sigma, mode="wrap")
        thr = np.quantile(f, porosity)
        fluid = f <= thr
        g = (~fluid).astype(np.uint8)
        if not percolates_z(g):
            continue
        if keep_largest:
            lab, n = ndimage.label(fluid)
            ids_b = set(np.unique(lab[0][lab[0] > 0]))
            ids_t = set(np.unique(lab[-1][lab[-1] > 0]))
            span = ids_b & ids_t
            if span:
                sizes = ndimage.sum(fluid, lab, index=list(span))
                best = list(span)[int(np.argmax(sizes))]
                g = (lab != best).astype(np.uint8)
        return g
    raise RuntimeError("gaussian_field: no percolating sample found")


def random_solid(shape, solid_fraction: float, seed: int) -> np.ndarray:
    """iid solid voxels (tests only need a fluid path, not physics)."""
    rng = np.random.default_rng(seed)
    return (rng.random(shape) < solid_fraction).astype(np.uint8)
