"""Seeded geometries and standard scenarios, driven through the SunlightLB C API.

Every function takes a :class:`~sunlightlb_gb300.binding.Library` so the
same set-up runs on the GPU library and on any other implementation of the
API.  Random numbers come from splitmix64 (Steele, Lea and Flood, 2014) so
a seed gives the same geometry on every machine.
"""

import math
import os
import tempfile

import numpy as np

MASK64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 generator; uniform() returns doubles in [0, 1)."""

    def __init__(self, seed):
        self.state = seed & MASK64

    def next(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next() >> 11) * (1.0 / (1 << 53)))

    def unit_vector(self):
        while True:
            v = [self.uniform(-1.0, 1.0) for _ in range(3)]
            n = math.sqrt(sum(c * c for c in v))
            if 1e-6 < n <= 1.0:
                return [c / n for c in v]


def sphere_nodes(shape, rad, centre):
    """Boolean mask of the nodes a reference insertsph(rad, centre) sets
    (rsq < rad^2, the test of reference src/lbobjs.c:214-215), periodic
    images excluded."""
    ni, nj, nk = shape
    ox, oy, oz = centre
    i = np.arange(ni, dtype=np.float64)[:, None, None]
    j = np.arange(nj, dtype=np.float64)[None, :, None]
    k = np.arange(nk, dtype=np.float64)[None, None, :]
    rsq = (i - ox) * (i - ox) + (j - oy) * (j - oy) + (k - oz) * (k - oz)
    return rsq < rad * rad


def images(shape, rad, centre):
    """Periodic images of a sphere whose node set meets the lattice."""
    out = []
    for di in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for dk in (-1, 0, 1):
                c = (centre[0] + di * shape[0], centre[1] + dj * shape[1], centre[2] + dk * shape[2])
                if all(-rad < c[a] < shape[a] - 1 + rad for a in range(3)):
                    out.append(c)
    return out


def _stamp(solid, rad, centre):
    """OR the nodes of a sphere (with periodic images) into solid, using a
    bounding box per image; returns the number of nodes newly set."""
    shape = solid.shape
    added = 0
    for c in images(shape, rad, centre):
        lo = [max(0, int(math.floor(c[a] - rad)) - 1) for a in range(3)]
        hi = [min(shape[a] - 1, int(math.ceil(c[a] + rad)) + 1) for a in range(3)]
        if any(lo[a] > hi[a] for a in range(3)):
            continue
        i = np.arange(lo[0], hi[0] + 1, dtype=np.float64)[:, None, None]
        j = np.arange(lo[1], hi[1] + 1, dtype=np.float64)[None, :, None]
        k = np.arange(lo[2], hi[2] + 1, dtype=np.float64)[None, None, :]
        rsq = (i - c[0]) * (i - c[0]) + (j - c[1]) * (j - c[1]) + (k - c[2]) * (k - c[2])
        box = solid[lo[0]:hi[0] + 1, lo[1]:hi[1] + 1, lo[2]:hi[2] + 1]
        inside = rsq < rad * rad
        added += int(np.count_nonzero(inside & ~box))
        box |= inside
    return added


def rsa_packing(n, phi, rmin, rmax, seed=1, overlap=False, max_tries=2_000_000):
    """Random sequential addition of spheres in a periodic n^3 box.

    Centres uniform in [0, n)^3, radii uniform in [rmin, rmax]; a sphere is
    accepted when its periodic minimum-image distance to every accepted one
    is at least the sum of the radii (any distance when overlap=True).
    Stops once the lattice solid fraction (nodes inside a sphere or an
    image) reaches phi.  Returns (spheres [(r, x, y, z)], solid mask)."""
    rng = SplitMix64(seed)
    solid = np.zeros((n, n, n), dtype=bool)
    spheres = []
    centres = np.zeros((0, 3))
    radii = np.zeros(0)
    tries = 0
    nset = 0
    target = phi * solid.size
    while nset < target:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"RSA stalled at solid fraction {nset / solid.size:.4f} < {phi}")
        c = np.array([rng.uniform(0.0, n) for _ in range(3)])
        r = rng.uniform(rmin, rmax)
        if not overlap and len(spheres):
            d = centres - c
            d -= n * np.round(d / n)
            if np.any(np.sqrt((d * d).sum(axis=1)) < radii + r):
                continue
        spheres.append((r, float(c[0]), float(c[1]), float(c[2])))
        centres = np.vstack([centres, c])
        radii = np.append(radii, r)
        nset += _stamp(solid, r, c)
    return spheres, solid


def packing_solid(n, spheres):
    solid = np.zeros((n, n, n), dtype=bool)
    for r, x, y, z in spheres:
        _stamp(solid, r, (x, y, z))
    return solid


def insert_spheres(L, lb, spheres, flatten=True):
    """insertsph for every sphere and each periodic image that meets the
    lattice (the scheme of examples/rcp_perm.pl:105-116), then flattenobj."""
    shape = (lb.esi, lb.esj, lb.esk)
    for r, x, y, z in spheres:
        for c in images(shape, r, (x, y, z)):
            L.insertsph(lb, r, c[0], c[1], c[2])
    if flatten:
        L.flattenobj(lb)


def insert_solid(L, lb, solid):
    """One object made of the given nodes, through insertlist (a node list
    file, reference src/lbobjs.c:128-165)."""
    idx = np.argwhere(solid)
    fd, path = tempfile.mkstemp(suffix=".lst", text=True)
    try:
        with os.fdopen(fd, "w") as f:
            np.savetxt(f, idx, fmt="%d")
        obj = L.insertlist(lb, path)
    finally:
        os.unlink(path)
    return obj


def sphere_drag(L, n=32, rad=4.5, force=1e-5, tau=1.0, precision=0):
    """Single fixed sphere at the box centre, Stokes flow, uniform body force
    along x (the small plain-method case)."""
    lb = L.newlb(n, n, n, "null")
    if L.extended:
        lb.precision = precision
    lb.tau = tau
    lb.stokes_flow = 1
    c = (n - 1) / 2.0
    obj = L.insertsph(lb, rad, c, c, c)
    L.syncobjs(lb)
    L.addbf(lb, force, 0.0, 0.0)
    return lb, obj


def permeability(lb, force):
    """Darcy constant k = vmean * eta / b (examples/rcp_perm.pl:161-165)."""
    eta = lb.rho0 * (lb.tau - 0.5) / 3.0
    return lb.vmeanx * eta / force


def packed_bed(L, n=128, phi=0.30, rmin=4.0, rmax=8.0, seed=1, force=1e-6, tau=1.0,
               precision=0, spheres=None, via_list=True):
    """Periodic random sphere packing, fixed objects, Stokes flow, body force
    along x (the packed-bed permeability case)."""
    if spheres is None:
        spheres, solid = rsa_packing(n, phi, rmin, rmax, seed)
    else:
        solid = packing_solid(n, spheres)
    lb = L.newlb(n, n, n, "null")
    if L.extended:
        lb.precision = precision
    lb.tau = tau
    lb.stokes_flow = 1
    if via_list:
        insert_solid(L, lb, solid)
        L.flattenobj(lb)
    else:
        insert_spheres(L, lb, spheres)
    L.syncobjs(lb)
    L.addbf(lb, force, 0.0, 0.0)
    return lb, spheres, solid
