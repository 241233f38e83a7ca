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


def _splitmix_block(state, count):
    """The next `count` outputs of a splitmix64 generator in `state` (the
    generator is a counter hash, so a block is computed at once); returns
    (new state, uint64 array)."""
    k = np.arange(1, count + 1, dtype=np.uint64)
    z = np.uint64(state) + k * np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    return (state + count * 0x9E3779B97F4A7C15) & MASK64, z


def _min_image_hits(cand, rc, cen, rad, n):
    """For each candidate row of cand (m x 3) with radius rc (m), whether any
    sphere of cen/rad (m x K x 3 / m x K, NaN radius = empty) overlaps it
    under the periodic minimum-image convention."""
    d = cen - cand[:, None, :]
    d -= n * np.round(d / n)
    dist = np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2])
    return np.any(dist < rad + rc[:, None], axis=1)


def rsa_packing(n, phi, rmin, rmax, seed=1, overlap=False, max_tries=50_000_000):
    """Random sequential addition of spheres in a periodic n^3 box, computed
    by the library's rsapacking (C, the same draws and decisions as
    rsa_packing_numpy below, bit for bit, ~20x faster).  Returns
    (spheres [(r, x, y, z)], solid mask (n, n, n) bool)."""
    import ctypes as C
    from . import library
    f = library().dll.rsapacking
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_ulonglong, C.c_int, C.c_long,
                  C.c_void_p, C.c_int, C.c_void_p]
    # room for the spheres: the solid volume over the smallest sphere's, and more
    cap = int(phi * n ** 3 / (4.0 / 3.0 * math.pi * max(rmin - 1.0, 0.5) ** 3)) * 2 + 1024
    out = np.zeros((cap, 4), dtype=np.float64)
    solid = np.zeros((n, n, n), dtype=np.uint8)
    m = f(n, phi, rmin, rmax, seed & MASK64, int(bool(overlap)), max_tries, out.ctypes.data, cap,
          solid.ctypes.data)
    if m == -1:
        raise RuntimeError(f"RSA stalled short of solid fraction {phi} (more than {max_tries} tries)")
    if m < 0:
        raise RuntimeError(f"rsapacking failed ({m})")
    return [tuple(float(v) for v in row) for row in out[:m]], solid.view(bool)


def rsa_packing_numpy(n, phi, rmin, rmax, seed=1, overlap=False, max_tries=50_000_000, block=4096):
    """Random sequential addition of spheres in a periodic n^3 box (numpy
    formulation, the definition rsapacking is tested against).

    Centres uniform in [0, n)^3, radii uniform in [rmin, rmax] (four
    splitmix64 draws per try: x, y, z, r); a sphere is accepted when its
    periodic minimum-image distance to every accepted one is at least the sum
    of the radii (any distance when overlap=True).  Stops once the lattice
    solid fraction (nodes inside a sphere or an image) reaches phi.  Returns
    (spheres [(r, x, y, z)], solid mask).

    Tries are drawn a block at a time and tested together against the
    spheres accepted before the block (binned in cubic cells of side
    >= 2 rmax, so only the 27 cells around a candidate matter); the few
    survivors are then taken in order and tested against the spheres
    accepted earlier in the same block, which gives exactly the sequential
    decisions."""
    state = seed & MASK64
    solid = np.zeros((n, n, n), dtype=bool)
    spheres = []
    ncell = max(1, int(n // (2.0 * rmax)))
    cw = n / ncell
    cap = 8
    grid = np.full((ncell, ncell, ncell, cap), -1, dtype=np.int64)
    fill = np.zeros((ncell, ncell, ncell), dtype=np.int64)
    cen = np.zeros((1024, 3))
    rad = np.zeros(1024)
    offs = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])
    tries = 0
    nset = 0
    target = phi * solid.size
    while nset < target:
        state, z = _splitmix_block(state, 4 * block)
        u = ((z >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))).reshape(block, 4)
        C = 0.0 + (n - 0.0) * u[:, :3]
        R = rmin + (rmax - rmin) * u[:, 3]
        alive = np.ones(block, dtype=bool)
        ns = len(spheres)
        if not overlap and ns:
            if ncell < 3:
                hit = _min_image_hits(C, R, np.broadcast_to(cen[:ns], (block, ns, 3)),
                                      np.broadcast_to(rad[:ns], (block, ns)), n)
            else:
                ci = np.minimum(ncell - 1, (C // cw).astype(np.int64))
                nb = (ci[:, None, :] + offs[None, :, :]) % ncell
                idx = grid[nb[..., 0], nb[..., 1], nb[..., 2]].reshape(block, -1)
                valid = idx >= 0
                safe = np.where(valid, idx, 0)
                r_nb = np.where(valid, rad[safe], np.nan)
                hit = _min_image_hits(C, R, cen[safe], r_nb, n)
            alive &= ~hit
        first_new = ns
        for t in np.nonzero(alive)[0] if not overlap else range(block):
            if tries + t + 1 > max_tries:
                raise RuntimeError(f"RSA stalled at solid fraction {nset / solid.size:.4f} < {phi}")
            c = C[t]
            r = float(R[t])
            if not overlap and len(spheres) > first_new:
                m = len(spheres)
                if _min_image_hits(c[None, :], np.array([r]), cen[None, first_new:m], rad[None, first_new:m], n)[0]:
                    continue
            m = len(spheres)
            if m == len(rad):
                cen = np.vstack([cen, np.zeros_like(cen)])
                rad = np.concatenate([rad, np.zeros_like(rad)])
            cen[m] = c
            rad[m] = r
            cell = tuple(min(ncell - 1, int(c[a] // cw)) for a in range(3))
            if fill[cell] == cap:
                grid = np.concatenate([grid, np.full(grid.shape, -1, dtype=np.int64)], axis=3)
                cap *= 2
            grid[cell + (fill[cell],)] = m
            fill[cell] += 1
            spheres.append((r, float(c[0]), float(c[1]), float(c[2])))
            nset += _stamp(solid, r, c)
            if nset >= target:
                break
        tries += block
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
    if L.has("insertspheres"):  # the node tests of all of them on the GPU
        rad, cen = [], []
        for r, x, y, z in spheres:
            for c in images(shape, r, (x, y, z)):
                rad.append(r)
                cen.append(c)
        if rad:
            cen = np.array(cen, dtype=np.float64)
            L.insertspheres(lb, len(rad), np.array(rad, dtype=np.float64), cen[:, 0], cen[:, 1], cen[:, 2])
    else:
        for r, x, y, z in spheres:
            for c in images(shape, r, (x, y, z)):
                L.insertsph(lb, r, c[0], c[1], c[2])
    if flatten:
        L.flattenobj(lb)


def insert_solid(L, lb, solid):
    """One object made of the given nodes: insertmask when the library has
    it, else insertlist (a node list file, reference src/lbobjs.c:128-165)."""
    if L.has("insertmask"):
        m = np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1)
        return L.insertmask(lb, m.ctypes.data)
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


def large_bed(L, n=512, phi=0.35, rmin=6.0, rmax=12.0, seed=4, precision=1, tau=1.0):
    """Periodic packed bed for flow with a passive scalar: seeded RSA
    spheres (each sphere plus its periodic images inserted with insertsph,
    then flattenobj, as examples/rcp_perm.pl:105-116 does), fixed objects.
    Returns (lb, spheres)."""
    spheres, _ = rsa_packing(n, phi, rmin, rmax, seed)
    lb = L.newlb(n, n, n, "null")
    if L.extended:
        lb.precision = precision
    lb.tau = tau
    lb.stokes_flow = 1
    insert_spheres(L, lb, spheres)
    L.syncobjs(lb)
    return lb, spheres


def pore_reynolds(lb, diameter):
    """Re = vmeanx * d / nu with nu = (tau - 1/2) / 3 (lattice units)."""
    return lb.vmeanx * diameter / ((lb.tau - 0.5) / 3.0)


def calibrated_flow(L, lb, diameter, re_target=1.0, b0=1e-6, stokes_tol=1e-5, tol=1e-7, check=100,
                    maxsteps=40000):
    """Body force along x that gives a pore Reynolds number re_target: a
    Stokes run at b0 to convergence fixes the linear response, b = b0 *
    re_target / Re(b0); the flow is then run with the inertial term
    (stokes_flow = 0) at b to convergence.  Returns a dict of the steps,
    forces and Reynolds numbers."""
    lb.stokes_flow = 1
    L.zerobf(lb)
    L.addbf(lb, b0, 0.0, 0.0)
    s0 = L.lbconverge(lb, check, stokes_tol, maxsteps)
    re0 = pore_reynolds(lb, diameter)
    b = b0 * re_target / re0
    lb.stokes_flow = 0
    L.zerobf(lb)
    L.addbf(lb, b, 0.0, 0.0)
    s1 = L.lbconverge(lb, check, tol, maxsteps)
    return {"stokes_steps": s0, "b_stokes": b0, "re_stokes": re0, "b": b, "steps": s1,
            "re": pore_reynolds(lb, diameter), "vmeanx": lb.vmeanx, "converged": s1 < maxsteps}


def tracer_breakthrough(L, lb, steps, precision=1, alpha=0.5, adprob=0.01, sample_every=500, source=1.0):
    """Passive scalar in the frozen flow of lb, carried along x through a
    column: newmp + mpinit, every boundary node adsorbing (adall) with
    probability adprob per encounter, a constant-concentration source plane
    x = 0 (p = source) and an absorbing plane x = esi - 1 (p = 0), both re-set
    before every update with mpwall.  The absorbing plane keeps the source
    from reaching the far end through the periodic wrap; the breakthrough
    curve is the mean tracer over the fluid nodes of the plane before it,
    x = esi - 2, every sample_every updates.  Returns (mp, curve, balances):
    curve = [(step, mean)], balances = [(step, fluid, adsorbed, all,
    injected)] with the tracer the two planes added (the absorbing plane
    counts negative)."""
    mp = L.newmp(lb, "null")
    if L.extended:
        mp.precision = precision
        mp.adprob = adprob
    mp.alpha = alpha
    L.mpinit(mp)
    L.adall(mp)
    sink = lb.esi - 1
    probe = max(0, lb.esi - 2)
    curve, balances = [], []
    for s in range(1, steps + 1):
        L.mpwall(mp, "x", 0, source)
        L.mpwall(mp, "x", sink, 0.0)
        L.mpstep(mp)
        if s % sample_every == 0 or s == steps:
            curve.append((s, L.mpplane(mp, "x", probe)))
            balances.append((s, L.mptotal(mp, "fluid"), L.mptotal(mp, "adsorbed"), L.mptotal(mp, "all"),
                             L.mptotal(mp, "injected")))
    return mp, curve, balances
