"""Scenario drivers shared by the tests: each runs the same call sequence of
the SunlightLB API on any library (GPU, oracle, reference build) and returns
what the tests compare."""

import numpy as np


def two_spheres(L, dims=(16, 17, 18), tau=0.8, stokes=1, skip=0, moving=0, steps=30,
                bf=(1e-4, 2e-5, 0.0), precision=0, measure=True, use_steps=False, psi=False):
    lb = L.newlb(dims[0], dims[1], dims[2], "null")
    if L.extended:
        lb.precision = precision
    lb.tau = tau
    lb.stokes_flow = stokes
    lb.skip_solid = skip
    lb.objects_moving = moving
    ni, nj, nk = dims
    o1 = L.insertsph(lb, max(1.0, 0.28 * min(dims)), 0.47 * ni, 0.47 * nj, 0.46 * nk)
    o2 = L.insertsph(lb, max(1.0, 0.16 * min(dims)), 0.06 * ni, 0.88 * nj, 0.17 * nk)
    assert o1 is not None and o2 is not None
    L.addbf(lb, *bf)
    if moving:
        o1.velx = 1e-3; o1.angz = 2e-4; o2.vely = -3e-4; o2.angx = 1e-4
        L.vspread(lb)
    if psi:
        w = np.linspace(0.5, 1.5, lb.nnodes)
        lb._keep_psi = w
        import ctypes as C
        lb.psi = w.ctypes.data_as(C.POINTER(C.c_double))
    if use_steps and L.has("lbsteps"):
        L.lbsteps(lb, steps)
    else:
        for _ in range(steps):
            L.lbstep(lb)
    if measure:
        L.measure(lb)
    return lb


def objects_ft(lb):
    return np.array([[o.frcx, o.frcy, o.frcz, o.trqx, o.trqy, o.trqz] for o in lb.objects()])


def couette(L, h=10, vel1=0.11, vel2=-0.07, tau=0.8, steps=5000, precision=0):
    """Planar Couette flow between moving walls (examples/planar_couette.pl)
    with the wall velocities spread to the nodes (vspread)."""
    lb = L.newlb(1, 1, 2 * (h + 1), "null")
    if L.extended:
        lb.precision = precision
    lb.stokes_flow = 1
    lb.objects_moving = 1
    lb.tau = tau
    w1 = L.insertwall(lb, "z", 0)
    w2 = L.insertwall(lb, "z", h + 1)
    w1.velx = vel1
    w2.velx = vel2
    L.vspread(lb)
    if L.has("lbsteps"):
        L.lbsteps(lb, steps)
    else:
        for _ in range(steps):
            L.lbstep(lb)
    L.measure(lb)
    eta = lb.rho0 * (lb.tau - 0.5) / 3.0
    return lb, w1, w2, 2 * eta * (vel1 - vel2) / h


FILE_OUTPUTS = (
    ("vel.bin", "lbsavevel", "binary"), ("vel.txt", "lbsavevel", "ascii"),
    ("frc.bin", "lbsavefrc", "binary"), ("frc.txt", "lbsavefrc", "ascii"), ("frc.lst", "lbsavefrc", "list"),
    ("map.lst", "lbsavemap", "list"), ("map.chr", "lbsavemap", "char"),
    ("obj.txt", "lbsaveobj", None), ("vsave.txt", "vsave", None),
    ("str.bin", "lbsavestr", "binary"), ("str.txt", "lbsavestr", "ascii"),
)


def write_files(L, lb, outdir):
    """Write every field and object file of the reference's file API
    (src/lbstore.c:227-678, src/lbmeasure.c:129-203) from lb into outdir, in
    a fixed order (lbsavestr advances the lattice one step, so it comes
    last); returns {file name: bytes}.  vsave writes the field that vzero and
    two vgrab calls (pre- and post-collision of one more step) accumulate."""
    import os
    out = {}
    for name, fn, typ in FILE_OUTPUTS:
        path = os.path.join(outdir, name)
        if fn == "vsave":
            L.vzero(lb)
            L.vgrab(lb, 0.5)
            L.bbl(lb); L.propagate(lb)
            L.vgrab(lb, 0.5)
            L.collide(lb)
            L.vsave(lb, path)
        elif typ is None:
            L.call(fn, lb, path)
        else:
            L.call(fn, lb, path, typ)
        with open(path, "rb") as f:
            out[name] = f.read()
    return out


def file_case(L, outdir, dims=(9, 10, 11), steps=12, moving=1, skip=0, stokes=1, tau=0.8):
    """A lattice with two spheres (moving walls by default), stepped and
    measured so that node forces exist, then written to every file type."""
    lb = two_spheres(L, dims=dims, steps=steps, moving=moving, skip=skip, stokes=stokes, tau=tau)
    return lb, write_files(L, lb, outdir)


def reload_case(L, files_dir, kind, dims=(9, 10, 11), moving=1, skip=0, stokes=1, tau=0.8):
    """A fresh lattice of the same geometry loaded from a written file:
    kind 'vel.bin' / 'vel.txt' through lbloadvel (then 3 steps), or
    'obj.txt' through lbloadobj (object positions and velocities)."""
    import os
    lb = two_spheres(L, dims=dims, steps=0, moving=moving, skip=skip, stokes=stokes, tau=tau, measure=False)
    path = os.path.join(files_dir, kind)
    if kind.startswith("vel"):
        lb.rescale = 0.75
        L.lbloadvel(lb, path, "binary" if kind.endswith(".bin") else "ascii")
        for _ in range(3):
            L.lbstep(lb)
        return lb, lb.pops()
    for o in lb.objects():
        o.posx = o.posy = o.posz = o.velx = o.angz = 0.0
    lb.rescale = 2.0
    L.lbloadobj(lb, path)
    return lb, objects_state(lb)


def objects_state(lb):
    return np.array([[o.id, o.base_obj.contents.id, o.posx, o.posy, o.posz, o.velx, o.vely, o.velz,
                      o.angx, o.angy, o.angz] for o in lb.objects()])


def mpsubs_case(L, outdir, n=10, steps=15):
    """Tracer set from a byte image by mpsubs over a sub-region (one run of
    data shorter than the region, so the short-data rows are exercised),
    then moment-propagation steps on a live flow."""
    import os
    lb = L.newlb(n, n + 1, n + 2, "null")
    lb.tau = 0.7
    L.insertsph(lb, 2.5, 4.5, 5.0, 6.0)
    L.addbf(lb, 1e-3, 2e-4, 0)
    for _ in range(6):
        L.lbstep(lb)
    mp = L.newmp(lb, "null")
    mp.alpha = 0.25
    L.mpinit(mp)
    region = (1, 7, 2, 9, 0, 11)
    count = (7 * 8 * 12) - 30  # the last 2.5 k-rows of the region get no data
    data = bytes((37 * i + 11) % 256 for i in range(count))
    path = os.path.join(outdir, "subs.dat")
    with open(path, "wb") as f:
        f.write(data)
    L.mpsubs(mp, path, *region, 0.8)
    if L.has("mppull"):
        L.mppull(mp)
    p0 = mp.field().copy()
    for s in range(steps):
        L.mpstep(mp)
        if s % 3 == 2:
            L.lbstep(lb)
    if L.has("mppull"):
        L.mppull(mp)
    return p0, mp.field().copy()


def translate_case(L, dims=(20, 18, 22), rad=3.6, centre=(17.3, 8.1, 1.7), step=(0.61, -0.43, 0.29), moves=6,
                   every=7, moving=1, stokes=1, skip=0, tau=0.8, precision=0, bf=(1e-4, 2e-5, 0.0),
                   ang=(0.0, 0.0, 1e-3), measure=True):
    """A sphere (with its periodic images, flattened into one object) near
    the periodic boundary, translated by `step` every `every` update steps
    (an odd count, so moves meet both storage layouts), `moves` times, then
    measured.  Returns (lb, obj)."""
    from sunlightlb_gb300 import workloads as W
    lb = L.newlb(dims[0], dims[1], dims[2], "null")
    if L.extended:
        lb.precision = precision
    lb.tau = tau
    lb.stokes_flow = stokes
    lb.skip_solid = skip
    lb.objects_moving = moving
    c = list(centre)
    for im in W.images(dims, rad, c):
        L.insertsph(lb, rad, im[0], im[1], im[2])
    obj = L.flattenobj(lb)
    obj.posx, obj.posy, obj.posz = c  # flattenobj leaves the centroid of the nodes
    obj.velx, obj.vely, obj.velz = (step[0] / every * 0.05, step[1] / every * 0.05, step[2] / every * 0.05)
    obj.angx, obj.angy, obj.angz = ang
    L.syncobjs(lb)
    if moving:
        L.vspread(lb)
    L.addbf(lb, *bf)
    for _ in range(moves):
        for _ in range(every):
            L.lbstep(lb)
        c = [c[a] + step[a] for a in range(3)]
        L.lbtranslate(lb, obj, rad, *c)
    if measure:
        for _ in range(every):
            L.lbstep(lb)
        L.measure(lb)
    return lb, obj


def object_ids(lb):
    ids = {o.address: o.id for o in lb.objects()}
    raw = lb.array("obj")
    return np.array([ids.get(int(p), -2) if p else -1 for p in raw])


def vacf_case(L, outdir, dims=(12, 13, 14), steps=25, direction="xx", second_init=False, psi=False, alpha=0.25,
              ads=False):
    """Tracer velocity autocorrelation (src/mpvacf.c) on a frozen flow past a
    sphere with an adsorbing patch: mpvacfinit (or mpvacfinit2), then per
    step an update of both tracer fields and mpvacf; returns (diffusion
    coefficient, P, P2, file bytes)."""
    import os
    lb = L.newlb(dims[0], dims[1], dims[2], "null")
    lb.tau = 0.7
    L.insertsph(lb, 3.2, 5.5, 6.0, 7.2)
    L.addbf(lb, 2e-3, 5e-4, -3e-4)
    if psi:
        w = np.linspace(0.6, 1.4, lb.nnodes)
        lb._keep_psi = w
        import ctypes as C
        lb.psi = w.ctypes.data_as(C.POINTER(C.c_double))
    for _ in range(30):
        L.lbstep(lb)
    mp, mp2 = L.newmp(lb, "null"), L.newmp(lb, "null")
    for m in (mp, mp2):
        m.alpha = alpha
        L.mpinit(m)
    if ads:  # adsorbing boundary nodes on half the sphere: their links are left out
        L.adslab(mp, -1.0, 5.5, -1.0, 20.0, -1.0, 20.0)
    if second_init:
        L.mpvacfinit(mp, mp2, direction, steps + 2)
        L.mpvacfinit2(mp, mp2)
    else:
        L.mpvacfinit(mp, mp2, direction, steps + 2)
    for _ in range(steps):
        L.mpstep(mp)
        L.mpstep(mp2)
        L.mpvacf(mp, mp2)
    path = os.path.join(outdir, "vacf.dat")
    d = L.mpvacfwr(mp, mp2, path, 5)
    if L.has("mppull"):
        L.mppull(mp)
        L.mppull(mp2)
    with open(path, "rb") as f:
        data = f.read()
    return d, mp.field().copy(), mp2.field().copy(), data
