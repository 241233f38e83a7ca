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
