"""GPU parity of the lattice Boltzmann update path against the CPU oracle.

FP64 populations must equal the oracle's bit for bit (the oracle itself
equals a strict build of the reference bit for bit, see test_oracle.py).
Reductions (mean flow, object force and torque) are summed in a different
order on the GPU, so they are compared to 1e-12 relative to their scale.
FP32 populations are compared to the FP64 oracle at the tolerances written
in each test.
"""

import numpy as np
import pytest

from scenarios import couette, objects_ft, two_spheres

pytestmark = pytest.mark.gpu

RED_TOL = 1e-12  # FP64 reductions: relative to the largest component


def close(a, b, tol):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= tol * scale


CASES = {
    "stokes": dict(),
    "navier_stokes": dict(stokes=0, tau=0.62),
    "skip_solid": dict(skip=1),
    "moving": dict(moving=1),
    "moving_ns_skip": dict(moving=1, stokes=0, skip=1, tau=0.6),
    "odd_steps": dict(steps=31),
    "thin_x": dict(dims=(2, 9, 11)),
    "thin_xy": dict(dims=(1, 2, 13), moving=1),
    "small": dict(dims=(3, 3, 3), steps=7),
    "ragged": dict(dims=(7, 13, 33), steps=12),
    # rows long enough for whole warps away from the lattice's faces (the
    # offset-table addressing of the pull-and-push update)
    "long_rows": dict(dims=(5, 7, 100), steps=9),
    "long_rows_moving_ns": dict(dims=(4, 6, 160), moving=1, stokes=0, tau=0.7, steps=10),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_bit_exact(gpu, orc, name):
    cfg = CASES[name]
    lg = two_spheres(gpu, **cfg)
    lo = two_spheres(orc, **cfg)
    pg, po = lg.pops(), lo.pops()
    assert np.array_equal(pg, po), f"max |diff| = {np.abs(pg - po).max():.3e}"
    assert lg.step == lo.step and lg.status == lo.status
    vg = [lg.vmeanx, lg.vmeany, lg.vmeanz]
    vo = [lo.vmeanx, lo.vmeany, lo.vmeanz]
    assert close(vg, vo, RED_TOL), (vg, vo)
    assert close(objects_ft(lg)[:, :3], objects_ft(lo)[:, :3], RED_TOL)
    assert close(objects_ft(lg)[:, 3:], objects_ft(lo)[:, 3:], RED_TOL)
    # node forces of the last measurement
    for f in ("fx", "fy", "fz"):
        assert close(lg.array(f), lo.array(f), RED_TOL)


def test_graph_steps_equal_single_steps(gpu):
    a = two_spheres(gpu, steps=260, use_steps=False, measure=False)
    b = two_spheres(gpu, steps=260, use_steps=True, measure=False)
    assert np.array_equal(a.pops(), b.pops())
    assert a.step == b.step == 260


def test_separate_phases(gpu, orc):
    """bbl / propagate / collide called one by one, mixed with lbstep and
    bblforce, as a driver of the reference may do."""
    out = []
    for L in (gpu, orc):
        lb = two_spheres(L, steps=5, measure=False, moving=1)
        L.bbl(lb); L.propagate(lb); L.collide(lb)
        L.lbstep(lb)
        L.zeroforce(lb)
        L.bblforce(lb); L.propagate(lb)
        L.accvmean(lb, 1.0)
        L.collide(lb)
        L.lbstep(lb)
        L.normforce(lb, 0.5)
        L.distribf(lb)
        out.append((lb.pops(), lb.vmeanx, objects_ft(lb), lb.array("fx").copy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert abs(out[0][1] - out[1][1]) <= RED_TOL * abs(out[1][1])
    assert close(out[0][2], out[1][2], RED_TOL)
    assert close(out[0][3], out[1][3], RED_TOL)


def test_psi_weighted_mean(gpu, orc):
    vg = two_spheres(gpu, psi=True, steps=9)
    vo = two_spheres(orc, psi=True, steps=9)
    assert close([vg.vmeanx, vg.vmeany], [vo.vmeanx, vo.vmeany], RED_TOL)


def test_nonuniform_body_force(gpu, orc):
    out = []
    for L in (gpu, orc):
        lb = two_spheres(L, steps=0, measure=False)
        bx = lb.array("bx")
        bx[: lb.nnodes // 3] *= 3.0
        L.lbpush(lb)
        for _ in range(11):
            L.lbstep(lb)
        L.measure(lb)
        out.append((lb.pops(), lb.vmeanx))
    assert np.array_equal(out[0][0], out[1][0])


def test_warm_start_from_velocity(gpu, orc):
    out = []
    for L in (gpu, orc):
        lb = two_spheres(L, steps=0, measure=False, stokes=0, tau=0.7)
        n = lb.nnodes
        x = np.arange(n, dtype=float)
        rho = 72.0 + 1e-3 * np.sin(x)
        ux, uy, uz = 1e-3 * np.cos(x), 2e-4 * np.sin(0.3 * x), -1e-4 * np.ones(n)
        L.lbsetvel(lb, rho, ux, uy, uz)
        L.lbsteps(lb, 4)
        out.append(lb.pops())
    assert np.array_equal(out[0], out[1])


def test_couette_wall_force_exact(gpu):
    """Planar Couette flow: wall force 2 eta (v1 - v2)/h, exact in LB
    (examples/planar_couette.pl; needs vspread, which the example omits)."""
    lb, w1, w2, expect = couette(gpu, steps=4000)
    assert abs(abs(w1.frcx) - expect) < 1e-9 * expect
    assert abs(abs(w2.frcx) - expect) < 1e-9 * expect
    assert w1.frcx * w2.frcx < 0


def test_fp32_close_to_fp64(gpu, orc):
    """FP32 populations with FP32 collision, FP64 reductions: mean flow and
    drag within 1e-4 relative of the FP64 oracle after 200 steps."""
    lg = two_spheres(gpu, steps=200, precision=1)
    lo = two_spheres(orc, steps=200)
    assert abs(lg.vmeanx - lo.vmeanx) <= 1e-4 * abs(lo.vmeanx)
    assert close(objects_ft(lg)[:, :3], objects_ft(lo)[:, :3], 1e-4)
    pg, po = lg.pops(), lo.pops()
    assert np.abs(pg - po).max() <= 1e-4 * np.abs(po).max()


def test_precision_switch_keeps_state(gpu):
    """Changing lb->precision between steps carries the state over: 20 FP64
    steps, one FP32 step, back to FP64 equals 21 FP64 steps to FP32
    rounding."""
    a = two_spheres(gpu, steps=20, measure=False)
    a.precision = 1
    gpu.lbstep(a)
    a.precision = 0
    b = two_spheres(gpu, steps=21, measure=False)
    pa, pb = a.pops(), b.pops()
    assert a.step == b.step == 21
    assert np.abs(pa - pb).max() < 1e-6 * np.abs(pb).max()


def test_large_lattice_many_objects(gpu, orc):
    """A lattice large enough for the host loops of the geometry upload to
    run in several ranges (3.1 M nodes), with 40 spheres spread over it: the
    dense object index keeps the first-seen order, so every object's force
    and torque and every population equal the oracle's (FP64, bit-exact
    populations)."""
    rng = np.random.default_rng(31)
    dims = (192, 128, 128)
    spheres = [(rng.uniform(3.0, 6.0), *(rng.uniform(0, d) for d in dims)) for _ in range(40)]
    lbs = []
    for L in (gpu, orc):
        lb = L.newlb(*dims, "null")
        if L.extended:
            lb.precision = 0
        lb.tau = 0.8
        for r, x, y, z in spheres:
            assert L.insertsph(lb, r, x, y, z) is not None
        L.addbf(lb, 1e-5, 2e-6, 0.0)
        for _ in range(3):
            L.lbstep(lb)
        L.measure(lb)
        lbs.append(lb)
    g, o = lbs
    assert np.array_equal(g.pops(), o.pops())
    fg, fo = objects_ft(g), objects_ft(o)
    assert fg.shape == fo.shape == (40, 6)
    assert close(fg[:, :3], fo[:, :3], RED_TOL)
    assert close(fg[:, 3:], fo[:, 3:], RED_TOL)


@pytest.mark.parametrize("precision", [0, 1])
def test_population_transfer_paths(gpu, precision):
    """Download and upload of the populations through both host paths --
    straight to and from the page-locked mirror lb->a, and through the
    device staging buffer for a pageable array -- give the same values."""
    import ctypes as C
    lb = two_spheres(gpu, dims=(20, 17, 33), steps=11, measure=False, precision=precision)
    gpu.lbpull(lb)
    pinned = lb.pops().copy()
    dev_fn = gpu.dll.slb_device
    dev_fn.argtypes = [C.c_void_p]
    dev_fn.restype = C.c_void_p
    get = gpu.dll.slbc_get_pops
    get.argtypes = [C.c_void_p, C.c_void_p]
    get.restype = C.c_int
    put = gpu.dll.slbc_put_pops
    put.argtypes = [C.c_void_p, C.c_void_p]
    put.restype = C.c_int
    dev = dev_fn(lb)
    pageable = np.zeros(15 * lb.nnodes)
    assert get(dev, pageable.ctypes.data) == 0
    assert np.array_equal(pageable, pinned.ravel())
    # a changed state uploaded from pageable memory reads back through the mirror
    changed = pageable * (1.0 + 1e-3 * np.sin(np.arange(pageable.size)))
    if precision == 1:
        changed = changed.astype(np.float32).astype(np.float64)
    assert put(dev, changed.ctypes.data) == 0
    a = lb.array("a")
    assert get(dev, a.ctypes.data) == 0
    assert np.array_equal(a.ravel(), changed)
