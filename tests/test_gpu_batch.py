"""Batches of lattices advanced in one persistent launch (batchsteps)
against the same lattices stepped one at a time (lbsteps) and against the
oracle: the populations must be identical bit for bit, FP32 and FP64."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DOMAINS = [  # dims, sphere radius, centre (fractions), velocity
    ((12, 13, 14), 3.0, (0.4, 0.5, 0.55), (1e-3, 0.0, 0.0)),
    ((16, 16, 16), 4.2, (0.3, 0.6, 0.5), (0.0, -7e-4, 3e-4)),
    ((9, 20, 11), 2.5, (0.5, 0.2, 0.5), (2e-4, 5e-4, -6e-4)),
    ((24, 24, 24), 5.5, (0.51, 0.49, 0.5), (-5e-4, 4e-4, 6e-4)),
    ((7, 7, 7), 2.0, (0.5, 0.5, 0.5), (0.0, 0.0, 1e-3)),
]


def domain(L, dims, rad, frac, vel, precision=1, moving=1, stokes=1, tau=1.0, bf=(2e-5, 0.0, 0.0)):
    lb = L.newlb(dims[0], dims[1], dims[2], "null")
    if L.extended:
        lb.precision = precision
    lb.tau = tau
    lb.stokes_flow = stokes
    lb.objects_moving = moving
    o = L.insertsph(lb, rad, frac[0] * dims[0], frac[1] * dims[1], frac[2] * dims[2])
    assert o is not None
    if moving:
        o.velx, o.vely, o.velz = vel
        o.angz = 1e-4
        L.vspread(lb)
    L.addbf(lb, *bf)
    L.lbstep(lb)  # into the collide-stream cycle
    return lb


def build(L, precision, **kw):
    return [domain(L, d, r, c, v, precision, **kw) for d, r, c, v in DOMAINS]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("steps", [37, 120])
@pytest.mark.parametrize("mode", [0, 1])
def test_batch_equals_one_at_a_time(gpu, precision, steps, mode):
    """mode 0: packed tiles (120 steps include two graph replays); mode 1:
    persistent launch."""
    batch = build(gpu, precision)
    alone = build(gpu, precision)
    b = gpu.newbatch()
    gpu.batchmode(b, mode)
    for lb in batch:
        gpu.batchadd(b, lb)
    assert gpu.batchsize(b) == len(DOMAINS)
    gpu.batchsteps(b, steps)
    for lb in alone:
        gpu.lbsteps(lb, steps)
    for lb1, lb2 in zip(batch, alone):
        assert lb1.step == lb2.step
        assert np.array_equal(lb1.pops(), lb2.pops())
        gpu.measure(lb1)
        gpu.measure(lb2)
        f1 = [(o.frcx, o.frcy, o.frcz, o.trqx, o.trqy, o.trqz) for o in lb1.objects()]
        f2 = [(o.frcx, o.frcy, o.frcz, o.trqx, o.trqy, o.trqz) for o in lb2.objects()]
        assert f1 == f2
    gpu.freebatch(b)


def test_batch_fp64_equals_oracle(gpu, orc):
    batch = build(gpu, 0)
    ref = build(orc, 0)
    b = gpu.newbatch()
    for lb in batch:
        gpu.batchadd(b, lb)
    gpu.batchsteps(b, 25)
    gpu.batchmode(b, 1)
    gpu.batchsteps(b, 30)  # the batch is reused, each lattice continues
    for lb in ref:
        for _ in range(55):
            orc.lbstep(lb)
    for lb1, lb2 in zip(batch, ref):
        assert np.array_equal(lb1.pops(), lb2.pops())
    gpu.freebatch(b)


def test_batch_mixed_classes_and_members(gpu):
    """Lattices with and without moving walls, uniform and per-node body
    forces (one launch per class), one member out of the collide-stream
    cycle (stepped on its own) and one of another precision."""
    kinds = [dict(moving=1), dict(moving=0), dict(moving=0, stokes=0, tau=0.7), dict(moving=1, stokes=0, tau=0.8)]
    batch, alone = [], []
    for n, (d, r, c, v) in enumerate(DOMAINS[:4]):
        batch.append(domain(gpu, d, r, c, v, 1, **kinds[n]))
        alone.append(domain(gpu, d, r, c, v, 1, **kinds[n]))
    for L in (batch, alone):
        # per-node body force on the third lattice (written into lb->bx and
        # handed over with lbpush)
        lb = L[2]
        bx = lb.array("bx")
        bx[:] = 1e-5 * (1.0 + 0.5 * np.sin(np.arange(lb.nnodes)))
        gpu.lbpush(lb)
        gpu.bbl(L[1])  # out of cycle
    other = domain(gpu, (10, 11, 12), 3.0, (0.5, 0.5, 0.5), (1e-3, 0, 0), 0)
    other2 = domain(gpu, (10, 11, 12), 3.0, (0.5, 0.5, 0.5), (1e-3, 0, 0), 0)
    b = gpu.newbatch()
    for lb in batch + [other]:
        gpu.batchadd(b, lb)
    gpu.batchsteps(b, 41)
    for lb in alone + [other2]:
        gpu.lbsteps(lb, 41)
    for lb1, lb2 in zip(batch + [other], alone + [other2]):
        assert np.array_equal(lb1.pops(), lb2.pops())
    gpu.freebatch(b)
