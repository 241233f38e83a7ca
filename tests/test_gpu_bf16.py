"""BF16 deviation storage (lb->precision = SLB_BF16) against the FP64 oracle.

Populations are stored as BF16 deviations from the equilibrium of each
node's FP32 moments.  At tau = 1 in Stokes flow the collision returns the
equilibrium exactly, so the variant is FP32-accurate; otherwise the BF16
rounding touches only the non-equilibrium part.  Tolerances are written in
each test.
"""

import numpy as np
import pytest

from scenarios import objects_ft, two_spheres

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_bf16_tau1_stokes_is_fp32_accurate(gpu, orc):
    g = two_spheres(gpu, tau=1.0, steps=150, precision=2)
    o = two_spheres(orc, tau=1.0, steps=150)
    assert rel(g.pops(), o.pops()) < 2e-5
    assert abs(g.vmeanx - o.vmeanx) <= 2e-5 * abs(o.vmeanx)
    assert rel(objects_ft(g)[:, :3], objects_ft(o)[:, :3]) < 2e-5


@pytest.mark.parametrize("cfg", [dict(tau=0.8), dict(tau=0.62, stokes=0), dict(tau=0.8, moving=1)])
def test_bf16_general_relaxation(gpu, orc, cfg):
    """tau != 1: the stored deviation is the non-equilibrium part; mean
    flow and drag within 2e-3 relative, populations within 2e-3 of their
    largest value, after 120 steps."""
    g = two_spheres(gpu, steps=120, precision=2, **cfg)
    o = two_spheres(orc, steps=120, **cfg)
    assert rel(g.pops(), o.pops()) < 2e-3
    assert abs(g.vmeanx - o.vmeanx) <= 2e-3 * abs(o.vmeanx)
    assert rel(objects_ft(g)[:, :3], objects_ft(o)[:, :3]) < 2e-3


def test_bf16_warm_start_and_graph_steps(gpu, orc):
    out = []
    for L, prec in ((gpu, 2), (orc, 0)):
        lb = two_spheres(L, steps=0, measure=False, tau=1.0)
        if L.extended:
            lb.precision = prec
        n = lb.nnodes
        x = np.arange(n, dtype=float)
        L.lbsetvel(lb, None, 1e-3 * np.cos(x), 2e-4 * np.sin(0.3 * x), -1e-4 * np.ones(n))
        L.lbsteps(lb, 130)
        L.measure(lb)
        out.append((lb.pops(), lb.vmeanx))
    assert rel(out[0][0], out[1][0]) < 2e-5
    assert abs(out[0][1] - out[1][1]) <= 2e-5 * abs(out[1][1])


def test_bf16_separate_phases_move_to_fp32(gpu, orc):
    """A separate bounce-back phase needs stored populations: the lattice
    moves to FP32 and keeps its state."""
    g = two_spheres(gpu, tau=1.0, steps=20, measure=False, precision=2)
    o = two_spheres(orc, tau=1.0, steps=20, measure=False)
    for L, lb in ((gpu, g), (orc, o)):
        L.bbl(lb); L.propagate(lb); L.collide(lb)
        L.lbsteps(lb, 10)
    assert g.precision == 1
    assert rel(g.pops(), o.pops()) < 2e-5


def test_bf16_skip_solid_moves_to_fp32(gpu, orc):
    """Solid nodes left unrelaxed keep streamed populations whose deviations
    are not paired (q and opp(q) differ), so BF16 storage cannot hold them:
    the lattice steps in FP32 and follows the oracle to FP32 accuracy."""
    g = two_spheres(gpu, tau=1.0, skip=1, steps=60, precision=2)
    o = two_spheres(orc, tau=1.0, skip=1, steps=60)
    assert g.precision == 1
    assert rel(g.pops(), o.pops()) < 2e-5
    assert rel(objects_ft(g)[:, :3], objects_ft(o)[:, :3]) < 2e-5


def _uploaded(gpu, orc, perturb):
    """The oracle's state after 40 steps at tau 0.8 (non-zero stress), with
    perturb applied, uploaded into a BF16 lattice and into a second oracle
    lattice; both then take 30 more steps."""
    src = two_spheres(orc, tau=0.8, steps=40, measure=False)
    state = src.pops()
    perturb(state)
    out = []
    for L, prec in ((gpu, 2), (orc, 0)):
        lb = two_spheres(L, tau=0.8, steps=0, measure=False, precision=prec)
        lb.pops()
        lb.array("a")[:] = state
        L.lbpush(lb)
        L.lbsteps(lb, 30)
        L.measure(lb)
        out.append(lb)
    return out


def test_bf16_upload_of_collided_state_stays_bf16(gpu, orc):
    """A post-collision state has paired deviations: it stays in BF16
    storage; after 30 more steps populations, mean flow and drag are within
    2e-3 (the BF16 rounding of the stress part)."""
    g, o = _uploaded(gpu, orc, lambda a: None)
    assert g.precision == 2
    assert rel(g.pops(), o.pops()) < 2e-3
    assert abs(g.vmeanx - o.vmeanx) <= 2e-3 * abs(o.vmeanx)
    assert rel(objects_ft(g)[:, :3], objects_ft(o)[:, :3]) < 2e-3


def test_bf16_upload_of_unpaired_state_moves_to_fp32(gpu, orc):
    """One population changed on one fluid node: its deviations are no
    longer paired, the upload moves the lattice to FP32 and the run follows
    the oracle to FP32 accuracy."""
    def bump(a):
        a[5, 1] += 1e-3
    g, o = _uploaded(gpu, orc, bump)
    assert g.precision == 1
    assert rel(g.pops(), o.pops()) < 2e-5
    assert abs(g.vmeanx - o.vmeanx) <= 2e-5 * abs(o.vmeanx)


@pytest.mark.parametrize("tau", [1.0, 0.8])
def test_bf16_thin_lattice_couette(gpu, orc, tau):
    """A 1 x 1 x 22 lattice (planar Couette flow between moving walls):
    every plane ring and halo of the paired-deviation step wraps onto the
    same few nodes.  Populations and wall stresses follow the FP64 oracle to
    2e-5 at tau = 1 (zero stress part) and 2e-3 at tau = 0.8."""
    from scenarios import couette
    g, gw1, gw2, _ = couette(gpu, tau=tau, steps=3000, precision=2)
    o, ow1, ow2, _ = couette(orc, tau=tau, steps=3000)
    tol = 2e-5 if tau == 1.0 else 2e-3
    assert g.precision == 2
    assert rel(g.pops(), o.pops()) < tol
    assert abs(gw1.frcx - ow1.frcx) <= tol * abs(ow1.frcx)
    assert abs(gw2.frcx - ow2.frcx) <= tol * abs(ow2.frcx)
