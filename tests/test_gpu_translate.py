"""Translating spheres (an extension with no counterpart in the reference,
which can only remove objects and insert new ones, src/lbobjs.c:433-453).

lbtranslate re-rasterises a spherical object on the GPU: nodes it leaves
become fluid at the equilibrium of density rho0 and the wall velocity, nodes
it reaches join it, and the flag words, boundary list, mask, body force and
wall velocities follow.  The CPU oracle restates the same rule (oracle/
orc_lb.c lbtranslate); FP64 populations must equal it bit for bit through
moves that meet both storage layouts, Stokes and Navier-Stokes, moving and
fixed walls; reductions to 1e-12; FP32 within 1e-4 of the FP64 oracle.
Batched lattices whose spheres are moved between batch steps equal the same
lattices stepped one at a time.
"""

import numpy as np
import pytest

import scenarios as S

pytestmark = pytest.mark.gpu

RED_TOL = 1e-12

CASES = {
    "stokes_moving": dict(),
    "navier_stokes": dict(stokes=0, tau=0.65),
    "fixed_walls": dict(moving=0),
    "even_moves": dict(every=8, moves=4),
    "fast": dict(step=(1.7, 0.9, -1.3), moves=3),
}


def close(a, b, tol):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", sorted(CASES))
def test_translate_fp64_bit_exact(gpu, orc, name):
    cfg = CASES[name]
    lg, og = S.translate_case(gpu, **cfg)
    lo, oo = S.translate_case(orc, **cfg)
    assert np.array_equal(S.object_ids(lg), S.object_ids(lo))
    assert np.array_equal(lg.array("mask"), lo.array("mask"))
    for f in ("bx", "by", "bz", "ux", "uy", "uz"):
        assert np.array_equal(lg.array(f), lo.array(f)), f
    pg, po = lg.pops(), lo.pops()
    assert np.array_equal(pg, po), np.abs(pg - po).max()
    assert close([lg.vmeanx, lg.vmeany, lg.vmeanz], [lo.vmeanx, lo.vmeany, lo.vmeanz], RED_TOL)
    assert close([og.frcx, og.frcy, og.frcz], [oo.frcx, oo.frcy, oo.frcz], RED_TOL)
    assert (og.posx, og.posy, og.posz) == (oo.posx, oo.posy, oo.posz)
    assert gpu.countfluid(lg) == orc.countfluid(lo)


def test_translate_fp32_close(gpu, orc):
    lg, og = S.translate_case(gpu, precision=1)
    lo, oo = S.translate_case(orc)
    assert np.array_equal(S.object_ids(lg), S.object_ids(lo))
    assert abs(lg.vmeanx - lo.vmeanx) <= 1e-4 * abs(lo.vmeanx)
    pg, po = lg.pops(), lo.pops()
    assert np.abs(pg - po).max() <= 1e-4 * np.abs(po).max()


def test_translate_in_batch_equals_alone(gpu):
    """Spheres of batched lattices moved between batch steps give the same
    FP32 state as the same lattices stepped one at a time."""
    def build(n):
        out = []
        for d in range(n):
            lb, obj = S.translate_case(gpu, dims=(16 + 4 * d, 18, 20), centre=(3.1 + d, 9.2, 10.4), moves=0,
                                       precision=1, measure=False)
            out.append((lb, obj))
        return out
    batch, alone = build(3), build(3)
    b = gpu.newbatch()
    for lb, _ in batch:
        gpu.batchadd(b, lb)
    for move in range(4):
        gpu.batchsteps(b, 9)
        for lb, _ in alone:
            gpu.lbsteps(lb, 9)
        for group in (batch, alone):
            for d, (lb, obj) in enumerate(group):
                gpu.lbtranslate(lb, obj, 3.6, obj.posx + 0.7, obj.posy - 0.3, obj.posz + 0.45 * d)
    for (l1, _), (l2, _) in zip(batch, alone):
        assert np.array_equal(S.object_ids(l1), S.object_ids(l2))
        assert np.array_equal(l1.pops(), l2.pops())
    gpu.freebatch(b)
