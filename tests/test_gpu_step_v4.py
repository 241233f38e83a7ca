"""The 128-bit form of the fused step (FP32 populations, 4 nodes along k
per thread, warp shuffles for the +-1 k shifts, scalar accesses at warp and
row edges and across bounce-back links) against the scalar form.

Both forms apply the same per-node arithmetic; the compiler may still
contract multiply-adds differently in the two kernels (FP32 arithmetic is
built with FMA), so the populations must agree to FP32 rounding -- 2e-6 of
their largest magnitude, a few units in the last place, where a misplaced
value would show as O(1) of it -- after any number of steps, on lattices
chosen to hit the
edge cases: rows of 8, 12, 20, 64 and 132 nodes along k (blocks of 2, 3, 5,
16 and 32+1 lanes along k, so warps span several rows or end inside one),
spheres across the periodic boundary, moving walls, Navier-Stokes,
skip_solid and a per-node body force.  The forced shapes go through
lbsettuning; the step counts are odd and even so both update kinds run.
"""

import ctypes as C

import numpy as np
import pytest

from scenarios import two_spheres

pytestmark = pytest.mark.gpu

VEC4 = -4
TOL = 2e-6


def run(gpu, cfg, shape, steps):
    lb = two_spheres(gpu, steps=0, measure=False, precision=1, **cfg)
    tune = (C.c_int * 4)(*shape)
    assert gpu.lbsettuning(lb, C.addressof(tune)) == 0
    for _ in range(steps):
        gpu.lbstep(lb)
    got = (C.c_int * 4)()
    gpu.lbtuning(lb, C.addressof(got))
    assert list(got) == list(shape)
    return lb


CASES = {
    "rows8": dict(dims=(9, 10, 8)),
    "rows12_moving": dict(dims=(7, 11, 12), moving=1),
    "rows20_ns": dict(dims=(6, 9, 20), stokes=0, tau=0.62),
    "rows64_skip": dict(dims=(5, 6, 64), skip=1),
    "rows132_moving_ns": dict(dims=(4, 5, 132), moving=1, stokes=0, tau=0.7),
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("steps", [7, 12])
def test_vec4_equals_scalar(gpu, name, steps):
    cfg = CASES[name]
    a = run(gpu, cfg, (VEC4, 128, VEC4, 128), steps)
    b = run(gpu, cfg, (1, 64, 1, 64), steps)
    pa, pb = a.pops(), b.pops()
    assert np.abs(pa - pb).max() <= TOL * np.abs(pb).max(), f"max |diff| = {np.abs(pa - pb).max():.3e}"
    gpu.measure(a)
    gpu.measure(b)
    assert abs(a.vmeanx - b.vmeanx) <= TOL * abs(b.vmeanx)


def test_vec4_nonuniform_body_force(gpu):
    out = []
    for shape in ((VEC4, 128, VEC4, 128), (2, 128, 1, 64)):
        lb = two_spheres(gpu, dims=(8, 9, 16), steps=0, measure=False, precision=1)
        bx = lb.array("bx")
        bx[: lb.nnodes // 3] *= 3.0
        gpu.lbpush(lb)
        tune = (C.c_int * 4)(*shape)
        assert gpu.lbsettuning(lb, C.addressof(tune)) == 0
        for _ in range(9):
            gpu.lbstep(lb)
        out.append(lb.pops())
    assert np.abs(out[0] - out[1]).max() <= TOL * np.abs(out[1]).max()


def test_vec4_rejected_where_it_does_not_apply(gpu):
    lb = two_spheres(gpu, dims=(6, 7, 10), steps=1, measure=False, precision=1)  # esk not a multiple of 4
    tune = (C.c_int * 4)(VEC4, 128, VEC4, 128)
    assert gpu.lbsettuning(lb, C.addressof(tune)) != 0
    lb64 = two_spheres(gpu, dims=(6, 7, 12), steps=1, measure=False, precision=0)  # FP64
    assert gpu.lbsettuning(lb64, C.addressof(tune)) != 0
