"""GPU parity of the moment-propagation (passive scalar) path.

The GPU gathers the tracer terms that the reference scatters and adds them
in the reference's order, so FP64 tracer fields equal the oracle's bit for
bit; sums over the lattice are compared to 1e-12 relative.  The partial
adsorption probability (an extension) is checked against the oracle's
restatement of it, and for mass conservation.
"""

import numpy as np
import pytest

from golden.make_golden import MP_CASES, mp_case

pytestmark = pytest.mark.gpu

TOL = 1e-12


def tracer_run(L, moving=0, ads=0, adprob=None, steps=40, n=12, interleave=True, precision=0,
               mp_precision=None, dims=None):
    d = dims or (n, n + 1, n + 3)
    lb = L.newlb(d[0], d[1], d[2], "null")
    if L.extended:
        lb.precision = precision
    lb.tau = 0.7
    lb.stokes_flow = 0
    lb.objects_moving = moving
    o1 = L.insertsph(lb, max(1.0, 0.29 * min(d)), 0.46 * d[0], 0.46 * d[1], 0.48 * d[2])
    L.addbf(lb, 1e-3, 2e-4, 0)
    if moving:
        o1.velx = 1e-2
        o1.angz = 2e-3
        L.vspread(lb)
    for _ in range(20):
        L.lbstep(lb)
    mp = L.newmp(lb, "null")
    if mp_precision is not None:
        mp.precision = mp_precision
    mp.alpha = 0.3
    if adprob is not None:
        mp.adprob = adprob
    L.mpinit(mp)
    if ads:
        L.adall(mp)
    L.mpwall(mp, "x", 0, 1.0)
    L.mpsph(mp, 2.0, 0.7 * d[0], 0.7 * d[1], 0.6 * d[2], 0.5)
    for s in range(steps):
        L.mpstep(mp)
        if interleave and s % 2:
            L.lbstep(lb)
            L.mprhoinit(mp)
    L.mppull(mp)
    return lb, mp


@pytest.mark.parametrize("name", sorted(MP_CASES))
def test_tracer_fp64_bit_exact(gpu, orc, name):
    rg = mp_case(gpu, **MP_CASES[name])
    ro = mp_case(orc, **MP_CASES[name])
    assert rg["p_sha256"] == ro["p_sha256"]
    for key in ("mpmean", "mpspread_x", "adtotal"):
        assert abs(rg[key] - ro[key]) <= TOL * max(abs(ro[key]), 1e-300), key


@pytest.mark.parametrize("dims", [(2, 7, 9), (1, 3, 12), (3, 3, 3), (9, 4, 2)])
def test_tracer_thin_lattices_bit_exact(gpu, orc, dims):
    """Wrap-around sources (the ranked summation order) in thin lattices."""
    pg = tracer_run(gpu, dims=dims, steps=15)[1].field().copy()
    po = tracer_run(orc, dims=dims, steps=15)[1].field().copy()
    assert np.array_equal(pg, po)


@pytest.mark.parametrize("P", [0.0, 0.01, 0.37])
def test_partial_adsorption_bit_exact(gpu, orc, P):
    pg = tracer_run(gpu, ads=1, adprob=P, moving=1)[1].field().copy()
    po = tracer_run(orc, ads=1, adprob=P, moving=1)[1].field().copy()
    assert np.array_equal(pg, po)


def test_tracer_mass_balance_frozen_flow(gpu):
    """Flow frozen: fluid + adsorbed tracer conserved to round-off."""
    for P in (1.0, 0.01):
        lb, mp = tracer_run(gpu, ads=1, adprob=P, steps=0, interleave=False)
        gpu.mpall(mp, 1.0)
        m0 = gpu.mptotal(mp, "fluid") + gpu.mptotal(mp, "adsorbed")
        for _ in range(200):
            gpu.mpstep(mp)
        m1 = gpu.mptotal(mp, "fluid") + gpu.mptotal(mp, "adsorbed")
        assert abs(m1 - m0) <= 1e-12 * m0, (P, m0, m1)


def test_tracer_fp32_close_to_fp64(gpu, orc):
    """FP32 flow and FP32 tracer against the FP64 oracle."""
    pg = tracer_run(gpu, precision=1, mp_precision=1, steps=60)[1].field().copy()
    po = tracer_run(orc, steps=60)[1].field().copy()
    assert np.abs(pg - po).max() <= 2e-5 * np.abs(po).max()


def test_tracer_utilities_match_oracle(gpu, orc):
    out = []
    for L in (gpu, orc):
        lb, mp = tracer_run(L, ads=1, steps=10)
        mp2 = L.newmp(lb, "null")
        mp2.alpha = 0.1
        L.mpinit(mp2)
        L.mpslab(mp2, 2.0, 7.0, -1.0, 20.0, 3.0, 9.0, 0.25)
        L.mpcyl(mp2, "z", 3.0, 6.0, 6.0, 0.75)
        L.mpcyl(mp2, "xh", 5.0, 6.0, 7.0, 0.05)
        L.mpcopy(mp, mp2)
        L.mprescale(mp2, 1.5)
        L.adzero(mp)
        vals = (L.mpmax(mp2), L.mpmin(mp2), L.mpmean(mp2), L.mpspread(mp2, "z"), L.adtotal(mp, "null", 1))
        L.mppull(mp2)
        L.mppull(mp)
        out.append((mp.field().copy(), mp2.field().copy(), vals))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    for a, b in zip(out[0][2], out[1][2]):
        assert abs(a - b) <= TOL * max(abs(b), 1e-300)


@pytest.mark.parametrize("mp_precision", [0, 1])
def test_source_plane_breakthrough_and_balance(gpu, orc, mp_precision):
    """Constant-concentration source plane re-set every step (mpwall), partial
    adsorption, frozen flow: the breakthrough samples (mpplane) and the
    injected tracer (mptotal "injected") match the oracle, and fluid +
    adsorbed tracer = injected to round-off."""
    out = []
    for L in (gpu, orc):
        lb, mp = tracer_run(L, ads=1, adprob=0.01, steps=0, interleave=False, precision=1 if L is gpu else 0,
                            mp_precision=mp_precision if L is gpu else None)
        L.mpinit(mp)
        L.adall(mp)
        curve = []
        for s in range(120):
            L.mpwall(mp, "x", 0, 1.0)
            L.mpstep(mp)
            if s % 10 == 9:
                curve.append(L.mpplane(mp, "x", lb.esi - 1))
        inj = L.mptotal(mp, "injected")
        held = L.mptotal(mp, "fluid") + L.mptotal(mp, "adsorbed")
        out.append((np.array(curve), inj, held))
    (cg, ig, hg), (co, io, ho) = out
    # the GPU flow is FP32 here: tolerances of an FP32 flow / FP32 tracer
    tol = 1e-4 if mp_precision else 2e-5
    assert np.abs(cg - co).max() <= tol * max(np.abs(co).max(), 1e-30)
    assert abs(ig - io) <= tol * io
    assert abs(ho - io) <= 1e-12 * io          # oracle: exact balance
    assert abs(hg - ig) <= (1e-5 if mp_precision else 1e-12) * ig


@pytest.mark.parametrize("cfg", [dict(moving=1), dict(ads=1), dict(ads=1, adprob=0.37),
                                 dict(moving=1, ads=1, adprob=0.37)])
def test_tracer_fp32_cases_close_to_fp64(gpu, orc, cfg):
    """FP32 tracer update (terms in link order, 1/rho snapshot) with moving
    walls and full or partial adsorption, flow steps between tracer steps
    (both AA layouts), against the FP64 oracle: within 2e-5 of the largest
    value after 60 updates."""
    pg = tracer_run(gpu, precision=1, mp_precision=1, steps=60, **cfg)[1].field().copy()
    po = tracer_run(orc, steps=60, **cfg)[1].field().copy()
    assert np.abs(pg - po).max() <= 2e-5 * np.abs(po).max()


def test_tracer_fp32_on_uploaded_flow(gpu, orc):
    """FP32 tracer updates on a flow just uploaded (the reference's layout),
    partial adsorption, against the FP64 oracle within 2e-5."""
    out = []
    for L, prec, mpp in ((gpu, 1, 1), (orc, 0, None)):
        lb, mp = tracer_run(L, precision=prec, mp_precision=mpp, steps=0, interleave=False, ads=1, adprob=0.37)
        lb.pops()
        L.lbpush(lb)
        for _ in range(30):
            L.mpstep(mp)
        L.mppull(mp)
        out.append(mp.field().copy())
    assert np.abs(out[0] - out[1]).max() <= 2e-5 * np.abs(out[1]).max()


def test_tracer_fp32_mass_balance_frozen_flow(gpu):
    """FP32 tracer, flow frozen (stencil update, columns normalised to 1,
    compensated accumulation on adsorbing solids): fluid + adsorbed tracer
    conserved to 2e-6 over 200 updates."""
    for P in (1.0, 0.01):
        lb, mp = tracer_run(gpu, ads=1, adprob=P, steps=0, interleave=False, precision=1, mp_precision=1)
        gpu.mpall(mp, 1.0)
        m0 = gpu.mptotal(mp, "fluid") + gpu.mptotal(mp, "adsorbed")
        for _ in range(200):
            gpu.mpstep(mp)
        m1 = gpu.mptotal(mp, "fluid") + gpu.mptotal(mp, "adsorbed")
        assert abs(m1 - m0) <= 2e-6 * m0, (P, m0, m1)


def test_tracer_fp32_stencil_tracks_fp64(gpu, orc):
    """Frozen flow, 200 FP32 updates (the stencil path from the second
    update on: FP32 coefficients, field kept as high + low parts) against
    the FP64 oracle: within 1e-6 of the largest value, with partial
    adsorption."""
    out = []
    for L, prec, mpp in ((gpu, 1, 1), (orc, 0, None)):
        lb, mp = tracer_run(L, precision=prec, mp_precision=mpp, steps=0, interleave=False, ads=1, adprob=0.37)
        for _ in range(200):
            L.mpstep(mp)
        L.mppull(mp)
        out.append(mp.field().copy())
    assert np.abs(out[0] - out[1]).max() <= 1e-6 * np.abs(out[1]).max()
