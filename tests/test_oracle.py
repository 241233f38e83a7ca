"""The CPU oracle pinned against builds of the reference (CPU only).

The golden fixtures of tests/golden/ were produced by tests/golden/make_golden.py
from two builds of the reference's own sources: a strict IEEE build (the
bit-exact target) and the as-shipped -O3 -ffast-math build.  The oracle must
reproduce the strict build's populations bit for bit and the shipped
build's results to 1e-12 relative; the known-answer runs of the reference's
examples must give the published numbers.
"""

import hashlib
import json
import os
import sys

import numpy as np
import pytest

from scenarios import objects_ft, two_spheres
from golden.make_golden import (LB_CASES, MP_CASES, mp_case, rcp_perm, sccp_sphere,
                                sphere_converge)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def digest(arr):
    a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64)) + 0.0
    return hashlib.sha256(a.tobytes()).hexdigest()


def rel_close(a, b, tol):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", sorted(LB_CASES))
def test_lb_case_matches_reference(orc, name):
    g = load("lb_cases.json")["cases"]
    lb = two_spheres(orc, **LB_CASES[name])
    a = lb.array("a")
    assert digest(a) == g["strict"][name]["pops_sha256"]
    assert lb.step == g["strict"][name]["step"]
    assert [lb.vmeanx, lb.vmeany, lb.vmeanz] == g["strict"][name]["vmean"]
    assert objects_ft(lb).tolist() == g["strict"][name]["objects_ft"]
    shipped = g["shipped"][name]
    assert rel_close([lb.vmeanx, lb.vmeany, lb.vmeanz], shipped["vmean"], 1e-12)
    assert rel_close(objects_ft(lb)[:, :3], np.array(shipped["objects_ft"])[:, :3], 1e-12)
    assert rel_close(a.ravel()[:: max(1, a.size // 16)][:16], shipped["pops_sample"], 1e-12)


@pytest.mark.parametrize("name", sorted(MP_CASES))
def test_mp_case_matches_reference(orc, name):
    g = load("mp_cases.json")["cases"]
    r = mp_case(orc, **MP_CASES[name])
    assert r["p_sha256"] == g["strict"][name]["p_sha256"]
    for key in ("mpmean", "mpspread_x", "adtotal"):
        assert r[key] == g["strict"][name][key]
        assert abs(r[key] - g["shipped"][name][key]) <= 1e-12 * max(abs(g["shipped"][name][key]), 1e-300)


def test_sccp_sphere_known_answer(orc):
    kat = load("kat.json")["kat"]["sccp_sphere"]
    r = sccp_sphere(orc)
    assert r["u_mean"] == kat["strict"]["u_mean"]
    assert round(r["u_mean"], 6) == kat["published"]["u_mean"]


def test_rcp_permeability_known_answer(orc):
    kat = load("kat.json")["kat"]["rcp_perm"]
    spheres = load("rcp144.json")["spheres"]
    r = rcp_perm(orc, spheres)
    assert r["k"] == kat["strict"]["k"]
    assert round(r["k"], 6) == kat["published"]["k"]
    assert round(r["vmeanx"], 6) == kat["published"]["vmeanx"]
    assert round(r["pore_fraction"], 2) == kat["published"]["pore_fraction"]


def test_plain_method_first_2000_steps(orc):
    kat = load("kat.json")["kat"]["sphere_converge"]
    r = sphere_converge(orc, stop_at=2000)
    assert r["vmeanx"] == kat["strict"]["vmeanx_at_2000"]


def test_oracle_equals_reference_build_live(orc, ref_strict):
    """Where the reference is built here: more geometries, compared live."""
    for cfg in (dict(dims=(9, 10, 11), steps=13, moving=1, stokes=0, tau=0.55),
                dict(dims=(4, 20, 6), steps=9, skip=1)):
        a = two_spheres(orc, **cfg)
        b = two_spheres(ref_strict, **cfg)
        assert np.array_equal(a.array("a"), b.array("a"))
        assert a.vmeanx == b.vmeanx


def test_partial_adsorption_conserves_mass(orc):
    """Extension (no reference counterpart): adsorption probability P.  With
    the flow frozen, fluid + adsorbed tracer is conserved to round-off for
    any P, and P = 1 is the reference's all-or-nothing adsorption."""
    L = orc
    lb = L.newlb(12, 13, 15, "null")
    lb.tau = 0.7
    L.insertsph(lb, 3.5, 5.5, 6.0, 7.2)
    L.addbf(lb, 1e-3, 2e-4, 0)
    for _ in range(20):
        L.lbstep(lb)
    for P in (0.0, 0.01, 0.37, 1.0):
        mp = L.newmp(lb, "null")
        mp.alpha = 0.3
        mp.adprob = P
        L.mpinit(mp)
        L.adall(mp)
        L.mpall(mp, 1.0)
        m0 = L.mptotal(mp, "all")
        for _ in range(60):
            L.mpstep(mp)
        m1 = L.mptotal(mp, "fluid") + L.mptotal(mp, "adsorbed")
        assert abs(m1 - m0) <= 1e-12 * m0, (P, m0, m1)
        if P == 0.0:
            assert L.mptotal(mp, "adsorbed") == 0.0
        L.adnone(mp)


def test_network_oracle_gradients_with_density_channel():
    """The network oracle's exact gradients, with a fourth (density) label
    channel, against central differences of its own loss (float64)."""
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import orc_unet
    rng = np.random.default_rng(3)
    w0 = w1 = w2 = w3 = 4
    shapes = {"e0a": (4, w0), "e0b": (w0, w0), "e1a": (w0, w1), "e1b": (w1, w1), "e2a": (w1, w2),
              "e2b": (w2, w2), "e3a": (w2, w3), "e3b": (w3, w3), "d2a": (w3 + w2, w2), "d2b": (w2, w2),
              "d1a": (w2 + w1, w1), "d1b": (w1, w1), "d0a": (w1 + w0, w0), "d0b": (w0, w0), "out": (w0, 4)}
    params = {k: (rng.normal(0, (2.0 / (27 * ci)) ** 0.5, (27, co, ci)), rng.normal(0, 0.1, co))
              for k, (ci, co) in shapes.items()}
    inp = (rng.random((1, 16, 16, 16, 4)) > 0.7).astype(np.float64)
    labels = rng.normal(0, 1, (1, 16, 16, 16, 4))
    loss, grads = orc_unet.forward_backward(params, inp, labels)
    h = 1e-6
    for name, idx in (("out", (13, 3, 2)), ("out", (0, 2, 1)), ("d0b", (5, 1, 2)), ("e0a", (26, 0, 0))):
        w, b = params[name]
        wp, wm = w.copy(), w.copy()
        wp[idx] += h
        wm[idx] -= h
        lp, _ = orc_unet.forward_backward({**params, name: (wp, b)}, inp, labels)
        lm, _ = orc_unet.forward_backward({**params, name: (wm, b)}, inp, labels)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - grads[name][0][idx]) <= 1e-5 * max(abs(fd), 1e-3), (name, idx, fd, grads[name][0][idx])
    b = params["out"][1]
    bp, bm = b.copy(), b.copy()
    bp[3] += h
    bm[3] -= h
    lp, _ = orc_unet.forward_backward({**params, "out": (params["out"][0], bp)}, inp, labels)
    lm, _ = orc_unet.forward_backward({**params, "out": (params["out"][0], bm)}, inp, labels)
    assert abs((lp - lm) / (2 * h) - grads["out"][1][3]) <= 1e-6


def _file_records(L):
    from golden.make_golden import file_records
    return file_records(L)


def test_file_api_matches_reference(orc):
    """Velocity, force, map, object and stress files written by the oracle
    are byte-identical to the strict reference build's (SHA-256 fixtures),
    and so are lattices reloaded from them (lbloadvel, lbloadobj) and the
    tracer set by mpsubs (src/lbstore.c:227-678, src/lbmeasure.c:129-203,
    src/mpobjs.c:188-226)."""
    g = load("files.json")["cases"]
    assert _file_records(orc) == g


def test_file_api_equals_reference_build_live(orc, ref_strict, tmp_path):
    """Where the reference is built here: the same files compared byte for
    byte, live, for one more configuration."""
    import scenarios as S
    cfg = dict(dims=(6, 13, 8), steps=7, moving=0, skip=0, stokes=0, tau=0.7)
    (tmp_path / "o").mkdir()
    (tmp_path / "r").mkdir()
    _, fo = S.file_case(orc, str(tmp_path / "o"), **cfg)
    _, fr = S.file_case(ref_strict, str(tmp_path / "r"), **cfg)
    assert fo.keys() == fr.keys()
    for k in fo:
        assert fo[k] == fr[k], k


def _time_lib(path):
    import ctypes as C
    lib = C.CDLL(path)
    f = lib.orc_time_steps
    f.restype = C.c_double
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_int,
                  C.c_void_p]
    return lib, f


@pytest.mark.parametrize("bits", ["64", "32"])
def test_timing_builds_step_like_reference(bits):
    """The CPU-baseline builds (the oracle under the reference's shipped
    -O3 -ffast-math flags, double and -D_SINGLE) advance a packed lattice
    like the reference's own sources compiled the same way: the population
    sums after 40 Navier-Stokes steps agree to the precision's round-off."""
    import ctypes as C
    from sunlightlb_gb300 import build as b
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    mine = os.path.join(root, "oracle", f"liboracle_time{bits}.so")
    ref = os.path.join(root, "oracle", "_ref", f"libref_time{bits}.so")
    if not os.path.exists(mine):
        b.build_oracle(with_reference=False)
    if not os.path.exists(ref):
        pytest.skip("reference build not available (built only where the reference sources are)")
    from sunlightlb_gb300 import workloads as W
    _, solid = W.rsa_packing(24, 0.3, 2.0, 4.0, 9)
    mask = np.ascontiguousarray(solid, dtype=np.uint8)
    sums = []
    for path in (mine, ref):
        lib, f = _time_lib(path)
        assert lib.orc_real_size() == int(bits) // 8
        cs = C.c_double()
        assert f(mask.ctypes.data, 24, 24, 24, 0.7, 0, 1e-3, 0, 40, C.byref(cs)) >= 0.0
        sums.append(cs.value)
    tol = 1e-10 if bits == "64" else 2e-4
    assert abs(sums[0] - sums[1]) <= tol * max(abs(sums[1]), 1e-30), sums


def test_translated_sphere_node_set(orc):
    """The translation rule (an extension without a reference counterpart):
    after each move the object's node set is exactly the sphere with its
    periodic images at the new centre (numpy rasterisation), the mask
    equals a full makemask of the new map, and the fluid count follows."""
    import scenarios as S
    from sunlightlb_gb300 import workloads as W
    dims, rad = (20, 18, 22), 3.6
    lb, obj = S.translate_case(orc, dims=dims, rad=rad, moves=5, measure=False)
    c = (obj.posx, obj.posy, obj.posz)
    want = np.zeros(dims, dtype=bool)
    for im in W.images(dims, rad, c):
        want |= W.sphere_nodes(dims, rad, im)
    got = S.object_ids(lb).reshape(dims) >= 0
    assert np.array_equal(got, want)
    mask = lb.array("mask").copy()
    orc.makemask(lb)
    assert np.array_equal(lb.array("mask"), mask)
    assert orc.countfluid(lb) == int((~want).sum())


VACF_CASES = [dict(), dict(direction="xy"), dict(direction="zz", psi=True), dict(second_init=True, direction="yx"),
              dict(ads=True, direction="yy", alpha=0.0)]


def test_vacf_matches_reference(orc, ref_strict, tmp_path):
    """The tracer velocity autocorrelation (src/mpvacf.c) restated: the
    diffusion coefficient, both tracer fields and the written file equal
    the strict reference build's bit for bit."""
    import scenarios as S
    for n, kw in enumerate(VACF_CASES):
        (tmp_path / f"o{n}").mkdir()
        (tmp_path / f"r{n}").mkdir()
        a = S.vacf_case(orc, str(tmp_path / f"o{n}"), **kw)
        b = S.vacf_case(ref_strict, str(tmp_path / f"r{n}"), **kw)
        assert a[0] == b[0], kw
        assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]), kw
        assert a[3] == b[3], kw


def test_vacf_golden(orc, tmp_path):
    import scenarios as S
    g = load("vacf.json")["cases"]
    for n, kw in enumerate(VACF_CASES):
        (tmp_path / f"o{n}").mkdir()
        d, p, p2, data = S.vacf_case(orc, str(tmp_path / f"o{n}"), **kw)
        rec = g[n]
        assert d == rec["diffusion"], kw
        assert digest(p) == rec["p_sha256"] and digest(p2) == rec["p2_sha256"], kw
