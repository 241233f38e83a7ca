"""Known-answer runs on the GPU: the reference's own example results, the
plain-method convergence case, and checkpoint files byte-compatible with
the reference's.

Values come from tests/golden/kat.json (produced from builds of the
reference by tests/golden/make_golden.py).  FP64 GPU results are compared
to the strict reference build to 1e-12 relative and to the published
digits; checkpoint files are compared byte for byte with the oracle's.
"""

import filecmp
import json
import os

import numpy as np
import pytest

from golden.make_golden import rcp_perm, sccp_sphere
from scenarios import two_spheres

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def kat():
    with open(os.path.join(GOLDEN, "kat.json")) as f:
        return json.load(f)["kat"]


def test_rcp_permeability(gpu):
    g = kat()["rcp_perm"]
    with open(os.path.join(GOLDEN, "rcp144.json")) as f:
        spheres = json.load(f)["spheres"]
    r = rcp_perm(gpu, spheres)
    assert abs(r["k"] - g["strict"]["k"]) <= 1e-12 * g["strict"]["k"]
    assert round(r["k"], 6) == g["published"]["k"]
    assert round(r["vmeanx"], 6) == g["published"]["vmeanx"]


def test_sccp_sphere_stokes(gpu):
    g = kat()["sccp_sphere"]
    r = sccp_sphere(gpu)
    assert abs(r["u_mean"] - g["strict"]["u_mean"]) <= 1e-12 * g["strict"]["u_mean"]
    assert round(r["u_mean"], 6) == g["published"]["u_mean"]


def test_plain_method_converges_like_reference(gpu):
    """32^3, sphere r 4.5 at the centre, body force 1e-5, tau 1, Stokes,
    checks every 100 steps until |dvmeanx|/|vmeanx| < 1e-8 (lbconverge)."""
    g = kat()["sphere_converge"]["strict"]
    lb = gpu.newlb(32, 32, 32, "null")
    lb.tau = 1.0
    lb.stokes_flow = 1
    obj = gpu.insertsph(lb, 4.5, 15.5, 15.5, 15.5)
    gpu.addbf(lb, 1e-5, 0.0, 0.0)
    steps = gpu.lbconverge(lb, 100, 1e-8, 60000)
    assert steps == g["steps"]
    assert abs(lb.vmeanx - g["vmeanx"]) <= 1e-12 * g["vmeanx"]
    assert abs(obj.frcx - g["frcx"]) <= 1e-12 * g["frcx"]
    assert abs(gpu.discrf(lb) - g["discrf"]) <= 1e-6 * g["discrf"]


def test_plain_method_fp32(gpu):
    """FP32 populations reach the FP64 drag and mean flow to 1e-4."""
    g = kat()["sphere_converge"]["strict"]
    lb = gpu.newlb(32, 32, 32, "null")
    lb.precision = 1
    lb.tau = 1.0
    lb.stokes_flow = 1
    obj = gpu.insertsph(lb, 4.5, 15.5, 15.5, 15.5)
    gpu.addbf(lb, 1e-5, 0.0, 0.0)
    gpu.lbconverge(lb, 100, 1e-8, 40000)
    assert abs(lb.vmeanx - g["vmeanx"]) <= 1e-4 * g["vmeanx"]
    assert abs(obj.frcx - g["frcx"]) <= 1e-4 * g["frcx"]


def test_checkpoint_files_match_oracle(gpu, orc, tmp_path):
    """lbsave / lbload (reference src/lbstore.c:36-218): the moment file
    written from the GPU equals the oracle's byte for byte, and reloading it
    (plain, rescaled, averaged) gives the oracle's populations."""
    out = []
    for L, tag in ((gpu, "g"), (orc, "o")):
        lb = two_spheres(L, steps=17, measure=False, stokes=0, tau=0.7)
        path = str(tmp_path / f"ck_{tag}.dms")
        L.lbsave(lb, path)
        L.lbstep(lb)
        lb.rescale = 1.5
        L.lbload(lb, path)
        L.lbstep(lb)
        lb.load_average = 1
        L.lbload(lb, path)
        out.append((path, lb.pops()))
    assert filecmp.cmp(out[0][0], out[1][0], shallow=False)
    assert np.array_equal(out[0][1], out[1][1])
