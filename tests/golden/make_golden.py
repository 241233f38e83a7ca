"""Generate the golden fixtures of tests/golden/ from builds of the reference.

Run where the reference sources exist (they are compiled by oracle/Makefile
into oracle/_ref/):

    make -C oracle ref && python tests/golden/make_golden.py [--files-only | --vacf-only]

(the reference checkout is $SLB_REFERENCE, default /root/reference).

Two reference builds are driven through the same C API calls as the GPU
library:
  strict   -O2 -fno-fast-math -ffp-contract=off (IEEE double, no FMA)
  shipped  the reference's own flags, -O3 -ffast-math (src/Makefile:39)
The strict build is the bit-exact target (populations are stored as the
SHA-256 of their float64 bytes, -0.0 folded to +0.0); the shipped build
gives the values the 1e-12 relative parity is checked against.

Fixtures (JSON):
  lb_cases.json     small update-path scenarios: population digest, mean
                    flow, object force and torque, node-force sums
  mp_cases.json     moment-propagation scenarios: tracer digest and totals
  kat.json          known-answer runs of the reference's examples and the
                    plain-method convergence case
  rcp144.json       the 144-sphere packing of examples/rcp_spheres.dat
  files.json        digests of the field, force, map, object and stress
                    files, of lattices reloaded from them, and of mpsubs
  vacf.json         tracer velocity autocorrelation: diffusion coefficient
                    and digests of both tracer fields
"""

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from sunlightlb_gb300.binding import Library  # noqa: E402
import scenarios as S  # noqa: E402

# the reference's checkout: SLB_REFERENCE overrides the default location
REF_ROOT = os.environ.get("SLB_REFERENCE", "/root/reference")
REF_EXAMPLES = os.path.join(REF_ROOT, "examples")


def digest(arr):
    a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64)) + 0.0  # -0.0 -> +0.0
    return hashlib.sha256(a.tobytes()).hexdigest()


def lb_record(lb):
    a = lb.array("a")
    ft = S.objects_ft(lb)
    return {
        "pops_sha256": digest(a),
        "pops_absmax": float(np.abs(a).max()),
        "pops_sample": [float(v) for v in a.ravel()[:: max(1, a.size // 16)][:16]],
        "vmean": [lb.vmeanx, lb.vmeany, lb.vmeanz],
        "objects_ft": ft.tolist(),
        "node_force_sum": [float(lb.array(f).sum()) for f in ("fx", "fy", "fz")],
        "step": lb.step,
    }


LB_CASES = {
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
    "psi": dict(psi=True, steps=9),
}


def mp_case(L, moving=0, ads=0, adprob=None, steps=40, n=12, interleave=True):
    lb = L.newlb(n, n + 1, n + 3, "null")
    lb.tau = 0.7
    lb.stokes_flow = 0
    lb.objects_moving = moving
    o1 = L.insertsph(lb, 3.5, 5.5, 6.0, 7.2)
    L.addbf(lb, 1e-3, 2e-4, 0)
    if moving:
        o1.velx = 1e-2
        o1.angz = 2e-3
        L.vspread(lb)
    for _ in range(20):
        L.lbstep(lb)
    mp = L.newmp(lb, "null")
    mp.alpha = 0.3
    if adprob is not None:
        mp.adprob = adprob
    L.mpinit(mp)
    if ads:
        L.adall(mp)
    L.mpwall(mp, "x", 0, 1.0)
    L.mpsph(mp, 2.0, 9, 9, 9, 0.5)
    for s in range(steps):
        L.mpstep(mp)
        if interleave and s % 2:
            L.lbstep(lb)
            L.mprhoinit(mp)
    L.mppull(mp) if L.has("mppull") else None
    p = mp.field()
    return {
        "p_sha256": digest(p),
        "p_sum": float(p.sum()),
        "mpmean": L.mpmean(mp),
        "mpspread_x": L.mpspread(mp, "x"),
        "adtotal": L.adtotal(mp, "null", 1),
    }


MP_CASES = {
    "stat": dict(),
    "move": dict(moving=1),
    "ads": dict(ads=1),
    "ads_move": dict(ads=1, moving=1),
    "frozen": dict(interleave=False, steps=30),
}


def run_lb_cases(L):
    return {name: lb_record(S.two_spheres(L, **cfg)) for name, cfg in LB_CASES.items()}


def run_mp_cases(L):
    return {name: mp_case(L, **cfg) for name, cfg in MP_CASES.items()}


def read_rcp():
    spheres = []
    with open(os.path.join(REF_EXAMPLES, "rcp_spheres.dat")) as f:
        for line in f:
            parts = line.split()
            if len(parts) == 4:
                spheres.append([float(v) for v in parts])
    return spheres


def rcp_perm(L, spheres, steps=1000):
    """examples/rcp_perm.pl:50-175 with addbf in place of the removed dpdx
    field: 45^3 box, 144 spheres (diameter 9), tau 0.8, skip_solid, grad 0.15;
    1000 steps, the extra step of lbsave, then measure."""
    sigma, length, grad = 9.0, 5.0, 0.15
    es = int(0.5 + length * sigma)
    scale = es / length
    lb = L.newlb(es, es, es, "null")
    lb.stokes_flow = 1
    lb.skip_solid = 1
    lb.tau = 0.80
    for r, x, y, z in spheres:
        while x < 0.0: x += length
        while y < 0.0: y += length
        while z < 0.0: z += length
        while x >= length: x -= length
        while y >= length: y -= length
        while z >= length: z -= length
        x, y, z = x * scale, y * scale, z * scale
        for ix in (-1, 0, 1):
            for iy in (-1, 0, 1):
                for iz in (-1, 0, 1):
                    ox, oy, oz = x + ix * es, y + iy * es, z + iz * es
                    if (-sigma < ox < es + sigma and -sigma < oy < es + sigma and -sigma < oz < es + sigma):
                        L.insertsph(lb, sigma / 2.0, ox, oy, oz)
    L.flattenobj(lb)
    L.addbf(lb, grad, 0.0, 0.0)
    for _ in range(steps):
        L.lbstep(lb)
    L.bbl(lb); L.propagate(lb); L.collide(lb)
    L.measure(lb)
    eta = lb.rho0 * (lb.tau - 0.5) / 3.0
    return {"vmeanx": lb.vmeanx, "k": lb.vmeanx * eta / grad,
            "pore_fraction": L.countfluid(lb) / lb.nnodes, "step": lb.step}


def sccp_sphere(L, steps=5000):
    """examples/sccp_sphere.pl:52-131, Stokes row: 17^3, tau 0.53125,
    skip_solid, a_nom = (17 - 0.4)/2 at the centre, grad 0.05."""
    es = 17
    lb = L.newlb(es, es, es, "null")
    lb.objects_moving = 0
    lb.vel_corrected = 1
    lb.skip_solid = 1
    lb.tau = 0.53125
    c = (es - 1.0) / 2.0
    L.insertsph(lb, (es - 0.4) / 2.0, c, c, c)
    lb.stokes_flow = 1
    L.addbf(lb, 0.05, 0.0, 0.0)
    for _ in range(steps):
        L.lbstep(lb)
    L.measure(lb)
    u = float(np.sqrt(lb.vmeanx ** 2 + lb.vmeany ** 2 + lb.vmeanz ** 2))
    return {"u_mean": u, "vmeanx": lb.vmeanx}


def sphere_converge(L, n=32, rad=4.5, force=1e-5, tol=1e-8, maxsteps=60000, stop_at=None):
    """The plain-method case: 32^3, one sphere r 4.5 at the box centre,
    body force 1e-5 along x, tau 1, Stokes; checks every 100 steps (98
    lbstep + measure) until |dvmeanx|/|vmeanx| < tol."""
    lb = L.newlb(n, n, n, "null")
    lb.tau = 1.0
    lb.stokes_flow = 1
    c = (n - 1) / 2.0
    obj = L.insertsph(lb, rad, c, c, c)
    L.addbf(lb, force, 0.0, 0.0)
    last, steps = None, 0
    history = []
    while steps < maxsteps:
        for _ in range(98):
            L.lbstep(lb)
        L.measure(lb)
        steps += 100
        history.append(lb.vmeanx)
        if stop_at is not None and steps >= stop_at:
            break
        if last is not None and abs(lb.vmeanx - last) < tol * abs(lb.vmeanx):
            break
        last = lb.vmeanx
    return {"steps": steps, "vmeanx": lb.vmeanx, "frcx": obj.frcx, "frcy": obj.frcy, "frcz": obj.frcz,
            "discrf": L.discrf(lb), "vmeanx_at_2000": history[19] if len(history) >= 20 else None}


FILE_CASES = {
    "moving": dict(),
    "skip_ns": dict(skip=1, stokes=0, tau=0.6),
}


def file_records(L):
    """SHA-256 of every file the reference's file API writes for each file
    case, of the populations after reloading the velocity files, of the
    object table after reloading the object file, and of the tracer after
    mpsubs and moment-propagation steps."""
    import tempfile
    out = {}
    for name, cfg in FILE_CASES.items():
        d = tempfile.mkdtemp()
        _, files = S.file_case(L, d, **cfg)
        rec = {"files": {k: hashlib.sha256(v).hexdigest() for k, v in files.items()}}
        for kind in ("vel.bin", "vel.txt", "obj.txt"):
            rec["reload_" + kind] = digest(S.reload_case(L, d, kind, **cfg)[1])
        out[name] = rec
    d = tempfile.mkdtemp()
    p0, p1 = S.mpsubs_case(L, d)
    out["mpsubs"] = {"p_injected": digest(p0), "p_after_steps": digest(p1)}
    return out


def write_vacf_fixture(strict):
    import tempfile
    sys.path.insert(0, os.path.dirname(HERE))
    from test_oracle import VACF_CASES
    cases = []
    for kw in VACF_CASES:
        d, p, p2, _ = S.vacf_case(strict, tempfile.mkdtemp(), **kw)
        cases.append({"config": kw, "diffusion": d, "p_sha256": digest(p), "p2_sha256": digest(p2)})
    with open(os.path.join(HERE, "vacf.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases}, f, indent=1)


def write_files_fixture(strict):
    with open(os.path.join(HERE, "files.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": file_records(strict)}, f, indent=1)


def main():
    ref_dir = os.path.join(ROOT, "oracle", "_ref")
    if "--files-only" in sys.argv:
        write_files_fixture(Library(os.path.join(ref_dir, "libref_strict.so"), extended=False))
        return
    if "--vacf-only" in sys.argv:
        write_vacf_fixture(Library(os.path.join(ref_dir, "libref_strict.so"), extended=False))
        return
    REF_STRICT = os.path.join(ref_dir, "libref_strict.so")
    REF_SHIPPED = os.path.join(ref_dir, "libref_shipped.so")
    strict = Library(REF_STRICT, extended=False)
    shipped = Library(REF_SHIPPED, extended=False)
    out = {}
    print("lb cases ...", flush=True)
    out["lb"] = {"strict": run_lb_cases(strict), "shipped": run_lb_cases(shipped)}
    print("mp cases ...", flush=True)
    out["mp"] = {"strict": run_mp_cases(strict), "shipped": run_mp_cases(shipped)}
    rcp = read_rcp()
    with open(os.path.join(HERE, "rcp144.json"), "w") as f:
        json.dump({"source": "examples/rcp_spheres.dat (radius, x, y, z in sphere diameters; box 5)",
                   "spheres": rcp}, f, indent=0)
    print("known answers ...", flush=True)
    kat = {
        "rcp_perm": {"published": {"vmeanx": 0.001607, "k": 0.077122, "pore_fraction": 0.40,
                                   "source": "examples/rcp_perm.pl:33-38"},
                     "strict": rcp_perm(strict, rcp), "shipped": rcp_perm(shipped, rcp)},
        "sccp_sphere": {"published": {"u_mean": 0.049391, "source": "examples/sccp_sphere.pl:31"},
                        "strict": sccp_sphere(strict), "shipped": sccp_sphere(shipped)},
        "sphere_converge": {"strict": sphere_converge(strict), "shipped": sphere_converge(shipped)},
    }
    with open(os.path.join(HERE, "lb_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": out["lb"]}, f, indent=1)
    with open(os.path.join(HERE, "mp_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": out["mp"]}, f, indent=1)
    write_files_fixture(strict)
    write_vacf_fixture(strict)
    with open(os.path.join(HERE, "kat.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "kat": kat}, f, indent=1)
    print(json.dumps(kat, indent=1))


if __name__ == "__main__":
    main()
