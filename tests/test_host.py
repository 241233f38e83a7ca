"""Host side of the GB300 library, on the CPU: the shared library loads and
exports every function the headers declare, set-up routines (objects,
geometry, mask, wall velocity, body force, adsorption marks) give exactly
the oracle's host arrays, and device calls fail loudly when there is no GPU.
None of these tests launches a kernel."""

import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    with open(os.path.join(ROOT, "include", header)) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set()
    for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text, re.M):
        names.add(m.group(1))
    return names


@pytest.mark.parametrize("header", ["sunlightlb.h", "slb_device.h"])
def test_library_exports_every_declared_function(gpu, header):
    names = declared_functions(header)
    assert len(names) > 10
    missing = [n for n in sorted(names) if not hasattr(gpu.dll, n)]
    assert not missing, f"{header}: not exported: {missing}"


def obj_ids(lb):
    """Object id per node (-1 fluid), independent of pointer values."""
    ids = {o.address: o.id for o in lb.objects()}
    raw = lb.array("obj")
    return np.array([ids.get(int(p), -2) if p else -1 for p in raw])


def same_host_state(a, b):
    assert np.array_equal(obj_ids(a), obj_ids(b))
    assert np.array_equal(a.array("mask"), b.array("mask"))
    assert a.next_id == b.next_id and a.changed_objects == b.changed_objects
    pa = [(o.id, o.posx, o.posy, o.posz) for o in a.objects()]
    pb = [(o.id, o.posx, o.posy, o.posz) for o in b.objects()]
    assert pa == pb
    for f in ("ux", "uy", "uz", "bx", "by", "bz"):
        assert np.array_equal(a.array(f), b.array(f)), f


def build_geometry(L, rng_seed):
    rng = np.random.default_rng(rng_seed)
    lb = L.newlb(11, 12, 13, "null")
    rets = []
    for _ in range(12):
        r = float(rng.uniform(-1.0, 6.0))
        c = [float(v) for v in rng.uniform(-4.0, 16.0, 3)]
        o = L.insertsph(lb, r, *c)
        rets.append(o is None)
    rets.append(L.insertcyl(lb, "y", 2.2, 3.0, 4.5) is None)
    rets.append(L.insertcyl(lb, "zh", 4.5, 5.0, 5.0) is None)
    rets.append(L.insertwall(lb, "x", 10) is None)
    rets.append(L.insertwall(lb, "k", 40) is None)       # out of range: empty object stays
    rets.append(L.insertslab(lb, 1.5, 4.5, -1.0, 3.2, 7.0, 12.5) is None)
    rets.append(L.insertslab(lb, 3.0, 3.5, 0, 1, 0, 1) is None)  # no node
    L.syncobjs(lb)
    return lb, rets


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_geometry_set_up_matches_oracle(gpu, orc, seed):
    a, ra = build_geometry(gpu, seed)
    b, rb = build_geometry(orc, seed)
    assert ra == rb
    same_host_state(a, b)
    assert gpu.countfluid(a) == orc.countfluid(b)
    for kind in ("links", "faces"):
        assert gpu.countmask(a, kind) == orc.countmask(b, kind)


def test_flatten_invert_remove_match_oracle(gpu, orc):
    out = []
    for L in (gpu, orc):
        lb, _ = build_geometry(L, 7)
        L.flattenobj(lb)
        s1 = (obj_ids(lb).copy(), [(o.id, o.posx, o.posy, o.posz) for o in lb.objects()])
        L.invertobj(lb)
        L.syncobjs(lb)
        s2 = (obj_ids(lb).copy(), lb.array("mask").copy(), [(o.id, o.posx) for o in lb.objects()])
        L.removeobjs(lb)
        s3 = (obj_ids(lb).copy(), lb.next_id)
        out.append((s1, s2, s3))
    (a1, a2, a3), (b1, b2, b3) = out
    assert np.array_equal(a1[0], b1[0]) and a1[1] == b1[1]
    assert np.array_equal(a2[0], b2[0]) and np.array_equal(a2[1], b2[1]) and a2[2] == b2[2]
    assert np.array_equal(a3[0], b3[0]) and a3[1] == b3[1]


def test_wall_velocity_and_body_force_match_oracle(gpu, orc):
    states = []
    for L in (gpu, orc):
        lb, _ = build_geometry(L, 4)
        for o in lb.objects():
            o.velx, o.vely, o.velz = 1e-3 * o.id, -2e-3, 5e-4
            o.angx, o.angy, o.angz = 1e-4, 2e-4 * o.id, -3e-4
        L.vspread(lb)
        L.vset(lb, 0, 0, 0, 0.1, 0.2, 0.3)
        L.vset(lb, 50, 0, 0, 0.1, 0.2, 0.3)
        L.addbf(lb, 1e-5, -2e-6, 3e-7)
        L.addbf(lb, 1e-5, 0.0, 0.0)
        states.append(lb)
    same_host_state(*states)
    gpu.zerobf(states[0]); orc.zerobf(states[1])
    same_host_state(*states)


def test_adsorption_marks_match_oracle(gpu, orc):
    masks = []
    for L in (gpu, orc):
        lb, _ = build_geometry(L, 5)
        mp = L.newmp(lb, "null")
        L.adsph(mp, 4.0, 5.0, 5.0, 5.0)
        L.adslab(mp, -1, 5, -1, 20, 3, 9)
        L.adcyl(mp, "x", 3.0, 6.0, 6.0)
        m1 = lb.array("mask").copy()
        L.adall(mp)
        m2 = lb.array("mask").copy()
        L.adnone(mp)
        masks.append((m1, m2, lb.array("mask").copy()))
    for x, y in zip(*masks):
        assert np.array_equal(x, y)


def test_insertsph_bounding_box_equals_full_scan(gpu, orc):
    """The library scans only a sphere's bounding box; the node set must be
    the reference's full-lattice scan for awkward radii and centres."""
    rng = np.random.default_rng(11)
    for _ in range(40):
        dims = [int(v) for v in rng.integers(1, 9, 3)]
        r = float(rng.choice([0.0, 0.5, 1.0, np.sqrt(2.0), 2.5, 7.9, 30.0, -3.0]))
        c = [float(v) for v in rng.uniform(-10, 18, 3)]
        res = []
        for L in (gpu, orc):
            lb = L.newlb(*dims, "null")
            o = L.insertsph(lb, r, *c)
            res.append((o is None, obj_ids(lb), lb.next_id))
        assert res[0][0] == res[1][0] and np.array_equal(res[0][1], res[1][1]) and res[0][2] == res[1][2]


def test_device_call_without_gpu_fails_loudly(gpu):
    """No CPU path: without a CUDA device the first device call exits with
    the reference's fatal-error convention and a clear message."""
    if gpu.dll.slbc_device_count() > 0:
        pytest.skip("a GPU is present")
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from sunlightlb_gb300.SunlightLB import *\n"
            "lb = newlb(8, 8, 8, 'null')\n"
            "insertsph(lb, 2.0, 3.5, 3.5, 3.5)\n"
            "lbstep(lb)\n"
            "print('still running')\n") % ROOT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "still running" not in r.stdout
    assert "no CUDA device" in r.stderr


def test_host_mirror_without_device(gpu):
    lb = gpu.newlb(4, 5, 6, "null")
    gpu.lbpull(lb)              # allocates the mirror, no device needed
    a = lb.array("a")
    assert a.shape == (120, 15) and not a.any()


def test_packings_are_seeded_and_stable():
    """The seeded packings every workload builds (the block-vectorised random
    sequential addition must keep the sequential decisions)."""
    import hashlib
    from sunlightlb_gb300 import workloads as W
    cases = [((128, 0.30, 4.0, 8.0, 1), {}, 986, "314597b4e685bbfd036c5c3fae1816ec"),
             ((64, 0.45, 3.0, 8.0, 12345), {"overlap": True}, 202, "c29cdae16782366f7e94f4213f942fd7")]
    for args, kw, n, digest in cases:
        for fn in (W.rsa_packing, W.rsa_packing_numpy):
            spheres, solid = fn(*args, **kw)
            assert len(spheres) == n
            assert hashlib.sha256(np.packbits(solid).tobytes()).hexdigest()[:32] == digest
            assert solid.mean() >= args[1]


def test_c_packing_equals_numpy_definition():
    """rsapacking (the library's C routine) takes the same decisions as the
    numpy formulation: identical sphere lists and masks on small, thin-cell,
    overlapping and large-radius cases."""
    from sunlightlb_gb300 import workloads as W
    for args, kw in (((40, 0.2, 3.0, 6.0, 5), {}), ((32, 0.3, 5.0, 12.0, 3), {}),
                     ((48, 0.45, 3.0, 8.0, 7), {"overlap": True}), ((72, 0.33, 2.0, 9.0, 11), {}),
                     ((50, 0.25, 6.0, 12.0, 2), {})):
        a, sa = W.rsa_packing(*args, **kw)
        b, sb = W.rsa_packing_numpy(*args, **kw)
        assert a == b, args
        assert np.array_equal(sa, sb), args


def test_flow_symmetries_algebra():
    """The augmentation's symmetries on a constant flow (1, 2, 3): signs and
    component swap, and each generator undone by applying it again."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    m = torch.zeros((4, 4, 4), dtype=torch.uint8)
    m[0, 1, 2] = 1
    lab = torch.tensor([1.0, 2.0, 3.0]).expand(4, 4, 4, 3).contiguous()
    want = {(1, 0, 0, 0): (1, -2, -3), (0, 1, 0, 0): (1, -2, 3), (0, 0, 1, 0): (1, 2, -3), (0, 0, 0, 1): (1, 3, 2)}
    where = {(1, 0, 0, 0): (3, 1, 2), (0, 1, 0, 0): (0, 2, 2), (0, 0, 1, 0): (0, 1, 1), (0, 0, 0, 1): (0, 2, 1)}
    for bits, u in want.items():
        m2, l2 = WS.symmetry(m, lab, *bits)
        assert torch.equal(l2[1, 2, 3], torch.tensor(u, dtype=torch.float32)), bits
        assert m2[where[bits]] == 1 and int(m2.sum()) == 1, bits
        m3, l3 = WS.symmetry(m2, l2, *bits)
        assert torch.equal(m3, m) and torch.equal(l3, lab), bits
    # a density channel moves with the nodes; the x reflection reverses the
    # force, so by Stokes linearity the whole solution -- the density
    # deviation included -- is negated; no other transform changes its sign
    lab4 = torch.cat([lab, torch.full((4, 4, 4, 1), 5.0)], dim=-1)
    lab4[0, 1, 2, 3] = 7.0
    for bits in want:
        m2, l2 = WS.symmetry(m, lab4, *bits)
        s = -1.0 if bits[0] else 1.0
        assert torch.equal(l2[..., :3], WS.symmetry(m, lab, *bits)[1]), bits
        assert float(l2[where[bits]][3]) == 7.0 * s and int((l2[..., 3] == 7.0 * s).sum()) == 1, bits
        assert int((l2[..., 3] == 5.0 * s).sum()) == 63, bits
    m2, l2 = WS.symmetry(m, lab4, 1, 1, 1, 1)
    assert float(l2[..., 3].sum()) == -(7.0 + 63 * 5.0)


def test_host_parallel_ranges_cover_once(gpu):
    """slb_parallel_for (the host loops of uploads and downloads): the
    ranges handed to the callback cover [0, n) exactly once, for sizes
    below, at and above the split threshold, on however many host threads
    the machine has."""
    import ctypes as C
    import threading
    fn_t = C.CFUNCTYPE(None, C.c_long, C.c_long, C.c_void_p)
    par = gpu.dll.slb_parallel_for
    par.argtypes = [C.c_long, C.c_long, fn_t, C.c_void_p]
    par.restype = None
    lock = threading.Lock()
    for n, grain in ((0, 16), (5, 16), (1000, 1), (1 << 20, 1 << 16), (3_000_001, 1 << 18)):
        seen = []

        def cb(lo, hi, ctx):
            with lock:
                seen.append((lo, hi))

        cfun = fn_t(cb)
        par(n, grain, cfun, None)
        seen.sort()
        covered = 0
        for lo, hi in seen:
            assert lo == covered and hi >= lo, (n, seen)
            covered = hi
        assert covered == n, (n, seen)


def test_wgrad_splits_fill_one_wave(gpu):
    """slbc_tc_wgrad_splits (host logic): for every layer shape of the
    network the K splits times the blocks per split fit the 152 SMs of a
    GB300 in one wave (one block per SM for cout <= 128, two for the
    256-channel layers); a block left over for a second wave doubles the
    launch.  Without a device the function assumes 152 SMs."""
    import ctypes as C
    if gpu.dll.slbc_device_count() > 0:
        pytest.skip("a GPU is present: the split count follows its SM count")
    f = gpu.dll.slbc_tc_wgrad_splits
    f.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_longlong]
    f.restype = C.c_int
    big = 1 << 40
    # (cin, cout): (splits, blocks per split)
    want = {(32, 32): (152, 1), (96, 32): (50, 3), (32, 64): (76, 2), (64, 64): (25, 6), (192, 64): (8, 18),
            (64, 128): (16, 9), (128, 128): (10, 15), (384, 128): (2, 54), (128, 256): (5, 54),
            (256, 256): (5, 54)}
    for (cin, cout), (splits, blocks) in want.items():
        got = f(cin, cout, big, big)
        assert got == splits, (cin, cout, got)
        per_sm = 2 if cout > 128 else 1
        assert got * blocks <= 152 * per_sm < (got + 1) * blocks, (cin, cout)
    # capped by the K tiles (at least 8 per split) and by the partial buffer
    assert f(32, 32, 80, big) == 10
    assert f(32, 32, big, 7) == 7
    assert f(32, 32, 3, big) == 1
