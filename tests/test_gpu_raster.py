"""GPU sphere rasterisation (insertspheres) against insertsph one sphere at
a time (reference src/lbobjs.c:204-232): the same object list (ids, centres)
and the same object map, node for node, on random sphere sets -- overlapping
spheres, spheres reaching past the lattice or lying wholly outside it,
negative and sub-node radii, spheres over objects already in the map -- and
on a seeded packing with its periodic images, against the GPU library's own
insertsph and the CPU oracle's."""

import numpy as np
import pytest

from scenarios import object_ids

pytestmark = pytest.mark.gpu


def sphere_set(seed, dims, n):
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.3, 5.0, n)
    r[::7] *= -1.0  # insertsph squares the radius
    c = np.stack([rng.uniform(-6, d + 6, n) for d in dims], axis=1)
    c[3] = (1e4, 0.0, 0.0)  # wholly outside: no object
    return r, c


def build(L, dims, r, c, batched, pre=False):
    lb = L.newlb(*dims, "null")
    if pre:
        L.insertslab(lb, 2.5, 7.5, -1.0, 30.0, 3.0, 9.0)
    if batched:
        made = L.insertspheres(lb, len(r), r, c[:, 0], c[:, 1], c[:, 2])
    else:
        made = sum(L.insertsph(lb, float(r[s]), *map(float, c[s])) is not None for s in range(len(r)))
    objs = [(o.id, o.posx, o.posy, o.posz) for o in lb.objects()]
    return made, object_ids(lb), objs, lb.next_id


@pytest.mark.parametrize("seed,dims,n,pre", [(1, (17, 19, 23), 40, False), (2, (9, 31, 12), 25, True),
                                            (3, (33, 8, 16), 60, False), (4, (5, 5, 5), 12, True)])
def test_insertspheres_equals_insertsph(gpu, orc, seed, dims, n, pre):
    r, c = sphere_set(seed, dims, n)
    got = build(gpu, dims, r, c, True, pre)
    for ref in (build(gpu, dims, r, c, False, pre), build(orc, dims, r, c, False, pre)):
        assert got[0] == ref[0]
        assert np.array_equal(got[1], ref[1])
        assert got[2] == ref[2]
        assert got[3] == ref[3]


def test_insertspheres_packing_with_images(gpu, orc):
    from sunlightlb_gb300 import workloads as W
    n = 48
    spheres, solid = W.rsa_packing(n, 0.3, 3.0, 6.0, 5)
    r, c = [], []
    for rad, x, y, z in spheres:
        for im in W.images((n, n, n), rad, (x, y, z)):
            r.append(rad)
            c.append(im)
    r, c = np.array(r), np.array(c)
    got = build(gpu, (n, n, n), r, c, True)
    ref = build(orc, (n, n, n), r, c, False)
    assert got[0] == ref[0] and np.array_equal(got[1], ref[1]) and got[2] == ref[2]
    assert np.array_equal(got[1].reshape(n, n, n) >= 0, solid)
