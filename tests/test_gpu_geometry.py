"""The solid boundary-node list built on the GPU (slbc_set_geometry_auto).

From the dense object index of every node the library builds the flag words
and the list of solid nodes with at least one fluid neighbour (over the 14
links, periodic), grouped by object with node order kept inside an object:
the list that force accumulation and distribf follow.  Checked against the
same definition in numpy, on random multi-object maps including thin and
non-cubic lattices.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LINKS = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
         (1, 1, 1), (-1, 1, 1), (1, -1, 1), (-1, -1, 1), (1, 1, -1), (-1, 1, -1), (1, -1, -1),
         (-1, -1, -1)]


def random_objects(dims, nobj, seed):
    rng = np.random.default_rng(seed)
    objidx = np.full(dims, -1, dtype=np.int32)
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    for o in range(nobj):
        for _ in range(3):  # a few periodic balls per object
            c = [rng.uniform(0, d) for d in dims]
            r = rng.uniform(1.0, max(1.5, 0.3 * min(dims)))
            d2 = 0.0
            for ax, g in enumerate((i, j, k)):
                dd = np.abs(g - c[ax])
                dd = np.minimum(dd, dims[ax] - dd)
                d2 = d2 + dd ** 2
            objidx[d2 < r * r] = o
    return objidx


def expected(objidx):
    solid = objidx >= 0
    fluid_nb = np.zeros_like(solid)
    for q in range(1, 15):
        fluid_nb |= ~np.roll(solid, shift=LINKS[q], axis=(0, 1, 2))
    nodes = np.flatnonzero((solid & fluid_nb).ravel())
    obj = objidx.ravel()[nodes]
    order = np.argsort(obj, kind="stable")
    return nodes[order], obj[order]


@pytest.mark.parametrize("dims,nobj,seed", [((12, 10, 14), 1, 0), ((40, 33, 70), 5, 1), ((3, 64, 5), 3, 2),
                                            ((64, 64, 64), 7, 3), ((1, 9, 40), 2, 4)])
def test_boundary_list_built_on_gpu(gpu, dims, nobj, seed):
    dll = gpu.dll
    dll.slbc_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
    dll.slbc_create.restype = C.c_int
    dll.slbc_destroy.argtypes = [C.c_void_p]
    f = dll.slbc_set_geometry_auto
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.POINTER(C.c_long)),
                  C.POINTER(C.POINTER(C.c_int)), C.POINTER(C.c_long)]
    f.restype = C.c_int
    dll.slbc_last_error.restype = C.c_char_p
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    objidx = random_objects(dims, nobj, seed)
    want_nodes, want_obj = expected(objidx)
    h = C.c_void_p()
    assert dll.slbc_create(C.byref(h), *dims, 1) == 0, dll.slbc_last_error()
    try:
        bn, bo, nb = C.POINTER(C.c_long)(), C.POINTER(C.c_int)(), C.c_long()
        flat = np.ascontiguousarray(objidx.ravel())
        rc = f(h, flat.ctypes.data, nobj, C.byref(bn), C.byref(bo), C.byref(nb))
        assert rc == 0, dll.slbc_last_error()
        try:
            got_nodes = np.ctypeslib.as_array(bn, shape=(nb.value,)).copy() if nb.value else np.zeros(0, int)
            got_obj = np.ctypeslib.as_array(bo, shape=(nb.value,)).copy() if nb.value else np.zeros(0, int)
        finally:
            libc.free(C.cast(bn, C.c_void_p))
            libc.free(C.cast(bo, C.c_void_p))
        assert nb.value == len(want_nodes)
        assert np.array_equal(got_nodes, want_nodes)
        assert np.array_equal(got_obj, want_obj)
    finally:
        dll.slbc_destroy(h)
