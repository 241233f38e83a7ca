"""The allocation-free mean-flow entry point (slbc_vsum_noalloc).

Callers that cannot allocate device memory where they need the mean flow
(an application that owns every device buffer through its own pool, a
time-stepping loop that must not call cudaMalloc) pass their own device
buffers; the entry point keeps its partial sums in a static device array.
This test builds the same lattice twice -- once through the allocating
entry points slbc_create / slbc_put_pops / slbc_vsum, once as plain device
buffers handed to slbc_vsum_noalloc -- and checks that two calls in a row
give slbc_vsum's sums (to 1e-12 relative; they use the same reduction
partition), that device free memory does not change across a call, and that
a reduction width beyond the static array is rejected.  It lives in a file
of its own, collected last, and passes alone or after the other tests.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_BLOCKS = 1216  # SLBC_VSUM_NOALLOC_MAX_BLOCKS in include/slb_device.h
TOL = 1e-12

LINKS = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
         (1, 1, 1), (-1, 1, 1), (1, -1, 1), (-1, -1, 1), (1, 1, -1), (-1, 1, -1), (1, -1, -1),
         (-1, -1, -1)]


class Params(C.Structure):
    _fields_ = [("tau", C.c_double), ("rho0", C.c_double), ("stokes_flow", C.c_int),
                ("skip_solid", C.c_int), ("objects_moving", C.c_int)]


def flag_words(solid):
    """Per-node flag words as the library defines them: bit 15 solid, bit q
    when the node and its neighbour x - c_q differ in solidity."""
    f = np.where(solid, 0x8000, 0).astype(np.int64)
    for q in range(1, 15):
        upstream = np.roll(solid, shift=LINKS[q], axis=(0, 1, 2))  # solid[x - c_q]
        f |= np.where(upstream != solid, 1 << q, 0)
    return f.astype(np.uint16).ravel()


def make_case(seed, dims=(12, 10, 14)):
    rng = np.random.default_rng(seed)
    n = int(np.prod(dims))
    i, j, k = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    solid = ((i - 5.5) ** 2 + (j - 4.0) ** 2 + (k - 6.5) ** 2) < 9.0
    a = 1e-4 * rng.standard_normal((n, 15))
    return dims, solid, a


def reference_sums(dll, dims, solid, a, precision, fac, bf):
    """slbc_vsum on a lattice created through the allocating entry points."""
    h = C.c_void_p()
    assert dll.slbc_create(C.byref(h), *dims, precision) == 0, dll.slbc_last_error()
    try:
        objidx = np.where(solid.ravel(), 0, -1).astype(np.int32)
        assert dll.slbc_set_geometry(h, objidx.ctypes.data, 1, None, None, 0) == 0
        par = Params(1.0, 72.0, 1, 0, 0)
        assert dll.slbc_set_params(h, C.byref(par)) == 0
        n = a.shape[0]
        b = [np.full(n, v) for v in bf]
        assert dll.slbc_set_bodyforce(h, b[0].ctypes.data, b[1].ctypes.data, b[2].ctypes.data) == 0
        aa = np.ascontiguousarray(a)
        assert dll.slbc_put_pops(h, aa.ctypes.data) == 0
        out = (C.c_double * 5)()
        assert dll.slbc_vsum(h, C.c_double(fac), None, out) == 0, dll.slbc_last_error()
        return np.array(out[:])
    finally:
        dll.slbc_destroy(h)


@pytest.fixture(scope="module")
def api():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import sunlightlb_gb300
    dll = sunlightlb_gb300.library().dll
    dll.slbc_last_error.restype = C.c_char_p
    dll.slbc_vsum_noalloc.restype = C.c_int
    dll.slbc_vsum_noalloc.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_void_p,
                                      C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                      C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_void_p,
                                      C.c_int, C.c_void_p, C.c_void_p]
    dll.slbc_vsum.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]
    dll.slbc_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
    dll.slbc_destroy.argtypes = [C.c_void_p]
    dll.slbc_set_geometry.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_long]
    dll.slbc_set_params.argtypes = [C.c_void_p, C.c_void_p]
    dll.slbc_set_bodyforce.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    dll.slbc_put_pops.argtypes = [C.c_void_p, C.c_void_p]
    return torch, dll


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_sums_equal_allocating_entry_point(api, precision):
    torch, dll = api
    dims, solid, a = make_case(3 + precision)
    n = a.shape[0]
    fac, bf = -0.5, (1e-5, -2e-6, 3e-7)
    expect = reference_sums(dll, dims, solid, a, precision, fac, bf)

    dtype = torch.float64 if precision == 0 else torch.float32
    npad = (n + 63) // 64 * 64
    pop = torch.zeros(15 * npad, dtype=dtype, device="cuda")
    soa = torch.from_numpy(np.ascontiguousarray(a.T)).to(dtype)  # pop[q*npad + x] = a[x][q]
    for q in range(15):
        pop[q * npad:q * npad + n] = soa[q].cuda()
    flags = torch.from_numpy(flag_words(solid).view(np.int16)).cuda()
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    nblocks = min((n + 255) // 256, MAX_BLOCKS)  # slbc_vsum's reduction width
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        rc = dll.slbc_vsum_noalloc(pop.data_ptr(), npad, precision, 0, flags.data_ptr(), *dims,
                                   72.0, fac, *bf, None, None, nblocks, out.data_ptr(), stream)
        assert rc == 0, dll.slbc_last_error()
        torch.cuda.synchronize()
        return out.cpu().numpy().copy()

    first = call()  # also looks up the static array's device address
    out.zero_()
    torch.cuda.synchronize()
    # device free memory is shared with every other process on the GPU: a
    # change seen once is measured again before it counts as an allocation
    for attempt in range(3):
        alloc_before = torch.cuda.memory_allocated()
        free_before = torch.cuda.mem_get_info()[0]
        second = call()
        free_after = torch.cuda.mem_get_info()[0]
        if free_after == free_before:
            break
    assert torch.cuda.memory_allocated() == alloc_before
    assert free_after == free_before, "the call allocated device memory"
    for got in (first, second):
        assert got[4] == expect[4] == np.count_nonzero(~solid)
        assert np.abs(got - expect).max() <= TOL * np.abs(expect).max(), (got, expect)


def test_noalloc_rejects_width_beyond_static_scratch(api):
    torch, dll = api
    buf = torch.zeros(64 * 15, dtype=torch.float64, device="cuda")
    flags = torch.zeros(64, dtype=torch.int16, device="cuda")
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    for bad in (0, MAX_BLOCKS + 1):
        rc = dll.slbc_vsum_noalloc(buf.data_ptr(), 64, 0, 0, flags.data_ptr(), 4, 4, 4, 72.0, 0.0,
                                   0.0, 0.0, 0.0, None, None, bad, out.data_ptr(), None)
        assert rc != 0
        assert str(MAX_BLOCKS) in dll.slbc_last_error().decode()
