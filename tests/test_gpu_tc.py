"""Tensor-core GEMM of the learned warm start (slbc_tc_gemm: tcgen05.mma
with BF16 operands staged by TMA, FP32 accumulation in TMEM) against a
plain PyTorch FP32 product of the same BF16 values.  Each product is exact
in FP32; only the summation order differs, so the tolerance is 1e-5 of the
largest entry."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def tc(gpu):
    f = gpu.dll.slbc_tc_gemm
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    s = gpu.dll.slbc_tc_status
    s.restype = C.c_int
    return f, s


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 512), (512, 256, 1088), (384, 128, 4096)])
def test_gemm_matches_fp32(gpu, M, N, K):
    torch = pytest.importorskip("torch")
    gemm, status = tc(gpu)
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    D = torch.full((M, N + 4), float("nan"), device="cuda")
    rc = gemm(A.data_ptr(), B.data_ptr(), D.data_ptr(), M, N, K, N + 4, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, gpu.dll.slbc_last_error
    assert status() == 0
    ref = A.float() @ B.float().t()
    got = D[:, :N]
    assert torch.isfinite(got).all()
    assert (got - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()
    assert torch.isnan(D[:, N:]).all()  # nothing written past N


def test_gemm_rejects_bad_shapes(gpu):
    torch = pytest.importorskip("torch")
    gemm, _ = tc(gpu)
    A = torch.zeros(128, 64, device="cuda", dtype=torch.bfloat16)
    D = torch.zeros(128, 128, device="cuda")
    assert gemm(A.data_ptr(), A.data_ptr(), D.data_ptr(), 100, 128, 64, 128, None) != 0
    assert gemm(A.data_ptr(), A.data_ptr(), D.data_ptr(), 128, 128, 48, 128, None) != 0


def conv_fns(gpu):
    f = gpu.dll.slbc_tc_conv3d
    f.restype = C.c_int
    f.argtypes = [C.c_void_p] + [C.c_int] * 7 + [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                                   C.c_int, C.c_void_p, C.c_void_p]
    h = gpu.dll.slbc_tc_halo
    h.restype = C.c_int
    h.argtypes = [C.c_void_p] + [C.c_int] * 7 + [C.c_void_p]
    return f, h


def to_padded(torch, x, ctot, coff):
    """(B, C, D, H, W) -> channels-last buffer with a 1-voxel halo (interior
    filled at channels [coff, coff + C), the rest zero)."""
    B, Cc, D, H, W = x.shape
    buf = torch.zeros(B, D + 2, H + 2, W + 2, ctot, device="cuda", dtype=torch.bfloat16)
    buf[:, 1:-1, 1:-1, 1:-1, coff:coff + Cc] = x.permute(0, 2, 3, 4, 1).to(torch.bfloat16)
    return buf


def gemm_weights(torch, wt):
    """torch weight (cout, cin, 3, 3, 3) -> w[tap][cin/32][cout][32], tap = 9 kz + 3 ky + kx."""
    cout, cin = wt.shape[:2]
    w = wt.permute(2, 3, 4, 0, 1).reshape(27, cout, cin // 32, 32).permute(0, 2, 1, 3)
    return w.contiguous().to(torch.bfloat16)


CONV_CASES = [  # B, D, H, W, cin, cout, in_ctot, in_coff, out_ctot, out_coff, relu, mask
    (2, 8, 8, 8, 32, 32, 32, 0, 32, 0, 0, 0),
    (1, 16, 16, 16, 64, 48, 96, 32, 64, 8, 1, 0),
    (1, 8, 32, 32, 96, 128, 96, 0, 128, 0, 1, 1),
    (1, 4, 4, 64, 32, 256, 32, 0, 256, 0, 0, 0),
    (1, 2, 2, 128, 32, 16, 40, 8, 24, 8, 0, 0),
    # narrower layers (32, 64 or 128 output channels, W % 16, H % 8, D % 2 == 0):
    # input-reuse tiles of 16 x 8 x 2 voxels
    (2, 8, 16, 16, 32, 32, 32, 0, 32, 0, 1, 0),
    (1, 4, 8, 32, 96, 32, 96, 0, 40, 8, 0, 1),
    (1, 6, 16, 32, 64, 64, 96, 32, 72, 8, 1, 0),
    (2, 2, 8, 16, 160, 64, 160, 0, 64, 0, 0, 1),
    (1, 4, 8, 16, 64, 128, 64, 0, 136, 8, 1, 0),
]


@pytest.mark.parametrize("case", CONV_CASES)
def test_conv3d_matches_torch(gpu, case):
    torch = pytest.importorskip("torch")
    F = torch.nn.functional
    conv, halo = conv_fns(gpu)
    B, D, H, W, cin, cout, in_ctot, in_coff, out_ctot, out_coff, relu, use_mask = case
    g = torch.Generator(device="cuda").manual_seed(sum(case))
    x = torch.randn(B, cin, D, H, W, device="cuda", generator=g).to(torch.bfloat16).float()
    wt = (torch.randn(cout, cin, 3, 3, 3, device="cuda", generator=g) / (27 * cin) ** 0.5).to(torch.bfloat16).float()
    bias = torch.randn(cout, device="cuda", generator=g) * 0.1
    st = torch.cuda.current_stream().cuda_stream
    xin = to_padded(torch, x, in_ctot, in_coff)
    assert halo(xin.data_ptr(), B, D, H, W, in_ctot, 0, in_ctot, st) == 0
    ref_pad = F.pad(x, (1, 1, 1, 1, 1, 1), mode="circular").permute(0, 2, 3, 4, 1)
    assert torch.equal(xin[..., in_coff:in_coff + cin].float(), ref_pad)  # the halo
    w = gemm_weights(torch, wt)
    out = torch.full((B, D + 2, H + 2, W + 2, out_ctot), 7.0, device="cuda", dtype=torch.bfloat16)
    ref = F.conv3d(F.pad(x, (1, 1, 1, 1, 1, 1), mode="circular"), wt, bias)
    if relu:
        ref = ref.clamp_min(0.0)
    mask_buf = None
    if use_mask:
        mk = torch.randn(B, cout, D, H, W, device="cuda", generator=g)
        mask_buf = to_padded(torch, mk, out_ctot, out_coff)
        ref = ref * (mk.to(torch.bfloat16).float() > 0)
    rc = conv(xin.data_ptr(), B, D, H, W, in_ctot, in_coff, cin, w.data_ptr(), bias.data_ptr(), cout,
              out.data_ptr(), out_ctot, out_coff, relu, mask_buf.data_ptr() if use_mask else None, st)
    assert rc == 0, gpu.dll.slbc_last_error
    assert gpu.dll.slbc_tc_status() == 0
    got = out[:, 1:-1, 1:-1, 1:-1, out_coff:out_coff + cout].float().permute(0, 4, 1, 2, 3)
    scale = ref.abs().max().item()
    assert ((got - ref).abs() <= 4e-3 * ref.abs() + 2e-3 * scale).all()
    # nothing outside the written interior slice
    untouched = out.clone()
    untouched[:, 1:-1, 1:-1, 1:-1, out_coff:out_coff + cout] = 7.0
    assert (untouched.float() == 7.0).all()


def wgrad_fns(gpu):
    cm = gpu.dll.slbc_tc_cmajor
    cm.restype = C.c_int
    cm.argtypes = [C.c_void_p] + [C.c_int] * 8 + [C.c_longlong, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    wg = gpu.dll.slbc_tc_wgrad
    wg.restype = C.c_int
    wg.argtypes = [C.c_void_p] * 4 + [C.c_int] * 5 + [C.c_longlong, C.c_int, C.c_int, C.c_void_p, C.c_longlong,
                                                     C.c_int, C.c_void_p, C.c_void_p]
    cmt = gpu.dll.slbc_tc_cmajor_tiles
    cmt.restype = C.c_int
    cmt.argtypes = [C.c_void_p] + [C.c_int] * 8 + [C.c_longlong, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    wgt = gpu.dll.slbc_tc_wgrad_tiles
    wgt.restype = C.c_int
    wgt.argtypes = [C.c_void_p] * 2 + [C.c_int] * 5 + [C.c_longlong, C.c_int, C.c_int, C.c_void_p, C.c_longlong,
                                                       C.c_int, C.c_void_p, C.c_void_p]
    return cm, wg, cmt, wgt


def flat_geometry(D, H, W):
    Wp = (W + 2 + 7) // 8 * 8
    pstride = ((D + 2) * (H + 2) * Wp + 63) // 64 * 64
    return Wp, pstride


WGRAD_CASES = [  # B, D, H, W, cin, cout, splits
    (1, 8, 8, 8, 32, 32, 3),
    (2, 16, 16, 16, 96, 64, 7),
    (1, 8, 16, 32, 64, 128, 5),
    (1, 8, 8, 8, 384, 256, 2),
    (1, 16, 16, 16, 32, 32, 40),
    # taps along N: partial last tap group (cin 128: 2 taps per block),
    # input channels in two chunks (cin 384), 3 taps per block (cin 192
    # is one tap per block), more splits than K tiles need
    (1, 8, 8, 16, 128, 128, 3),
    (1, 8, 8, 8, 384, 128, 2),
    (2, 8, 8, 8, 192, 64, 4),
    (1, 8, 8, 8, 64, 32, 200),
]


@pytest.mark.parametrize("B,D,H,W,nch", [(1, 8, 8, 8, 32), (2, 8, 16, 8, 128)])
def test_cmajor_tiles_layout(gpu, B, D, H, W, nch):
    """slbc_tc_cmajor_tiles writes the same rows as slbc_tc_cmajor, regrouped
    as [tile][copy][channel][64]."""
    torch = pytest.importorskip("torch")
    _, halo = conv_fns(gpu)
    cm, _, cmt, _ = wgrad_fns(gpu)
    g = torch.Generator(device="cuda").manual_seed(B * 100 + nch)
    y = torch.randn(B, nch, D, H, W, device="cuda", generator=g).to(torch.bfloat16).float()
    st = torch.cuda.current_stream().cuda_stream
    yb = to_padded(torch, y, nch, 0)
    assert halo(yb.data_ptr(), B, D, H, W, nch, 0, nch, st) == 0
    Wp, pstride = flat_geometry(D, H, W)
    cols = B * pstride
    plain = torch.empty(3, nch, cols, device="cuda", dtype=torch.bfloat16)
    tiles = torch.full((cols // 64, 3, nch, 64), 7.0, device="cuda", dtype=torch.bfloat16)
    for i, shift in enumerate((-1, 0, 1)):
        assert cm(yb.data_ptr(), B, D, H, W, nch, 0, nch, Wp, pstride, shift, 0, plain[i].data_ptr(), st) == 0
        assert cmt(yb.data_ptr(), B, D, H, W, nch, 0, nch, Wp, pstride, shift, i, 3, tiles.data_ptr(), st) == 0
    torch.cuda.synchronize()
    want = plain.view(3, nch, cols // 64, 64).permute(2, 0, 1, 3)
    assert torch.equal(tiles, want)


@pytest.mark.parametrize("layout", ["copies_apart", "copies_one_buffer", "tiles"])
@pytest.mark.parametrize("case", WGRAD_CASES)
def test_wgrad_matches_torch(gpu, case, layout):
    """Against torch's weight gradient, with dY's three copies in separate
    allocations, equally spaced in one (one TMA box per stage for them), or
    as K-tile blocks (slbc_tc_cmajor_tiles + slbc_tc_wgrad_tiles)."""
    torch = pytest.importorskip("torch")
    F = torch.nn.functional
    _, halo = conv_fns(gpu)
    cm, wg, cmt, wgt = wgrad_fns(gpu)
    B, D, H, W, cin, cout, splits = case
    g = torch.Generator(device="cuda").manual_seed(sum(case) + 11)
    x = torch.randn(B, cin, D, H, W, device="cuda", generator=g).to(torch.bfloat16).float()
    dy = torch.randn(B, cout, D, H, W, device="cuda", generator=g).to(torch.bfloat16).float()
    st = torch.cuda.current_stream().cuda_stream
    xb = to_padded(torch, x, cin, 0)
    yb = to_padded(torch, dy, cout, 0)
    assert halo(xb.data_ptr(), B, D, H, W, cin, 0, cin, st) == 0
    assert halo(yb.data_ptr(), B, D, H, W, cout, 0, cout, st) == 0
    Wp, pstride = flat_geometry(D, H, W)
    xt = torch.empty(cin, B * pstride, device="cuda", dtype=torch.bfloat16)
    assert cm(xb.data_ptr(), B, D, H, W, cin, 0, cin, Wp, pstride, 0, 1, xt.data_ptr(), st) == 0
    if layout == "tiles" and cout > 128:
        pytest.skip("K-tile blocks: cout 32, 64 or 128")
    dys = []
    whole = torch.empty(3, cout, B * pstride, device="cuda", dtype=torch.bfloat16)
    for i, shift in enumerate((-1, 0, 1)):
        if layout == "tiles":
            assert cmt(yb.data_ptr(), B, D, H, W, cout, 0, cout, Wp, pstride, shift, i, 3, whole.data_ptr(), st) == 0
            continue
        t = whole[i] if layout == "copies_one_buffer" else torch.empty(cout, B * pstride, device="cuda",
                                                                      dtype=torch.bfloat16)
        assert cm(yb.data_ptr(), B, D, H, W, cout, 0, cout, Wp, pstride, shift, 0, t.data_ptr(), st) == 0
        dys.append(t)
    partial = torch.empty(splits * 27 * cout * cin, device="cuda")
    dw = torch.empty(27, cout, cin, device="cuda")
    if layout == "tiles":
        rc = wgt(whole.data_ptr(), xt.data_ptr(), B, D, H, W, Wp, pstride, cin, cout, partial.data_ptr(),
                 partial.numel(), splits, dw.data_ptr(), st)
    else:
        rc = wg(dys[0].data_ptr(), dys[1].data_ptr(), dys[2].data_ptr(), xt.data_ptr(), B, D, H, W, Wp, pstride,
                cin, cout, partial.data_ptr(), partial.numel(), splits, dw.data_ptr(), st)
    assert rc == 0, gpu.dll.slbc_last_error
    assert gpu.dll.slbc_tc_status() == 0
    ref = torch.nn.grad.conv3d_weight(F.pad(x, (1, 1, 1, 1, 1, 1), mode="circular"), (cout, cin, 3, 3, 3), dy)
    ref = ref.permute(2, 3, 4, 0, 1).reshape(27, cout, cin)
    assert (dw - ref).abs().max().item() <= 1e-4 * ref.abs().max().item()

