"""The learned warm start's network: loss and every weight and bias
gradient of the tensor-core training step against the CPU oracle
(oracle/orc_unet.py, float64 on the same BF16-rounded weights and inputs).
Activations are BF16 between layers on the GPU, so the comparison is on the
relative L2 norm of each layer's gradient (5%) and of the loss (2%)."""

import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import orc_unet
    return orc_unet


@pytest.mark.parametrize("nch,widths,B", [(3, (32, 32, 32, 32), 2), (4, (32, 32, 32, 32), 2),
                                          (4, (32, 64, 128, 256), 1)])
def test_unet_gradients_match_cpu_oracle(gpu, nch, widths, B):
    """nch label channels: the velocity, and with 4 the density deviation;
    the network's own widths 32 -> 64 -> 128 -> 256 as well as a narrow
    form."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    orc = oracle()
    D, H, W = 32, 32, 64
    net = WS.UNet(gpu, D, H, W, batch=B, widths=widths, seed=3, features=0)
    rng = np.random.default_rng(5)
    solid = (rng.random((B, D, H, W)) > 0.7).astype(np.uint8)
    zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    lab = np.stack([np.sin(2 * np.pi * xx / W) * np.cos(2 * np.pi * yy / H),
                    0.5 * np.cos(2 * np.pi * zz / D), 0.2 * np.sin(2 * np.pi * (xx + zz) / W),
                    0.3 * np.cos(2 * np.pi * (yy + zz) / H)][:nch], axis=-1)
    labels = np.broadcast_to(lab, (B, D, H, W, nch)) * (1 - solid[..., None])
    labels = np.ascontiguousarray(labels, dtype=np.float32)
    m_dev = torch.as_tensor(solid, device="cuda")
    l_dev = torch.as_tensor(labels, device="cuda")
    net.encode(m_dev)
    net.forward()
    loss = float(net.loss_and_backward(l_dev).item())
    assert net.status() == 0
    params = {}
    for name, *_ in net.layers:
        p = net.params[name]
        params[name] = (p["w"].to(torch.bfloat16).double().cpu().numpy(), p["b"].double().cpu().numpy())
    inp = np.zeros((B, D, H, W, WS.IN_CH))
    inp[..., 0] = solid
    ref_loss, ref = orc.forward_backward(params, inp, labels.astype(np.float64))
    assert abs(loss - ref_loss) <= 0.02 * ref_loss, (loss, ref_loss)
    for name, *_ in net.layers:
        gw = net.params[name]["gw"].double().cpu().numpy()
        gb = net.params[name]["gb"].double().cpu().numpy()
        rw, rb = ref[name]
        assert np.linalg.norm(gw - rw) <= 0.05 * np.linalg.norm(rw), name
        assert np.linalg.norm(gb - rb) <= 0.05 * np.linalg.norm(rb) + 1e-12, name


def test_wall_distance_features(gpu):
    """Input channels 1 and 2: periodic distance to the nearest solid node
    (searched within 5, capped there) / 5 and its square; 0 on solid nodes."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    B, D, H, W = 1, 32, 32, 64
    net = WS.UNet(gpu, D, H, W, batch=B, widths=(32, 32, 32, 32), seed=3)
    rng = np.random.default_rng(9)
    solid = (rng.random((B, D, H, W)) > 0.97).astype(np.uint8)
    net.encode(torch.as_tensor(solid, device="cuda"))
    got = net.buf["IN"][0, 1:-1, 1:-1, 1:-1, :3].float().cpu().numpy()
    best = np.full((D, H, W), 25.0)
    s = solid[0].astype(bool)
    for dz in range(-5, 6):
        for dy in range(-5, 6):
            for dx in range(-5, 6):
                d2 = dx * dx + dy * dy + dz * dz
                if d2 >= 25:
                    continue
                hit = np.roll(s, shift=(-dz, -dy, -dx), axis=(0, 1, 2))
                best = np.where(hit & (d2 < best), d2, best)
    d = np.where(s, 0.0, np.sqrt(best) / 5.0)
    assert np.array_equal(got[..., 0], s.astype(np.float32))
    assert np.abs(got[..., 1] - d).max() <= 4e-3
    assert np.abs(got[..., 2] - np.where(s, 0.0, d * d)).max() <= 4e-3


def test_wall_distance_features_wide(gpu):
    """features = 2: the distance searched to 12 (capped there) / 12 and its
    square in channels 1 and 2, min(d, 5) / 5 in channel 3 -- against the
    cube search over periodic images with numpy."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    k = WS.Kernels(gpu.dll)
    B, D, H, W = 2, 20, 24, 30
    rng = np.random.default_rng(17)
    solid = (rng.random((B, D, H, W)) > 0.995).astype(np.uint8)
    out = torch.zeros((B, D + 2, H + 2, W + 2, 32), device="cuda", dtype=torch.bfloat16)
    k.nn_encode(torch.as_tensor(solid, device="cuda").data_ptr(), B, D, H, W, out.data_ptr(), 32, 2,
                torch.cuda.current_stream().cuda_stream)
    got = out[:, 1:-1, 1:-1, 1:-1, :].float().cpu().numpy()
    R = 12
    for b in range(B):
        s = solid[b].astype(bool)
        best = np.full((D, H, W), float(R * R))
        for dz in range(-R, R + 1):
            for dy in range(-R, R + 1):
                for dx in range(-R, R + 1):
                    d2 = dx * dx + dy * dy + dz * dz
                    if d2 >= R * R:
                        continue
                    hit = np.roll(s, shift=(-dz, -dy, -dx), axis=(0, 1, 2))
                    best = np.where(hit & (d2 < best), d2, best)
        dist = np.sqrt(best)
        d = np.where(s, 0.0, dist / R)
        assert np.array_equal(got[b, ..., 0], s.astype(np.float32))
        assert np.abs(got[b, ..., 1] - d).max() <= 4e-3
        assert np.abs(got[b, ..., 2] - np.where(s, 0.0, d * d)).max() <= 4e-3
        assert np.abs(got[b, ..., 3] - np.where(s, 0.0, np.minimum(dist, 5.0) / 5.0)).max() <= 4e-3
        assert not got[b, ..., 4:].any()


@pytest.mark.parametrize("B,D,H,W,frac", [(2, 4, 8, 16, 0.98), (1, 12, 3, 40, 0.995), (3, 16, 16, 16, 0.9)])
def test_wall_distance_small_and_wrapped(gpu, B, D, H, W, frac):
    """The separable distance passes on grids thinner than the search cube
    (offsets wrap onto the same node more than once) and on batches: equal
    to the cube search over periodic images."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    k = WS.Kernels(gpu.dll)
    rng = np.random.default_rng(B * 1000 + D * 10 + W)
    solid = (rng.random((B, D, H, W)) > frac).astype(np.uint8)
    out = torch.zeros((B, D + 2, H + 2, W + 2, 32), device="cuda", dtype=torch.bfloat16)
    k.nn_encode(torch.as_tensor(solid, device="cuda").data_ptr(), B, D, H, W, out.data_ptr(), 32, 1,
                torch.cuda.current_stream().cuda_stream)
    got = out[:, 1:-1, 1:-1, 1:-1, :].float().cpu().numpy()
    for b in range(B):
        s = solid[b].astype(bool)
        best = np.full((D, H, W), 25.0)
        for dz in range(-5, 6):
            for dy in range(-5, 6):
                for dx in range(-5, 6):
                    d2 = dx * dx + dy * dy + dz * dz
                    if d2 >= 25:
                        continue
                    hit = np.roll(s, shift=(-dz, -dy, -dx), axis=(0, 1, 2))
                    best = np.where(hit & (d2 < best), d2, best)
        d = np.where(s, 0.0, np.sqrt(best) / 5.0)
        assert np.array_equal(got[b, ..., 0], s.astype(np.float32))
        assert np.abs(got[b, ..., 1] - d).max() <= 4e-3
        assert np.abs(got[b, ..., 2] - np.where(s, 0.0, d * d)).max() <= 4e-3
        assert not got[b, ..., 3:].any()


def test_training_lowers_the_loss(gpu):
    """A few Adam steps on one batch reduce its loss."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    B, D, H, W = 2, 32, 32, 64
    net = WS.UNet(gpu, D, H, W, batch=B, widths=(32, 32, 32, 32), seed=4)
    rng = np.random.default_rng(6)
    solid = (rng.random((B, D, H, W)) > 0.75).astype(np.uint8)
    labels = (rng.random((B, D, H, W, 3)).astype(np.float32) * 0.5) * (1 - solid[..., None])
    m_dev = torch.as_tensor(solid, device="cuda")
    l_dev = torch.as_tensor(labels, device="cuda")
    hist = WS.train(net, m_dev, l_dev, iters=60, lr=2e-3, seed=1, log_every=1, warmup=10)
    assert net.status() == 0
    first = np.mean([l for _, l in hist[:5]])
    last = np.mean([l for _, l in hist[-5:]])
    assert last < 0.7 * first, (first, last)


def test_projection_loss_term(gpu):
    """slbc_nn_proj: loss += (w / B) sum_n s_n^2 and grad += 2 w s_n
    label_n / (q_n B) with s_n = <label_n, pred_n - label_n> / q_n, q_n =
    <label_n, label_n> over the 3 velocity channels of 4-channel labels,
    against float64 torch on the same data (BF16 gradient rounding)."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    k = WS.Kernels(gpu.dll)
    B, D, H, W, ctot, lch, w = 3, 8, 8, 16, 32, 4, 7.5
    g = torch.Generator(device="cuda").manual_seed(12)
    lab = torch.randn(B, D, H, W, lch, device="cuda", generator=g)
    pred = torch.zeros(B, D + 2, H + 2, W + 2, ctot, device="cuda")
    pred[:, 1:-1, 1:-1, 1:-1, :lch] = lab * (1.0 + 0.05 * torch.arange(1, B + 1, device="cuda").view(B, 1, 1, 1, 1))
    pred[:, 1:-1, 1:-1, 1:-1, :lch] += 0.1 * torch.randn(B, D, H, W, lch, device="cuda", generator=g)
    base = 0.01 * torch.randn(B, D + 2, H + 2, W + 2, ctot, device="cuda", generator=g)
    grad = base.to(torch.bfloat16)
    q = lab[..., :3].double().pow(2).sum(dim=(1, 2, 3, 4))
    dot = torch.zeros(B, device="cuda", dtype=torch.float64)
    loss = torch.full((1,), 0.25, device="cuda", dtype=torch.float64)
    st = torch.cuda.current_stream().cuda_stream
    k.nn_proj(pred.data_ptr(), ctot, lab.data_ptr(), lch, 3, q.data_ptr(), B, D, H, W, w, grad.data_ptr(), ctot,
              dot.data_ptr(), loss.data_ptr(), st)
    torch.cuda.synchronize()
    p = pred[:, 1:-1, 1:-1, 1:-1, :3].double()
    s = ((p - lab[..., :3].double()) * lab[..., :3].double()).sum(dim=(1, 2, 3, 4)) / q
    assert abs(float(loss) - (0.25 + w / B * float((s * s).sum()))) <= 1e-9 * (1.0 + float(loss))
    want = base.to(torch.bfloat16).double()
    want[:, 1:-1, 1:-1, 1:-1, :3] += (2.0 * w * s / (q * B)).view(B, 1, 1, 1, 1) * lab[..., :3].double()
    got = grad.double()
    # channels 3.. and the halo untouched; channels 0..2 within BF16 rounding
    assert torch.equal(got[..., 3:], base.to(torch.bfloat16).double()[..., 3:])
    assert torch.equal(got[:, 0], want[:, 0])
    err = (got - want).abs().max().item()
    assert err <= 2 ** -7 * want.abs().max().item(), err


def test_plane_flux_correction(gpu):
    """slbc_nn_plane_flux against float64 numpy: every x plane's velocity
    scaled by qh / q[i] (qh the harmonic mean of the plane fluxes q of u_x),
    the fluid nodes' density deviation raised by 3 p[i] with p the
    midpoint-rule sum of force (1 - qh / q) over the planes before, zero
    mean; afterwards every plane carries qh.  A state with a plane flux <= 0
    is left as it is (spread -1)."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    k = WS.Kernels(gpu.dll)
    D, H, W, force = 12, 6, 10, 1e-6
    rng = np.random.default_rng(4)
    solid = (rng.random((D, H, W)) < 0.3).astype(np.uint8)
    u0 = rng.random((3, D, H, W)) * (1 - solid) * 1e-4
    u0[0] *= (1.0 + 0.4 * np.sin(np.arange(D) / 2.0))[:, None, None]
    d0 = rng.standard_normal((D, H, W)) * 1e-6 * (1 - solid)
    st = torch.cuda.current_stream().cuda_stream
    sdev = torch.as_tensor(solid, device="cuda")
    u = torch.as_tensor(u0.astype(np.float32).ravel(), device="cuda")
    dr = torch.as_tensor(d0.astype(np.float32).ravel(), device="cuda")
    work = torch.zeros(3 * D + 1, device="cuda", dtype=torch.float64)
    k.nn_plane_flux(u.data_ptr(), dr.data_ptr(), sdev.data_ptr(), D, H, W, force, 1.0, work.data_ptr(), st)
    torch.cuda.synchronize()
    u32 = u0.astype(np.float32).astype(np.float64)
    q = u32[0].sum(axis=(1, 2))
    qh = D / (1.0 / q).sum()
    g = force * (1.0 - qh / q)
    p = np.cumsum(g) - 0.5 * g
    p -= p.mean()
    want_u = u32 * (qh / q)[None, :, None, None]
    want_d = d0.astype(np.float32).astype(np.float64) + 3.0 * p[:, None, None] * (1 - solid)
    got_u = u.cpu().numpy().astype(np.float64).reshape(3, D, H, W)
    got_d = dr.cpu().numpy().astype(np.float64).reshape(D, H, W)
    assert np.abs(got_u - want_u).max() <= 1e-6 * np.abs(want_u).max()
    assert np.abs(got_d - want_d).max() <= 1e-6 * np.abs(want_d).max()
    planes = got_u[0].sum(axis=(1, 2))
    assert np.abs(planes - qh).max() <= 1e-5 * qh
    assert abs(float(work[3 * D]) - (q.max() - q.min()) / q.mean()) <= 1e-9
    # a plane without positive flux: nothing changes
    u1 = u0.copy()
    u1[0, 3] = 0.0
    u = torch.as_tensor(u1.astype(np.float32).ravel(), device="cuda")
    dr = torch.as_tensor(d0.astype(np.float32).ravel(), device="cuda")
    k.nn_plane_flux(u.data_ptr(), dr.data_ptr(), sdev.data_ptr(), D, H, W, force, 1.0, work.data_ptr(), st)
    torch.cuda.synchronize()
    assert np.array_equal(u.cpu().numpy(), u1.astype(np.float32).ravel())
    assert np.array_equal(dr.cpu().numpy(), d0.astype(np.float32).ravel())
    assert float(work[3 * D]) == -1.0
    # a gain multiplies the corrected state: velocity, density and pressure
    u = torch.as_tensor(u0.astype(np.float32).ravel(), device="cuda")
    dr = torch.as_tensor(d0.astype(np.float32).ravel(), device="cuda")
    k.nn_plane_flux(u.data_ptr(), dr.data_ptr(), sdev.data_ptr(), D, H, W, force, 0.75, work.data_ptr(), st)
    torch.cuda.synchronize()
    got_u = u.cpu().numpy().astype(np.float64).reshape(3, D, H, W)
    got_d = dr.cpu().numpy().astype(np.float64).reshape(D, H, W)
    assert np.abs(got_u - 0.75 * want_u).max() <= 1e-6 * np.abs(want_u).max()
    assert np.abs(got_d - 0.75 * want_d).max() <= 1e-6 * np.abs(want_d).max()


def test_cross_flux_correction(gpu):
    """slbc_nn_cross_flux against float64 numpy: u_y gets (mean - Q_y[j]) /
    M[j] |u| in y plane j (Q the plane flux, M the plane sum of |u|), u_z
    the same over z planes; afterwards every y plane carries the mean y
    flux and every z plane the mean z flux, u_x and the x plane fluxes are
    unchanged, and solid nodes (u = 0) stay 0."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    k = WS.Kernels(gpu.dll)
    D, H, W = 10, 12, 14
    rng = np.random.default_rng(8)
    solid = rng.random((D, H, W)) < 0.3
    u0 = (rng.random((3, D, H, W)) - 0.3) * ~solid * 1e-4
    u0[1] += 2e-5 * np.sin(np.arange(H) / 2.0)[None, :, None] * ~solid
    u0[2] += 3e-5 * np.cos(np.arange(W) / 3.0)[None, None, :] * ~solid
    st = torch.cuda.current_stream().cuda_stream
    u = torch.as_tensor(u0.astype(np.float32).ravel(), device="cuda")
    work = torch.zeros(3 * (H + W), device="cuda", dtype=torch.float64)
    k.nn_cross_flux(u.data_ptr(), D, H, W, work.data_ptr(), st)
    torch.cuda.synchronize()
    u32 = u0.astype(np.float32).astype(np.float64)
    sp = np.sqrt((u32 ** 2).sum(axis=0))
    qy, my = u32[1].sum(axis=(0, 2)), sp.sum(axis=(0, 2))
    qz, mz = u32[2].sum(axis=(0, 1)), sp.sum(axis=(0, 1))
    want = u32.copy()
    want[1] += ((qy.mean() - qy) / my)[None, :, None] * sp
    want[2] += ((qz.mean() - qz) / mz)[None, None, :] * sp
    got = u.cpu().numpy().astype(np.float64).reshape(3, D, H, W)
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()
    assert np.array_equal(got[0], u32[0])
    assert not got[:, solid].any()
    scale = np.abs(u32).sum(axis=(1, 2, 3)).max() / D
    assert np.abs(got[1].sum(axis=(0, 2)) - qy.mean()).max() <= 1e-5 * scale
    assert np.abs(got[2].sum(axis=(0, 1)) - qz.mean()).max() <= 1e-5 * scale


def test_gradient_clipping(gpu):
    """Device-side clipping against the running gradient norm: the first
    call sets the running norm, a 10x spike is scaled to 3x the running
    norm, a non-finite gradient is zeroed without touching the running norm."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    net = WS.UNet(gpu, 32, 32, 64, batch=1, widths=(32, 32, 32, 32), seed=2)
    net._alloc_grads()
    grads = [net.params[name]["g" + key] for name, *_ in net.layers for key in ("w", "b")]
    count = sum(g.numel() for g in grads)

    def fill(v):
        for g in grads:
            g.fill_(v)

    def norm():
        return float(torch.sqrt(sum((g.double() ** 2).sum() for g in grads)))

    v = 2.0 ** -10  # exact in FP32, so the norms below are exact
    fill(v)
    n1 = v * np.sqrt(count)
    net.clip_grads(3.0, 0.98)
    assert abs(norm() - n1) <= 1e-6 * n1
    run = n1
    assert abs(float(net.clip_state[1]) - run) <= 1e-6 * run  # decay passed as FP32
    fill(10 * v)  # 10x spike
    net.clip_grads(3.0, 0.98)
    assert abs(norm() - 3.0 * n1) <= 1e-5 * n1
    run = 0.98 * run + 0.02 * 3.0 * n1
    assert abs(float(net.clip_state[1]) - run) <= 1e-6 * run  # decay passed as FP32
    fill(v)
    grads[3][0] = float("nan")
    net.clip_grads(3.0, 0.98)
    assert all(not g.any() for g in grads)
    assert abs(float(net.clip_state[1]) - run) <= 1e-6 * run  # decay passed as FP32
    assert float(net.clip_state[0]) == 0.0


def test_symmetries_map_flows_to_flows(gpu):
    """The training augmentation: each symmetry applied to a bed and its
    converged flow gives the converged flow of the transformed bed
    (FP64 lattices; a wrong sign or component swap shows as an error of
    the size of u_y, u_z)."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    n = 24
    solid = WS.packing(n, 0.25, 11)
    cases = [(1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 0), (0, 0, 0, 1), (1, 1, 0, 1), (1, 1, 1, 1)]
    m0 = torch.as_tensor(solid.astype(np.uint8), device="cuda")
    (f0,), _ = WS.converged_flows(gpu, [solid], tol=1e-11, maxsteps=40000, precision=0, density=True)
    l0 = WS.to_labels(f0, (n, n, n))
    assert l0.shape[-1] == 4
    moved = [WS.symmetry(m0, l0, *c) for c in cases]
    fields, _ = WS.converged_flows(gpu, [m.cpu().numpy().astype(bool) for m, _ in moved], tol=1e-11, maxsteps=40000,
                                   precision=0, density=True)
    scale = float(l0[..., :3].abs().max())
    side = float(l0[..., 1:3].abs().max())
    dscale = float(l0[..., 3].abs().max())
    assert side > 0.05 * scale  # the transverse components are not negligible
    assert dscale > 0.0
    for c, (m, l), f in zip(cases, moved, fields):
        got = WS.to_labels(f, (n, n, n))
        assert float((got[..., :3] - l[..., :3]).abs().max()) <= 1e-6 * scale, c
        # the density channel at its own scale: a wrong sign shows as 2x
        assert float((got[..., 3] - l[..., 3]).abs().max()) <= 1e-5 * dscale, c


def test_trained_network_beats_plain_start(gpu):
    """What the learned part gains over the method without it: a network
    trained briefly (1000 iterations) on 128 converged 64^3 packings starts
    three held-out packings closer to their converged permeability than
    the plain start from rest, and they reach it (within 1e-3) in fewer
    steps (0.80x of the plain steps in recent runs: training order of the
    atomic bias-gradient sums varies, so the bound is 0.9x; the shipped
    network's wall-time gain is test_committed_network_saves_wall_time)."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    n, force = 64, 1e-6
    specs = WS.packing_specs(131, 5, phi_range=(0.1, 0.4))
    solids = [WS.packing(n, phi, sd) for phi, sd in specs]
    train, held = solids[:128], solids[128:]
    fields, _ = WS.converged_flows(gpu, train, force=force, tol=1e-7, maxsteps=20000)
    masks = torch.as_tensor(np.stack(train).astype(np.uint8), device="cuda")
    labels = torch.stack([WS.to_labels(f, (n, n, n)) for f in fields])
    del fields
    sw = 1.0 / labels.pow(2).mean(dim=(1, 2, 3, 4)).clamp_min(1e-12)
    net = WS.UNet(gpu, n, n, n, batch=4, seed=1)
    WS.train(net, masks, labels, 1000, lr=1e-3, seed=2, sample_w=sw, lr_min=1e-5)
    assert net.status() == 0
    inf = WS.UNet(gpu, n, n, n, batch=1, params=net.params)
    rows = []
    for s in held:
        traj = WS.permeability_run(gpu, s, force)
        k = traj[-1][1]
        u = WS.predict_velocity(inf, torch.as_tensor(s.astype(np.uint8), device="cuda"), force, WS.ETA_TAU1)
        trw = WS.permeability_run(gpu, s, force, k_ref=k, warm_u=u, rel=1e-3)
        rows.append((WS.first_within(traj, k, 1e-3)[0], WS.first_within(trw, k, 1e-3)[0],
                     abs(traj[0][1] - k) / k, abs(trw[0][1] - k) / k))
    plain_steps, warm_steps, plain_err, warm_err = (sum(c) for c in zip(*rows))
    assert warm_err < 0.5 * plain_err, rows
    assert warm_steps < 0.9 * plain_steps, rows


def test_committed_network_saves_wall_time(gpu):
    """The shipped network (sunlightlb_gb300/data/warm_unet.npz) against the
    plain start on 10 held-out 128^3 packings at the permeability tolerance
    of 1e-4, checks every 50 steps, inference timed: total wall time and
    steps both lower with the warm start.  Measured 2.1x total wall and 2.4x
    steps on these packings; the test holds 1.6x and 2x (wall clocks vary
    a little between GPUs)."""
    pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    if not os.path.exists(WS.WEIGHTS):
        pytest.skip("no committed network")
    rows, _ = WS.held_out_comparison(gpu, 10, side=128, check=50, rel=1e-4)
    assert all(r["plain_steps"] and r["warm_steps"] for r in rows), rows
    wall = sum(r["plain_wall_s"] for r in rows) / sum(r["warm_wall_s"] for r in rows)
    steps = sum(r["plain_steps"] for r in rows) / sum(r["warm_steps"] for r in rows)
    assert wall >= 1.6 and steps >= 2.0, (wall, steps, rows)


def test_state_warm_start_rebuilds_converged_state(gpu):
    """lbstate / lbsetstatedev: the velocity and density deviation of a
    converged FP32 lattice, set back with u_x - F / (2 rho0) on fluid nodes,
    give the converged permeability within 1e-4 after 10 steps; without a
    density field lbsetstatedev equals lbsetveldev."""
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    n, force = 32, 1e-6
    solid = WS.packing(n, 0.3, 21)
    traj = WS.permeability_run(gpu, solid, force)
    k = traj[-1][1]
    def lattice():
        lb = gpu.newlb(n, n, n, "null")
        lb.precision = 1
        lb.tau = 1.0
        lb.stokes_flow = 1
        WS.W.insert_solid(gpu, lb, solid)
        gpu.syncobjs(lb)
        gpu.addbf(lb, force, 0.0, 0.0)
        gpu.lbsteps(lb, 2)
        return lb

    src = lattice()
    gpu.lbsteps(src, traj[-1][0])
    u = torch.empty(3 * n ** 3, device="cuda", dtype=torch.float32)
    drho = torch.empty(n ** 3, device="cuda", dtype=torch.float32)
    gpu.lbstate(src, u.data_ptr(), drho.data_ptr())
    torch.cuda.synchronize()
    gpu.freelb(src)
    fluid = torch.as_tensor(~solid.reshape(-1), device="cuda")
    assert float(drho[~fluid].abs().max()) == 0.0 and float(drho[fluid].abs().max()) > 0.0
    us = u.clone()
    us[:n ** 3][fluid] -= force / (2 * 72.0)
    eta = 72.0 * 0.5 / 3.0

    def k_after(set_state):
        lb = lattice()
        set_state(lb)
        gpu.lbsteps(lb, 8)
        gpu.measure(lb)
        kk = lb.vmeanx * eta / force
        gpu.lbpull(lb)
        a = lb.array("a").copy()
        gpu.freelb(lb)
        return kk, a

    k_state, _ = k_after(lambda lb: gpu.lbsetstatedev(lb, us.data_ptr(), drho.data_ptr()))
    assert abs(k_state - k) <= 1e-4 * k, (k_state, k)
    _, a_vel = k_after(lambda lb: gpu.lbsetveldev(lb, us.data_ptr()))
    _, a_state0 = k_after(lambda lb: gpu.lbsetstatedev(lb, us.data_ptr(), None))
    assert np.array_equal(a_vel, a_state0)
