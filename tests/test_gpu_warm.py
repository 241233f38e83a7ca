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


def test_unet_gradients_match_cpu_oracle(gpu):
    torch = pytest.importorskip("torch")
    from sunlightlb_gb300 import warmstart as WS
    orc = oracle()
    B, D, H, W = 2, 32, 32, 64
    net = WS.UNet(gpu, D, H, W, batch=B, widths=(32, 32, 32, 32), seed=3, features=0)
    rng = np.random.default_rng(5)
    solid = (rng.random((B, D, H, W)) > 0.7).astype(np.uint8)
    zz, yy, xx = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    lab = np.stack([np.sin(2 * np.pi * xx / W) * np.cos(2 * np.pi * yy / H),
                    0.5 * np.cos(2 * np.pi * zz / D), 0.2 * np.sin(2 * np.pi * (xx + zz) / W)], axis=-1)
    labels = np.broadcast_to(lab, (B, D, H, W, 3)) * (1 - solid[..., None])
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
    hist = WS.train(net, m_dev, l_dev, iters=60, lr=2e-3, seed=1, log_every=1)
    assert net.status() == 0
    first = np.mean([l for _, l in hist[:5]])
    last = np.mean([l for _, l in hist[-5:]])
    assert last < 0.7 * first, (first, last)
