"""CPU oracle of the learned warm start's network (test infrastructure only).

A float64 numpy restatement of the encoder-decoder that
sunlightlb_gb300/warmstart.py runs on the tensor cores: the same layer
list, periodic 3x3x3 convolutions (tap = 9 dz + 3 dy + dx for the neighbour
offset (dx-1, dy-1, dz-1)), ReLU, 2x2x2 average pooling, nearest
upsampling, channel concatenation (upsampled part first, skip part after),
the mean-square loss over the label channels (velocity 0..2, and the
density deviation 3 when the labels carry it), and the exact gradients
of all of it.  There is no counterpart in the reference (its lattice
Boltzmann code has no learned part); the GPU gradients are checked against
this.  Arrays are channels-last without halo: (B, D, H, W, C).
"""

import numpy as np


def _shift(x, off):
    """x at v + off for every voxel v (periodic), off = (dx, dy, dz)."""
    dx, dy, dz = off
    return np.roll(x, shift=(-dz, -dy, -dx), axis=(1, 2, 3))


def _offsets():
    return [((t % 3) - 1, ((t // 3) % 3) - 1, (t // 9) - 1) for t in range(27)]


def conv(x, w, b):
    """w[tap][cout][cin], b[cout]."""
    out = np.zeros(x.shape[:4] + (w.shape[1],))
    for t, off in enumerate(_offsets()):
        out += _shift(x, off) @ w[t].T
    return out + b


def conv_backward(x, w, g):
    """(dW, db, dX) of conv for the output gradient g."""
    dw = np.zeros_like(w)
    dx = np.zeros_like(x)
    gf = g.reshape(-1, g.shape[-1])
    for t, off in enumerate(_offsets()):
        xs = _shift(x, off).reshape(-1, x.shape[-1])
        dw[t] = gf.T @ xs
        dx += _shift((g @ w[t]), (-off[0], -off[1], -off[2]))
    return dw, g.sum(axis=(0, 1, 2, 3)), dx


def pool(x):
    B, D, H, W, C = x.shape
    return x.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4, 6))


def pool_backward(g):
    return np.repeat(np.repeat(np.repeat(g, 2, axis=1), 2, axis=2), 2, axis=3) / 8.0


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, axis=1), 2, axis=2), 2, axis=3)


def up_backward(g):
    B, D, H, W, C = g.shape
    return g.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4, 6))


def relu(x):
    return np.maximum(x, 0.0)


def forward_backward(params, inp, labels):
    """params: {layer: (w, b)} (float64), inp: (B, D, H, W, 32) input
    encoding, labels: (B, D, H, W, C), C = 3 or 4.  Returns (loss,
    {layer: (dw, db)})."""
    P = params
    a = {}
    a["A0"] = relu(conv(inp, *P["e0a"]))
    s0 = relu(conv(a["A0"], *P["e0b"]))
    a["P1"] = pool(s0)
    a["A1"] = relu(conv(a["P1"], *P["e1a"]))
    s1 = relu(conv(a["A1"], *P["e1b"]))
    a["P2"] = pool(s1)
    a["A2"] = relu(conv(a["P2"], *P["e2a"]))
    s2 = relu(conv(a["A2"], *P["e2b"]))
    a["P3"] = pool(s2)
    a["A3"] = relu(conv(a["P3"], *P["e3a"]))
    b3 = relu(conv(a["A3"], *P["e3b"]))
    c2 = np.concatenate([up(b3), s2], axis=-1)
    e2 = relu(conv(c2, *P["d2a"]))
    d2 = relu(conv(e2, *P["d2b"]))
    c1 = np.concatenate([up(d2), s1], axis=-1)
    e1 = relu(conv(c1, *P["d1a"]))
    d1 = relu(conv(e1, *P["d1b"]))
    c0 = np.concatenate([up(d1), s0], axis=-1)
    e0 = relu(conv(c0, *P["d0a"]))
    d0 = relu(conv(e0, *P["d0b"]))
    out = conv(d0, *P["out"])
    nch = labels.shape[-1]
    n = labels[..., 0].size * nch
    diff = out[..., :nch] - labels
    loss = float((diff ** 2).sum() / n)
    g_out = np.zeros_like(out)
    g_out[..., :nch] = 2.0 * diff / n
    grads = {}

    def back(name, x, g, y=None):
        """layer backward; g at the output pre-activation (already masked)"""
        dw, db, dx = conv_backward(x, P[name][0], g)
        grads[name] = (dw, db)
        return dx

    g = back("out", d0, g_out) * (d0 > 0)
    g = back("d0b", e0, g) * (e0 > 0)
    gc0 = back("d0a", c0, g)
    wu0 = d1.shape[-1]
    g = up_backward(gc0[..., :wu0]) * (d1 > 0)
    g = back("d1b", e1, g) * (e1 > 0)
    gc1 = back("d1a", c1, g)
    wu1 = d2.shape[-1]
    g = up_backward(gc1[..., :wu1]) * (d2 > 0)
    g = back("d2b", e2, g) * (e2 > 0)
    gc2 = back("d2a", c2, g)
    wu2 = b3.shape[-1]
    g = up_backward(gc2[..., :wu2]) * (b3 > 0)
    g = back("e3b", a["A3"], g) * (a["A3"] > 0)
    g = back("e3a", a["P3"], g)
    g = (pool_backward(g) + gc2[..., wu2:]) * (s2 > 0)
    g = back("e2b", a["A2"], g) * (a["A2"] > 0)
    g = back("e2a", a["P2"], g)
    g = (pool_backward(g) + gc1[..., wu1:]) * (s1 > 0)
    g = back("e1b", a["A1"], g) * (a["A1"] > 0)
    g = back("e1a", a["P1"], g)
    g = (pool_backward(g) + gc0[..., wu0:]) * (s0 > 0)
    g = back("e0b", a["A0"], g) * (a["A0"] > 0)
    back("e0a", inp, g)
    return loss, grads
