"""Learned warm start of the permeability calculation.

A 3-D convolutional encoder-decoder maps a binary solid mask to the
zero-Reynolds steady velocity of a periodic packing (in units of the Darcy
response, q = u * eta / b, so one network serves every body force and
viscosity).  The lattice is then warm-started at equilibrium with
rho = rho0 and that velocity (lbsetveldev) and the unchanged lattice
Boltzmann iteration removes the residual; plain initialisation stays the
fallback whenever the warm start is not faster.

Network: four resolution levels (widths 32, 64, 128, 256 by default), two
periodic 3x3x3 convolutions with ReLU per level on the way down and up,
2x2x2 average pooling, nearest upsampling, skip connections by channel
concatenation, a last 3x3x3 convolution to the 3 velocity components.
BF16 weights and activations, FP32 accumulation: every convolution, its
input gradient and its weight gradient run on the tensor cores
(slbc_tc_conv3d / slbc_tc_wgrad, tcgen05.mma); pooling, upsampling, masks,
bias gradients, the loss and Adam are the library's own CUDA kernels
(slbc_nn_*).  Buffers are device tensors (torch is used for memory only):
channels-last with a one-voxel periodic halo.

Training data are generated by the solver itself (batched lattices, FP32
populations, converged flow at body force b), see converged_flows.
"""

import ctypes as C
import math
import os
import time

import numpy as np

from . import workloads as W

ETA_TAU1 = 72.0 * (1.0 - 0.5) / 3.0   # rho0 (tau - 1/2) / 3 at tau = 1, rho0 = 72
IN_CH = 32                             # input channels (channel 0 = solid mask)
OUT_CH = 32                            # output channels (0..2 = velocity, 3 = density when trained with it)
DRHO_UNIT = 12.0                       # density labels: (rho - rho0) / (DRHO_UNIT * body force)


class Kernels:
    """ctypes signatures of the tensor-core and glue entry points."""

    def __init__(self, dll):
        p, i, ll, f, d = C.c_void_p, C.c_int, C.c_longlong, C.c_float, C.c_double
        sig = {
            "slbc_tc_conv3d": [p] + [i] * 7 + [p, p, i, p, i, i, i, p, p],
            "slbc_tc_conv3d_f32": [p] + [i] * 7 + [p, p, i, p, i, i, p],
            "slbc_tc_halo": [p] + [i] * 7 + [p],
            "slbc_tc_cmajor": [p] + [i] * 8 + [ll, i, i, p, p],
            "slbc_tc_wgrad": [p] * 4 + [i] * 5 + [ll, i, i, p, ll, i, p, p],
            "slbc_tc_cmajor_tiles": [p] + [i] * 8 + [ll, i, i, i, p, p],
            "slbc_tc_wgrad_tiles": [p] * 2 + [i] * 5 + [ll, i, i, p, ll, i, p, p],
            "slbc_nn_pool": [p, i, i, p, i, i] + [i] * 5 + [p],
            "slbc_nn_pool_bwd": [p, i, i, p, i, i, p, i, i, p, i, i] + [i] * 5 + [p],
            "slbc_nn_up": [p, i, i, p, i, i] + [i] * 5 + [p],
            "slbc_nn_up_bwd": [p, i, i, p, i, i, p, i, i] + [i] * 5 + [p],
            "slbc_nn_bias_grad": [p, i, i] + [i] * 5 + [p, p],
            "slbc_nn_wfwd": [p, i, i, p, p],
            "slbc_nn_wdgrad": [p, i, i, i, i, p, p],
            "slbc_nn_adam": [p, p, p, p, ll, f, f, f, f, i, p],
            "slbc_nn_mse": [p, i, p, i, p, i, i, i, i, p, i, p, p],
            "slbc_nn_proj": [p, i, p, i, i, p, i, i, i, i, f, p, i, p, p, p],
            "slbc_nn_sqsum": [p, ll, p, p],
            "slbc_nn_clip": [p, f, f, p],
            "slbc_nn_scale": [p, ll, p, p],
            "slbc_nn_encode": [p, i, i, i, i, p, i, i, p],
            "slbc_nn_decode": [p, i, p, i, i, i, f, f, p, f, p, p],
            "slbc_nn_plane_flux": [p, p, p, i, i, i, f, f, p, p],
            "slbc_nn_cross_flux": [p, i, i, i, p, p],
            "slbc_tc_status": [],
        }
        self.dll = dll
        for name, args in sig.items():
            fn = getattr(dll, name)
            fn.argtypes = args
            fn.restype = C.c_int
            setattr(self, name[5:], self._checked(name, fn))
        dll.slbc_last_error.restype = C.c_char_p
        # a count, not a status
        self.tc_wgrad_splits = dll.slbc_tc_wgrad_splits
        self.tc_wgrad_splits.argtypes = [i, i, ll, ll]
        self.tc_wgrad_splits.restype = C.c_int

    def _checked(self, name, fn):
        def call(*a):
            rc = fn(*a)
            if rc != 0 and name != "slbc_tc_status":
                raise RuntimeError(f"{name}: {self.dll.slbc_last_error().decode()}")
            return rc
        return call


def flat_geometry(D, H, W_):
    """Row pitch and sample stride of the channel-major weight-gradient copies."""
    Wp = (W_ + 2 + 7) // 8 * 8
    return Wp, ((D + 2) * (H + 2) * Wp + 63) // 64 * 64


class UNet:
    """The encoder-decoder on a batch of B grids D x H x W (powers of two,
    the coarsest level D*H*W/512 >= 128 voxels)."""

    def __init__(self, lib, D, H, W_, batch, widths=(32, 64, 128, 256), seed=0, params=None, features=1):
        import torch
        self.torch = torch
        # input: mask (0), mask + wall distance searched to 5 (1), or to 12
        # with the near-wall distance beside it (2)
        self.features = features
        self.k = Kernels(lib.dll)
        self.D, self.H, self.W, self.B = D, H, W_, batch
        self.widths = w0, w1, w2, w3 = widths
        self.dev = torch.device("cuda")
        self.stream = torch.cuda.current_stream().cuda_stream
        # layer: (name, level, cin, cout, src, src_coff, dst, dst_coff, relu)
        self.layers = [
            ("e0a", 0, IN_CH, w0, "IN", 0, "A0", 0, 1),
            ("e0b", 0, w0, w0, "A0", 0, "C0", w1, 1),
            ("e1a", 1, w0, w1, "P1", 0, "A1", 0, 1),
            ("e1b", 1, w1, w1, "A1", 0, "C1", w2, 1),
            ("e2a", 2, w1, w2, "P2", 0, "A2", 0, 1),
            ("e2b", 2, w2, w2, "A2", 0, "C2", w3, 1),
            ("e3a", 3, w2, w3, "P3", 0, "A3", 0, 1),
            ("e3b", 3, w3, w3, "A3", 0, "B3", 0, 1),
            ("d2a", 2, w3 + w2, w2, "C2", 0, "E2", 0, 1),
            ("d2b", 2, w2, w2, "E2", 0, "D2", 0, 1),
            ("d1a", 1, w2 + w1, w1, "C1", 0, "E1", 0, 1),
            ("d1b", 1, w1, w1, "E1", 0, "D1", 0, 1),
            ("d0a", 0, w1 + w0, w0, "C0", 0, "E0", 0, 1),
            ("d0b", 0, w0, w0, "E0", 0, "D0", 0, 1),
            ("out", 0, w0, OUT_CH, "D0", 0, "OUT", 0, 0),
        ]
        self.buf_spec = {  # name: (level, channels)
            "IN": (0, IN_CH), "A0": (0, w0), "C0": (0, w1 + w0), "E0": (0, w0), "D0": (0, w0),
            "P1": (1, w0), "A1": (1, w1), "C1": (1, w2 + w1), "E1": (1, w1), "D1": (1, w1),
            "P2": (2, w1), "A2": (2, w2), "C2": (2, w3 + w2), "E2": (2, w2), "D2": (2, w2),
            "P3": (3, w2), "A3": (3, w3), "B3": (3, w3),
        }
        self.buf = {n: self._act(lv, c) for n, (lv, c) in self.buf_spec.items()}
        self.buf["OUT"] = torch.zeros(self._shape(0, OUT_CH), device=self.dev, dtype=torch.float32)
        self.grad = None
        self.clip_state = None
        self.params = params if params is not None else self._init_params(seed)
        self.wf = {}
        self.wd = {}
        self.refresh_weights()
        self.t = 0

    # ---- buffers -----------------------------------------------------------
    def dims(self, level):
        return self.D >> level, self.H >> level, self.W >> level

    def _shape(self, level, ch):
        d, h, w = self.dims(level)
        return (self.B, d + 2, h + 2, w + 2, ch)

    def _act(self, level, ch):
        return self.torch.zeros(self._shape(level, ch), device=self.dev, dtype=self.torch.bfloat16)

    def _init_params(self, seed):
        torch = self.torch
        g = torch.Generator(device="cpu").manual_seed(seed)
        P = {}
        for name, lv, cin, cout, *_ in self.layers:
            std = math.sqrt(2.0 / (27 * cin))
            if name == "e0a":
                std = math.sqrt(2.0 / (27 * (1 + {0: 0, 1: 2, 2: 3}[self.features])))  # live input channels
            w = torch.randn(27, cout, cin, generator=g) * std
            b = torch.zeros(cout)
            if name == "out":
                w *= 0.1
                w[:, 3:, :] = 0.0
            P[name] = {"w": w.to(self.dev), "b": b.to(self.dev)}
            for key in ("w", "b"):
                P[name]["m" + key] = torch.zeros_like(P[name][key])
                P[name]["v" + key] = torch.zeros_like(P[name][key])
        return P

    def refresh_weights(self):
        """BF16 tensor-core layouts of the FP32 master weights."""
        torch = self.torch
        for name, lv, cin, cout, *_ in self.layers:
            m = self.params[name]["w"]
            wf = self.wf.get(name)
            if wf is None:
                wf = self.wf[name] = torch.empty(27 * cin * cout, device=self.dev, dtype=torch.bfloat16)
            self.k.nn_wfwd(m.data_ptr(), cout, cin, wf.data_ptr(), self.stream)
            if name == "e0a":
                continue  # no input gradient needed
            chunks = self.wd.get(name)
            if chunks is None:
                nci = cin if cin <= 256 else cin // 2
                chunks = self.wd[name] = [(c0, nci, torch.empty(27 * nci * cout, device=self.dev,
                                                                 dtype=torch.bfloat16)) for c0 in range(0, cin, nci)]
            for c0, nci, t in chunks:
                self.k.nn_wdgrad(m.data_ptr(), cout, cin, c0, nci, t.data_ptr(), self.stream)

    def _halo(self, name, coff=0, nch=None):
        t = self.buf[name] if name in self.buf else self.grad[name]
        lv, ch = self.buf_spec.get(name, (None, None)) if name in self.buf else self.grad_spec[name]
        d, h, w = self.dims(lv)
        self.k.tc_halo(t.data_ptr(), self.B, d, h, w, t.shape[-1], coff, nch or t.shape[-1], self.stream)

    # ---- forward -------------------------------------------------------------
    def encode(self, solid_u8):
        """solid_u8: device uint8 tensor (B, D, H, W)."""
        k = self.k
        k.nn_encode(solid_u8.data_ptr(), self.B, self.D, self.H, self.W, self.buf["IN"].data_ptr(), IN_CH,
                    self.features, self.stream)
        self._halo("IN")

    def forward(self):
        k, w0, w1, w2, w3 = self.k, *self.widths
        B = self.B
        for name, lv, cin, cout, src, scoff, dst, dcoff, relu in self.layers:
            d, h, w = self.dims(lv)
            s, t = self.buf[src], self.buf[dst]
            p = self.params[name]
            if name == "out":
                k.tc_conv3d_f32(s.data_ptr(), B, d, h, w, s.shape[-1], scoff, cin, self.wf[name].data_ptr(),
                                p["b"].data_ptr(), cout, t.data_ptr(), t.shape[-1], dcoff, self.stream)
                continue
            k.tc_conv3d(s.data_ptr(), B, d, h, w, s.shape[-1], scoff, cin, self.wf[name].data_ptr(),
                        p["b"].data_ptr(), cout, t.data_ptr(), t.shape[-1], dcoff, relu, None, self.stream)
            self._halo(dst, dcoff, cout)
            if name in ("e0b", "e1b", "e2b"):  # pool the skip slice down a level
                nxt = {"e0b": "P1", "e1b": "P2", "e2b": "P3"}[name]
                pt = self.buf[nxt]
                k.nn_pool(t.data_ptr(), t.shape[-1], dcoff, pt.data_ptr(), pt.shape[-1], 0, B, d, h, w, cout,
                          self.stream)
                self._halo(nxt)
            if name in ("e3b", "d2b", "d1b"):  # upsample into the next concat buffer
                up = {"e3b": "C2", "d2b": "C1", "d1b": "C0"}[name]
                ut = self.buf[up]
                ud, uh, uw = self.dims(lv - 1)
                k.nn_up(t.data_ptr(), t.shape[-1], 0, ut.data_ptr(), ut.shape[-1], 0, B, ud, uh, uw, cout,
                        self.stream)
                self._halo(up, 0, cout)
        return self.buf["OUT"]

    # ---- backward --------------------------------------------------------------
    def _alloc_grads(self):
        torch = self.torch
        w0, w1, w2, w3 = self.widths
        self.grad_spec = {
            "gOUT": (0, OUT_CH), "gD0": (0, w0), "gE0": (0, w0), "gC0": (0, w1 + w0), "gS0": (0, w0), "gA0": (0, w0),
            "gD1": (1, w1), "gE1": (1, w1), "gC1": (1, w2 + w1), "gS1": (1, w1), "gA1": (1, w1), "gP1": (1, w0),
            "gD2": (2, w2), "gE2": (2, w2), "gC2": (2, w3 + w2), "gS2": (2, w2), "gA2": (2, w2), "gP2": (2, w1),
            "gB3": (3, w3), "gA3": (3, w3), "gP3": (3, w2),
        }
        self.grad = {n: self._act(lv, c) for n, (lv, c) in self.grad_spec.items()}
        Wp, ps = flat_geometry(self.D, self.H, self.W)
        maxc = max(c for _, c in self.buf_spec.values())
        self.cm_x = torch.empty(maxc * self.B * ps, device=self.dev, dtype=torch.bfloat16)
        # the three x-shifted copies of an output gradient: K-tile blocks
        # (cout <= 128), else three equally spaced channel-major copies
        self.cm_g = torch.empty(3 * w3 * self.B * ps, device=self.dev, dtype=torch.bfloat16)
        self.ws_floats = 1 << 26
        self.ws = torch.empty(self.ws_floats, device=self.dev, dtype=torch.float32)
        self.loss_acc = torch.zeros(1, device=self.dev, dtype=torch.float64)
        self.proj_dot = torch.zeros(self.B, device=self.dev, dtype=torch.float64)
        for name, *_ in self.layers:
            p = self.params[name]
            p["gw"] = torch.zeros_like(p["w"])
            p["gb"] = torch.zeros_like(p["b"])

    def _wgrad(self, name, g_name, x_name, x_coff=0):
        """weight and bias gradients of layer `name` from the gradient at its
        output (g_name, channels [0, cout)) and its input (x_name slice)."""
        k = self.k
        _, lv, cin, cout, *_ = next(l for l in self.layers if l[0] == name)
        d, h, w = self.dims(lv)
        Wp, ps = flat_geometry(d, h, w)
        g = self.grad[g_name]
        x = self.buf[x_name]
        tiles = cout <= 128
        n = cout * self.B * ps
        cm_g = [self.cm_g[i * n:(i + 1) * n] for i in range(3)]
        for i, shift in enumerate((-1, 0, 1)):
            if tiles:
                k.tc_cmajor_tiles(g.data_ptr(), self.B, d, h, w, g.shape[-1], 0, cout, Wp, ps, shift, i, 3,
                                  self.cm_g.data_ptr(), self.stream)
            else:
                k.tc_cmajor(g.data_ptr(), self.B, d, h, w, g.shape[-1], 0, cout, Wp, ps, shift, 0,
                            cm_g[i].data_ptr(), self.stream)
        k.tc_cmajor(x.data_ptr(), self.B, d, h, w, x.shape[-1], x_coff, cin, Wp, ps, 0, 1, self.cm_x.data_ptr(),
                    self.stream)
        splits = k.tc_wgrad_splits(cin, cout, self.B * ps // 64, self.ws_floats // (27 * cout * cin))
        p = self.params[name]
        if tiles:
            k.tc_wgrad_tiles(self.cm_g.data_ptr(), self.cm_x.data_ptr(), self.B, d, h, w, Wp, ps, cin, cout,
                             self.ws.data_ptr(), self.ws_floats, splits, p["gw"].data_ptr(), self.stream)
        else:
            k.tc_wgrad(cm_g[0].data_ptr(), cm_g[1].data_ptr(), cm_g[2].data_ptr(), self.cm_x.data_ptr(),
                       self.B, d, h, w, Wp, ps, cin, cout, self.ws.data_ptr(), self.ws_floats, splits,
                       p["gw"].data_ptr(), self.stream)
        p["gb"].zero_()
        k.nn_bias_grad(g.data_ptr(), g.shape[-1], 0, self.B, d, h, w, cout, p["gb"].data_ptr(), self.stream)

    def _dgrad(self, name, g_name, out_name, mask_name=None):
        """gradient at the input of layer `name` into grad[out_name], times
        (mask > 0) when the input is a ReLU output mask_name."""
        k = self.k
        _, lv, cin, cout, *_ = next(l for l in self.layers if l[0] == name)
        d, h, w = self.dims(lv)
        g, o = self.grad[g_name], self.grad[out_name]
        m = self.buf[mask_name] if mask_name else None
        for c0, nci, wt in self.wd[name]:
            k.tc_conv3d(g.data_ptr(), self.B, d, h, w, g.shape[-1], 0, cout, wt.data_ptr(), None, nci,
                        o.data_ptr(), o.shape[-1], c0, 0, m.data_ptr() if m is not None else None, self.stream)
        self._halo(out_name)

    def loss_and_backward(self, labels, sample_w=None, proj=None):
        """labels: device FP32 (B, D, H, W, 3 or 4); sample_w: optional device
        FP32 (B,) loss weights; proj: optional (weight, lab_sq) adding weight
        times the mean squared projection of the velocity error on the
        label (lab_sq: device FP64 (B,) label energies over the 3 velocity
        channels, slbc_nn_proj).  Returns the loss (device scalar, FP64)."""
        if self.grad is None:
            self._alloc_grads()
        k, G, X = self.k, self.grad, self.buf
        B, (w0, w1, w2, w3) = self.B, self.widths
        self.loss_acc.zero_()
        k.nn_mse(X["OUT"].data_ptr(), OUT_CH, labels.data_ptr(), labels.shape[-1],
                 sample_w.data_ptr() if sample_w is not None else None, B, self.D, self.H, self.W, G["gOUT"].data_ptr(),
                 OUT_CH, self.loss_acc.data_ptr(), self.stream)
        if proj is not None and proj[0] > 0:
            k.nn_proj(X["OUT"].data_ptr(), OUT_CH, labels.data_ptr(), labels.shape[-1], 3, proj[1].data_ptr(), B,
                      self.D, self.H, self.W, float(proj[0]), G["gOUT"].data_ptr(), OUT_CH, self.proj_dot.data_ptr(),
                      self.loss_acc.data_ptr(), self.stream)
        self._halo("gOUT")
        # level 0 decoder
        self._wgrad("out", "gOUT", "D0")
        self._dgrad("out", "gOUT", "gD0", "D0")
        self._wgrad("d0b", "gD0", "E0")
        self._dgrad("d0b", "gD0", "gE0", "E0")
        self._wgrad("d0a", "gE0", "C0")
        self._dgrad("d0a", "gE0", "gC0")
        d1, h1, wd1 = self.dims(0)
        k.nn_up_bwd(G["gC0"].data_ptr(), w1 + w0, 0, G["gD1"].data_ptr(), w1, 0, X["D1"].data_ptr(), w1, 0, B,
                    d1, h1, wd1, w1, self.stream)
        self._halo("gD1")
        self._wgrad("d1b", "gD1", "E1")
        self._dgrad("d1b", "gD1", "gE1", "E1")
        self._wgrad("d1a", "gE1", "C1")
        self._dgrad("d1a", "gE1", "gC1")
        d, h, w = self.dims(1)
        k.nn_up_bwd(G["gC1"].data_ptr(), w2 + w1, 0, G["gD2"].data_ptr(), w2, 0, X["D2"].data_ptr(), w2, 0, B,
                    d, h, w, w2, self.stream)
        self._halo("gD2")
        self._wgrad("d2b", "gD2", "E2")
        self._dgrad("d2b", "gD2", "gE2", "E2")
        self._wgrad("d2a", "gE2", "C2")
        self._dgrad("d2a", "gE2", "gC2")
        d, h, w = self.dims(2)
        k.nn_up_bwd(G["gC2"].data_ptr(), w3 + w2, 0, G["gB3"].data_ptr(), w3, 0, X["B3"].data_ptr(), w3, 0, B,
                    d, h, w, w3, self.stream)
        self._halo("gB3")
        # level 3 and the encoder
        self._wgrad("e3b", "gB3", "A3")
        self._dgrad("e3b", "gB3", "gA3", "A3")
        self._wgrad("e3a", "gA3", "P3")
        self._dgrad("e3a", "gA3", "gP3")
        for lv, (gp, gc, skip_c, gs, xa, ga, lay_b, lay_a, xp, gpn, cskip) in enumerate([
                ("gP3", "gC2", w3, "gS2", "A2", "gA2", "e2b", "e2a", "P2", "gP2", w2),
                ("gP2", "gC1", w2, "gS1", "A1", "gA1", "e1b", "e1a", "P1", "gP1", w1),
                ("gP1", "gC0", w1, "gS0", "A0", "gA0", "e0b", "e0a", "IN", None, w0)]):
            level = 2 - lv
            d, h, w = self.dims(level)
            cb = {2: "C2", 1: "C1", 0: "C0"}[level]
            ctot = X[cb].shape[-1]
            k.nn_pool_bwd(G[gp].data_ptr(), G[gp].shape[-1], 0, G[gs].data_ptr(), cskip, 0, G[gc].data_ptr(), ctot,
                          skip_c, X[cb].data_ptr(), ctot, skip_c, B, d, h, w, cskip, self.stream)
            self._halo(gs)
            self._wgrad(lay_b, gs, xa)
            self._dgrad(lay_b, gs, ga, xa)
            self._wgrad(lay_a, ga, xp)
            if gpn is not None:
                self._dgrad(lay_a, ga, gpn)
        return self.loss_acc

    def clip_grads(self, factor=3.0, decay=0.98):
        """Scale all gradients down to at most `factor` times their running
        norm (device-side: no host synchronisation)."""
        if self.clip_state is None:
            self.clip_state = self.torch.zeros(3, device=self.dev, dtype=self.torch.float64)
        st = self.clip_state.data_ptr()
        grads = [self.params[name]["g" + key] for name, *_ in self.layers for key in ("w", "b")]
        for g in grads:
            self.k.nn_sqsum(g.data_ptr(), g.numel(), st, self.stream)
        self.k.nn_clip(st, factor, decay, self.stream)
        for g in grads:
            self.k.nn_scale(g.data_ptr(), g.numel(), st, self.stream)

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.t += 1
        for name, *_ in self.layers:
            p = self.params[name]
            for key in ("w", "b"):
                self.k.nn_adam(p[key].data_ptr(), p["g" + key].data_ptr(), p["m" + key].data_ptr(),
                               p["v" + key].data_ptr(), p[key].numel(), lr, b1, b2, eps, self.t, self.stream)
        self.refresh_weights()

    def status(self):
        return self.k.tc_status()


# ---- data ------------------------------------------------------------------------

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "warm_unet.npz")


def save_weights(net, path, meta=None):
    """The network's weights and biases as BF16 bit patterns (the precision
    the tensor-core kernels use) in an .npz file, with the widths and any
    metadata (a JSON string)."""
    import json
    arrays = {}
    for name, *_ in net.layers:
        for key in ("w", "b"):
            t = net.params[name][key].detach().float().contiguous().cpu()
            bits = t.view(-1).numpy().view(np.uint32)
            # round to nearest even BF16
            rounded = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)
            arrays[f"{name}.{key}"] = rounded.reshape(tuple(t.shape))
    arrays["widths"] = np.array(net.widths, dtype=np.int32)
    arrays["features"] = np.array([net.features], dtype=np.int32)
    arrays["meta"] = np.frombuffer(json.dumps(meta or {}).encode(), dtype=np.uint8)
    tmp = path + ".tmp.npz"
    np.savez_compressed(tmp, **arrays)
    os.replace(tmp, path)


def load_weights(path=WEIGHTS):
    """(params, widths, features, meta) of a file written by save_weights;
    params as FP32 device tensors, the form UNet(params=...) takes."""
    import json
    import torch
    z = np.load(path)
    params = {}
    for key in z.files:
        if "." not in key:
            continue
        name, kind = key.split(".")
        f32 = (z[key].astype(np.uint32) << 16).view(np.float32)
        params.setdefault(name, {})[kind] = torch.as_tensor(f32.copy(), device="cuda")
    meta = json.loads(bytes(z["meta"]).decode()) if "meta" in z.files else {}
    return params, tuple(int(v) for v in z["widths"]), int(z["features"][0]), meta


def with_adam_state(params):
    """params of load_weights with zero Adam moments, ready for training
    (fine-tuning a saved network)."""
    import torch
    for p in params.values():
        for key in ("w", "b"):
            p["m" + key] = torch.zeros_like(p[key])
            p["v" + key] = torch.zeros_like(p[key])
    return params


def packing_specs(n, seed, phi_range=(0.1, 0.5), r_range=(3.0, 8.0)):
    """Seeded (phi, packing seed) pairs; spheres may overlap (a Boolean model),
    since non-overlapping random addition stalls near phi = 0.38."""
    rng = W.SplitMix64(seed)
    return [(rng.uniform(*phi_range), int(rng.next() & 0x7FFFFFFF)) for _ in range(n)]


def packing(side, phi, seed, r_range=(3.0, 8.0)):
    return W.rsa_packing(side, phi, r_range[0], r_range[1], seed, overlap=True)[1]


def converged_flows(L, solids, force=1e-6, tol=1e-6, check=200, maxsteps=40000, chunk=256, precision=1,
                    density=False):
    """Steady Stokes flow of every packing (tau = 1, body force along x),
    advanced as batches of `chunk` lattices; a lattice leaves the batch once
    the relative change of its mean flow between checks is below tol.
    Returns (velocity fields as device FP32 tensors (3, N) in units of the
    Darcy response q = u * eta / b, steps per lattice); with density a
    fourth row holds the density deviation in units of DRHO_UNIT * b."""
    import torch
    fields, steps = [None] * len(solids), [0] * len(solids)
    for start in range(0, len(solids), chunk):
        idx = list(range(start, min(start + chunk, len(solids))))
        lbs = {}
        for i in idx:
            s = solids[i]
            lb = L.newlb(s.shape[0], s.shape[1], s.shape[2], "null")
            lb.precision = precision
            lb.tau = 1.0
            lb.stokes_flow = 1
            W.insert_solid(L, lb, s)
            L.syncobjs(lb)
            L.addbf(lb, force, 0.0, 0.0)
            lbs[i] = lb
        prev = {i: None for i in idx}
        active = list(idx)
        while active:
            b = L.newbatch()
            for i in active:
                L.batchadd(b, lbs[i])
            L.batchsteps(b, check - 2)
            L.freebatch(b)
            still = []
            for i in active:
                L.measure(lbs[i])
                steps[i] += check
                v = lbs[i].vmeanx
                done = prev[i] is not None and abs(v - prev[i]) <= tol * abs(v) or steps[i] >= maxsteps
                prev[i] = v
                if not done:
                    still.append(i)
            active = still
        for i in idx:
            lb = lbs[i]
            u = torch.empty((4 if density else 3) * lb.nnodes, device="cuda", dtype=torch.float32)
            if density:
                L.lbstate(lb, u.data_ptr(), u[3 * lb.nnodes:].data_ptr())
            else:
                L.lbvelocity(lb, u.data_ptr())
            torch.cuda.synchronize()
            f = u.view(-1, lb.nnodes)
            f[:3] *= ETA_TAU1 / force
            if density:
                f[3] *= 1.0 / (DRHO_UNIT * force)
            fields[i] = f
            L.freelb(lb)
    return fields, steps


def to_labels(field, shape):
    """(C, N) -> (D, H, W, C)."""
    return field.view(field.shape[0], *shape).permute(1, 2, 3, 0).contiguous()


# ---- warm start -------------------------------------------------------------------

def predict_velocity(net, solid_u8, force, eta, rho0=72.0, force_shift=1.0):
    """Velocity field (3 x N device FP32, layout of lbsetveldev) predicted by
    a batch-1 network for a solid mask (device uint8 (D, H, W)), body force
    `force` along x.  The labels are the converged fields lbvelocity reads
    from post-collision states, while lbsetveldev takes the velocity of the
    state before the collision that adds the force: a converged state is
    rebuilt exactly from u - F / (2 rho) and its own density (10 steps to
    k within 1e-4, against 120-850 without the shift).  With rho = rho0
    everywhere (the network predicts no density) the whole force, u - F /
    rho0, measured best: on 100 held-out 128^3 packings the mean steps
    ratio to the plain start was 2.73x unshifted, 3.01x with F / 2 and
    3.20x with F.  So u_x is set with force_shift * force / rho0 taken off
    on fluid nodes."""
    import torch
    net.encode(solid_u8.view(1, *solid_u8.shape))
    out = net.forward()
    n = solid_u8.numel()
    u = torch.empty(3 * n, device="cuda", dtype=torch.float32)
    net.k.nn_decode(out.data_ptr(), OUT_CH, solid_u8.data_ptr(), net.D, net.H, net.W, force / eta,
                    force_shift * force / rho0, u.data_ptr(), 0.0, None, net.stream)
    return u


def predict_state(net, solid_u8, force, eta, rho0=72.0, force_shift=0.5, plane_flux=True, info=None, gain=1.0,
                  cross_flux=False):
    """Velocity (3 x N) and density deviation (N) device FP32 fields from a
    network trained on labels with density (converged_flows(density=True)):
    with its own density a converged state is rebuilt exactly from
    u - F / (2 rho), so force_shift defaults to 1/2 here.  plane_flux: the
    x flux made the same through every x plane (slbc_nn_plane_flux), as
    mass conservation requires of the converged flow; the network, which
    sees part of the bed, predicts each slab as if the whole body force
    drove it.  On 59 held-out 128^3 packings this took the total wall time
    to k within 1e-4 from 2.18x to 2.32x less than the plain start.  info
    (a dict) receives the relative spread of the plane fluxes before.  gain
    multiplies the state after the plane-flux step (plane_flux must be on
    for it; a global gain calibrated so that warm states start with the
    converged mean flow, 0.991 for the committed network, measured worse:
    the fast transients of the first steps take flux with them).
    cross_flux: afterwards the y and z plane fluxes of u_y and u_z made
    uniform too (slbc_nn_cross_flux)."""
    import torch
    net.encode(solid_u8.view(1, *solid_u8.shape))
    out = net.forward()
    n = solid_u8.numel()
    u = torch.empty(3 * n, device="cuda", dtype=torch.float32)
    drho = torch.empty(n, device="cuda", dtype=torch.float32)
    net.k.nn_decode(out.data_ptr(), OUT_CH, solid_u8.data_ptr(), net.D, net.H, net.W, force / eta,
                    force_shift * force / rho0, u.data_ptr(), DRHO_UNIT * force, drho.data_ptr(), net.stream)
    if not plane_flux and gain != 1.0:
        raise ValueError("predict_state: a gain needs the plane-flux step")
    if plane_flux:
        work = torch.empty(3 * net.D + 1, device="cuda", dtype=torch.float64)
        net.k.nn_plane_flux(u.data_ptr(), drho.data_ptr(), solid_u8.data_ptr(), net.D, net.H, net.W, force,
                            float(gain), work.data_ptr(), net.stream)
        if info is not None:
            info["plane_flux_spread"] = float(work[3 * net.D])
    if cross_flux:
        work = torch.empty(3 * (net.H + net.W), device="cuda", dtype=torch.float64)
        net.k.nn_cross_flux(u.data_ptr(), net.D, net.H, net.W, work.data_ptr(), net.stream)
    return u, drho


def set_warm(L, lb, warm_u, warm_drho, scale=1.0):
    """Warm state through lbsetstatedev (velocity and density deviation) or
    lbsetveldev (velocity only), both fields multiplied by `scale`."""
    if scale != 1.0:
        warm_u = warm_u * scale
        warm_drho = warm_drho * scale if warm_drho is not None else None
    if warm_drho is not None:
        L.lbsetstatedev(lb, warm_u.data_ptr(), warm_drho.data_ptr())
    else:
        L.lbsetveldev(lb, warm_u.data_ptr())


def wall_force_balance(L, lb, obj, body):
    """Relative imbalance F_wall / F_body - 1 along x after one measure (two
    steps): F_wall the momentum exchanged over the bounce-back links of the
    bed's object, F_body = body = force * (fluid nodes), equal at steady
    state."""
    L.measure(lb)
    return obj.frcx / body - 1.0


def permeability_run(L, solid, force, k_ref=None, warm_u=None, tol=1e-8, rel=1e-4, check=100, maxsteps=60000,
                     warm_drho=None, correct=0, probe=0, stats=None):
    """Packed bed (device uint8 or numpy mask) until the relative change of
    the mean flow between checks is below tol (plain) or, given k_ref, until
    the permeability is within `rel` of k_ref; warm_u (device velocities,
    lbsetveldev layout) warm-starts the lattice, with warm_drho (device
    density deviations) through lbsetstatedev.  Returns the trajectory
    [(steps, k, wall seconds)] measured every `check` steps; the wall clock
    starts before the warm start.

    correct > 0 adds a force-balance correction of the warm start's mean
    flow: `correct` steps after the warm state, one measure compares the
    wall force with the body force.  In Stokes flow the wall force is linear
    in the flow, so a prediction of the right shape but a mean flow (1 +
    eps) times the converged one feels (1 + eps) times the body force; the
    warm state is set again scaled by 1 / (1 + eps) and the steps and time
    spent count towards the run (measured on held-out 128^3 packings: no
    gain, because the wall force answers the prediction's near-wall error
    rather than its mean-flow error).  probe > 0 (with k_ref) instead records,
    for `probe` measures in a row after the warm state, the force imbalance
    beside the permeability error: returns [(steps, imbalance, k error)].
    A dict `stats` receives the force imbalance of the final state
    ("imbalance_final")."""
    import torch
    mask = solid.cpu().numpy() if hasattr(solid, "cpu") else solid
    lb = L.newlb(mask.shape[0], mask.shape[1], mask.shape[2], "null")
    lb.precision = 1
    lb.tau = 1.0
    lb.stokes_flow = 1
    obj = W.insert_solid(L, lb, mask)
    L.syncobjs(lb)
    L.addbf(lb, force, 0.0, 0.0)
    body = force * L.countfluid(lb)
    L.lbsteps(lb, 2)  # upload and tuning outside the timed region
    torch.cuda.synchronize()
    eta = lb.rho0 * (lb.tau - 0.5) / 3.0
    t0 = time.perf_counter()
    steps, prev, traj = 0, None, []
    if warm_u is not None:
        set_warm(L, lb, warm_u, warm_drho)
        if probe > 0:
            rows = []
            for n in range(probe):
                imb = wall_force_balance(L, lb, obj, body)
                rows.append((2 * (n + 1), imb, (lb.vmeanx * eta / force - k_ref) / k_ref))
            L.freelb(lb)
            return rows
        if correct > 0:
            if correct > 2:
                L.lbsteps(lb, correct - 2)
            eps = wall_force_balance(L, lb, obj, body)
            steps += max(correct, 2)
            set_warm(L, lb, warm_u, warm_drho, 1.0 / (1.0 + eps))
    elif probe > 0:
        L.freelb(lb)
        return []
    while steps < maxsteps:
        L.lbsteps(lb, check - 2)
        L.measure(lb)
        steps += check
        k = lb.vmeanx * eta / force
        traj.append((steps, k, time.perf_counter() - t0))
        if k_ref is not None:
            if abs(k - k_ref) <= rel * abs(k_ref):
                break
        elif prev is not None and abs(lb.vmeanx - prev) <= tol * abs(lb.vmeanx):
            break
        prev = lb.vmeanx
    if stats is not None:
        stats["imbalance_final"] = obj.frcx / body - 1.0
    L.freelb(lb)
    return traj


def conv_layer_times(lib, side, batch, widths=(32, 64, 128, 256), reps=20):
    """Forward-convolution time of every layer shape of the network on
    `batch` grids of side^3 (CUDA events over `reps` launches on random
    BF16 data): [(level, cin, cout, ms, TFLOP/s)]."""
    import torch
    k = Kernels(lib.dll)
    dev = torch.device("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    w0, w1, w2, w3 = widths
    shapes = [(0, IN_CH, w0), (0, w0, w0), (0, w1 + w0, w0), (0, w0, w0), (0, w0, OUT_CH),
              (1, w0, w1), (1, w1, w1), (1, w2 + w1, w1), (1, w1, w1),
              (2, w1, w2), (2, w2, w2), (2, w3 + w2, w2), (2, w2, w2),
              (3, w2, w3), (3, w3, w3)]
    out = []
    for lv, cin, cout in shapes:
        d = side >> lv
        x = torch.randn((batch, d + 2, d + 2, d + 2, cin), device=dev).to(torch.bfloat16)
        y = torch.zeros((batch, d + 2, d + 2, d + 2, cout), device=dev, dtype=torch.bfloat16)
        w = (torch.randn(27 * cin * cout, device=dev) * 0.01).to(torch.bfloat16)
        b = torch.zeros(cout, device=dev)
        args = (x.data_ptr(), batch, d, d, d, cin, 0, cin, w.data_ptr(), b.data_ptr(), cout, y.data_ptr(), cout, 0,
                1, None, stream)
        for _ in range(3):
            k.tc_conv3d(*args)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            k.tc_conv3d(*args)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out.append((lv, cin, cout, ms, 2.0 * 27 * cin * cout * batch * d ** 3 / (ms * 1e-3) / 1e12))
    return out


def wgrad_layer_times(lib, side, batch, widths=(32, 64, 128, 256), reps=20):
    """Weight-gradient time (slbc_tc_wgrad_tiles for cout <= 128, else
    slbc_tc_wgrad, alone, from ready copies of dY and X; the split sum
    included) of every layer shape of the network on
    `batch` grids of side^3, CUDA events over `reps` calls on random BF16
    data: [(level, cin, cout, splits, ms, TFLOP/s)], FLOPs 2 * 27 * cin *
    cout * interior voxels."""
    import torch
    k = Kernels(lib.dll)
    dev = torch.device("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    w0, w1, w2, w3 = widths
    shapes = [(0, IN_CH, w0), (0, w1 + w0, w0), (0, w0, w0), (1, w0, w1), (1, w1, w1), (1, w2 + w1, w1),
              (2, w1, w2), (2, w2, w2), (2, w3 + w2, w2), (3, w2, w3), (3, w3, w3)]
    ws_floats = 1 << 26
    ws = torch.empty(ws_floats, device=dev, dtype=torch.float32)
    out = []
    for lv, cin, cout in shapes:
        d = side >> lv
        Wp, ps = flat_geometry(d, d, d)
        xt = torch.randn(cin, batch * ps, device=dev).to(torch.bfloat16)
        dys = torch.randn(3, cout, batch * ps, device=dev).to(torch.bfloat16)
        dw = torch.empty(27 * cout * cin, device=dev, dtype=torch.float32)
        splits = k.tc_wgrad_splits(cin, cout, batch * ps // 64, ws_floats // (27 * cout * cin))
        tail = (batch, d, d, d, Wp, ps, cin, cout, ws.data_ptr(), ws_floats, splits, dw.data_ptr(), stream)
        if cout <= 128:  # K-tile blocks, as UNet lays them out
            fn, args = k.tc_wgrad_tiles, (dys.data_ptr(), xt.data_ptr()) + tail
        else:
            fn, args = k.tc_wgrad, (dys[0].data_ptr(), dys[1].data_ptr(), dys[2].data_ptr(), xt.data_ptr()) + tail
        for _ in range(3):
            fn(*args)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn(*args)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out.append((lv, cin, cout, splits, ms, 2.0 * 27 * cin * cout * batch * d ** 3 / (ms * 1e-3) / 1e12))
    if k.tc_status() != 0:
        raise RuntimeError("wgrad_layer_times: a tensor-core pipeline wait gave up")
    return out


PACKING_SEED, PACKING_FORCE = 3, 1e-6  # the packings and body force the committed network was trained on


def held_out_comparison(L, count, side=128, check=50, rel=1e-4, weights=WEIGHTS):
    """The saved network (weights) against the plain start on the first
    `count` held-out side^3 packings of its training distribution (those
    after its training set, seed PACKING_SEED): per packing the steps and
    wall time to permeability within `rel` of the plain converged value,
    checks every `check` steps in both arms, inference timed in the warm
    arm.  Returns (rows, meta) with rows of dicts."""
    import torch
    params, widths, features, meta = load_weights(weights)
    ntrain = int(meta.get("train_samples", 0))
    specs = packing_specs(ntrain + count, PACKING_SEED)[ntrain:ntrain + count]
    inf = UNet(L, side, side, side, batch=1, widths=widths, params=params, features=features)
    rows = []
    for phi, sd in specs:
        solid = packing(side, phi, sd)
        traj = permeability_run(L, solid, PACKING_FORCE)
        k_conv = traj[-1][1]
        sdev = torch.as_tensor(solid.astype(np.uint8), device="cuda")
        plain = first_within(permeability_run(L, solid, PACKING_FORCE, k_ref=k_conv, check=check, rel=rel), k_conv,
                             rel)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        u, drho = predict_state(inf, sdev, PACKING_FORCE, ETA_TAU1)
        torch.cuda.synchronize()
        t_inf = time.perf_counter() - t0
        warm = first_within(permeability_run(L, solid, PACKING_FORCE, k_ref=k_conv, warm_u=u, warm_drho=drho,
                                             check=check, rel=rel), k_conv, rel)
        rows.append({"phi": round(phi, 4), "k": k_conv, "plain_steps": plain[0] if plain else None,
                     "plain_wall_s": round(plain[1], 4) if plain else None,
                     "warm_steps": warm[0] if warm else None,
                     "warm_wall_s": round(warm[1] + t_inf, 4) if warm else None, "inference_s": round(t_inf, 4)})
    return rows, meta


def first_within(traj, k_ref, rel):
    """(steps, wall) of the first check within rel of k_ref, else None."""
    for steps, k, wall in traj:
        if abs(k - k_ref) <= rel * abs(k_ref):
            return steps, wall
    return None


def symmetry(mask, label, flip_x, flip_y, flip_z, swap_yz):
    """One of the 16 symmetries of the periodic packed-bed problem with the
    body force along x, applied to a mask (D, H, W) over (x, y, z) and its
    steady flow (D, H, W, 3).  Reflecting y (or z) negates u_y (u_z);
    swapping y and z swaps u_y and u_z; reflecting x reverses the force, so
    by linearity of Stokes flow the solution of the reflected bed is the
    reflected solution negated as a whole: u_x kept, u_y and u_z negated,
    and a density (pressure) channel after the three velocity components
    negated too.  Other transforms move the density with the nodes."""
    import torch
    dims, sign = [], [1.0, 1.0, 1.0]
    extra = label.shape[-1] - 3
    scalar_sign = 1.0
    if flip_x:
        dims.append(0)
        sign[1], sign[2] = -sign[1], -sign[2]
        scalar_sign = -1.0
    if flip_y:
        dims.append(1)
        sign[1] = -sign[1]
    if flip_z:
        dims.append(2)
        sign[2] = -sign[2]
    if dims:
        mask, label = mask.flip(dims), label.flip(dims)
    label = label * torch.tensor(sign + [scalar_sign] * extra, device=label.device, dtype=label.dtype)
    if swap_yz:
        mask = mask.transpose(1, 2)
        label = label.transpose(1, 2)[..., [0, 2, 1] + list(range(3, 3 + extra))]
    return mask.contiguous(), label.contiguous()


def train(net, masks, labels, iters, lr=1e-3, seed=0, log_every=0, sample_w=None, lr_min=None, warmup=100, clip=3.0,
          augment=False, proj_weight=0.0):
    """Adam on mini-batches of net.B samples drawn (seeded) from masks
    (device uint8 (N, D, H, W)) and labels (device FP32 (N, D, H, W, 3)),
    optional per-sample loss weights (device FP32 (N,)); with lr_min the
    learning rate decays from lr to lr_min along a half cosine.  The rate
    ramps up linearly over the first `warmup` iterations and the gradients
    are clipped to `clip` times their running norm (0: off): without these,
    some seeds of the 1e-3 rate fell into a plateau near loss 0.25 early on.
    With augment, every drawn sample goes through a random one of the 16
    symmetries of the problem (cubic grids only).  proj_weight > 0 adds the
    squared projection of each sample's velocity error on its label
    (slbc_nn_proj): the component of the error along the converged flow,
    which the lattice removes slowest after a warm start.
    Returns the loss every log_every iterations (and the last)."""
    import torch
    rng = np.random.default_rng(seed)
    n = masks.shape[0]
    hist = []
    lab_sq = labels[..., :3].double().pow(2).sum(dim=(1, 2, 3, 4)) if proj_weight > 0 else None
    for it in range(1, iters + 1):
        idx = torch.as_tensor(rng.choice(n, size=net.B, replace=n < net.B), device=masks.device)
        mb = masks.index_select(0, idx).contiguous()
        lab = labels.index_select(0, idx).contiguous()
        sw = sample_w.index_select(0, idx).contiguous() if sample_w is not None else None
        proj = (proj_weight, lab_sq.index_select(0, idx).contiguous()) if lab_sq is not None else None
        if augment and mb.shape[1] == mb.shape[2] == mb.shape[3]:
            for b, bits in enumerate(rng.integers(0, 2, size=(net.B, 4))):
                mb[b], lab[b] = symmetry(mb[b], lab[b], *bits)
        net.encode(mb)
        net.forward()
        loss = net.loss_and_backward(lab, sw, proj)
        if clip:
            net.clip_grads(clip)
        rate = lr if lr_min is None else lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * (it - 1) / iters))
        if it <= warmup:
            rate *= it / warmup
        net.adam(rate)
        if (log_every and it % log_every == 0) or it == iters:
            hist.append((it, float(loss.item())))
    return hist
