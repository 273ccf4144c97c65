"""Learned warm start: the U-Net that predicts the initial field of a 2-D
Laplace Jacobi solve from its Dirichlet border.

Every operation runs in libstencil_gb300.so (include/unet.h): BF16 tensor-core
implicit-GEMM 3x3 convolutions (forward, data gradient, weight gradient) with
FP32 accumulation, pooling, upsampling, ReLU, the output head, the masked MSE
loss and Adam on FP32 master weights.  This module sequences those calls and
owns the buffers (torch CUDA tensors, used as plain device memory).

Architecture (4 levels, 32 base channels, 3x3 convolutions, ReLU):
  enc0 32-32 | pool | enc1 64-64 | pool | enc2 128-128 | pool | bottom 256-256
  up + cat(enc2) 384 -> 128-128 | up + cat(enc1) 192 -> 64-64 |
  up + cat(enc0) 96 -> 32-32 | 1x1 head -> 1
The two bottom convolutions take their taps 2 and 4 cells apart (dilation):
the receptive field then reaches about 80 cells from each output cell, so at
the 128 x 128 training size every interior cell sees all four borders (with
undilated taps it reaches 48, and the centre of the grid sees none).
Inputs (3 of 32 padded channels): the border field, the border mask and the
transfinite (Coons) interpolation of the border.  The head predicts the
correction to the Coons field on interior cells.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import lib as _lib

IN_CH = 32
DILATION = {"ba": 2, "bb": 4}  # layers whose taps are spread (default 1)
LAYERS = [  # name, cin, cout
    ("e0a", IN_CH, 32), ("e0b", 32, 32),
    ("e1a", 32, 64), ("e1b", 64, 64),
    ("e2a", 64, 128), ("e2b", 128, 128),
    ("ba", 128, 256), ("bb", 256, 256),
    ("d2a", 384, 128), ("d2b", 128, 128),
    ("d1a", 192, 64), ("d1b", 64, 64),
    ("d0a", 96, 32), ("d0b", 32, 32),
]


class Act(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("n", ctypes.c_int), ("h", ctypes.c_int),
                ("w", ctypes.c_int), ("c_stride", ctypes.c_int), ("c_off", ctypes.c_int),
                ("c", ctypes.c_int), ("reserved", ctypes.c_int)]


_sig_done = False


def _L():
    global _sig_done
    L = _lib.load()
    if not _sig_done:
        A = ctypes.POINTER(Act)
        vp, i, f, ll = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_longlong
        sig = {
            "unet_conv3x3_fwd": [A, vp, vp, A, i, vp],
            "unet_conv3x3_fwd_dil": [A, vp, vp, A, i, i, vp],
            "unet_conv3x3_fwd_engine": [A, vp, vp, A, i, i, i, vp],
            "unet_conv3x3_wgrad_dil": [A, A, vp, vp, i, vp],
            "unet_conv3x3_wgrad_engine": [A, A, vp, vp, i, i, vp, ctypes.c_size_t, vp],
            "unet_wgrad_workspace_bytes": [A, A, ctypes.POINTER(ctypes.c_size_t)],
            "unet_flip_weights": [vp, vp, i, i, vp],
            "unet_conv3x3_wgrad": [A, A, vp, vp, vp],
            "unet_relu_bwd": [A, A, vp],
            "unet_maxpool2_fwd": [A, A, vp],
            "unet_maxpool2_bwd": [A, A, A, A, vp],
            "unet_upsample2_fwd": [A, A, vp],
            "unet_upsample2_bwd": [A, A, vp],
            "unet_add": [A, A, vp],
            "unet_head_fwd": [A, vp, vp, vp, vp],
            "unet_head_bwd": [A, vp, vp, A, vp, vp, vp],
            "unet_features": [vp, i, i, i, A, vp, vp],
            "unet_mse": [vp, vp, vp, i, i, i, f, vp, vp, vp],
            "unet_adam": [vp, vp, vp, vp, vp, ll, f, f, f, f, i, vp],
            "unet_assemble": [vp, vp, vp, i, i, i, vp, vp],
            "unet_to_bf16": [vp, vp, ll, vp],
            "unet_coons_fill": [vp, i, i, i, vp, vp],
            "unet_resample_border": [vp, i, i, i, i, i, vp, vp],
            "unet_upsample_bilinear": [vp, i, i, i, vp, i, i, vp, vp],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _sig_done = True
    return L


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def view(t, c_off=0, c=None):
    """An NHWC BF16 view of tensor t (shape [n, h, w, c_stride])."""
    n, h, w, cs = t.shape
    return Act(t.data_ptr(), n, h, w, cs, c_off, cs - c_off if c is None else c, 0)


def _chk(rc, where):
    _lib.check(rc, where)


class UNet:
    """Parameters, optimizer state and per-shape activation buffers."""

    def __init__(self, device="cuda", seed=0):
        import torch
        self.device = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        self.params = {}
        for name, cin, cout in LAYERS:
            std = math.sqrt(2.0 / (9 * cin))
            w = (torch.randn(cout, 9, cin, generator=g) * std).float()
            if name == "e0a":
                w[:, :, 3:] = 0.0  # padded input channels
            self.params[name] = {
                "w": w.to(self.device).contiguous(),
                "b": torch.zeros(cout, device=self.device),
            }
        self.head_w = (torch.randn(32, generator=g) * 0.01).float().to(self.device)
        self.head_b = torch.zeros(1, device=self.device)
        self._alloc_state()
        self.bufs = {}
        self.step = 0

    # -- parameters --------------------------------------------------------
    def _alloc_state(self):
        import torch
        for name, cin, cout in LAYERS:
            P = self.params[name]
            P["wb"] = torch.empty(P["w"].shape, dtype=torch.bfloat16, device=self.device)
            P["wt"] = torch.empty((cin, 9, cout), dtype=torch.bfloat16, device=self.device)
            for k in ("w", "b"):
                P["d" + k] = torch.zeros_like(P[k])
                P["m" + k] = torch.zeros_like(P[k])
                P["v" + k] = torch.zeros_like(P[k])
        self.head = {"w": self.head_w, "b": self.head_b}
        for k in ("w", "b"):
            self.head["d" + k] = torch.zeros_like(self.head[k])
            self.head["m" + k] = torch.zeros_like(self.head[k])
            self.head["v" + k] = torch.zeros_like(self.head[k])
        self.sync_bf16()

    def sync_bf16(self, stream=None):
        s = _stream(stream)
        L = _L()
        for name, cin, cout in LAYERS:
            P = self.params[name]
            _chk(L.unet_to_bf16(_p(P["w"]), _p(P["wb"]), P["w"].numel(), s), "unet_to_bf16")

    def state_dict(self):
        out = {}
        for name, _, _ in LAYERS:
            out[name + ".w"] = self.params[name]["w"].cpu().numpy()
            out[name + ".b"] = self.params[name]["b"].cpu().numpy()
        out["head.w"] = self.head["w"].cpu().numpy()
        out["head.b"] = self.head["b"].cpu().numpy()
        return out

    def load_state_dict(self, d):
        import torch
        for name, _, _ in LAYERS:
            self.params[name]["w"].copy_(torch.from_numpy(np.asarray(d[name + ".w"])))
            self.params[name]["b"].copy_(torch.from_numpy(np.asarray(d[name + ".b"])))
        self.head["w"].copy_(torch.from_numpy(np.asarray(d["head.w"])))
        self.head["b"].copy_(torch.from_numpy(np.asarray(d["head.b"])))
        self.sync_bf16()

    def save(self, path):
        np.savez(path, **self.state_dict())

    def load(self, path):
        self.load_state_dict(dict(np.load(path)))

    # -- buffers -----------------------------------------------------------
    def _buffers(self, n, h, w):
        import torch
        key = (n, h, w)
        if key in self.bufs:
            return self.bufs[key]
        if h % 8 or w % 8:
            raise ValueError("grid sides must be multiples of 8")
        bf = dict(dtype=torch.bfloat16, device=self.device)
        B = {}
        shapes = {
            "x0": (n, h, w, IN_CH), "e0a": (n, h, w, 32), "cat0": (n, h, w, 96),
            "p0": (n, h // 2, w // 2, 32), "e1a": (n, h // 2, w // 2, 64),
            "cat1": (n, h // 2, w // 2, 192), "p1": (n, h // 4, w // 4, 64),
            "e2a": (n, h // 4, w // 4, 128), "cat2": (n, h // 4, w // 4, 384),
            "p2": (n, h // 8, w // 8, 128), "ba": (n, h // 8, w // 8, 256),
            "bb": (n, h // 8, w // 8, 256), "d2a": (n, h // 4, w // 4, 128),
            "d2b": (n, h // 4, w // 4, 128), "d1a": (n, h // 2, w // 2, 64),
            "d1b": (n, h // 2, w // 2, 64), "d0a": (n, h, w, 32), "d0b": (n, h, w, 32),
        }
        for k, shp in shapes.items():
            B[k] = torch.empty(shp, **bf)
            if k not in ("x0",):
                B["g_" + k] = torch.empty(shp, **bf)
        for k in ("g_e0b", "g_e1b", "g_e2b"):
            pass
        B["g_e0b"] = torch.empty((n, h, w, 32), **bf)
        B["g_e1b"] = torch.empty((n, h // 2, w // 2, 64), **bf)
        B["g_e2b"] = torch.empty((n, h // 4, w // 4, 128), **bf)
        B["g_tmp32"] = torch.empty((n, h, w, 32), **bf)
        B["coons"] = torch.empty((n, h, w), dtype=torch.float32, device=self.device)
        B["out"] = torch.empty((n, h, w), dtype=torch.float32, device=self.device)
        B["dout"] = torch.empty((n, h, w), dtype=torch.float32, device=self.device)
        B["loss"] = torch.zeros(1, dtype=torch.float32, device=self.device)
        self.bufs[key] = B
        return B

    # -- forward -----------------------------------------------------------
    def _conv(self, name, x, y, s):
        P = self.params[name]
        _chk(_L().unet_conv3x3_fwd_dil(ctypes.byref(x), _p(P["wb"]), _p(P["b"]), ctypes.byref(y), 1,
                                       DILATION.get(name, 1), s),
             "conv " + name)

    def forward(self, fields, stream=None):
        """fields: fp32 [n, h, w] with the Dirichlet border on the outer ring.
        Returns (out, coons, buffers): out fp32 [n, h, w] = predicted correction."""
        s = _stream(stream)
        L = _L()
        n, h, w = fields.shape
        B = self._buffers(n, h, w)
        _chk(L.unet_features(_p(fields), n, h, w, ctypes.byref(view(B["x0"])), _p(B["coons"]), s),
             "unet_features")
        V = view
        self._conv("e0a", V(B["x0"]), V(B["e0a"]), s)
        self._conv("e0b", V(B["e0a"]), V(B["cat0"], 64, 32), s)
        _chk(L.unet_maxpool2_fwd(ctypes.byref(V(B["cat0"], 64, 32)), ctypes.byref(V(B["p0"])), s), "pool0")
        self._conv("e1a", V(B["p0"]), V(B["e1a"]), s)
        self._conv("e1b", V(B["e1a"]), V(B["cat1"], 128, 64), s)
        _chk(L.unet_maxpool2_fwd(ctypes.byref(V(B["cat1"], 128, 64)), ctypes.byref(V(B["p1"])), s), "pool1")
        self._conv("e2a", V(B["p1"]), V(B["e2a"]), s)
        self._conv("e2b", V(B["e2a"]), V(B["cat2"], 256, 128), s)
        _chk(L.unet_maxpool2_fwd(ctypes.byref(V(B["cat2"], 256, 128)), ctypes.byref(V(B["p2"])), s), "pool2")
        self._conv("ba", V(B["p2"]), V(B["ba"]), s)
        self._conv("bb", V(B["ba"]), V(B["bb"]), s)
        _chk(L.unet_upsample2_fwd(ctypes.byref(V(B["bb"])), ctypes.byref(V(B["cat2"], 0, 256)), s), "up2")
        self._conv("d2a", V(B["cat2"]), V(B["d2a"]), s)
        self._conv("d2b", V(B["d2a"]), V(B["d2b"]), s)
        _chk(L.unet_upsample2_fwd(ctypes.byref(V(B["d2b"])), ctypes.byref(V(B["cat1"], 0, 128)), s), "up1")
        self._conv("d1a", V(B["cat1"]), V(B["d1a"]), s)
        self._conv("d1b", V(B["d1a"]), V(B["d1b"]), s)
        _chk(L.unet_upsample2_fwd(ctypes.byref(V(B["d1b"])), ctypes.byref(V(B["cat0"], 0, 64)), s), "up0")
        self._conv("d0a", V(B["cat0"]), V(B["d0a"]), s)
        self._conv("d0b", V(B["d0a"]), V(B["d0b"]), s)
        _chk(L.unet_head_fwd(ctypes.byref(V(B["d0b"])), _p(self.head["w"]), _p(self.head["b"]),
                             _p(B["out"]), s), "head")
        return B["out"], B["coons"], B

    # -- backward ----------------------------------------------------------
    def _conv_bwd(self, name, x, y, gy, gx, s):
        """gy holds dL/dy (post-ReLU output y); accumulates dW/db, writes dL/dx into gx."""
        L = _L()
        P = self.params[name]
        _chk(L.unet_relu_bwd(ctypes.byref(gy), ctypes.byref(y), s), "relu_bwd " + name)
        d = DILATION.get(name, 1)
        ws = self._wgrad_ws(x, gy)
        _chk(L.unet_conv3x3_wgrad_engine(ctypes.byref(x), ctypes.byref(gy), _p(P["dw"]), _p(P["db"]), d, 0,
                                         _p(ws), ws.numel(), s),
             "wgrad " + name)
        if gx is not None:
            cin, cout = P["w"].shape[2], P["w"].shape[0]
            _chk(L.unet_flip_weights(_p(P["wb"]), _p(P["wt"]), cout, cin, s), "flip " + name)
            _chk(L.unet_conv3x3_fwd_dil(ctypes.byref(gy), _p(P["wt"]), None, ctypes.byref(gx), 0, d, s),
                 "dgrad " + name)

    def _wgrad_ws(self, x, gy):
        """Device workspace for the tcgen05 weight gradient (channel-major
        copies of the layer's input and output gradient), grown on demand."""
        import torch
        need = ctypes.c_size_t()
        _chk(_L().unet_wgrad_workspace_bytes(ctypes.byref(x), ctypes.byref(gy), ctypes.byref(need)),
             "wgrad workspace")
        ws = getattr(self, "_ws", None)
        if ws is None or ws.numel() < need.value:
            self._ws = ws = torch.empty(need.value, dtype=torch.uint8, device=self.device)
        return ws

    def zero_grad(self):
        for name, _, _ in LAYERS:
            self.params[name]["dw"].zero_()
            self.params[name]["db"].zero_()
        self.head["dw"].zero_()
        self.head["db"].zero_()

    def backward(self, B, stream=None):
        """Gradients of the loss whose dL/d(out) is in B['dout']."""
        s = _stream(stream)
        L = _L()
        V = view
        _chk(L.unet_head_bwd(ctypes.byref(V(B["d0b"])), _p(self.head["w"]), _p(B["dout"]),
                             ctypes.byref(V(B["g_d0b"])), _p(self.head["dw"]), _p(self.head["db"]), s),
             "head_bwd")
        self._conv_bwd("d0b", V(B["d0a"]), V(B["d0b"]), V(B["g_d0b"]), V(B["g_d0a"]), s)
        self._conv_bwd("d0a", V(B["cat0"]), V(B["d0a"]), V(B["g_d0a"]), V(B["g_cat0"]), s)
        _chk(L.unet_upsample2_bwd(ctypes.byref(V(B["g_cat0"], 0, 64)), ctypes.byref(V(B["g_d1b"])), s), "up0 bwd")
        self._conv_bwd("d1b", V(B["d1a"]), V(B["d1b"]), V(B["g_d1b"]), V(B["g_d1a"]), s)
        self._conv_bwd("d1a", V(B["cat1"]), V(B["d1a"]), V(B["g_d1a"]), V(B["g_cat1"]), s)
        _chk(L.unet_upsample2_bwd(ctypes.byref(V(B["g_cat1"], 0, 128)), ctypes.byref(V(B["g_d2b"])), s), "up1 bwd")
        self._conv_bwd("d2b", V(B["d2a"]), V(B["d2b"]), V(B["g_d2b"]), V(B["g_d2a"]), s)
        self._conv_bwd("d2a", V(B["cat2"]), V(B["d2a"]), V(B["g_d2a"]), V(B["g_cat2"]), s)
        _chk(L.unet_upsample2_bwd(ctypes.byref(V(B["g_cat2"], 0, 256)), ctypes.byref(V(B["g_bb"])), s), "up2 bwd")
        self._conv_bwd("bb", V(B["ba"]), V(B["bb"]), V(B["g_bb"]), V(B["g_ba"]), s)
        self._conv_bwd("ba", V(B["p2"]), V(B["ba"]), V(B["g_ba"]), V(B["g_p2"]), s)
        # level 2: pool gradient + skip gradient
        _chk(L.unet_maxpool2_bwd(ctypes.byref(V(B["cat2"], 256, 128)), ctypes.byref(V(B["p2"])),
                                 ctypes.byref(V(B["g_p2"])), ctypes.byref(V(B["g_e2b"])), s), "pool2 bwd")
        _chk(L.unet_add(ctypes.byref(V(B["g_e2b"])), ctypes.byref(V(B["g_cat2"], 256, 128)), s), "add2")
        self._conv_bwd("e2b", V(B["e2a"]), V(B["cat2"], 256, 128), V(B["g_e2b"]), V(B["g_e2a"]), s)
        self._conv_bwd("e2a", V(B["p1"]), V(B["e2a"]), V(B["g_e2a"]), V(B["g_p1"]), s)
        _chk(L.unet_maxpool2_bwd(ctypes.byref(V(B["cat1"], 128, 64)), ctypes.byref(V(B["p1"])),
                                 ctypes.byref(V(B["g_p1"])), ctypes.byref(V(B["g_e1b"])), s), "pool1 bwd")
        _chk(L.unet_add(ctypes.byref(V(B["g_e1b"])), ctypes.byref(V(B["g_cat1"], 128, 64)), s), "add1")
        self._conv_bwd("e1b", V(B["e1a"]), V(B["cat1"], 128, 64), V(B["g_e1b"]), V(B["g_e1a"]), s)
        self._conv_bwd("e1a", V(B["p0"]), V(B["e1a"]), V(B["g_e1a"]), V(B["g_p0"]), s)
        _chk(L.unet_maxpool2_bwd(ctypes.byref(V(B["cat0"], 64, 32)), ctypes.byref(V(B["p0"])),
                                 ctypes.byref(V(B["g_p0"])), ctypes.byref(V(B["g_e0b"])), s), "pool0 bwd")
        _chk(L.unet_add(ctypes.byref(V(B["g_e0b"])), ctypes.byref(V(B["g_cat0"], 64, 32)), s), "add0")
        self._conv_bwd("e0b", V(B["e0a"]), V(B["cat0"], 64, 32), V(B["g_e0b"]), V(B["g_e0a"]), s)
        self._conv_bwd("e0a", V(B["x0"]), V(B["e0a"]), V(B["g_e0a"]), None, s)

    def loss_and_grad(self, fields, targets, stream=None):
        """Masked MSE of (coons + out) against targets over interior cells;
        fills B['dout'] and returns the loss tensor (device, fp32 sum)."""
        s = _stream(stream)
        out, coons, B = self.forward(fields, stream)
        n, h, w = fields.shape
        B["loss"].zero_()
        scale = 1.0 / (n * (h - 2) * (w - 2))
        _chk(_L().unet_mse(_p(out), _p(coons), _p(targets), n, h, w, scale, _p(B["loss"]),
                           _p(B["dout"]), s), "unet_mse")
        return B

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
        s = _stream(stream)
        L = _L()
        self.step += 1
        for name, _, _ in LAYERS:
            P = self.params[name]
            _chk(L.unet_adam(_p(P["w"]), _p(P["dw"]), _p(P["mw"]), _p(P["vw"]), _p(P["wb"]),
                             P["w"].numel(), lr, beta1, beta2, eps, self.step, s), "adam")
            _chk(L.unet_adam(_p(P["b"]), _p(P["db"]), _p(P["mb"]), _p(P["vb"]), None,
                             P["b"].numel(), lr, beta1, beta2, eps, self.step, s), "adam")
        for k in ("w", "b"):
            _chk(L.unet_adam(_p(self.head[k]), _p(self.head["d" + k]), _p(self.head["m" + k]),
                             _p(self.head["v" + k]), None, self.head[k].numel(), lr, beta1, beta2,
                             eps, self.step, s), "adam")

    def predict(self, fields, stream=None):
        """Initial fields: the border, and coons + prediction inside (fp32 [n, h, w])."""
        import torch
        s = _stream(stream)
        out, coons, B = self.forward(fields, stream)
        u = torch.empty_like(fields)
        n, h, w = fields.shape
        _chk(_L().unet_assemble(_p(fields), _p(coons), _p(out), n, h, w, _p(u), s), "assemble")
        return u


def coons_fill(fields, stream=None):
    """Border kept, interior = transfinite interpolation of the border
    (fields fp32 [n, h, w]; one kernel)."""
    import torch
    n, h, w = fields.shape
    u = torch.empty_like(fields)
    _chk(_L().unet_coons_fill(_p(fields), n, h, w, _p(u), _stream(stream)), "unet_coons_fill")
    return u


def resample_border(fields, h, w, stream=None):
    """Coarse h x w problems: the fine border sampled at the nearest positions, zero interior."""
    import torch
    n, H, W = fields.shape
    c = torch.empty((n, h, w), dtype=torch.float32, device=fields.device)
    _chk(_L().unet_resample_border(_p(fields), n, H, W, h, w, _p(c), _stream(stream)),
         "unet_resample_border")
    return c


def upsample_bilinear(coarse, fields, stream=None):
    """Fine fields: bilinear (corners aligned) interpolation of coarse inside,
    the fine border of `fields` on the band."""
    import torch
    n, h, w = coarse.shape
    _, H, W = fields.shape
    u = torch.empty_like(fields)
    _chk(_L().unet_upsample_bilinear(_p(coarse), n, h, w, _p(fields), H, W, _p(u), _stream(stream)),
         "unet_upsample_bilinear")
    return u


def _stream(stream):
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)
