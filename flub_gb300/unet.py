"""Learned warm start: a 3-level 3D U-Net (16/32/64 channels, 3x3x3
convolutions, BF16 activations and weights, FP32 accumulation) whose output is
CG's initial guess.  No reference counterpart: flub's MGPCG always starts from
x = 0 (multigrid/mgpcg.py:380-390 clears x before the loop); a guess can only
change the iteration count, because the solve still stops at the same
squared-residual tolerance, relative to the right-hand side.

Every operation of the forward pass, the backward pass and Adam runs as a
kernel of this library (include/flub_gb300.h, "Learned warm start"); torch
only owns the device memory.

Layout: activations channels-last [B, X, Y, Z, C] BF16; convolution weights
[27, Cout, Cin] (tap = (dx+1)*9 + (dy+1)*3 + (dz+1)); FP32 master parameters
with Adam moments; a BF16 copy of each weight for the forward pass and a
flipped, transposed BF16 copy [27, Cin, Cout] for the data gradient, both
written by the Adam kernel.

Network (N = the grid, channels in brackets):
    in[16]   = (div / rms, fluid mask, solid mask, 13 zeros)        N
    e0       = relu conv(relu conv(in))                      [16]   N
    e1       = relu conv(relu conv(pool e0))                 [32]   N/2
    m        = relu conv(relu conv(pool e1))                 [64]   N/4
    d1       = relu conv(relu conv(up m  (+) e1))            [32]   N/2
    d0       = relu conv(relu conv(up d1 (+) e0))            [16]   N
    out      = 1x1x1 head(d0) -> x / rms  (FP32)
where (+) is the decoder's skip connection, accumulated by the convolution
kernel from two sources.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib

BF16 = torch.bfloat16

# name, cin0, cin1 (skip source, 0 = none), cout, level
LAYERS = (
    ("enc0a", 16, 0, 16, 0),
    ("enc0b", 16, 0, 16, 0),
    ("enc1a", 16, 0, 32, 1),
    ("enc1b", 32, 0, 32, 1),
    ("mid_a", 32, 0, 64, 2),
    ("mid_b", 64, 0, 64, 2),
    ("dec1a", 64, 32, 32, 1),
    ("dec1b", 32, 0, 32, 1),
    ("dec0a", 32, 16, 16, 0),
    ("dec0b", 16, 0, 16, 0),
)
IN_CHANNELS = 16


def _s():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _check_act(t, C, name):
    if t.dtype != BF16 or not t.is_cuda or not t.is_contiguous() or t.shape[-1] != C or t.dim() != 5:
        raise ValueError(f"{name}: expected a contiguous CUDA bf16 [B, X, Y, Z, {C}] tensor, got "
                         f"{tuple(t.shape)} {t.dtype}")


# ------------------------------------------------------------------ op wrappers

def conv3d(x0, w0, x1=None, w1=None, bias=None, relu=True, out=None):
    """y = [relu](conv(x0, w0) + conv(x1, w1) + bias), 3x3x3, zero padding."""
    B, NX, NY, NZ, c0 = x0.shape
    cout = w0.shape[1]
    _check_act(x0, w0.shape[2], "x0")
    c1 = 0
    if x1 is not None:
        _check_act(x1, w1.shape[2], "x1")
        c1 = x1.shape[-1]
    if out is None:
        out = torch.empty((B, NX, NY, NZ, cout), dtype=BF16, device=x0.device)
    _lib.call("flub_conv3d_bf16", _p(x0), c0, _p(w0), _p(x1), c1, _p(w1), _p(bias), _p(out), cout, B, NX, NY, NZ,
              1 if relu else 0, _s())
    return out


def conv3d_wgrad(x, dy, dw, db=None):
    B, NX, NY, NZ, cin = x.shape
    cout = dy.shape[-1]
    _lib.call("flub_conv3d_wgrad", _p(x), cin, _p(dy), cout, _p(dw), _p(db), B, NX, NY, NZ, _s())


def conv_error(reset=True):
    v = ctypes.c_int32(0)
    _lib.call("flub_conv_error", ctypes.byref(v), 1 if reset else 0)
    return int(v.value)


def pool2(x, out=None):
    B, NX, NY, NZ, C = x.shape
    if out is None:
        out = torch.empty((B, NX // 2, NY // 2, NZ // 2, C), dtype=BF16, device=x.device)
    _lib.call("flub_pool2_bf16", _p(x), _p(out), B, NX, NY, NZ, C, _s())
    return out


def pool2_bwd(dy, dx, accumulate):
    B, NX, NY, NZ, C = dx.shape
    _lib.call("flub_pool2_bwd_bf16", _p(dy), _p(dx), B, NX, NY, NZ, C, 1 if accumulate else 0, _s())
    return dx


def up2(x, out=None):
    B, cx, cy, cz, C = x.shape
    if out is None:
        out = torch.empty((B, 2 * cx, 2 * cy, 2 * cz, C), dtype=BF16, device=x.device)
    _lib.call("flub_up2_bf16", _p(x), _p(out), B, 2 * cx, 2 * cy, 2 * cz, C, _s())
    return out


def up2_bwd(dy, out=None):
    B, NX, NY, NZ, C = dy.shape
    if out is None:
        out = torch.empty((B, NX // 2, NY // 2, NZ // 2, C), dtype=BF16, device=dy.device)
    _lib.call("flub_up2_bwd_bf16", _p(dy), _p(out), B, NX, NY, NZ, C, _s())
    return out


def relu_bwd(dy, y, out=None):
    out = dy if out is None else out
    _lib.call("flub_relu_bwd_bf16", _p(dy), _p(y), _p(out), dy.numel(), _s())
    return out


def unet_input(div, tag, inv_scale=None, out=None):
    """div FP32 / tag int32 of shape [B, X, Y, Z] -> BF16 [B, X, Y, Z, 16]."""
    B = div.shape[0]
    ncell = div[0].numel()
    if inv_scale is None:
        inv_scale = torch.empty(B, dtype=torch.float32, device=div.device)
    if out is None:
        out = torch.empty(tuple(div.shape) + (IN_CHANNELS,), dtype=BF16, device=div.device)
    work = torch.empty(2 * 152 * B, dtype=torch.float64, device=div.device)
    _lib.call("flub_unet_input", _p(div), _p(tag), B, ncell, _p(inv_scale), _p(work), _p(out), _s())
    return out, inv_scale


def head_fwd(x, w, b, out=None):
    n = x.numel() // x.shape[-1]
    if out is None:
        out = torch.empty(x.shape[:-1], dtype=torch.float32, device=x.device)
    _lib.call("flub_head_fwd", _p(x), _p(w), _p(b), _p(out), n, _s())
    return out


def head_bwd(x, w, dout, dw, db, dx=None):
    n = x.numel() // x.shape[-1]
    if dx is None:
        dx = torch.empty_like(x)
    _lib.call("flub_head_bwd", _p(x), _p(w), _p(dout), _p(dx), _p(dw), _p(db), n, _s())
    return dx


def unet_loss(pred, x, tag, inv_scale, inv_count=None, relative=False, dpred=None, loss=None):
    """Masked MSE of the normalised prediction; relative=True weights each
    sample by 1 / |target|^2 (mean relative squared error)."""
    B = pred.shape[0]
    ncell = pred[0].numel()
    if dpred is None:
        dpred = torch.empty_like(pred)
    if loss is None:
        loss = torch.zeros(1, dtype=torch.float64, device=pred.device)
    norm = torch.empty(B, dtype=torch.float64, device=pred.device) if relative else None
    _lib.call("flub_unet_loss", _p(pred), _p(x), _p(tag), _p(inv_scale), ncell, B,
              float(inv_count) if inv_count is not None else 0.0, _p(norm), _p(dpred), _p(loss), _s())
    return dpred, loss


def unet_output(out, tag, inv_scale, gain=1.0, x0=None):
    B = out.shape[0]
    ncell = out[0].numel()
    if x0 is None:
        x0 = torch.empty_like(out)
    _lib.call("flub_unet_output", _p(out), _p(tag), _p(inv_scale), ncell, B, float(gain), _p(x0), _s())
    return x0


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8, w16=None, w16t=None):
    cout = cin = 0
    if w16 is not None:
        cout, cin = int(w16.shape[1]), int(w16.shape[2])
    _lib.call("flub_adam", _p(p), _p(g), _p(m), _p(v), p.numel(), float(lr), float(b1), float(b2), float(eps),
              int(step), _p(w16), _p(w16t), cout, cin, _s())


# ------------------------------------------------------------------ the network

class _Param:
    """FP32 master + gradient + Adam moments (+ BF16 copies for a conv weight)."""

    def __init__(self, value, conv):
        self.p = value.contiguous()
        self.g = torch.zeros_like(self.p)
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.conv = conv
        if conv:
            t, co, ci = self.p.shape
            self.w16 = torch.empty((t, co, ci), dtype=BF16, device=self.p.device)
            self.w16t = torch.empty((t, ci, co), dtype=BF16, device=self.p.device)
            self.refresh()

    def refresh(self):
        """BF16 copy and flipped transposed copy from the FP32 master."""
        if self.conv:
            self.w16.copy_(self.p.to(BF16))
            self.w16t.copy_(self.p.flip(0).transpose(1, 2).to(BF16))


class UNet3D:
    def __init__(self, device=None, seed=0):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        gen = torch.Generator().manual_seed(seed)
        self.params = {}
        for name, c0, c1, co, _lvl in LAYERS:
            fan_in = 27 * (c0 + c1)
            std = math.sqrt(2.0 / fan_in)
            self.params[name + ".w0"] = _Param((torch.randn((27, co, c0), generator=gen) * std).to(self.device), True)
            if c1:
                self.params[name + ".w1"] = _Param((torch.randn((27, co, c1), generator=gen) * std).to(self.device),
                                                   True)
            self.params[name + ".b"] = _Param(torch.zeros(co, device=self.device), False)
        self.params["head.w"] = _Param((torch.randn(16, generator=gen) * 0.25).to(self.device), False)
        self.params["head.b"] = _Param(torch.zeros(1, device=self.device), False)
        self.step_count = 0
        self._acts = None

    # ---------------------------------------------------------------- state
    def state_dict(self):
        return {k: v.p.detach().cpu().numpy().copy() for k, v in self.params.items()}

    def load_state_dict(self, sd):
        for k, v in self.params.items():
            a = torch.as_tensor(np.asarray(sd[k], dtype=np.float32))
            if tuple(a.shape) != tuple(v.p.shape):
                raise ValueError(f"{k}: shape {tuple(a.shape)}, expected {tuple(v.p.shape)}")
            v.p.copy_(a.to(self.device))
            v.refresh()

    def save(self, path):
        np.savez(path, **self.state_dict())

    @classmethod
    def load(cls, path, device=None):
        net = cls(device=device)
        with np.load(path) as z:
            net.load_state_dict({k: z[k] for k in z.files})
        return net

    def num_parameters(self):
        return sum(v.p.numel() for v in self.params.values())

    @staticmethod
    def check_shape(shape):
        """Grid extents the network accepts: every level's convolution needs
        NZ to divide 128 (or be a multiple of it) and NY a multiple of 128/NZ."""
        nx, ny, nz = shape
        for l in range(3):
            X, Y, Z = nx >> l, ny >> l, nz >> l
            if (X << l, Y << l, Z << l) != (nx, ny, nz) or min(X, Y, Z) < 1:
                return False
            zb = Z if Z < 128 else 128
            if 128 % zb or Z % zb or Y % (128 // zb):
                return False
        return True

    # ---------------------------------------------------------------- forward
    def _w(self, name):
        return self.params[name].w16

    def _b(self, name):
        return self.params[name].p

    def forward(self, div, tag, keep=False):
        """div [B, X, Y, Z] FP32, tag int32 (0 air, 1 fluid, 2 solid).  Returns
        (out, inv_scale): out is the normalised prediction x * inv_scale[b]."""
        if div.dim() == 3:
            div, tag = div.unsqueeze(0), tag.unsqueeze(0)
        if not self.check_shape(tuple(div.shape[1:])):
            raise ValueError(f"UNet3D: unsupported grid {tuple(div.shape[1:])}")
        a = {}
        inp, inv_scale = unet_input(div.contiguous(), tag.contiguous())
        a["in"] = inp
        c = lambda x, n, x1=None: conv3d(x, self._w(n + ".w0"), x1,
                                         self.params[n + ".w1"].w16 if x1 is not None else None, self._b(n + ".b"))
        a["e0a"] = c(inp, "enc0a")
        a["e0"] = c(a["e0a"], "enc0b")
        a["p0"] = pool2(a["e0"])
        a["e1a"] = c(a["p0"], "enc1a")
        a["e1"] = c(a["e1a"], "enc1b")
        a["p1"] = pool2(a["e1"])
        a["ma"] = c(a["p1"], "mid_a")
        a["m"] = c(a["ma"], "mid_b")
        a["u1"] = up2(a["m"])
        a["d1a"] = c(a["u1"], "dec1a", a["e1"])
        a["d1"] = c(a["d1a"], "dec1b")
        a["u0"] = up2(a["d1"])
        a["d0a"] = c(a["u0"], "dec0a", a["e0"])
        a["d0"] = c(a["d0a"], "dec0b")
        out = head_fwd(a["d0"], self.params["head.w"].p, self.params["head.b"].p)
        self._acts = a if keep else None
        return out, inv_scale

    def predict(self, div, tag, gain=1.0, out=None):
        """Pressure guess in the units of div (x0 for the solve); 0 off fluid."""
        o, inv = self.forward(div, tag)
        return unet_output(o, tag if tag.dim() == o.dim() else tag.unsqueeze(0), inv, gain,
                           out if out is not None else None)

    # ---------------------------------------------------------------- backward
    def zero_grad(self):
        for v in self.params.values():
            v.g.zero_()

    def backward(self, dout):
        """Accumulate parameter gradients from d loss / d out (FP32, the shape
        of out).  Needs forward(..., keep=True)."""
        a = self._acts
        if a is None:
            raise RuntimeError("backward() needs forward(keep=True)")
        P = self.params

        def conv_back(name, x0, dy, x1=None, need_dx=True):
            # dy is already through the ReLU gradient
            conv3d_wgrad(x0, dy, P[name + ".w0"].g, P[name + ".b"].g)
            if x1 is not None:
                conv3d_wgrad(x1, dy, P[name + ".w1"].g, None)
            if not need_dx:
                return None, None
            dx0 = conv3d(dy, P[name + ".w0"].w16t, relu=False)
            dx1 = conv3d(dy, P[name + ".w1"].w16t, relu=False) if x1 is not None else None
            return dx0, dx1

        g = head_bwd(a["d0"], P["head.w"].p, dout, P["head.w"].g, P["head.b"].g)
        g = relu_bwd(g, a["d0"])
        g, _ = conv_back("dec0b", a["d0a"], g)
        g = relu_bwd(g, a["d0a"])
        g_u0, g_e0 = conv_back("dec0a", a["u0"], g, a["e0"])
        g = relu_bwd(up2_bwd(g_u0), a["d1"])
        g, _ = conv_back("dec1b", a["d1a"], g)
        g = relu_bwd(g, a["d1a"])
        g_u1, g_e1 = conv_back("dec1a", a["u1"], g, a["e1"])
        g = relu_bwd(up2_bwd(g_u1), a["m"])
        g, _ = conv_back("mid_b", a["ma"], g)
        g = relu_bwd(g, a["ma"])
        g, _ = conv_back("mid_a", a["p1"], g)
        g = relu_bwd(pool2_bwd(g, g_e1, accumulate=True), a["e1"])
        g, _ = conv_back("enc1b", a["e1a"], g)
        g = relu_bwd(g, a["e1a"])
        g, _ = conv_back("enc1a", a["p0"], g)
        g = relu_bwd(pool2_bwd(g, g_e0, accumulate=True), a["e0"])
        g, _ = conv_back("enc0b", a["e0a"], g)
        g = relu_bwd(g, a["e0a"])
        conv_back("enc0a", a["in"], g, need_dx=False)

    def loss_and_grad(self, div, tag, x, relative=True):
        """Masked MSE of the normalised prediction against x (the converged
        solution), by default relative per sample (mean of
        |pred - t|^2 / |t|^2); accumulates gradients.  Returns the loss
        (device scalar)."""
        if div.dim() == 3:
            div, tag, x = div.unsqueeze(0), tag.unsqueeze(0), x.unsqueeze(0)
        out, inv = self.forward(div, tag, keep=True)
        inv_count = None
        if not relative:
            inv_count = 1.0 / max(int((tag == 1).sum().item()), 1)
        dout, loss = unet_loss(out, x.contiguous(), tag.contiguous(), inv, inv_count, relative=relative)
        self.backward(dout)
        self._acts = None
        return loss

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        for v in self.params.values():
            adam(v.p, v.g, v.m, v.v, self.step_count, lr, b1, b2, eps,
                 v.w16 if v.conv else None, v.w16t if v.conv else None)
