"""CPU reference of the learned warm start's U-Net (test infrastructure: only
the tests use it, as the checker of the GPU kernels).

The network of flub_gb300/unet.py restated with torch.nn.functional on the CPU
in float64, with autograd for the gradients.  No reference counterpart (flub
has no learned warm start).  With ``bf16=True`` the weights and every
activation are rounded to bfloat16 where the GPU path stores them, so the
forward pass can be compared tightly; gradients are always float64.

Weights are taken in the GPU layout [27, Cout, Cin] (tap = (dx+1)*9 + (dy+1)*3
+ (dz+1)) and converted to torch's [Cout, Cin, 3, 3, 3]; activations are
channels-last [B, X, Y, Z, C] at the interface.
"""
import torch
import torch.nn.functional as F

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


def rb(t, on=True):
    """Round to bfloat16 (value kept in float64) when on."""
    return t.to(torch.bfloat16).to(torch.float64) if on else t


def w_to_torch(w):
    """[27, Cout, Cin] -> [Cout, Cin, 3, 3, 3]."""
    t, co, ci = w.shape
    return w.reshape(3, 3, 3, co, ci).permute(3, 4, 0, 1, 2).contiguous()


def to_ncdhw(x):
    return x.permute(0, 4, 1, 2, 3).contiguous()


def to_ndhwc(x):
    return x.permute(0, 2, 3, 4, 1).contiguous()


def conv3d(x0, w0, x1=None, w1=None, bias=None, relu=True):
    """Channels-last float64 3x3x3 convolution with an optional second source."""
    y = F.conv3d(to_ncdhw(x0), w_to_torch(w0), padding=1)
    if x1 is not None:
        y = y + F.conv3d(to_ncdhw(x1), w_to_torch(w1), padding=1)
    y = to_ndhwc(y)
    if bias is not None:
        y = y + bias
    return torch.relu(y) if relu else y


def pool2(x):
    return to_ndhwc(F.avg_pool3d(to_ncdhw(x), 2))


def up2(x):
    return x.repeat_interleave(2, 1).repeat_interleave(2, 2).repeat_interleave(2, 3)


def unet_input(div, tag):
    """div / rms over fluid, fluid mask, solid mask, 13 zero channels; and
    inv_scale per sample."""
    B = div.shape[0]
    fl = (tag == 1)
    inv = torch.ones(B, dtype=torch.float64)
    for b in range(B):
        c = int(fl[b].sum())
        s = float((div[b].double()[fl[b]] ** 2).sum())
        if c > 0 and s > 0:
            inv[b] = 1.0 / (s / c) ** 0.5
    x = torch.zeros(tuple(div.shape) + (16,), dtype=torch.float64)
    x[..., 0] = torch.where(fl, div.double() * inv.view(B, 1, 1, 1), 0.0)
    x[..., 1] = fl.double()
    x[..., 2] = (tag == 2).double()
    return x, inv


def forward(params, div, tag, bf16=True):
    """params: dict name -> float64 tensor (GPU layout).  Returns (out, inv)."""
    P = {k: (rb(v, bf16) if v.dim() == 3 else v) for k, v in params.items()}
    x, inv = unet_input(div, tag)
    x = rb(x, bf16)

    def c(inp, n, x1=None):
        return rb(conv3d(inp, P[n + ".w0"], x1, P.get(n + ".w1") if x1 is not None else None, P[n + ".b"]), bf16)

    e0 = c(c(x, "enc0a"), "enc0b")
    e1 = c(c(rb(pool2(e0), bf16), "enc1a"), "enc1b")
    m = c(c(rb(pool2(e1), bf16), "mid_a"), "mid_b")
    d1 = c(c(up2(m), "dec1a", e1), "dec1b")
    d0 = c(c(up2(d1), "dec0a", e0), "dec0b")
    out = (d0 * P["head.w"]).sum(-1) + P["head.b"]
    return out, inv


def loss_fn(out, x, tag, inv, relative=False):
    """Masked MSE of the normalised prediction: the mean over the batch's fluid
    cells, or (relative=True) the mean over samples of |out - t|^2 / |t|^2."""
    fl = tag == 1
    B = out.shape[0]
    t = x.double() * inv.view(B, 1, 1, 1)
    d = out - t
    if not relative:
        return (d[fl] ** 2).sum() / max(int(fl.sum()), 1)
    total = 0.0
    for b in range(B):
        nb = float((t[b][fl[b]] ** 2).sum())
        if nb > 0:
            total = total + (d[b][fl[b]] ** 2).sum() / (B * nb)
    return total


def loss_and_grads(params, div, tag, x, bf16=True, relative=True):
    """Float64 loss and d loss / d param for every parameter."""
    leaf = {k: v.detach().clone().double().requires_grad_(True) for k, v in params.items()}
    out, inv = forward(leaf, div, tag, bf16=bf16)
    loss = loss_fn(out, x, tag, inv, relative=relative)
    loss.backward()
    return float(loss.detach()), {k: v.grad.detach() for k, v in leaf.items()}, out.detach()
