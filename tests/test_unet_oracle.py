"""CPU checks of the U-Net reference (oracle/unet_ref.py) itself: its
autograd gradients against central finite differences in float64, its
convolution against a direct loop, and the host-side shape rules."""
import numpy as np
import pytest
import torch

from oracle import unet_ref as R


def _params(seed):
    g = torch.Generator().manual_seed(seed)
    P = {}
    for name, c0, c1, co, _ in R.LAYERS:
        P[name + ".w0"] = torch.randn((27, co, c0), generator=g, dtype=torch.float64) * (2.0 / (27 * (c0 + c1))) ** 0.5
        if c1:
            P[name + ".w1"] = torch.randn((27, co, c1), generator=g, dtype=torch.float64) * (2.0 / (27 * (c0 + c1))) ** 0.5
        P[name + ".b"] = torch.randn(co, generator=g, dtype=torch.float64) * 0.05
    P["head.w"] = torch.randn(16, generator=g, dtype=torch.float64) * 0.25
    P["head.b"] = torch.zeros(1, dtype=torch.float64)
    return P


def _scene(seed, shape=(4, 4, 8), B=1):
    g = torch.Generator().manual_seed(seed)
    tag = torch.ones((B,) + shape, dtype=torch.int32)
    tag[..., -2:] = 0
    tag[:, 0, 0] = 2
    div = torch.where(tag == 1, torch.randn((B,) + shape, generator=g, dtype=torch.float64), 0.0)
    x = torch.where(tag == 1, torch.randn((B,) + shape, generator=g, dtype=torch.float64), 0.0)
    return div, tag, x


def test_conv3d_matches_direct_loop():
    g = torch.Generator().manual_seed(0)
    x = torch.randn((1, 3, 4, 5, 16), generator=g, dtype=torch.float64)
    w = torch.randn((27, 16, 16), generator=g, dtype=torch.float64)
    y = R.conv3d(x, w, relu=False)
    ref = torch.zeros_like(y)
    X, Y, Z = 3, 4, 5
    for i in range(X):
        for j in range(Y):
            for k in range(Z):
                for t in range(27):
                    dx, dy, dz = t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1
                    ii, jj, kk = i + dx, j + dy, k + dz
                    if 0 <= ii < X and 0 <= jj < Y and 0 <= kk < Z:
                        ref[0, i, j, k] += w[t] @ x[0, ii, jj, kk]
    assert torch.allclose(y, ref, rtol=1e-12, atol=1e-12)


def test_gradients_match_finite_differences():
    """Directional derivative of the float64 loss along a random parameter
    direction: autograd vs a central difference."""
    P = _params(1)
    div, tag, x = _scene(2)
    loss, grads, _ = R.loss_and_grads(P, div, tag, x, bf16=False)
    inv = R.unet_input(div, tag)[1]

    def loss_at(Q):
        return float(R.loss_fn(R.forward(Q, div, tag, bf16=False)[0], x, tag, inv, relative=True))

    g = torch.Generator().manual_seed(3)
    for trial in range(3):
        d = {k: torch.randn(v.shape, generator=g, dtype=torch.float64) for k, v in P.items()}
        eps = 1e-6
        fd = (loss_at({k: P[k] + eps * d[k] for k in P}) - loss_at({k: P[k] - eps * d[k] for k in P})) / (2 * eps)
        an = sum(float((grads[k] * d[k]).sum()) for k in P)
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-3), (trial, fd, an)


def test_shape_rules():
    from flub_gb300.unet import UNet3D
    assert UNet3D.check_shape((128, 128, 128))
    assert UNet3D.check_shape((256, 256, 256))
    assert UNet3D.check_shape((8, 32, 64))
    assert not UNet3D.check_shape((32, 32, 32))  # 8^3 level: fewer than 128 cells per (x) plane
    assert not UNet3D.check_shape((30, 32, 64))
