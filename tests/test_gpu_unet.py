"""GPU tests of the learned warm start's kernels: the tcgen05 convolution, the
CUDA-core U-Net operations and Adam, each against the float64 CPU reference
(oracle/unet_ref.py), and the whole network's gradients."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

BF16 = torch.bfloat16


def _dev():
    return torch.device("cuda", 0)


def _bf(t):
    return t.to(BF16)


def _rand(shape, gen, scale=1.0):
    return (torch.randn(shape, generator=gen, dtype=torch.float64) * scale)


def _rel(a, b):
    a = a.double().cpu()
    b = b.double().cpu()
    return float((a - b).norm() / max(float(b.norm()), 1e-30))


CONV_CASES = [
    # (B, X, Y, Z, cin0, cin1, cout)
    (1, 4, 8, 16, 16, 0, 16),
    (2, 3, 4, 32, 16, 0, 32),
    (1, 2, 2, 64, 32, 0, 64),
    (1, 2, 1, 128, 64, 0, 64),
    (2, 2, 8, 16, 64, 0, 32),
    (1, 3, 4, 32, 32, 0, 16),
    (1, 2, 8, 16, 64, 0, 16),
    (1, 4, 4, 32, 64, 32, 32),
    (2, 2, 8, 16, 32, 16, 16),
    # NY % 16 == 0 and NZ % 8 == 0: the halo-plane kernel (NZ = 24 only there)
    (1, 5, 16, 8, 16, 0, 16),
    (2, 4, 32, 16, 16, 0, 32),
    (1, 3, 16, 24, 32, 16, 16),
    (1, 6, 16, 16, 64, 32, 32),
    (1, 2, 16, 8, 64, 0, 64),
]


@pytest.mark.parametrize("case", CONV_CASES)
def test_conv3d_matches_float64(case):
    from flub_gb300 import unet as U
    from oracle import unet_ref as R
    B, X, Y, Z, c0, c1, co = case
    g = torch.Generator().manual_seed(hash(case) % 1000)
    x0 = _bf(_rand((B, X, Y, Z, c0), g))
    w0 = _bf(_rand((27, co, c0), g, 1.0 / math.sqrt(27 * c0)))
    x1 = _bf(_rand((B, X, Y, Z, c1), g)) if c1 else None
    w1 = _bf(_rand((27, co, c1), g, 1.0 / math.sqrt(27 * c1))) if c1 else None
    bias = _rand((co,), g, 0.1).float()
    for relu in (False, True):
        U.conv_error(reset=True)
        y = U.conv3d(x0.to(_dev()), w0.to(_dev()), x1.to(_dev()) if c1 else None, w1.to(_dev()) if c1 else None,
                     bias.to(_dev()), relu=relu)
        torch.cuda.synchronize()
        assert U.conv_error() == 0
        ref = R.conv3d(x0.double(), w0.double(), x1.double() if c1 else None, w1.double() if c1 else None,
                       bias.double(), relu=relu)
        err = (y.double().cpu() - ref).abs()
        # FP32 accumulation, BF16 output: a few BF16 ulps of the output scale
        assert float(err.max()) <= 1e-2 * float(ref.abs().max()) + 1e-6, (case, relu, float(err.max()))
        assert _rel(y, ref) <= 4e-3, (case, relu)


@pytest.mark.parametrize("case", [(1, 64, 64, 64, 16, 0, 16), (1, 64, 64, 64, 32, 16, 16), (1, 32, 32, 32, 64, 32, 32),
                                  (2, 32, 32, 32, 16, 0, 32)])
def test_conv3d_halo_planes_at_network_sizes(case, monkeypatch):
    """The U-Net's own layer shapes, where the halo-plane kernel marches up
    to 8 x planes per CTA: against float64 and against the tap-tile kernel
    (FLUB_CONV_HALO=0), which accumulates the same products in another order."""
    from flub_gb300 import unet as U
    from oracle import unet_ref as R
    B, X, Y, Z, c0, c1, co = case
    g = torch.Generator().manual_seed(11)
    x0 = _bf(_rand((B, X, Y, Z, c0), g))
    w0 = _bf(_rand((27, co, c0), g, 1.0 / math.sqrt(27 * c0)))
    x1 = _bf(_rand((B, X, Y, Z, c1), g)) if c1 else None
    w1 = _bf(_rand((27, co, c1), g, 1.0 / math.sqrt(27 * c1))) if c1 else None
    bias = _rand((co,), g, 0.1).float()
    args = (x0.to(_dev()), w0.to(_dev()), x1.to(_dev()) if c1 else None, w1.to(_dev()) if c1 else None,
            bias.to(_dev()))
    U.conv_error(reset=True)
    y = U.conv3d(*args, relu=True)
    monkeypatch.setenv("FLUB_CONV_HALO", "0")
    y_tap = U.conv3d(*args, relu=True)
    monkeypatch.delenv("FLUB_CONV_HALO")
    torch.cuda.synchronize()
    assert U.conv_error() == 0
    ref = R.conv3d(x0.double(), w0.double(), x1.double() if c1 else None, w1.double() if c1 else None,
                   bias.double(), relu=True)
    assert _rel(y, ref) <= 4e-3
    assert float((y.double().cpu() - ref).abs().max()) <= 1e-2 * float(ref.abs().max())
    # the two kernels round the same FP32 sums differently: at most a BF16 ulp or two apart
    d = (y.double() - y_tap.double()).abs()
    assert float(d.max()) <= 2.0 ** -6 * float(y_tap.double().abs().max())


@pytest.mark.parametrize("case", [(1, 4, 8, 16, 16, 16), (2, 2, 4, 32, 32, 64), (1, 2, 2, 64, 64, 32),
                                  (1, 2, 8, 16, 64, 64), (1, 3, 4, 32, 16, 32)])
def test_conv3d_wgrad_matches_float64(case):
    from flub_gb300 import unet as U
    from oracle import unet_ref as R
    B, X, Y, Z, ci, co = case
    g = torch.Generator().manual_seed(7 + ci + co)
    x = _bf(_rand((B, X, Y, Z, ci), g))
    dy = _bf(_rand((B, X, Y, Z, co), g))
    w = torch.zeros((27, co, ci), dtype=torch.float64, requires_grad=True)
    b = torch.zeros(co, dtype=torch.float64, requires_grad=True)
    y = R.conv3d(x.double(), w, bias=b, relu=False)
    (y * dy.double()).sum().backward()
    dw = torch.full((27, co, ci), 0.5, dtype=torch.float32, device=_dev())  # accumulates onto 0.5
    db = torch.full((co,), 0.25, dtype=torch.float32, device=_dev())
    U.conv3d_wgrad(x.to(_dev()), dy.to(_dev()), dw, db)
    torch.cuda.synchronize()
    assert _rel(dw.double().cpu() - 0.5, w.grad) <= 1e-5
    assert _rel(db.double().cpu() - 0.25, b.grad) <= 1e-5


def test_conv3d_data_gradient_is_flipped_transposed_conv():
    from flub_gb300 import unet as U
    from oracle import unet_ref as R
    g = torch.Generator().manual_seed(3)
    B, X, Y, Z, ci, co = 1, 3, 4, 32, 32, 16
    w = _rand((27, co, ci), g, 0.1)
    p = U._Param(w.float().to(_dev()), True)
    dy = _bf(_rand((B, X, Y, Z, co), g))
    xx = torch.zeros((B, X, Y, Z, ci), dtype=torch.float64, requires_grad=True)
    y = R.conv3d(xx, p.w16.double().cpu(), relu=False)
    (y * dy.double()).sum().backward()
    dx = U.conv3d(dy.to(_dev()), p.w16t, relu=False)
    torch.cuda.synchronize()
    assert _rel(dx, xx.grad) <= 4e-3


def test_pool_up_relu_head_ops():
    from flub_gb300 import unet as U
    from oracle import unet_ref as R
    g = torch.Generator().manual_seed(5)
    x = _bf(_rand((2, 4, 6, 8, 32), g))
    xd = x.to(_dev())
    pr = R.pool2(x.double())
    assert float((U.pool2(xd).double().cpu() - pr).abs().max()) <= 2.0 ** -8 * float(pr.abs().max())
    assert torch.equal(U.up2(xd).cpu(), R.up2(x))
    # the 8 children summed in FP32 in (di, dj, dk) order, then / 8, rounded to BF16
    xf, s = x.float(), 0.0
    for d in range(8):
        s = s + xf[:, d >> 2::2, (d >> 1) & 1::2, d & 1::2, :]
    assert torch.equal(U.pool2(xd).cpu(), (s * 0.125).to(BF16))
    # a channel count that is not a multiple of 8 (element-wise kernels)
    x12 = _bf(_rand((1, 4, 6, 2, 12), g))
    assert torch.equal(U.up2(x12.to(_dev())).cpu(), R.up2(x12))
    s12 = 0.0
    for d in range(8):
        s12 = s12 + x12.float()[:, d >> 2::2, (d >> 1) & 1::2, d & 1::2, :]
    assert torch.equal(U.pool2(x12.to(_dev())).cpu(), (s12 * 0.125).to(BF16))
    # gradients
    dyc = _bf(_rand((2, 2, 3, 4, 32), g))
    dx = torch.zeros_like(xd)
    U.pool2_bwd(dyc.to(_dev()), dx, accumulate=False)
    assert torch.equal(dx.cpu(), (R.up2(dyc.double()) / 8).to(BF16))
    U.pool2_bwd(dyc.to(_dev()), dx, accumulate=True)
    assert torch.allclose(dx.double().cpu(), R.up2(dyc.double()) / 4, rtol=1e-2, atol=0)
    dyf = _bf(_rand((2, 4, 6, 8, 32), g))
    s = U.up2_bwd(dyf.to(_dev())).double().cpu()
    ref = R.pool2(dyf.double()) * 8
    assert (s - ref).abs().max() <= 1e-2 * ref.abs().max()
    y = _bf(_rand((2, 4, 6, 8, 32), g)).relu()
    r = U.relu_bwd(dyf.to(_dev()).clone(), y.to(_dev()))
    assert torch.equal(r.cpu(), torch.where(y > 0, dyf, torch.zeros_like(dyf)))
    # head
    x16 = _bf(_rand((2, 4, 6, 8, 16), g))
    w = _rand((16,), g).float()
    b = torch.tensor([0.3])
    out = U.head_fwd(x16.to(_dev()), w.to(_dev()), b.to(_dev()))
    ref = (x16.double() * w.double()).sum(-1) + 0.3
    assert float((out.double().cpu() - ref).abs().max()) <= 1e-5 * float(ref.abs().max())
    dout = _rand((2, 4, 6, 8), g).float()
    dw = torch.zeros(16, device=_dev())
    db = torch.zeros(1, device=_dev())
    dx = U.head_bwd(x16.to(_dev()), w.to(_dev()), dout.to(_dev()), dw, db)
    assert _rel(dw, (dout.double().unsqueeze(-1) * x16.double()).sum((0, 1, 2, 3))) <= 1e-5
    assert abs(float(db) - float(dout.double().sum())) <= 1e-4 * float(dout.double().abs().sum())
    assert _rel(dx, dout.double().unsqueeze(-1) * w.double()) <= 4e-3


def test_input_loss_output():
    from flub_gb300 import unet as U
    from oracle import unet_ref as R
    g = torch.Generator().manual_seed(9)
    shape = (2, 4, 8, 16)
    div = _rand(shape, g).float()
    tag = torch.randint(0, 3, shape, generator=g, dtype=torch.int32)
    tag[1] = 0  # a sample without fluid: inv_scale 1, zero loss
    inp, inv = U.unet_input(div.to(_dev()), tag.to(_dev()))
    rinp, rinv = R.unet_input(div, tag)
    assert torch.allclose(inv.double().cpu(), rinv, rtol=1e-6)
    assert torch.equal(inp.cpu()[..., 1:], rinp[..., 1:].to(BF16))
    assert float((inp.double().cpu()[..., 0] - rinp[..., 0]).abs().max()) <= 2.0 ** -8 * float(rinp[..., 0].abs().max())
    pred = _rand(shape, g).float()
    x = _rand(shape, g).float()
    cnt = int((tag == 1).sum())
    for relative in (False, True):
        dpred, loss = U.unet_loss(pred.to(_dev()), x.to(_dev()), tag.to(_dev()), inv, 1.0 / cnt, relative=relative)
        pr = pred.double().requires_grad_(True)
        lr = R.loss_fn(pr, x, tag, rinv, relative=relative)
        lr.backward()
        assert abs(float(loss) - float(lr.detach())) <= 1e-5 * float(lr.detach())
        assert _rel(dpred, pr.grad) <= 1e-5
    x0 = U.unet_output(pred.to(_dev()), tag.to(_dev()), inv, gain=0.5)
    ref = torch.where(tag == 1, pred.double() / rinv.view(2, 1, 1, 1) * 0.5, 0.0)
    assert _rel(x0, ref) <= 1e-6


def test_adam_matches_reference_formula_and_writes_bf16_copies():
    from flub_gb300 import unet as U
    g = torch.Generator().manual_seed(11)
    w = _rand((27, 32, 16), g, 0.1).float()
    p = U._Param(w.to(_dev()), True)
    m = torch.zeros_like(w, dtype=torch.float64)
    v = torch.zeros_like(w, dtype=torch.float64)
    ref = w.double().clone()
    for step in range(1, 4):
        grad = _rand((27, 32, 16), g, 0.01).float()
        p.g.copy_(grad.to(_dev()))
        U.adam(p.p, p.g, p.m, p.v, step, 1e-3, w16=p.w16, w16t=p.w16t)
        m = 0.9 * m + 0.1 * grad.double()
        v = 0.999 * v + 0.001 * grad.double() ** 2
        ref = ref - 1e-3 * (m / (1 - 0.9 ** step)) / ((v / (1 - 0.999 ** step)).sqrt() + 1e-8)
    torch.cuda.synchronize()
    assert float((p.p.double().cpu() - ref).abs().max()) <= 1e-6
    assert torch.equal(p.w16.cpu(), p.p.cpu().to(BF16))
    assert torch.equal(p.w16t.cpu(), p.p.cpu().flip(0).transpose(1, 2).to(BF16))


def _small_batch(seed, shape=(8, 32, 64), B=2):
    g = torch.Generator().manual_seed(seed)
    tag = torch.ones((B,) + shape, dtype=torch.int32)
    tag[:, :, :, shape[2] // 2:] = 0
    tag[:, 0] = 2
    tag[:, :, :4, :8] = 2
    div = torch.where(tag == 1, _rand((B,) + shape, g), 0.0).float()
    x = torch.where(tag == 1, _rand((B,) + shape, g), 0.0).float()
    return div, tag, x


def test_unet_forward_matches_reference():
    from flub_gb300 import unet as U
    from oracle import unet_ref as R
    net = U.UNet3D(device=_dev(), seed=1)
    div, tag, _ = _small_batch(1)
    out, inv = net.forward(div.to(_dev()), tag.to(_dev()))
    torch.cuda.synchronize()
    assert U.conv_error() == 0
    params = {k: torch.as_tensor(v).double() for k, v in net.state_dict().items()}
    rout, rinv = R.forward(params, div, tag, bf16=True)
    assert torch.allclose(inv.double().cpu(), rinv, rtol=1e-6)
    assert _rel(out, rout) <= 2e-2


def test_unet_gradients_match_reference():
    """Every parameter gradient of the GPU backward pass against float64
    autograd on the CPU (BF16 activations and activation gradients on the GPU
    limit the agreement to about a percent)."""
    from flub_gb300 import unet as U
    from oracle import unet_ref as R
    net = U.UNet3D(device=_dev(), seed=2)
    # a non-trivial head so every layer receives gradient
    div, tag, x = _small_batch(2)
    net.zero_grad()
    loss = net.loss_and_grad(div.to(_dev()), tag.to(_dev()), x.to(_dev()))
    torch.cuda.synchronize()
    assert U.conv_error() == 0
    params = {k: torch.as_tensor(v).double() for k, v in net.state_dict().items()}
    rloss, rgrads, _ = R.loss_and_grads(params, div, tag, x, bf16=True)
    assert abs(float(loss) - rloss) <= 2e-2 * rloss
    for k, v in net.params.items():
        gg = v.g.double().cpu()
        rg = rgrads[k]
        cos = float((gg * rg).sum() / (gg.norm() * rg.norm() + 1e-30))
        assert cos >= 0.98, (k, cos)
        assert _rel(gg, rg) <= 0.1, (k, _rel(gg, rg))


def test_unet_training_reduces_loss():
    from flub_gb300 import unet as U
    net = U.UNet3D(device=_dev(), seed=3)
    div, tag, _ = _small_batch(4)
    # target: a smooth function of the input the network can fit
    x = torch.nn.functional.avg_pool3d(div.unsqueeze(1).double(), 3, 1, 1).squeeze(1).float()
    x = torch.where(tag == 1, x, 0.0)
    d, t, xx = div.to(_dev()), tag.to(_dev()), x.to(_dev())
    losses = []
    for _ in range(30):
        net.zero_grad()
        losses.append(float(net.loss_and_grad(d, t, xx)))
        net.adam_step(lr=1e-3)
    assert losses[-1] < 0.5 * losses[0], losses


def test_learned_pipeline_small():
    """Data generation by the plain solver, a few training steps, and the
    cold/warm evaluation at 64^3: every solve converges to the same tolerance,
    and the scaled guess never starts above the cold residual in energy."""
    from flub_gb300 import learned
    from flub_gb300.unet import UNet3D
    dev = _dev()
    data = learned.generate(6, 64, seed0=123, device=dev)
    assert (data.iters > 0).all()
    net = UNet3D(device=dev, seed=0)
    losses = learned.train(net, data, epochs=4, batch=2, lr=1e-3, seed=0)
    assert len(losses) == 12 and all(math.isfinite(l) for l in losses)
    summary, rows = learned.evaluate(net, data, "fp32")
    assert summary["all_converged"]
    for r in rows:
        assert math.isfinite(r["gamma"])
        assert r["warm"] <= r["cold"] + 2, r
        assert r["err_warm"] <= 1e-3 and r["err_cold"] <= 1e-3, r


def _prolong_ref(xc, tc, tf):
    """Cell-centred trilinear prolongation (tags: 0 air, 1 fluid, 2 solid):
    fine fluid cell 2I + e takes weights 3/4 (cell I) and 1/4 (cell I - 1 for
    e = 0, I + 1 for e = 1) per axis over the coarse cells inside the domain
    that are not solid, renormalised; air contributes 0."""
    out = np.zeros(tf.shape)
    for i, j, k in zip(*np.nonzero(tf == 1)):
        s = w = 0.0
        for a in (0, 1):
            for b in (0, 1):
                for e in (0, 1):
                    ii = i // 2 + (a * (1 if i & 1 else -1))
                    jj = j // 2 + (b * (1 if j & 1 else -1))
                    kk = k // 2 + (e * (1 if k & 1 else -1))
                    if not (0 <= ii < tc.shape[0] and 0 <= jj < tc.shape[1] and 0 <= kk < tc.shape[2]):
                        continue
                    if tc[ii, jj, kk] == 2:
                        continue
                    wt = (0.25 if a else 0.75) * (0.25 if b else 0.75) * (0.25 if e else 0.75)
                    w += wt
                    if tc[ii, jj, kk] == 1:
                        s += wt * xc[ii, jj, kk]
        out[i, j, k] = s / w if w > 0 else 0.0
    return out


def test_warm_start_support_kernels_match_reference_formulas():
    """Level tags, restriction, trilinear prolongation and the device-scaled
    guess against plain float64 restatements on the CPU."""
    from flub_gb300 import MGPCG, scenes
    from flub_gb300 import kernels as K
    from flub_gb300.fields import Field, MACGrid
    from oracle import np_oracle
    sc = scenes.random_scene(32, 7)
    dev = _dev()
    tag = K.classify(torch.as_tensor(sc.phi).to(dev), sc.prims, sc.h, sc.h0)
    tagf = tag.f if hasattr(tag, "f") else tag
    vel = MACGrid(*(Field(torch.as_tensor(a).to(dev), d=d + 1) for d, a in enumerate((sc.u, sc.v, sc.w))))
    velr = MACGrid(*(Field(torch.as_tensor(a).to(dev), d=d + 1) for d, a in enumerate((sc.ur, sc.vr, sc.wr))))
    div = K.divergence(vel, velr, tag, scale=-1.0 / sc.h)
    mg = MGPCG(3, sc.shape, sc.levels, float, device=dev)
    mg.set_tags(tag)
    mg.init(div, -sc.h0)
    mg.mask_interior()
    t0 = tagf.cpu().numpy()
    t1 = mg.level_tags(1).cpu().numpy()
    assert np.array_equal(t1, np_oracle.tag_levels(t0, 2)[1])
    b = mg.r0.view(sc.shape).clone()
    bc = mg.restrict_vector(1, b).cpu().double().numpy()
    ref = b.cpu().double().numpy().reshape(16, 2, 16, 2, 16, 2).sum((1, 3, 5))
    ref[t1 != 1] = 0
    assert np.allclose(bc, ref, rtol=1e-5, atol=1e-6 * np.abs(ref).max())
    # trilinear prolongation of a linear function is exact away from walls
    I = np.arange(16)[:, None, None] + 0 * np.arange(16)[None, :, None] + 0 * np.arange(16)[None, None, :]
    lin = (1.0 + 0.5 * I).astype(np.float32)
    allfluid = MGPCG(3, (32, 32, 32), 3, float, device=dev)
    allfluid.set_tags(torch.ones((32, 32, 32), dtype=torch.int32, device=dev))
    f = allfluid.prolong_vector(1, torch.as_tensor(lin).to(dev)).cpu().numpy()
    i = np.arange(32)
    exact = 1.0 + 0.5 * ((i + 0.5) / 2 - 0.5)
    assert np.allclose(f[1:-1, 5, 5], exact[1:-1], atol=1e-6)
    # with solid, air and fluid cells: the renormalised weights of a float64 restatement
    c1 = np.random.default_rng(8).standard_normal(t1.shape).astype(np.float32)
    got = mg.prolong_vector(1, torch.as_tensor(c1).to(dev)).cpu().double().numpy()
    assert np.allclose(got, _prolong_ref(c1.astype(np.float64), t1, t0), rtol=0, atol=1e-6 * np.abs(c1).max())
    # scaled guess: gamma = (d . b) / (d . L d)
    g = torch.Generator(device=dev).manual_seed(1)
    d = torch.randn(sc.shape, generator=g, device=dev) * (tagf == 1)
    mg.set_initial_guess_scaled(d)
    info = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    dn = d.cpu().double().numpy()
    gamma = float((dn * b.cpu().double().numpy()).sum() / (dn * np_oracle.matvec(dn, t0)).sum())
    assert abs(info["x0_scale"] - gamma) <= 1e-5 * abs(gamma)
    assert info["converged"]


def test_trained_network_saves_iterations():
    """The committed network against the method without it on held-out 128^3
    scenes (seeds outside the training range): every solve reaches the same
    tolerance, and the warm start needs fewer CG iterations on average."""
    import os
    from flub_gb300 import learned
    from flub_gb300.unet import UNet3D
    if not os.path.exists(learned.WEIGHTS):
        pytest.skip("no trained weights in the tree")
    dev = _dev()
    net = UNet3D.load(learned.WEIGHTS, device=dev)
    data = learned.generate(6, 128, seed0=950000, device=dev)
    summary, rows = learned.evaluate(net, data, "fp32")
    assert summary["all_converged"]
    assert summary["saved_mean"] >= 0.5, summary
    for r in rows:
        assert r["warm"] <= r["cold"], r
        assert r["err_warm"] <= 1e-5, r
        assert r["err_net"] < 0.5, r


def test_warm_start_graph_equals_eager():
    """The captured-graph guess is the eager guess, bit for bit, and a warm
    solve through it converges to the same tolerance."""
    from flub_gb300 import Projection, learned
    from flub_gb300.unet import UNet3D
    from flub_gb300.fields import Field, MACGrid
    from flub_gb300 import scenes
    dev = _dev()
    net = UNet3D(device=dev, seed=5)
    sc = scenes.dam(128, 2)
    d_ = lambda a: torch.as_tensor(a).to(dev)
    outs = {}
    for graph in (False, True):
        proj = Projection(sc.shape, sc.levels, precision="mixed", schedule="v22")
        vel = MACGrid(*(Field(d_(a), d=i + 1) for i, a in enumerate((sc.u, sc.v, sc.w))))
        velr = MACGrid(*(Field(d_(a), d=i + 1) for i, a in enumerate((sc.ur, sc.vr, sc.wr))))
        ws = learned.WarmStart(net, graph=graph)
        info = proj.project(vel, velr, d_(sc.phi), sc.prims, warm_start=ws)
        # a second projection of the original velocities (a graph replay on new inputs)
        vel = MACGrid(*(Field(d_(a), d=i + 1) for i, a in enumerate((sc.u, sc.v, sc.w))))
        info2 = proj.project(vel, velr, d_(sc.phi), sc.prims, warm_start=ws)
        assert info["converged"] and info2["converged"]
        outs[graph] = (info["x0_scale"], info2["x0_scale"], proj.p.f.cpu())
    assert outs[False][0] == outs[True][0] and outs[False][1] == outs[True][1]
    assert torch.equal(outs[False][2], outs[True][2])
