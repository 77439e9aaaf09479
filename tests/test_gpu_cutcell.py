"""GPU parity of the rigid-coupling producers and the cut-cell projection
variants against the oracle (bit-exact): precompute_solid_vel
(rigid_coupling.py:51-70), phi_to_fraction + fraction_quad (geometry.py,
utils/util.py), divergence_fractional_3d (divergence.py:4-42) and
u/v/w_subtract_gradient_batty_3d (subtract_gradient.py:7-122)."""
import numpy as np
import pytest
import torch

import oracle as O
from flub_gb300 import (divergence_fractional_3d, launch, phi_prims, phi_to_fraction_3d, precompute_solid_vel,
                        scenes, u_subtract_gradient_batty_3d, v_subtract_gradient_batty_3d,
                        w_subtract_gradient_batty_3d)
from flub_gb300.fields import Field, IntField, MACGrid, MACGridInt

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def _shapes(n):
    return [(n + 1, n, n), (n, n + 1, n), (n, n, n + 1)]


def _bodies():
    x = np.array([[0.6, 0.3, 0.45], [0.3, 0.6, 0.5]], np.float32)
    v = np.array([[0.2, -0.5, 0.1], [0.0, 0.3, -0.2]], np.float32)
    w = np.array([[0.0, 1.5, -0.7], [2.0, 0.0, 0.4]], np.float32)
    return x, v, w


@pytest.mark.parametrize("n", [16, 40])
def test_solid_vel_bit_exact(n):
    rng = np.random.default_rng(n)
    bx, bv, bw = _bodies()
    owners = [rng.integers(-1, 3, size=s).astype(np.int32) for s in _shapes(n)]  # includes an out-of-range owner 2
    vel_rigid = MACGrid(*(Field(torch.zeros(s, device="cuda"), d=d + 1) for d, s in enumerate(_shapes(n))))
    vel_owner = MACGridInt(*(IntField(dev(o), d=d + 1) for d, o in enumerate(owners)))
    for d in (1, 2, 3):
        f = (vel_rigid.u, vel_rigid.v, vel_rigid.w)[d - 1].f
        launch(precompute_solid_vel, dim=tuple(f.shape), inputs=[bx, bv, bw, vel_rigid, vel_owner, d])
        ref = np.zeros(_shapes(n)[d - 1], np.float32)
        O.solid_vel(ref, owners[d - 1], d, 1.0 / n, bx, bv, bw)
        assert np.array_equal(host(f), ref), d


def _face_sdf(n, prims):
    """Face-centre and node SDF of the primitives (the inputs phi_to_fraction reads)."""
    h = 1.0 / n
    nodes = torch.empty((n + 1, n + 1, n + 1), device="cuda")
    phi_prims(nodes, prims, h, h, (0.0, 0.0, 0.0))
    faces = []
    for d, s in enumerate(_shapes(n)):
        f = torch.empty(s, device="cuda")
        st = [0.5, 0.5, 0.5]
        st[d] = 0.0
        phi_prims(f, prims, h, h, tuple(st))
        faces.append(f)
    return nodes, faces


@pytest.mark.parametrize("name", ["dam64", "rand48"])
def test_phi_to_fraction_bit_exact(name):
    s = {"dam64": lambda: scenes.dam(64, 2), "rand48": lambda: scenes.random_scene(48, 9)}[name]()
    n = s.shape[0]
    nodes, faces = _face_sdf(n, s.prims)
    ref_in = [host(f).copy() for f in faces]
    frac = MACGrid(*(Field(f, d=d + 1) for d, f in enumerate(faces)))
    nodes_h = host(nodes)
    for d in (1, 2, 3):
        launch(phi_to_fraction_3d, dim=tuple(faces[d - 1].shape), inputs=[Field(nodes), frac, d])
        ref = O.phi_to_fraction(nodes_h, ref_in[d - 1], d)
        out = host(faces[d - 1])
        assert np.array_equal(out, ref), d
        assert ((out == 0.0) | ((out >= 0.1) & (out <= 1.0))).all()


@pytest.mark.parametrize("n", [24, 64])
def test_divergence_fractional_bit_exact(n):
    rng = np.random.default_rng(n + 1)
    vel = [rng.standard_normal(s).astype(np.float32) for s in _shapes(n)]
    frac = [np.where(rng.random(s) < 0.3, rng.random(s), 1.0).astype(np.float32) for s in _shapes(n)]
    rig = [rng.standard_normal(s).astype(np.float32) for s in _shapes(n)]
    ref = O.divergence_fractional(*vel, *frac, *rig)
    div = torch.empty((n, n, n), device="cuda")
    launch(divergence_fractional_3d, dim=(n, n, n), inputs=[*(dev(a) for a in vel), div, *(dev(a) for a in frac),
                                                             *(dev(a) for a in rig)])
    assert np.array_equal(host(div), ref)


@pytest.mark.parametrize("lo", [0.0, 0.25])
def test_subtract_gradient_batty_bit_exact(lo):
    n = 32
    rng = np.random.default_rng(5)
    s = scenes.dam(n, 3)
    phi = s.phi
    p = rng.standard_normal((n, n, n)).astype(np.float32)
    kernels = (u_subtract_gradient_batty_3d, v_subtract_gradient_batty_3d, w_subtract_gradient_batty_3d)
    for d, sh in enumerate(_shapes(n), start=1):
        uf = rng.standard_normal(sh).astype(np.float32)
        fr = np.where(rng.random(sh) < 0.1, 0.0, rng.random(sh)).astype(np.float32)
        ur = rng.standard_normal(sh).astype(np.float32)
        ref = uf.copy()
        O.subtract_gradient_batty(ref, p, fr, phi, ur, d, lo, 1.0 / n)
        ug = dev(uf)
        launch(kernels[d - 1], dim=sh, inputs=[ug, dev(p), dev(fr), dev(phi), dev(ur), lo, 1.0, 1.0 / n])
        assert np.array_equal(host(ug), ref), d
