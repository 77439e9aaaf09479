"""The CUDA path of the widening rows against fixtures computed by the
reference's own kernels (tests/golden/refw_*.npz, made by
tests/golden/make_ref_widen.py): bit for bit, on the fixtures' inputs, with
the reference's constants (dt = 0.01, h0 = 1/256)."""
import numpy as np
import pytest
import torch

from flub_gb300 import kernels as K
from flub_gb300 import (divergence_fractional_3d, launch, phi_to_fraction_3d, precompute_solid_vel,
                        u_subtract_gradient_batty_3d, v_subtract_gradient_batty_3d, w_subtract_gradient_batty_3d)
from flub_gb300.fields import Field, IntField, MACGrid, MACGridInt
from tests.golden import make_ref_widen as W

pytestmark = pytest.mark.gpu

STAGGER = {0: (0.5, 0.5, 0.5), 1: (0.0, 0.5, 0.5), 2: (0.5, 0.0, 0.5), 3: (0.5, 0.5, 0.0)}


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def _mac(arrs):
    return MACGrid(*(Field(dev(a), stagger=STAGGER[d + 1], d=d + 1) for d, a in enumerate(arrs)))


def _eq(t, ref):
    got = host(t)
    return got.shape == ref.shape and got.dtype == ref.dtype and np.array_equal(got, ref)


def test_advection_matches_reference():
    f = W.load("adv")
    dt, h0 = float(f["dt"]), float(f["h0"])
    vel = _mac([f["u"], f["v"], f["w"]])
    new_phi = torch.zeros(f["phi"].shape, device="cuda")
    K.advect_phi_field(vel, Field(dev(f["phi"])), Field(new_phi), dt, h0)
    assert _eq(new_phi, f["advect_phi"])
    out = _mac([np.zeros_like(f[k]) for k in "uvw"])
    K.advect_uv_mc(vel, out, dt, h0, h0)
    for k, a in zip("uvw", (out.u.f, out.v.f, out.w.f)):
        assert _eq(a, f["advect_mc_" + k]), k
    qn = torch.zeros(f["q"].shape, device="cuda")
    K.advect_simple(vel.u.f, vel.v.f, vel.w.f, dev(f["q"]), qn, dt, h0)
    assert _eq(qn, f["advect_simple"])


def test_extrapolation_matches_reference():
    f = W.load("ext")
    vel = _mac([f[k] for k in "uvw"])
    tags = MACGridInt(*(IntField(dev(f[k]), d=d + 1) for d, k in enumerate(("tu", "tv", "tw"))))
    K.extrapolate(vel, tags, Field(dev(f["phi"])), int(f["n_cells"]))
    for k, a, t in zip("uvw", (vel.u.f, vel.v.f, vel.w.f), (tags.u.f, tags.v.f, tags.w.f)):
        assert _eq(a, f["ext_" + k]), k
        assert _eq(t, f["ext_t" + k]), k


@pytest.mark.parametrize("sb", [1, 0])
def test_redistance_matches_reference(sb):
    f = W.load("red")
    h0 = float(f["h0"])
    out = torch.empty(f["phi"].shape, device="cuda")
    K.init_distance(dev(f["phi"]), h0, sb, out=out)
    assert _eq(out, f[f"init_sb{sb}"])
    g = dev(f["phi"])
    K.redistance(g, h0, sb, 2)
    assert _eq(g, f[f"redistance_sb{sb}"])


def test_cut_cells_match_reference():
    f = W.load("cut")
    shape = tuple(int(a) for a in f["shape"])
    nx = shape[0]
    frac = _mac([f["fc_" + k] for k in "uvw"])
    for d, k, t in zip((1, 2, 3), "uvw", (frac.u.f, frac.v.f, frac.w.f)):
        launch(phi_to_fraction_3d, dim=tuple(t.shape), inputs=[Field(dev(f["phin"])), frac, d])
        assert _eq(t, f["frac_" + k]), k
    div = torch.empty(shape, device="cuda")
    launch(divergence_fractional_3d, dim=shape,
           inputs=[*(dev(f[k]) for k in "uvw"), div, *(dev(f["frac_" + k]) for k in "uvw"),
                   *(dev(f[k + "r"]) for k in "uvw")])
    assert _eq(div, f["div_frac"])
    kern = (u_subtract_gradient_batty_3d, v_subtract_gradient_batty_3d, w_subtract_gradient_batty_3d)
    for d, k in zip((1, 2, 3), "uvw"):
        ug = dev(f[k])
        launch(kern[d - 1], dim=tuple(ug.shape),
               inputs=[ug, dev(f["p"]), dev(f["frac_" + k]), dev(f["phic"]), dev(f[k + "r"]), 0.0, 1.0, 1.0 / nx])
        assert _eq(ug, f["batty_" + k]), k
    vel_rigid = _mac([np.full(f["solid_" + k].shape, 9.0, np.float32) for k in "uvw"])
    vel_owner = MACGridInt(*(IntField(dev(f["own_" + k]), d=d + 1) for d, k in enumerate("uvw")))
    for d, k, t in zip((1, 2, 3), "uvw", (vel_rigid.u.f, vel_rigid.v.f, vel_rigid.w.f)):
        K.solid_vel(vel_rigid, vel_owner, d, f["bx"], f["bv"], f["bw"], h0=float(f["h0"]))
        assert _eq(t, f["solid_" + k]), k
