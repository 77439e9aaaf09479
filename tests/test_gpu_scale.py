"""The 512^3 dam break (the benchmark scene scaled up, generated on the
device): the light-schedule FP32 and learned + mixed-precision solves
converge, and their pressures agree.  At this size the FP64 host oracle would
take minutes, so the checks are size-independent: the solver's own residual
test, the true residual ||b - L x|| / ||b|| evaluated in FP64 (a gross-error
check only: rounding even the exact solution to FP32 leaves ~1e-3 there,
since ||x|| / ||b|| ~ 1e4 at this size), and the agreement of two differently
computed solutions (FP32 V(2,2) vs FP16 V-cycle with a learned guess)."""
import os

import pytest
import torch

from flub_gb300 import Projection, learned, scenes
from flub_gb300.fields import Field, MACGrid

pytestmark = pytest.mark.gpu

RTOL_PRESSURE = 1e-5


def _shift(a, axis, d, fill):
    """b[idx] = a[idx + d along axis], fill outside the domain."""
    b = torch.full_like(a, fill)
    n = a.shape[axis]
    if d > 0:
        b.narrow(axis, 0, n - 1).copy_(a.narrow(axis, 1, n - 1))
    else:
        b.narrow(axis, 1, n - 1).copy_(a.narrow(axis, 0, n - 1))
    return b


def _lap64(x, tag):
    """The matvec of multigrid/mgpcg.py:118-142 (neighbor_dot_tag) in FP64:
    per fluid cell, the sum over in-domain non-solid neighbours of
    (neighbour value, 0 for air) - own value."""
    out = torch.zeros_like(x)
    for axis in range(3):
        for d in (1, -1):
            nt = _shift(tag, axis, d, 2)
            nx = _shift(x, axis, d, 0.0)
            out += torch.where(nt < 2, torch.where(nt == 0, torch.zeros_like(x), nx) - x, torch.zeros_like(x))
    return torch.where(tag == 1, out, torch.zeros_like(out))


def _true_residual(proj):
    """||b - L x|| / ||b|| in FP64 for the FP32 solution x."""
    mg = proj.mg
    tag = proj.tag.f
    div = proj.div.f
    b = torch.where(tag == 1, div * torch.tensor(-proj.h0, dtype=torch.float32, device=div.device),
                    torch.zeros_like(div)).double()
    res = b - _lap64(mg.x.view(mg.shape).double(), tag)
    return float(res.norm() / b.norm())


def test_dam512_light_and_learned_mixed_agree():
    s = scenes.dam_device(512, 2, "cuda")
    v0 = [a.clone() for a in (s.u, s.v, s.w)]
    vr = MACGrid(*(Field(a, d=d + 1) for d, a in enumerate((s.ur, s.vr, s.wr))))
    out = {}
    for name, prec, use_net in (("plain-v22", "fp32", False), ("learned+mixed-v22", "mixed", True)):
        if use_net and not os.path.exists(learned.WEIGHTS):
            pytest.skip("no trained weights in the tree")
        vel = MACGrid(*(Field(a.clone(), d=d + 1) for d, a in enumerate(v0)))
        proj = Projection(s.shape, s.levels, precision=prec, schedule="v22")
        ws = learned.WarmStart(learned.UNet3D.load(learned.WEIGHTS)) if use_net else None
        info = proj.project(vel, vr, s.phi, s.prims, max_iters=200, eps=1e-12, abs_tol=0.0, rel_tol=1e-12,
                            smoother="phases", warm_start=ws)
        assert info["converged"] and info["rtr"] < 1e-12 * info["rtr0"], (name, info)
        assert _true_residual(proj) < 1e-3, name
        out[name] = proj.p.f.double().clone()
        assert proj.max_abs_div(vel, vr) < 1e-2
        del proj
        torch.cuda.empty_cache()
    a, b = out["plain-v22"], out["learned+mixed-v22"]
    assert float((a - b).norm() / a.norm()) < RTOL_PRESSURE
