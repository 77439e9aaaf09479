"""The whole projection step on the GPU: the classification of Dh()
(example_fluid.py:96-114 with water_3d.py:55-56), divergence()
(example_fluid.py:84-94), call_mgpcg() (water_3d.py:58-68) and the velocity
update of project() (example_fluid.py:120-147), on persistent device buffers.

The scalings of the reference are kept as FP32 operations: div *= -1/h,
r0 = -h0 * div, p = x * h0 and the update reads p * (1/h0).
"""
import torch

from . import kernels as K
from .fields import Field, IntField, MACGrid
from .mgpcg import MGPCG


class Projection:
    def __init__(self, shape, n_mg_levels, precision="fp32", device=None, h=None, schedule="reference"):
        self.shape = tuple(shape)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.h = float(h) if h is not None else 1.0 / self.shape[0]  # const_param.py:59 h = 1 / gridx
        self.h0 = self.h
        self.mg = MGPCG(3, self.shape, n_mg_levels, float, precision=precision, device=self.device,
                        schedule=schedule)
        mk = lambda dt: torch.empty(self.shape, dtype=dt, device=self.device)
        self.tag = IntField(mk(torch.int32))
        self.div = Field(mk(torch.float32))
        self.p = Field(mk(torch.float32))

    def classify(self, phi, prims):
        K.classify(phi, prims, self.h, self.h0, tag=self.tag)
        return self.tag

    def project(self, vel: MACGrid, vel_rigid: MACGrid, phi=None, prims=(), tag=None, max_iters=200, eps=1e-12,
                abs_tol=0.0, rel_tol=1e-12, smoother="phases", x0=None, warm_start=None, sync=True):
        """Project ``vel`` in place.  Either the level set ``phi`` (+ solid
        primitives) or ready ``tag``s must be given.  ``x0`` (a pressure guess
        in solver units) or ``warm_start`` (a learned.WarmStart) start CG from
        a guess; the tolerance stays relative to the right-hand side.  Returns
        the solve info (sync=True) or None (the work is only enqueued)."""
        if tag is not None:
            self.tag.f.copy_(tag.f if hasattr(tag, "f") else tag)
        else:
            self.classify(phi, prims)
        K.divergence(vel, vel_rigid, self.tag, div=self.div, scale=-1.0 / self.h)
        mg = self.mg
        mg.set_tags(self.tag)
        mg.init(self.div, -self.h0)
        mg.mask_interior()
        if x0 is not None:
            mg.set_initial_guess(x0)
        elif warm_start is not None:
            warm_start.apply(mg)
        mg.solve(max_iters, eps, abs_tol, rel_tol, smoother=smoother, sync=False)
        mg.get_x(self.p.f, self.h0)
        K.subtract_gradient(vel, vel_rigid, self.p, self.tag, p_scale=1.0 / self.h0)
        return mg.info() if sync else None

    def max_abs_div(self, vel, vel_rigid):
        """Post-projection check (example_fluid.py:146-147): max |div u| over fluid cells."""
        d = K.divergence(vel, vel_rigid, self.tag, scale=1.0)
        return float(d.abs().max().item()) if d.numel() else 0.0
