"""GPU parity of the velocity extrapolation (extrapolate.py, utils/util.py
set_unknown, water_3d.py extrapolate) against the oracle: bit-exact values
and flags, through the reference's launch form and the fused call."""
import numpy as np
import pytest
import torch

import oracle as O
from flub_gb300 import (Projection, extrapolate, extrapolate_3d, flush_1_3d, launch, scenes, set_unknown,
                        set_unknown_3d)
from flub_gb300.fields import Field, IntField, MACGrid, MACGridInt

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def _mac(u, v, w):
    return MACGrid(Field(dev(u), d=1), Field(dev(v), d=2), Field(dev(w), d=3))


def _macint(tu, tv, tw):
    return MACGridInt(IntField(dev(tu), d=1), IntField(dev(tv), d=2), IntField(dev(tw), d=3))


def _projected(scene):
    """Velocities after a projection (the input extrapolation sees in water_3d.step)."""
    proj = Projection(scene.shape, scene.levels)
    vel, velr = _mac(scene.u, scene.v, scene.w), _mac(scene.ur, scene.vr, scene.wr)
    proj.project(vel, velr, dev(scene.phi), scene.prims)
    return [host(a) for a in (vel.u.f, vel.v.f, vel.w.f)]


SCENES = {
    "dam64": lambda: scenes.dam(64, seed=4, levels=4),
    "rand32": lambda: scenes.random_scene(32, 31, levels=3),
    "sphere32": lambda: scenes.sphere(32, seed=5, levels=3),
}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_set_unknown_bit_exact(name):
    s = SCENES[name]()
    rng = np.random.default_rng(1)
    # the last face layer keeps whatever flags it had
    flags = [rng.integers(-1, 2, size=f.shape).astype(np.int32) for f in (s.u, s.v, s.w)]
    ref = [f.copy() for f in flags]
    O.set_unknown(s.phi, *ref)
    tags = _macint(*flags)
    launch(set_unknown_3d, dim=s.shape, inputs=[Field(dev(s.phi)), tags])
    for a, b in zip((tags.u.f, tags.v.f, tags.w.f), ref):
        assert np.array_equal(host(a), b)


@pytest.mark.parametrize("name", sorted(SCENES))
def test_extrapolate_by_1_launch_form_bit_exact(name):
    """wp.launch(extrapolate_3d, dim=shapeu, inputs=[vel, tag, 1]) ... and
    flush_1_3d, as extrapolate.py:39-47 calls them."""
    s = SCENES[name]()
    faces = _projected(s)
    flags = [np.zeros(f.shape, np.int32) for f in faces]
    O.set_unknown(s.phi, *flags)
    ref = [f.copy() for f in faces]
    rflags = [f.copy() for f in flags]
    for q, t in zip(ref, rflags):
        O.extrapolate_axis(q, t)
    vel, tags = _mac(*faces), _macint(*flags)
    for d, f in enumerate((vel.u.f, vel.v.f, vel.w.f)):
        launch(extrapolate_3d, dim=tuple(f.shape), inputs=[vel, tags, d + 1])
    for a, b in zip((vel.u.f, vel.v.f, vel.w.f), ref):
        assert np.array_equal(host(a), b)
    for a, b in zip((tags.u.f, tags.v.f, tags.w.f), rflags):
        assert np.array_equal(host(a), b)  # extrapolated faces carry -1 before the flush
    for t, r in zip((tags.u, tags.v, tags.w), rflags):
        launch(flush_1_3d, dim=tuple(t.f.shape), inputs=[t])
        O.flush_unknown(r)
        assert np.array_equal(host(t.f), r)


@pytest.mark.parametrize("name", sorted(SCENES))
def test_fused_extrapolation_bit_exact(name):
    """water_3d.py:70-73 with n_cells = 16 * res / 128 passes (at least 2)."""
    s = SCENES[name]()
    n_cells = max(2, 16 * s.shape[0] // 128)
    faces = _projected(s)
    flags = [np.zeros(f.shape, np.int32) for f in faces]
    ref = [f.copy() for f in faces]
    rflags = [f.copy() for f in flags]
    O.extrapolate(*ref, *rflags, s.phi, n_cells)
    vel, tags = _mac(*faces), _macint(*flags)
    extrapolate(vel, tags, Field(dev(s.phi)), n_cells)
    for a, b in zip((vel.u.f, vel.v.f, vel.w.f), ref):
        assert np.array_equal(host(a), b)
    for a, b in zip((tags.u.f, tags.v.f, tags.w.f), rflags):
        assert np.array_equal(host(a), b)
    # something was extrapolated and something was zeroed
    changed = sum(int((host(a) != f).sum()) for a, f in zip((vel.u.f, vel.v.f, vel.w.f), faces))
    assert changed > 0


def test_extrapolation_rejects_bad_arguments():
    from flub_gb300 import FlubError
    from flub_gb300 import _lib
    with pytest.raises(FlubError):
        _lib.call("flub_extrapolate_axis", None, None, 4, 4, 4, 1, None)
    with pytest.raises(FlubError):
        _lib.call("flub_extrapolate", *([None] * 7), 4, 4, 4, -1, None)
