"""The allocation-free V-cycle (flub_vcycle_noalloc), for callers that cannot
allocate device memory themselves -- e.g. a plugin inside a host application
that owns all device memory, or a real-time caller that cannot afford
cudaMalloc.  It keeps its level hierarchy in a fixed 2 MiB device array inside
the library (grids up to 64^3 cells).

Called through the C ABI and compared with the regular path
(flub_mg_set_tags + flub_mg_apply_preconditioner, which uses a workspace),
bit for bit as the other V-cycle parity tests compare, on two calls in a row.
This file is collected last so that a stop-at-first-failure run has already
run every other test."""
import ctypes

import numpy as np
import pytest
import torch

import oracle as O
from flub_gb300 import MGPCG, _lib, scenes

pytestmark = pytest.mark.gpu


def _case(scene):
    tag, _ = O.classify(scene.phi, scene.prims, scene.h, scene.h0)
    div = O.divergence(scene.u, scene.v, scene.w, scene.ur, scene.vr, scene.wr, tag)
    r = np.where(tag == 1, div, 0).astype(np.float32)
    return torch.from_numpy(tag).cuda(), torch.from_numpy(r).cuda()


def _noalloc(tag, r, levels):
    lib = _lib.load()
    z = torch.full_like(r, float("nan"))  # every element must be written
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.flub_vcycle_noalloc(ctypes.c_void_p(tag.data_ptr()), ctypes.c_void_p(r.data_ptr()),
                                 ctypes.c_void_p(z.data_ptr()), *tag.shape, levels, stream)
    _lib.check(st, "flub_vcycle_noalloc")
    torch.cuda.synchronize()
    return z


def _regular(tag, r, levels):
    mg = MGPCG(3, tuple(tag.shape), levels)
    mg.set_tags(tag)
    z = mg.apply_preconditioner(r)
    torch.cuda.synchronize()
    return z


def test_noalloc_vcycle_matches_regular_path_twice():
    # two calls in a row on different scenes and sizes: the second call must not
    # see anything the first one left in the shared array
    for scene in (scenes.dam(64, seed=41, levels=4), scenes.random_scene(32, 42, levels=3)):
        tag, r = _case(scene)
        z_free = _noalloc(tag, r, scene.levels)
        z_ref = _regular(tag, r, scene.levels)
        assert torch.equal(z_free, z_ref)
        assert torch.isfinite(z_free).all()


@pytest.mark.parametrize("no_cluster", ["0", "1"])
def test_noalloc_vcycle_non_cubic_ragged_grid(no_cluster, monkeypatch):
    """A non-cubic grid whose coarse level has nz % 8 != 0 (the scalar sweep and
    restriction kernels), with the thread-block-cluster coarse levels and
    without them (FLUB_NO_CLUSTER=1: global sweeps and the one-block tail)."""
    monkeypatch.setenv("FLUB_NO_CLUSTER", no_cluster)
    shape = (16, 32, 24)
    rng = np.random.default_rng(43)
    phi = (rng.uniform(-1, 1, shape) + 0.4).astype(np.float32)
    tag = O.tag_dirichlet(phi)
    tag[rng.random(shape) < 0.05] = 2
    r = np.where(tag == 1, rng.standard_normal(shape), 0).astype(np.float32)
    tag_d, r_d = torch.from_numpy(tag).cuda(), torch.from_numpy(r).cuda()
    for _ in range(2):
        z_free = _noalloc(tag_d, r_d, 2)
        assert torch.equal(z_free, _regular(tag_d, r_d, 2))
        assert np.array_equal(z_free.cpu().numpy(), O.vcycle(r, O.tag_levels(tag, 2), np.float32))


def test_noalloc_vcycle_rejects_grids_over_the_limit():
    lib = _lib.load()
    shape = (128, 64, 64)  # 524288 cells > 64^3
    tag = torch.ones(shape, dtype=torch.int32, device="cuda")
    r = torch.zeros(shape, device="cuda")
    st = lib.flub_vcycle_noalloc(ctypes.c_void_p(tag.data_ptr()), ctypes.c_void_p(r.data_ptr()),
                                 ctypes.c_void_p(r.data_ptr()), *shape, 4, None)
    assert st == 1
    assert b"allocation-free limit" in lib.flub_last_error()
