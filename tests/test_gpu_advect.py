"""GPU parity of the advection kernels against the oracle (bit-exact):
_advect_mc_1/2/3 and their fused form, advect_mc, advect_uv_mc, advect_3d,
advect_phi and advect_simple_3d (advect.py:10-138, utils/util.py:20-160)."""
import numpy as np
import pytest
import torch

import oracle as O
from flub_gb300 import (FlubError, _advect_mc_1, _advect_mc_2, _advect_mc_3, advect_3d, advect_mc, advect_phi,
                        advect_simple_3d, advect_uv_mc, launch)
from flub_gb300.fields import Field, MACGrid

pytestmark = pytest.mark.gpu

F = np.float32


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def _vel_np(n, scale, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    return [(scale * rng.standard_normal(s)).astype(F) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz),
                                                                (nx, ny, nz + 1))]


def _mac(arrs):
    return MACGrid(*(Field(dev(a), stagger=O.STAGGER[d + 1], d=d + 1) for d, a in enumerate(arrs)))


def _field_shape(n, d):
    nx, ny, nz = n
    return {0: n, 1: (nx + 1, ny, nz), 2: (nx, ny + 1, nz), 3: (nx, ny, nz + 1)}[d]


# velocity scale: traces of up to ~8 cells at dt = 0.01, h = 1/n, some leaving the grid
CASES = [((16, 16, 16), 20.0), ((24, 12, 40), 12.0), ((64, 16, 64), 30.0), ((7, 5, 9), 6.0)]


@pytest.mark.parametrize("n,scale", CASES)
@pytest.mark.parametrize("d", [0, 1, 2, 3])
def test_advect_mc_fused_bit_exact(n, scale, d):
    vel = _vel_np(n, scale, 100 + d)
    q = np.random.default_rng(d).standard_normal(_field_shape(n, d)).astype(F)
    h = 1.0 / n[0]
    ref = O.advect_mc(*vel, q, O.STAGGER[d], 0.01, h)
    out = torch.zeros(q.shape, device="cuda")
    advect_mc(_mac(vel), Field(dev(q), stagger=O.STAGGER[d], d=d), Field(out, stagger=O.STAGGER[d], d=d))
    assert np.array_equal(host(out), ref)


@pytest.mark.parametrize("n,scale", CASES[:2])
def test_advect_mc_three_stages_bit_exact(n, scale):
    """The reference's three launches, each against the oracle's stage, and
    their result equal to the fused launch."""
    d = 1
    vel = _vel_np(n, scale, 7)
    q = np.random.default_rng(8).standard_normal(_field_shape(n, d)).astype(F)
    h = 1.0 / n[0]
    mac = _mac(vel)
    q_in = Field(dev(q), stagger=O.STAGGER[d], d=d)
    q_out = Field(torch.zeros(q.shape, device="cuda"), stagger=O.STAGGER[d], d=d)
    q_tmp = torch.zeros(q.shape, device="cuda")
    r_out, r_tmp = np.zeros_like(q), np.zeros_like(q)
    for stage, kern in ((1, _advect_mc_1), (2, _advect_mc_2), (3, _advect_mc_3)):
        launch(kern, dim=q.shape, inputs=[mac, q_in, q_out, q_tmp])
        O.advect_mc(*vel, q, O.STAGGER[d], 0.01, h, stage=stage, q_out=r_out, q_tmp=r_tmp)
        assert np.array_equal(host(q_out.f), r_out), stage
        assert np.array_equal(host(q_tmp), r_tmp), stage
    fused = torch.zeros(q.shape, device="cuda")
    advect_mc(mac, q_in, Field(fused, stagger=O.STAGGER[d], d=d))
    assert np.array_equal(host(fused), host(q_out.f))


def test_advect_mc_centred_limiter_bit_exact():
    n = (32, 16, 24)
    vel = _vel_np(n, 10.0, 9)
    q = np.random.default_rng(10).standard_normal(n).astype(F)
    ref = O.advect_mc(*vel, q, O.STAGGER[0], 0.01, 1.0 / 32, minmax_h=1.0)
    out = torch.zeros(n, device="cuda")
    advect_mc(_mac(vel), Field(dev(q)), Field(out), minmax_h=1.0)
    assert np.array_equal(host(out), ref)


@pytest.mark.parametrize("n", [(32, 8, 32), (20, 20, 20)])
def test_advect_uv_mc_and_advect_3d_bit_exact(n):
    vel = _vel_np(n, 15.0, 11)
    q = np.random.default_rng(12).standard_normal(n).astype(F)
    h = 1.0 / n[0]
    ref_vel = O.advect_velocity_mc(*vel, 0.01, h)
    ref_q = O.advect_mc(*vel, q, O.STAGGER[0], 0.01, h)
    out = _mac([np.zeros_like(a) for a in vel])
    advect_uv_mc(_mac(vel), out)
    for a, r in zip((out.u.f, out.v.f, out.w.f), ref_vel):
        assert np.array_equal(host(a), r)
    new_vel = _mac([np.zeros_like(a) for a in vel])
    new_q = Field(torch.zeros(n, device="cuda"))
    advect_3d(_mac(vel), Field(dev(q)), new_vel, new_q)
    assert np.array_equal(host(new_q.f), ref_q)
    for a, r in zip((new_vel.u.f, new_vel.v.f, new_vel.w.f), ref_vel):
        assert np.array_equal(host(a), r)


@pytest.mark.parametrize("n,scale", CASES)
def test_advect_phi_bit_exact(n, scale):
    vel = _vel_np(n, scale, 13)
    phi = np.random.default_rng(14).standard_normal(n).astype(F)
    h = 1.0 / n[0]
    ref = O.advect_phi(*vel, phi, 0.01, h)
    out = torch.zeros(n, device="cuda")
    launch(advect_phi, dim=n, inputs=[_mac(vel), Field(dev(phi)), Field(out)])
    got = host(out)
    assert np.array_equal(got, ref)
    assert (got == F(h)).any() or scale < 10      # some traces leave the grid


@pytest.mark.parametrize("n,scale", CASES)
def test_advect_simple_bit_exact(n, scale):
    vel = _vel_np(n, scale, 15)
    q = np.random.default_rng(16).standard_normal(n).astype(F)
    ref = O.advect_simple(*vel, q, 0.02, 0.05)
    out = torch.zeros(n, device="cuda")
    launch(advect_simple_3d, dim=n, inputs=[*(dev(a) for a in vel), dev(q), out, 0.02, 0.05])
    assert np.array_equal(host(out), ref)


def test_advect_one_cell_grid():
    n = (1, 1, 1)
    vel = _vel_np(n, 50.0, 17)
    q = np.array([[[0.75]]], F)
    ref = O.advect_mc(*vel, q, O.STAGGER[0], 0.01, 1.0)
    out = torch.zeros(n, device="cuda")
    advect_mc(_mac(vel), Field(dev(q)), Field(out))
    assert np.array_equal(host(out), ref)


def test_advect_rejects_aliasing_and_bad_args():
    n = (8, 8, 8)
    vel = _mac(_vel_np(n, 1.0, 18))
    q = Field(torch.zeros(n, device="cuda"))
    with pytest.raises(FlubError):
        advect_mc(vel, q, q)
    with pytest.raises(FlubError):
        advect_uv_mc(vel, vel)
    with pytest.raises(FlubError):
        advect_mc(vel, q, Field(torch.zeros(n, device="cuda")), h0=0.0)


@pytest.mark.parametrize("scale", [1e7, 1e30])
def test_advect_far_outside_and_nan_bit_exact(scale):
    """Traces that leave the grid by millions of cells (or saturate the index
    range), and a NaN velocity component: the same values as the oracle."""
    n = (12, 10, 14)
    vel = _vel_np(n, 1.0, 19)
    vel[0][3, 4, 5] = scale
    vel[1][6, 2, 7] = -scale
    vel[2][5, 5, 5] = np.nan
    q = np.random.default_rng(20).standard_normal(n).astype(F)
    h = 1.0 / 12
    ref = O.advect_mc(*vel, q, O.STAGGER[0], 0.01, h)
    out = torch.zeros(n, device="cuda")
    advect_mc(_mac(vel), Field(dev(q)), Field(out))
    got = host(out)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.array_equal(got[~np.isnan(ref)], ref[~np.isnan(ref)])
    assert np.isnan(ref).any()
