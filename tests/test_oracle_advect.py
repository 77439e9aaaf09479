"""The advection oracle (oracle/flub_oracle.c) pinned by known answers and by
an independent NumPy restatement (oracle/np_advect.py): advect.py:10-138,
utils/util.py:20-160.  CPU only."""
import numpy as np
import pytest

import oracle as O
from oracle import np_advect as NA

F = np.float32


def _vel(n, scale, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    return tuple((scale * rng.standard_normal(s)).astype(F) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz),
                                                                    (nx, ny, nz + 1)))


def _uniform(n, U):
    nx, ny, nz = n
    return (np.full((nx + 1, ny, nz), U[0], F), np.full((nx, ny + 1, nz), U[1], F), np.full((nx, ny, nz + 1), U[2], F))


def test_sample_velocity_reproduces_linear_fields():
    n = (10, 12, 14)
    nx, ny, nz = n
    # u(x, y, z) = 0.1 + 0.2 x - 0.3 y + 0.05 z at face positions (i, j+0.5, k+0.5), and so on
    def lin(shape, off, c):
        i, j, k = np.meshgrid(*(np.arange(s, dtype=np.float64) for s in shape), indexing="ij")
        return (c[0] + c[1] * (i + off[0]) + c[2] * (j + off[1]) + c[3] * (k + off[2])).astype(F)
    cu, cv, cw = (0.1, 0.2, -0.3, 0.05), (-0.2, 0.01, 0.1, 0.3), (0.5, -0.1, 0.02, -0.04)
    u = lin((nx + 1, ny, nz), (0, 0.5, 0.5), cu)
    v = lin((nx, ny + 1, nz), (0.5, 0, 0.5), cv)
    w = lin((nx, ny, nz + 1), (0.5, 0.5, 0), cw)
    for p in [(3.3, 4.7, 5.1), (5.0, 6.5, 7.25), (1.9, 2.2, 8.8)]:
        got = O.sample_velocity(u, v, w, p)
        want = [c[0] + c[1] * p[0] + c[2] * p[1] + c[3] * p[2] for c in (cu, cv, cw)]
        np.testing.assert_allclose(got, want, rtol=0, atol=2e-6)


def test_backtrace_of_a_uniform_field_is_a_shift():
    n = (16, 16, 16)
    U = (1.5, -0.75, 0.25)
    u, v, w = _uniform(n, U)
    dt, h = 0.01, 1.0 / 16
    p = O.backtrace(u, v, w, (8.0, 8.5, 8.5), dt, h)
    np.testing.assert_allclose(p, [8.0 - dt / h * U[0], 8.5 - dt / h * U[1], 8.5 - dt / h * U[2]], atol=2e-6)


def test_backtrace_rk3_order_on_a_rotation():
    """Solid rotation about the centre: the RK3 trace lands on the circle;
    the error falls by about 2^3 or more when dt halves."""
    n = 48
    c = n / 2
    om = 1.0
    i, j, k = np.meshgrid(*(np.arange(s, dtype=np.float64) for s in (n + 1, n, n)), indexing="ij")
    u = (-om * ((j + 0.5) - c)).astype(F)          # u = -omega (y - c), grid units per unit time
    i, j, k = np.meshgrid(*(np.arange(s, dtype=np.float64) for s in (n, n + 1, n)), indexing="ij")
    v = (om * ((i + 0.5) - c)).astype(F)
    w = np.zeros((n, n, n + 1), F)
    p0 = np.array([c + 10.0, c, c], np.float64)
    errs = []
    for dt in (0.2, 0.1):
        p = O.backtrace(u, v, w, p0, dt, 1.0)       # h = 1: velocity already in grid units
        ang = -om * dt
        exact = [c + 10.0 * np.cos(ang), c + 10.0 * np.sin(ang), c]
        errs.append(np.abs(p - exact).max())
    assert errs[0] < 2e-3 and errs[1] < errs[0] / 6.0, errs


def test_tricubic_reproduces_cubic_polynomials():
    q_shape = (12, 11, 13)
    i, j, k = np.meshgrid(*(np.arange(s, dtype=np.float64) for s in q_shape), indexing="ij")
    f = lambda x, y, z: 0.5 + 0.01 * x ** 3 - 0.02 * y ** 2 * z + 0.03 * z ** 3 - 0.1 * x * y
    q = f(i, j, k).astype(F)
    for s, t, r in [(5.3, 4.7, 6.1), (2.0, 3.5, 7.9), (8.25, 6.75, 4.5)]:
        assert O.tricubic(q, s, t, r) == pytest.approx(f(s, t, r), abs=2e-4)


def test_tricubic_interpolates_at_nodes():
    q = np.random.default_rng(3).standard_normal((9, 8, 7)).astype(F)
    for ijk in [(3, 4, 2), (1, 1, 1), (0, 0, 0), (8, 7, 6)]:
        assert O.tricubic(q, *map(float, ijk)) == q[ijk]


@pytest.mark.parametrize("stage", [0, 1, 2, 3])
def test_advect_mc_keeps_a_constant_field(stage):
    n = (10, 9, 11)
    u, v, w = _vel(n, 3.0, 1)
    q = np.full((11, 9, 11), 0.625, F)
    q_out = np.full_like(q, 0.625)
    q_tmp = np.full_like(q, 0.625)
    out = O.advect_mc(u, v, w, q, O.STAGGER[1], 0.01, 1.0 / 10, stage=stage, q_out=q_out, q_tmp=q_tmp)
    # the cubic weights of utils/util.py:122-129 sum to 1 only up to FP32 rounding
    np.testing.assert_allclose(out, 0.625, rtol=0, atol=4 * np.spacing(F(0.625)))


def test_advect_mc_limiter_reads_the_far_corner():
    """sample_minmax divides the (grid-unit) position by h0 again, so for feet
    at >= 1 cell from the origin its 8 values are the clamped far corner, whose
    min and max are equal: the MacCormack value is always replaced by the
    semi-Lagrangian one there.  With minmax_h = 1 the bounds come from the
    cell around the foot and the correction survives where it is in bounds."""
    n = (12, 12, 12)
    u, v, w = _vel(n, 2.0, 4)
    rng = np.random.default_rng(5)
    q = rng.standard_normal((12, 12, 12)).astype(F)
    h = 1.0 / 12
    sl = O.advect_mc(u, v, w, q, O.STAGGER[0], 0.01, h, stage=1)
    mc = O.advect_mc(u, v, w, q, O.STAGGER[0], 0.01, h)
    p = NA._grid_points(q.shape, O.STAGGER[0])
    foot = NA.backtrace(u, v, w, p, 0.01, h)
    far = (foot[0] >= 1) & (foot[1] >= 1) & (foot[2] >= 1)
    assert far.sum() > 1000
    assert np.array_equal(mc[far], sl[far])
    mc1 = O.advect_mc(u, v, w, q, O.STAGGER[0], 0.01, h, minmax_h=1.0)
    changed = mc1 != sl
    assert changed.mean() > 0.2
    lo, hi = NA.sample_minmax(q, foot, 1.0, O.STAGGER[0])
    assert ((mc1[changed] > lo[changed]) & (mc1[changed] < hi[changed])).all()


def test_advect_phi_outside_is_h0():
    n = (8, 8, 8)
    u, v, w = _uniform(n, (-40.0, 0.0, 0.0))       # traces leave through x = nx
    phi = np.random.default_rng(6).standard_normal(n).astype(F)
    h = 1.0 / 8
    out = O.advect_phi(u, v, w, phi, 0.01, h)
    # foot x = i + 0.5 + 0.01 * 40 / h = i + 3.7: outside for i >= 5
    assert (out[5:] == F(h)).all()
    assert not (out[:4] == F(h)).any()


@pytest.mark.parametrize("d", [0, 1, 2, 3])
def test_c_oracle_matches_numpy_mc(d):
    n = (9, 7, 11)
    u, v, w = _vel(n, 4.0, 10 + d)
    shape = {0: n, 1: (10, 7, 11), 2: (9, 8, 11), 3: (9, 7, 12)}[d]
    q = np.random.default_rng(20 + d).standard_normal(shape).astype(F)
    for mh in (None, 1.0):
        c = O.advect_mc(u, v, w, q, O.STAGGER[d], 0.01, 1.0 / 9, minmax_h=mh)
        py = NA.advect_mc(u, v, w, q, O.STAGGER[d], 0.01, 1.0 / 9, minmax_h=mh)
        assert np.array_equal(c, py)


def test_c_oracle_matches_numpy_phi_and_simple():
    n = (10, 8, 9)
    u, v, w = _vel(n, 6.0, 30)
    q = np.random.default_rng(31).standard_normal(n).astype(F)
    assert np.array_equal(O.advect_phi(u, v, w, q, 0.01, 0.1), NA.advect_phi(u, v, w, q, 0.01, 0.1))
    assert np.array_equal(O.advect_simple(u, v, w, q, 0.01, 0.1), NA.advect_simple(u, v, w, q, 0.01, 0.1))


def test_advect_simple_shifts_linear_fields():
    """A uniform velocity carries a linear field exactly (interior cells)."""
    n = (12, 12, 12)
    U = (0.5, 0.25, -0.5)
    u, v, w = _uniform(n, U)
    i, j, k = np.meshgrid(*(np.arange(s, dtype=np.float64) for s in n), indexing="ij")
    lin = lambda x, y, z: 1.0 + 0.3 * x - 0.2 * y + 0.1 * z
    q = lin(i + 0.5, j + 0.5, k + 0.5).astype(F)
    h, dt = 1.0 / 12, 0.05
    out = O.advect_simple(u, v, w, q, dt, h)
    s = dt / h
    want = lin(i + 0.5 - s * U[0], j + 0.5 - s * U[1], k + 0.5 - s * U[2])
    np.testing.assert_allclose(out[2:-2, 2:-2, 2:-2], want[2:-2, 2:-2, 2:-2], atol=2e-5)


def test_c_oracle_matches_numpy_far_outside_and_nan():
    n = (8, 9, 10)
    u, v, w = _vel(n, 1.0, 40)
    u[3, 4, 5] = 1e30
    v[2, 2, 2] = -1e7
    w[4, 4, 4] = np.nan
    q = np.random.default_rng(41).standard_normal(n).astype(F)
    c = O.advect_mc(u, v, w, q, O.STAGGER[0], 0.01, 1.0 / 8)
    py = NA.advect_mc(u, v, w, q, O.STAGGER[0], 0.01, 1.0 / 8)
    assert np.array_equal(np.isnan(c), np.isnan(py)) and np.isnan(c).any()
    assert np.array_equal(c[~np.isnan(c)], py[~np.isnan(py)])
