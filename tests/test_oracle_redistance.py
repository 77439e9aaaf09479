"""The redistance oracle (oracle/flub_oracle.c) pinned by known answers and by
an independent NumPy restatement (oracle/np_redistance.py):
redistance.py:7-136, utils/util.py:403-412.  CPU only."""
import numpy as np
import pytest

import oracle as O
from oracle import np_redistance as NR

F = np.float32


def _sphere(n, c, R, h, warp=0.5, noise=0.0, seed=0):
    i, j, k = np.meshgrid(*(np.arange(s) + 0.5 for s in n), indexing="ij")
    r = np.sqrt((i - c[0]) ** 2 + (j - c[1]) ** 2 + (k - c[2]) ** 2)
    true = (r - R) * h
    phi = true * (1 + warp * np.sin(i / 3.0))
    if noise:
        phi = phi + noise * h * np.random.default_rng(seed).standard_normal(n)
    return phi.astype(F), true


@pytest.mark.parametrize("n", [(14, 12, 16), (9, 11, 7)])
@pytest.mark.parametrize("set_boundary", [0, 1])
def test_c_oracle_matches_numpy(n, set_boundary):
    h = 1.0 / n[0]
    phi, _ = _sphere(n, (n[0] / 2 - 0.7, n[1] / 2 + 0.2, n[2] / 2 - 0.3), min(n) / 3.2, h, noise=0.05)
    assert np.array_equal(O.redistance_init(phi, h, set_boundary), NR.init_distance(phi, h, set_boundary))
    a = O.redistance_init(phi, h, set_boundary)
    b = a.copy()
    for d in O.REDISTANCE_DIRECTIONS:
        for odd in (0, 1):
            O.redistance_sweep(a, *d, odd, h)
            NR.sweep(b, *d, odd, h)
            assert np.array_equal(a, b), (d, odd)
    assert np.array_equal(O.redistance(phi, h, set_boundary), NR.redistance(phi, h, set_boundary))


def test_init_distance_kat():
    """A cell at +0.5 h next to one at -1.5 h: the zero crossing is a quarter
    of a cell away, so the cell gets 0.25 h; the negative one gets -0.75 h;
    cells with no sign change next to them get +-2."""
    h = 0.1
    phi = np.full((7, 5, 5), 3 * h, F)
    phi[:3] = -1.5 * h
    phi[3] = 0.5 * h
    out = O.redistance_init(phi, h, 1)
    assert out[3, 2, 2] == pytest.approx(0.25 * h, abs=1e-7)
    assert out[2, 2, 2] == pytest.approx(-0.75 * h, abs=1e-7)
    assert out[5, 2, 2] == F(2.0)
    assert out[1, 2, 2] == F(-2.0)
    # set_boundary = 0 leaves the boundary layer alone
    out0 = O.redistance_init(phi, h, 0)
    assert np.array_equal(out0[0], phi[0]) and np.array_equal(out0[:, :, -1], phi[:, :, -1])


def test_plane_positive_side_is_exact():
    """phi = 3 (x - x0): the positive side becomes the distance to the plane
    to FP32 precision; near the plane the negative side does too."""
    n = (32, 32, 32)
    h = 1.0 / 32
    i, j, k = np.meshgrid(*(np.arange(s) + 0.5 for s in n), indexing="ij")
    true = (i - 13.3) * h
    out = O.redistance((3.0 * true).astype(F), h, 1)
    inner = (slice(1, -1),) * 3
    pos = (true > 0)[inner]
    np.testing.assert_allclose(out[inner][pos], true[inner][pos], rtol=0, atol=1e-6)
    band = (slice(10, 14), slice(6, -6), slice(6, -6))
    np.testing.assert_allclose(out[band], true[band], rtol=0, atol=1e-6)
    assert np.array_equal(np.sign(out), np.sign(true))


def test_sphere_band_is_within_a_fraction_of_a_cell():
    n = (32, 32, 32)
    h = 1.0 / 32
    phi, true = _sphere(n, (15.2, 16.7, 14.1), 8.3, h)
    out = O.redistance(phi, h, 1)
    band = (np.abs(true) < 6 * h) & (np.abs(true) > h)
    band[0], band[-1], band[:, 0], band[:, -1], band[:, :, 0], band[:, :, -1] = (False,) * 6
    err = np.abs(out - true)[band] / h
    assert err.max() < 0.75 and err.mean() < 0.3
    g = np.gradient(out.astype(np.float64), h)
    gn = np.sqrt(sum(a * a for a in g))[band]
    assert 0.95 < np.median(gn) < 1.08


def test_sweep_parity_matches_the_reference_loop():
    """The cells one _sweep launch changes have parity (odd + the n - 1 of
    every mirrored axis) & 1."""
    n = (6, 7, 8)
    h = 0.05
    phi, _ = _sphere(n, (3.1, 3.4, 3.9), 2.2, h)
    base = O.redistance_init(phi, h, 1)
    i, j, k = np.meshgrid(*(np.arange(s) for s in n), indexing="ij")
    for d in O.REDISTANCE_DIRECTIONS:
        for odd in (0, 1):
            a = base.copy()
            O.redistance_sweep(a, *d, odd, h)
            colour = (odd + sum(s - 1 for s, inc in zip(n, d) if inc < 0)) & 1
            changed = a != base
            assert changed.any()
            assert (((i + j + k) & 1)[changed] == colour).all()
