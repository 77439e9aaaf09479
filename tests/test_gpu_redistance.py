"""GPU parity of the level-set redistance against the oracle (bit-exact):
_init_distance, every _sweep launch and the whole redistance
(redistance.py:7-136)."""
import numpy as np
import pytest
import torch

import oracle as O
from flub_gb300 import FlubError, _init_distance, _sweep, init_distance, launch, redistance

pytestmark = pytest.mark.gpu

F = np.float32


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def _field(n, seed, noise=0.05):
    i, j, k = np.meshgrid(*(np.arange(s) + 0.5 for s in n), indexing="ij")
    rng = np.random.default_rng(seed)
    h = 1.0 / n[0]
    c = [s / 2 + rng.uniform(-1, 1) for s in n]
    r = np.sqrt((i - c[0]) ** 2 + (j - c[1]) ** 2 + (k - c[2]) ** 2)
    phi = (r - min(n) / 3.3) * h * (1 + 0.5 * np.sin(i / 3.0)) + noise * h * rng.standard_normal(n)
    # a second, flat interface (a water surface) across the box
    phi = np.minimum(phi, (j - n[1] * 0.35) * h * 1.7)
    return phi.astype(F), h


SHAPES = [(32, 32, 32), (40, 24, 56), (17, 9, 13), (64, 16, 64)]


@pytest.mark.parametrize("n", SHAPES)
@pytest.mark.parametrize("set_boundary", [0, 1])
def test_init_distance_bit_exact(n, set_boundary):
    phi, h = _field(n, 1)
    ref = O.redistance_init(phi, h, set_boundary)
    g = dev(phi)
    launch(_init_distance, dim=n, inputs=[g, h, set_boundary])
    assert np.array_equal(host(g), ref)
    out = torch.empty_like(g)
    init_distance(dev(phi), h, set_boundary, out=out)
    assert np.array_equal(host(out), ref)


@pytest.mark.parametrize("n", [(17, 9, 13), (24, 20, 16)])
def test_every_sweep_launch_bit_exact(n):
    phi, h = _field(n, 2)
    a = O.redistance_init(phi, h, 1)
    g = dev(a)
    for d in O.REDISTANCE_DIRECTIONS:
        for odd in (0, 1):
            O.redistance_sweep(a, *d, odd, h)
            launch(_sweep, dim=n, inputs=[g, *d, odd, h])
            assert np.array_equal(host(g), a), (d, odd)


@pytest.mark.parametrize("n", SHAPES)
@pytest.mark.parametrize("set_boundary", [0, 1])
def test_redistance_bit_exact(n, set_boundary):
    phi, h = _field(n, 3)
    ref = O.redistance(phi, h, set_boundary)
    g = dev(phi)
    redistance(g, h, set_boundary)
    assert np.array_equal(host(g), ref)


@pytest.mark.parametrize("n_rounds", [0, 1, 3])
def test_redistance_rounds_bit_exact(n_rounds):
    n = (24, 16, 20)
    phi, h = _field(n, 4)
    ref = O.redistance(phi, h, 1, n_rounds=n_rounds)
    g = dev(phi)
    redistance(g, h, 1, n_rounds=n_rounds)
    assert np.array_equal(host(g), ref)


@pytest.mark.parametrize("n", [(1, 1, 1), (2, 3, 4), (3, 3, 3)])
def test_redistance_tiny_grids(n):
    phi = np.random.default_rng(5).standard_normal(n).astype(F)
    ref = O.redistance(phi, 0.25, 1)
    g = dev(phi)
    redistance(g, 0.25, 1)
    assert np.array_equal(host(g), ref)


def test_redistance_rejects_bad_arguments():
    g = torch.zeros((8, 8, 8), device="cuda")
    with pytest.raises(FlubError):
        launch(_sweep, dim=(8, 8, 8), inputs=[g, 2, 1, 1, 0, 0.1])
    with pytest.raises(FlubError):
        init_distance(g, 0.1, 1, out=g)
