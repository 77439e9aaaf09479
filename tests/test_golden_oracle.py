"""The oracle reproduces the committed golden fixtures (tests/golden/*.npz)
bit for bit from their stored inputs: a regression pin on the checker."""
import numpy as np
import pytest

import oracle as O
from flub_gb300 import scenes
from tests.golden.make_golden import CASES, load


class _S:
    def __init__(self, d):
        self.phi, self.prims = d["phi"], d["prims"]
        self.u, self.v, self.w, self.ur, self.vr, self.wr = (d[k] for k in ("u", "v", "w", "ur", "vr", "wr"))
        self.levels = int(d["levels"])
        self.h = self.h0 = float(d["h"])
        self.shape = self.phi.shape


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_fixture(name):
    d = load(name)
    out = O.project(_S(d), max_iters=200, rel_tol=1e-12, abs_tol=0.0)
    for k in ("tag", "phi_rigid", "div", "r0"):
        assert np.array_equal(out[k], d[k]), k
    assert out["iters"] == int(d["iters"])
    assert np.array_equal(out["x"], d["x"])
    for k in ("u", "v", "w"):
        assert np.array_equal(out[k], d[k + "_out"]), k
    z = O.vcycle(d["r0"], O.tag_levels(d["tag"], int(d["levels"])), np.float32)
    assert np.array_equal(z, d["vcycle_r0"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_scene_is_regenerable(name):
    """The stored inputs come from the seeded generators (up to last-bit libm
    differences between platforms)."""
    d = load(name)
    s = CASES[name]()
    assert s.phi.shape == d["phi"].shape
    assert np.allclose(s.u, d["u"], atol=1e-6) and np.allclose(s.v, d["v"], atol=1e-6)
    assert np.array_equal(s.prims.view(np.uint8), d["prims"].view(np.uint8))
