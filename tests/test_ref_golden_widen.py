"""The oracle's widening rows against fixtures computed by the reference's own
code.

tests/golden/refw_*.npz hold the results of the unmodified reference kernels
(advect.py, extrapolate.py with utils/util.py set_unknown, redistance.py,
geometry.py phi_to_fraction, divergence.py divergence_fractional_3d,
subtract_gradient.py u/v/w_subtract_gradient_batty_3d, rigid_coupling.py
precompute_solid_vel), run on the CPU through the stand-in for ``warp``
(tests/golden/make_ref_widen.py).  Every output must match bit for bit on a
10 x 12 x 14 grid: MacCormack and semi-Lagrangian advection with traces that
leave the grid, three passes of velocity extrapolation with their flags,
redistancing with and without the boundary cells, face fractions, the
fractional divergence, the cut-face pressure-gradient update and the solid
face velocities of two bodies.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

import oracle as O
from tests.golden import make_ref_widen as W


def _eq(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a, b)


def test_advection_matches_reference():
    f = W.load("adv")
    dt, h0 = float(f["dt"]), float(f["h0"])
    assert _eq(O.advect_phi(f["u"], f["v"], f["w"], f["phi"], dt, h0), f["advect_phi"])
    for k, a in zip("uvw", O.advect_velocity_mc(f["u"], f["v"], f["w"], dt, h0, minmax_h=h0)):
        assert _eq(a, f["advect_mc_" + k]), k
    assert _eq(O.advect_simple(f["u"], f["v"], f["w"], f["q"], dt, h0), f["advect_simple"])


def test_extrapolation_matches_reference():
    f = W.load("ext")
    u, v, w = (f[k].copy() for k in "uvw")
    tu, tv, tw = (f[k].copy() for k in ("tu", "tv", "tw"))
    O.extrapolate(u, v, w, tu, tv, tw, f["phi"], int(f["n_cells"]))
    for k, a, t in zip("uvw", (u, v, w), (tu, tv, tw)):
        assert _eq(a, f["ext_" + k]), k
        assert _eq(t, f["ext_t" + k]), k
    # the passes reached cells that were unknown, and some stayed unknown
    assert (f["ext_tu"] == 1).any() and (f["ext_tu"] == 0).any()


def test_redistance_matches_reference():
    f = W.load("red")
    h0 = float(f["h0"])
    for sb in (1, 0):
        assert _eq(O.redistance_init(f["phi"], h0, sb), f[f"init_sb{sb}"]), sb
        assert _eq(O.redistance(f["phi"], h0, sb, 2), f[f"redistance_sb{sb}"]), sb


def test_cut_cells_match_reference():
    f = W.load("cut")
    nx = int(f["shape"][0])
    fr = []
    for d, k in zip((1, 2, 3), "uvw"):
        a = f["fc_" + k].copy()
        O.phi_to_fraction(f["phin"], a, d)
        assert _eq(a, f["frac_" + k]), k
        fr.append(a)
    # faces fully open, fully closed and cut
    assert (fr[0] == 1).any() and (fr[0] == 0).any() and ((fr[0] > 0) & (fr[0] < 1)).any()
    div = O.divergence_fractional(f["u"], f["v"], f["w"], *fr, f["ur"], f["vr"], f["wr"])
    assert _eq(div, f["div_frac"])
    for d, k in zip((1, 2, 3), "uvw"):
        uf = f[k].copy()
        O.subtract_gradient_batty(uf, f["p"], fr[d - 1], f["phic"], f[k + "r"], d, 0.0, 1.0 / nx)
        assert _eq(uf, f["batty_" + k]), k
    for d, k in zip((1, 2, 3), "uvw"):
        ur = np.full(f["solid_" + k].shape, 9.0, np.float32)
        O.solid_vel(ur, f["own_" + k], d, float(f["h0"]), f["bx"], f["bv"], f["bw"])
        assert _eq(ur, f["solid_" + k]), k


@pytest.mark.skipif(not os.path.isdir(os.path.join(W.DEFAULT_REFERENCE, "multigrid")),
                    reason="the reference tree is not on this machine")
@pytest.mark.parametrize("name", ["red", "cut"])
def test_widen_fixture_regenerates_from_reference(name):
    """A fixture recomputed from the reference tree in a child process equals
    the committed file in every array."""
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        fresh = pool.apply(W.compute_case, (name, W.DEFAULT_REFERENCE))
    stored = W.load(name)
    assert sorted(fresh) == sorted(stored)
    for k in stored:
        assert _eq(np.asarray(fresh[k]), stored[k]), k
