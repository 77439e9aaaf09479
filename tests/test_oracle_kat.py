"""Pins the CPU oracle against known answers derived by hand from the
reference's kernels, and against the independent NumPy restatement.

Each known answer below is worked out from the reference source cited in its
docstring; none comes from running the oracle."""
import numpy as np
import pytest

import oracle as O
from oracle import np_oracle as N
from flub_gb300 import scenes


def line(tags):
    """A 1 x 1 x n grid."""
    return np.asarray(tags, np.int32).reshape(1, 1, -1)


# ---------------------------------------------------------------- classification

def test_tag_dirichlet_kat():
    """geometry.py:335-344: phi > 0 -> air (0), else fluid (1); phi = 0 is fluid."""
    phi = np.array([-1.0, 0.0, 1e-30, 2.0, -0.0], np.float32).reshape(1, 1, 5)
    assert O.tag_dirichlet(phi).ravel().tolist() == [1, 1, 0, 0, 1]


def test_tag_neumann_kat():
    """geometry.py:390-397: solid where phi_rigid < 0, other tags untouched."""
    tag = np.array([0, 1, 0, 1], np.int32).reshape(1, 1, 4)
    O.tag_neumann(np.array([-1, -1, 0, 1], np.float32).reshape(1, 1, 4), tag)
    assert tag.ravel().tolist() == [2, 2, 0, 1]


def test_phi_prims_sphere_kat():
    """geometry.py:82-113,148-169,225-239 for a sphere r = 0.25 at the centre of a
    4^3 grid (h = h0 = 0.25, cell centres 0.125 + 0.25 i)."""
    prims = scenes.make_prims([dict(geometry=2, x=(0.5, 0.5, 0.5), radius=0.25)])
    phi = O.phi_prims((4, 4, 4), 0.25, 0.25, prims)
    assert phi[1, 1, 1] == pytest.approx(0.125 * np.sqrt(3) - 0.25, abs=1e-7)      # inside
    assert phi[0, 0, 0] == 2.0                                                      # sdf 0.3995 >= h0
    assert phi[0, 1, 1] == pytest.approx(np.sqrt(0.171875) - 0.25, abs=1e-7)       # 0.1646 < h0


def test_phi_prims_box_kat():
    """geometry.py:17-32 _sdf_cube, box of half extent 0.25 at the centre of 4^3."""
    prims = scenes.make_prims([dict(geometry=1, x=(0.5, 0.5, 0.5), radius=0.25)])
    phi = O.phi_prims((4, 4, 4), 0.25, 0.25, prims)
    assert phi[1, 1, 1] == np.float32(-0.125)
    assert phi[0, 0, 0] == pytest.approx(0.125 * np.sqrt(3), abs=1e-7)
    assert phi[0, 1, 1] == np.float32(0.125)
    # no primitive -> 2.0 everywhere
    assert np.all(O.phi_prims((2, 2, 2), 0.5, 0.5, scenes.make_prims([])) == 2.0)


def test_phi_prims_keeps_min_below_h0():
    """sdf_argmin_prims: the running value starts at 2.0 and takes an SDF only if
    it is below min(h0, running)."""
    prims = scenes.make_prims([dict(geometry=2, x=(0.5, 0.5, 0.5), radius=0.3),
                               dict(geometry=2, x=(0.5, 0.5, 0.5), radius=0.1)])
    phi = O.phi_prims((4, 4, 4), 0.25, 0.25, prims)
    # at (1,1,1): distances 0.2165 - 0.3 = -0.0835 and 0.2165 - 0.1 = 0.1165 -> min -0.0835
    assert phi[1, 1, 1] == pytest.approx(0.125 * np.sqrt(3) - 0.3, abs=1e-7)


# ---------------------------------------------------------------- divergence / gradient

def _faces(shape, u=None):
    nx, ny, nz = shape
    f = [np.zeros((nx + 1, ny, nz), np.float32), np.zeros((nx, ny + 1, nz), np.float32),
         np.zeros((nx, ny, nz + 1), np.float32)]
    if u is not None:
        f[0][:] = np.asarray(u, np.float32).reshape(nx + 1, ny, nz)
    return f


def test_divergence_kat():
    """divergence.py:43-99 on a 2 x 1 x 1 grid: boundary faces count 0; a face
    whose outer neighbour is solid takes the rigid velocity."""
    u, v, w = _faces((2, 1, 1), [5, 7, 11])
    ur, vr, wr = _faces((2, 1, 1), [0, 3, 0])
    div = O.divergence(u, v, w, ur, vr, wr, np.array([1, 1], np.int32).reshape(2, 1, 1))
    assert div.ravel().tolist() == [7.0, -7.0]
    div = O.divergence(u, v, w, ur, vr, wr, np.array([1, 2], np.int32).reshape(2, 1, 1))
    assert div.ravel().tolist() == [3.0, -7.0]
    # a single cell: all six faces are on the domain boundary
    one = _faces((1, 1, 1))
    one[0][:] = 9.0
    assert O.divergence(*one, *_faces((1, 1, 1)), np.ones((1, 1, 1), np.int32)).item() == 0.0


def test_mask_and_scale_kat():
    """divergence.py:173-180 and utils/util.py:162-165."""
    d = np.array([1.0, 2.0, 3.0], np.float32).reshape(1, 1, 3)
    O.mask_with_tag(d, np.array([1, 0, 2], np.int32).reshape(1, 1, 3))
    O.scale(d, np.float32(-4.0))
    assert d.ravel().tolist() == [-4.0, 0.0, 0.0]


@pytest.mark.parametrize("tags,expect", [([1, 1], 4.0), ([1, 2], 3.0), ([2, 0], 3.0), ([0, 0], 0.0),
                                         ([0, 1], 4.0)])
def test_subtract_gradient_kat(tags, expect):
    """subtract_gradient.py:37-68 on a 2 x 1 x 1 grid, u = [5, 7, 11], p = [1, 4]:
    solid either side -> rigid (3); fluid either side -> 7 - (4 - 1); else 0;
    boundary faces 0."""
    u = np.array([5, 7, 11], np.float32).reshape(3, 1, 1)
    ur = np.array([0, 3, 0], np.float32).reshape(3, 1, 1)
    p = np.array([1, 4], np.float32).reshape(2, 1, 1)
    O.subtract_gradient(u, ur, p, np.array(tags, np.int32).reshape(2, 1, 1), 1)
    assert u.ravel().tolist() == [0.0, expect, 0.0]


# ---------------------------------------------------------------- multigrid pieces

def test_matvec_kat():
    """mgpcg.py:118-142 on the line [fluid, fluid, air, solid], x = [1, 2, 3, 4]:
    cell 0: (2 - 1) = 1 (the wall neighbour adds 0); cell 1: (0 - 2) + (1 - 2) = -3;
    non-fluid cells give 0."""
    tag = line([1, 1, 0, 2])
    x = np.array([1, 2, 3, 4], np.float32).reshape(1, 1, 4)
    assert O.matvec(x, tag).ravel().tolist() == [1.0, -3.0, 0.0, 0.0]
    assert N.matvec(x, tag).ravel().tolist() == [1.0, -3.0, 0.0, 0.0]


def test_divd_kat():
    """mgpcg.py:51-58 / 144-160: in-domain non-solid neighbours of fluid cells."""
    assert N.divd(line([1, 1, 0, 2])).ravel().tolist() == [1.0, 2.0, 0.0, 0.0]


def test_smooth_kat():
    """mgpcg.py:72-86: phase 0 updates (i+j+k) odd cells, phase 1 even ones.
    Line [F, F, A, S], r = [1, 1, 0, 0], z = 0:
    phase 0: z1 = (1 + 0) / 2 = 0.5, z3 (solid, divd 0) = 0;
    phase 1: z0 = (1 + (0.5 - 0)) / 1 = 1.5, z2 (air) = 0."""
    tag = line([1, 1, 0, 2])
    r = np.array([1, 1, 0, 0], np.float32).reshape(1, 1, 4)
    z = np.zeros_like(r)
    O.smooth(z, r, tag, 0)
    assert z.ravel().tolist() == [0.0, 0.5, 0.0, 0.0]
    O.smooth(z, r, tag, 1)
    assert z.ravel().tolist() == [1.5, 0.5, 0.0, 0.0]


def test_restrict_tag_kat():
    """mgpcg.py:162-174: any air -> 0, else any fluid -> 1, else 2."""
    for children, expect in [([2] * 8, 2), ([2] * 7 + [0], 0), ([2] * 7 + [1], 1), ([1] * 7 + [0], 0)]:
        t = np.array(children, np.int32).reshape(2, 2, 2)
        assert O.tag_levels(t, 2)[1].item() == expect
        assert N.restrict_tag(t).item() == expect


def test_restrict_kat():
    """mgpcg.py:94-101: coarse r = sum of children's r + L z if the coarse cell is
    fluid, else 0.  All fluid 2^3, z = 0: 1 + 2 + ... + 8 = 36."""
    tag = np.ones((2, 2, 2), np.int32)
    r = np.arange(1, 9, dtype=np.float32).reshape(2, 2, 2)
    z = np.zeros_like(r)
    assert O.restrict(r, z, tag, np.ones((1, 1, 1), np.int32)).item() == 36.0
    assert O.restrict(r, z, tag, np.zeros((1, 1, 1), np.int32)).item() == 0.0
    # with z: L z at child (0,0,0) for z = e_000 is -3 (three fluid neighbours), at
    # each of its three neighbours +1 -> the sum of L z over the block is 0.
    z[0, 0, 0] = 1.0
    assert O.restrict(r, z, tag, np.ones((1, 1, 1), np.int32)).item() == 36.0


def test_prolong_kat():
    zf = np.zeros((2, 2, 2), np.float32)
    O.prolong(zf, np.array([[[2.5]]], np.float32))
    assert np.all(zf == 2.5)


# ---------------------------------------------------------------- solver

def _explicit_solution(tag, b):
    """Direct solve of L x = b on the fluid cells via the assembled matrix."""
    fl = np.flatnonzero(tag.ravel() == 1)
    n = tag.size
    cols = []
    for q in fl:
        e = np.zeros(n)
        e[q] = 1.0
        cols.append(N.matvec(e.reshape(tag.shape), tag).ravel()[fl])
    A = np.array(cols).T
    x = np.zeros(n)
    x[fl] = np.linalg.solve(A, b.ravel()[fl])
    return x.reshape(tag.shape)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_pcg_solves_the_system(seed):
    """mgpcg.py:378-462: the converged x satisfies L x = b (checked against a
    dense direct solve of the assembled operator)."""
    from scipy import ndimage
    rng = np.random.default_rng(seed)
    tag = rng.choice([0, 1, 1, 1, 2], size=(4, 4, 4)).astype(np.int32)
    # every fluid component must touch air, else L is singular on it
    lab, n = ndimage.label(tag == 1)
    air_nb = ndimage.binary_dilation(tag == 0)
    for c in range(1, n + 1):
        comp = lab == c
        if not np.any(comp & air_nb):
            tag[tuple(np.argwhere(comp)[0])] = 0
    b = np.where(tag == 1, rng.standard_normal(tag.shape), 0.0)
    tags = O.tag_levels(tag, 2)
    # eps = 0: the reference's default eps = 1e-12 in zTr/(old_zTr + eps) distorts
    # beta once zTr itself falls to ~1e-12, which this tiny system reaches
    res = O.pcg(b, tags, max_iters=200, eps=0.0, rel_tol=1e-24, abs_tol=0.0, dtype=np.float64)
    assert res["converged"]
    xd = _explicit_solution(tag, b)
    assert np.allclose(N.matvec(xd, tag), b)
    assert np.linalg.norm(res["x"] - xd) <= 1e-9 * np.linalg.norm(xd)


def test_vcycle_is_symmetric():
    """The V-cycle (pre/post smoothing mirrored, R = P^T) is a symmetric operator."""
    s = scenes.random_scene(16, 5, levels=3)
    tag, _ = O.classify(s.phi, s.prims, s.h, s.h0)
    tags = O.tag_levels(tag, 3)
    rng = np.random.default_rng(0)
    a = np.where(tag == 1, rng.standard_normal(tag.shape), 0.0)
    b = np.where(tag == 1, rng.standard_normal(tag.shape), 0.0)
    ma, mb = O.vcycle(a, tags, np.float64), O.vcycle(b, tags, np.float64)
    assert abs(np.sum(b * ma) - np.sum(a * mb)) <= 1e-12 * abs(np.sum(b * ma))
    # and positive definite on the fluid (it approximates (-L)^-1)
    assert np.sum(a * ma) > 0


def test_divergence_of_gradient_is_L():
    """On fluid cells D(G p) = L p (the identity behind the projection): the
    divergence of the velocity update equals L p."""
    s = scenes.random_scene(16, 9, levels=3)
    tag, _ = O.classify(s.phi, s.prims, s.h, s.h0)
    rng = np.random.default_rng(1)
    # the solve leaves p = 0 off the fluid (air is p = 0 Dirichlet)
    p = np.where(tag == 1, rng.standard_normal(tag.shape), 0.0)
    zero = [np.zeros_like(a, np.float64) for a in (s.u, s.v, s.w)]
    g = [-N.subtract_gradient(zero[d], zero[d], p, tag, d + 1) for d in range(3)]  # G p (faces)
    d = N.divergence(*g, *zero, tag)
    lp = N.matvec(p, tag)
    fl = tag == 1
    assert np.allclose(d[fl], lp[fl], atol=1e-10)


# ---------------------------------------------------------------- C oracle vs NumPy oracle

@pytest.mark.parametrize("maker", [lambda: scenes.box(16, seed=3, levels=3), lambda: scenes.sphere(16, levels=2),
                                   lambda: scenes.dam(16, levels=3), lambda: scenes.random_scene(16, 11, levels=3)])
def test_c_oracle_matches_numpy(maker):
    s = maker()
    tag, _ = O.classify(s.phi, s.prims, s.h, s.h0)
    div = O.divergence(s.u, s.v, s.w, s.ur, s.vr, s.wr, tag)
    assert np.allclose(div, N.divergence(s.u, s.v, s.w, s.ur, s.vr, s.wr, tag), atol=1e-5)
    tags = O.tag_levels(tag, s.levels)
    assert all(np.array_equal(a, b) for a, b in zip(tags, N.tag_levels(tag, s.levels)))
    b = np.where(tag == 1, div, 0).astype(np.float64)
    assert np.array_equal(O.matvec(b, tag), N.matvec(b, tag))
    assert np.allclose(O.vcycle(b, tags, np.float64), N.vcycle(b, tags), rtol=1e-12, atol=1e-12)
    rc = O.pcg(b, tags, dtype=np.float64)
    rn = N.pcg(b, tags)
    assert rc["iters"] == rn["iters"]
    assert np.linalg.norm(rc["x"] - rn["x"]) <= 1e-9 * np.linalg.norm(rn["x"])


def test_fp32_oracle_tracks_fp64():
    s = scenes.box(32, seed=4, levels=3)
    res32 = O.project(s)
    res64 = O.project(s, dtype=np.float64)
    assert res32["converged"] and res64["converged"]
    assert abs(res32["iters"] - res64["iters"]) <= 1
    e = np.linalg.norm(res32["x"] - res64["x"]) / np.linalg.norm(res64["x"])
    assert e < 1e-5


def test_fraction_mode_removes_mean():
    """mgpcg.py:191-205: zero_centered leaves a zero-mean residual on the fluid."""
    s = scenes.box(16, seed=2, levels=2)
    tag, _ = O.classify(s.phi, s.prims, s.h, s.h0)
    tag[tag == 0] = 1  # all fluid: the all-Neumann problem "fraction" is for
    div = O.divergence(s.u, s.v, s.w, s.ur, s.vr, s.wr, tag)
    tags = O.tag_levels(tag, 2)
    res = O.pcg(div.astype(np.float64), tags, max_iters=200, eps=0.0, rel_tol=1e-20, abs_tol=0.0,
                smoother="fraction", dtype=np.float64)
    r = res["r"]
    assert abs(r[tag == 1].mean()) < 1e-12
    assert res["converged"]


def test_max_iters_zero_and_one():
    s = scenes.box(16, seed=1, levels=2)
    tag, _ = O.classify(s.phi, s.prims, s.h, s.h0)
    div = O.divergence(s.u, s.v, s.w, s.ur, s.vr, s.wr, tag)
    b = np.where(tag == 1, div, 0).astype(np.float32)
    tags = O.tag_levels(tag, 2)
    r0 = O.pcg(b, tags, max_iters=0)
    assert r0["iters"] == 0 and not r0["converged"] and np.all(r0["x"] == 0)
    r1 = O.pcg(b, tags, max_iters=1)
    assert r1["iters"] == 1 and np.any(r1["x"] != 0)


# ---------------------------------------------------------------- velocity extrapolation (extrapolate.py)

def test_set_unknown_kat():
    phi = np.array([[[-1.0, 0.0]]], np.float32)  # (1, 1, 2): fluid, surface
    tu = np.full((2, 1, 2), 7, np.int32)
    tv = np.full((1, 2, 2), 7, np.int32)
    tw = np.full((1, 1, 3), 7, np.int32)
    O.set_unknown(phi, tu, tv, tw)
    assert tu[0].tolist() == [[0, 1]] and tu[1].tolist() == [[7, 7]]       # last layer untouched
    assert tv[0, 0].tolist() == [0, 1] and tv[0, 1].tolist() == [7, 7]
    assert tw[0, 0].tolist() == [0, 1, 7]


def test_extrapolate_axis_kat():
    q = np.zeros((3, 3, 3), np.float32)
    t = np.ones((3, 3, 3), np.int32)
    t[0, 0, 0], q[0, 0, 0] = 0, 6.0
    t[2, 2, 2], q[2, 2, 2] = 0, 3.0
    O.extrapolate_axis(q, t)
    assert q[1, 1, 1] == 4.5 and t[1, 1, 1] == -1          # both known corners
    assert q[0, 0, 1] == 6.0 and q[1, 2, 2] == 3.0
    assert q[0, 2, 0] == 0.0 and t[0, 2, 0] == 1            # no known neighbour: zeroed, still unknown
    assert q[0, 0, 0] == 6.0 and t[0, 0, 0] == 0            # known faces untouched
    O.flush_unknown(t)
    assert set(np.unique(t)) <= {0, 1}


def test_extrapolation_passes_repeat_the_first():
    """flush_1_3d turns -1 back into 1, so the known set never grows and every
    pass recomputes the first one (the reference's behaviour, reproduced)."""
    rng = np.random.default_rng(3)
    phi = rng.standard_normal((6, 5, 4)).astype(np.float32)
    faces = [rng.standard_normal(s).astype(np.float32) for s in ((7, 5, 4), (6, 6, 4), (6, 5, 5))]
    flags = [np.zeros(f.shape, np.int32) for f in faces]
    one = [f.copy() for f in faces]
    t1 = [f.copy() for f in flags]
    O.extrapolate(*one, *t1, phi, 1)
    many = [f.copy() for f in faces]
    t4 = [f.copy() for f in flags]
    O.extrapolate(*many, *t4, phi, 4)
    for a, b in zip(one, many):
        assert np.array_equal(a, b)
    for a, b in zip(t1, t4):
        assert np.array_equal(a, b)


# ---------------------------------------------------------------- rigid face velocities, cut cells

def test_fraction_edge_triangle_quad_kat():
    # all positive / all negative / half-plane through the face centre
    assert O.fraction_quad(1, 1, 1, 1, 1) == 1.0
    assert O.fraction_quad(-1, -1, -1, -1, -1) == 0.0
    assert O.fraction_quad(1, -1, -1, 1, 0.0) == 0.5
    # small positive slivers are cut to 0 (edge fraction < 0.1, face fraction < 0.1)
    assert O.fraction_quad(0.05, -1, -1, -1, -1) == 0.0


def test_solid_vel_kat():
    # one body rotating about z with omega = (0, 0, 2) at x = (0.5, 0.5, 0.5), v = (1, 0, 0)
    n = 4
    h0 = 1.0 / n
    ur = np.zeros((n + 1, n, n), np.float32)
    owner = np.zeros(ur.shape, np.int32)
    owner[:, :, 0] = -1
    O.solid_vel(ur, owner, 1, h0, [[0.5, 0.5, 0.5]], [[1.0, 0.0, 0.0]], [[0.0, 0.0, 2.0]])
    # u = v_x + (omega x p)_x = 1 - 2 * p_y with p_y = (j + 0.5) h0 - 0.5
    for i in range(n + 1):
        for j in range(n):
            for k in range(n):
                inside = 0.01 * h0 < i * h0 < 1 - 0.01 * h0 and owner[i, j, k] != -1
                expect = 1.0 - 2.0 * ((j + 0.5) * h0 - 0.5) if inside else 0.0
                assert ur[i, j, k] == pytest.approx(expect, abs=1e-6)


def test_divergence_fractional_full_fluid_is_plain_divergence():
    rng = np.random.default_rng(8)
    s = (5, 4, 3)
    u = rng.standard_normal((6, 4, 3)).astype(np.float32)
    v = rng.standard_normal((5, 5, 3)).astype(np.float32)
    w = rng.standard_normal((5, 4, 4)).astype(np.float32)
    ones = [np.ones_like(a) for a in (u, v, w)]
    zeros = [np.zeros_like(a) for a in (u, v, w)]
    d = O.divergence_fractional(u, v, w, *ones, *zeros)
    ref = (u[1:] - u[:-1]) + (v[:, 1:] - v[:, :-1]) + (w[:, :, 1:] - w[:, :, :-1])
    assert np.allclose(d, ref, atol=1e-5)
    # fully solid faces: only the rigid velocities count
    d2 = O.divergence_fractional(u, v, w, *zeros, *[a * 0 + 2.0 for a in (u, v, w)])
    assert np.allclose(d2, 0.0)


def test_subtract_gradient_batty_kat():
    nx, ny, nz = 4, 1, 1
    phi = np.array([-1.0, -1.0, 0.5, 1.0], np.float32).reshape(nx, ny, nz)   # fluid, fluid, air, air
    p = np.array([3.0, 1.0, 9.0, 9.0], np.float32).reshape(nx, ny, nz)
    uf = np.zeros((nx + 1, ny, nz), np.float32)
    frac = np.ones_like(uf)
    ur = np.full_like(uf, 7.0)
    O.subtract_gradient_batty(uf, p, frac, phi, ur, 1, 0.0, 1.0 / nx)
    assert uf[1, 0, 0] == pytest.approx(-(1.0 - 3.0))                   # fluid-fluid: theta = 1
    theta = 1.0 - 0.5 / 1.5                                              # fluid (-1) next to air (0.5)
    assert uf[2, 0, 0] == pytest.approx(-(0.0 - 1.0) / theta)            # ghost pressure 0 in the air
    assert uf[3, 0, 0] == 0.0                                            # air-air
    assert uf[0, 0, 0] == 0.0 and uf[4, 0, 0] == 0.0                     # domain boundary, lo = 0
    frac[1] = 0.0
    uf[:] = 0.0
    O.subtract_gradient_batty(uf, p, frac, phi, ur, 1, 0.0, 1.0 / nx)
    assert uf[1, 0, 0] == 7.0                                            # zero fraction: rigid velocity


def test_fp64_bottom_changes_only_the_rounding():
    """The FP64 bottom (no reference counterpart) leaves the V-cycle within FP32
    rounding of the FP32 one, and exactly equal to it when the bottom is
    already exact (no fluid at the bottom)."""
    from flub_gb300 import scenes
    s = scenes.dam(32, seed=60, levels=3)
    tag, _ = O.classify(s.phi, s.prims, s.h, s.h0)
    div = O.divergence(s.u, s.v, s.w, s.ur, s.vr, s.wr, tag)
    r0 = np.where(tag == 1, div, 0).astype(np.float32)
    tags = O.tag_levels(tag, 3)
    z32 = O.vcycle(r0, tags, np.float32)
    with O.bottom_fp64():
        z64 = O.vcycle(r0, tags, np.float32)
    assert not np.array_equal(z32, z64)
    assert np.linalg.norm(z64 - z32) <= 1e-5 * np.linalg.norm(z32)
    assert np.array_equal(O.vcycle(r0, tags, np.float32), z32)  # the switch is restored on exit
