"""GPU parity: every kernel of the path, called through the C ABI, against the
CPU oracle on the same inputs.

Bit-exact (np.array_equal) for integer work (tags) and for the FP32 kernels whose
operation order the oracle mirrors (classification SDF, divergence, gradient,
matvec, one V-cycle).  Solves are compared within tolerance: the FP64 inner
products are summed in a different order on the GPU, so alpha/beta can differ
in the last bit; the iteration count must agree within 1 and the pressure
must be within relative L2 1e-5 of the FP64 oracle's solve (same algorithm,
same tolerance)."""
import os

import numpy as np
import pytest
import torch

import oracle as O
from flub_gb300 import MGPCG, Projection, launch, scenes
from flub_gb300 import kernels as K
from flub_gb300._lib import FlubError
from flub_gb300.fields import Field, IntField, MACGrid
from tests.golden.make_golden import CASES, load

pytestmark = pytest.mark.gpu

PRESSURE_RTOL = 1e-5  # relative L2 of the pressure vs the FP64 oracle


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def mac(u, v, w):
    return MACGrid(Field(dev(u), d=1), Field(dev(v), d=2), Field(dev(w), d=3))


SCENES = {
    "box32": lambda: scenes.box(32, seed=21, levels=3),
    "sphere32": lambda: scenes.sphere(32, seed=22, levels=3),
    "dam32": lambda: scenes.dam(32, seed=23, levels=3),
    "dam64": lambda: scenes.dam(64, seed=24, levels=4),
    "rand32": lambda: scenes.random_scene(32, 25, levels=3),
    "rand32b": lambda: scenes.random_scene(32, 26, levels=4),
}


@pytest.fixture(scope="module", params=sorted(SCENES))
def scene(request):
    return SCENES[request.param]()


# ---------------------------------------------------------------- classification

def test_classify_bit_exact(scene):
    tag_o, phr_o = O.classify(scene.phi, scene.prims, scene.h, scene.h0)
    phr = torch.empty(scene.shape, dtype=torch.float32, device="cuda")
    tag = K.classify(dev(scene.phi), scene.prims, scene.h, scene.h0, phi_rigid=phr)
    assert np.array_equal(host(tag), tag_o)
    assert np.array_equal(host(phr), phr_o)


@pytest.mark.parametrize("shape", [(20, 24, 32), (20, 24, 30)])
def test_classify_every_primitive_kind_bit_exact(shape):
    """Rotated boxes (geometry 1 and 3), a sphere (2), the two-box primitive
    (4), the constant ones (5 and an unknown kind) and overlaps between them,
    on a grid with nz % 4 == 0 (four cells per thread) and one without."""
    def unit(q):
        q = np.asarray(q, np.float64)
        return tuple((q / np.linalg.norm(q)).astype(np.float32))
    prims = scenes.make_prims([
        dict(geometry=1, x=(0.3, 0.4, 0.5), radius=(0.12, 0.2, 0.08), q=unit((0.1, 0.3, -0.2, 0.9))),
        dict(geometry=3, x=(0.6, 0.5, 0.4), radius=0.1, q=unit((-0.4, 0.1, 0.2, 0.8))),
        dict(geometry=2, x=(0.45, 0.6, 0.55), radius=0.17),
        dict(geometry=4, x=(0.7, 0.3, 0.6), radius=(0.15, 0.04, 0.06), q=unit((0.2, -0.1, 0.5, 0.7))),
        dict(geometry=5, x=(0.1, 0.1, 0.1), radius=0.1),
        dict(geometry=7, x=(0.9, 0.9, 0.9), radius=0.1),
    ])
    rng = np.random.default_rng(17)
    phi = rng.standard_normal(shape).astype(np.float32) * 0.1
    h, h0 = 1.0 / shape[0], 0.05
    tag_o, phr_o = O.classify(phi, prims, h, h0)
    assert (tag_o == 2).any() and (tag_o == 0).any() and (tag_o == 1).any()
    phr = torch.empty(shape, dtype=torch.float32, device="cuda")
    tag = K.classify(dev(phi), prims, h, h0, phi_rigid=phr)
    assert np.array_equal(host(tag), tag_o)
    assert np.array_equal(host(phr), phr_o)


def test_classify_unfused_kernels_bit_exact(scene):
    tag_o, phr_o = O.classify(scene.phi, scene.prims, scene.h, scene.h0)
    tag = IntField(torch.empty(scene.shape, dtype=torch.int32, device="cuda"))
    phi = Field(dev(scene.phi))
    phr = torch.full(scene.shape, 1.0, device="cuda")
    launch(K._tag_dirichlet, scene.shape, [tag, phi])
    prims = scenes.make_prims([]) if len(scene.prims) == 0 else scene.prims
    launch(K.precompute_grid_point_phi_prims, scene.shape,
           [phr, None, prims["x"], prims["q"], [dict(geometry=g, radius=r) for g, r in
                                               zip(prims["geometry"], prims["radius"])], (0.5, 0.5, 0.5)])
    launch(K._tag_neumann, scene.shape, [tag, Field(phr)])
    assert np.array_equal(host(tag.f), tag_o)
    assert np.array_equal(host(phr), phr_o)


# ---------------------------------------------------------------- divergence / gradient

def test_divergence_bit_exact(scene):
    tag_o, _ = O.classify(scene.phi, scene.prims, scene.h, scene.h0)
    div_o = O.divergence(scene.u, scene.v, scene.w, scene.ur, scene.vr, scene.wr, tag_o)
    vel, velr = mac(scene.u, scene.v, scene.w), mac(scene.ur, scene.vr, scene.wr)
    div = Field(torch.empty(scene.shape, device="cuda"))
    launch(K.divergence_tag, scene.shape, [vel, div, velr, IntField(dev(tag_o))])
    assert np.array_equal(host(div.f), div_o)
    # mask + scale (example_fluid.py:90-93), unfused and fused
    launch(K.mask_with_tag, scene.shape, [div, IntField(dev(tag_o))])
    launch(K.scale_by_3d, scene.shape, [div, -1.0 / scene.h])
    O.mask_with_tag(div_o, tag_o)
    O.scale(div_o, np.float32(-1.0 / scene.h))
    assert np.array_equal(host(div.f), div_o)
    fused = K.divergence(vel, velr, dev(tag_o), scale=-1.0 / scene.h)
    assert np.array_equal(host(fused), div_o)


@pytest.mark.parametrize("shape", [(12, 20, 28), (12, 20, 30), (9, 7, 4)])
def test_divergence_ragged_shapes_bit_exact(shape):
    """Plain and fused (masked, scaled) divergence on random tags (air, fluid
    and solid mixed everywhere) at nz % 4 == 0 (four cells per thread) and not."""
    rng = np.random.default_rng(37)
    nx, ny, nz = shape
    tag = rng.integers(0, 3, shape).astype(np.int32)
    vel = [rng.standard_normal(s).astype(np.float32) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    velr = [rng.standard_normal(a.shape).astype(np.float32) for a in vel]
    div_o = O.divergence(*vel, *velr, tag)
    vd, vrd = mac(*vel), mac(*velr)
    div = Field(torch.empty(shape, device="cuda"))
    launch(K.divergence_tag, shape, [vd, div, vrd, IntField(dev(tag))])
    assert np.array_equal(host(div.f), div_o)
    O.mask_with_tag(div_o, tag)
    O.scale(div_o, np.float32(-3.0))
    assert np.array_equal(host(K.divergence(vd, vrd, dev(tag), scale=-3.0)), div_o)


def test_subtract_gradient_bit_exact(scene):
    tag_o, _ = O.classify(scene.phi, scene.prims, scene.h, scene.h0)
    rng = np.random.default_rng(5)
    p = rng.standard_normal(scene.shape).astype(np.float32)
    outs = [np.array(a, copy=True) for a in (scene.u, scene.v, scene.w)]
    for d, (a, ar) in enumerate(zip(outs, (scene.ur, scene.vr, scene.wr))):
        O.subtract_gradient(a, ar, p, tag_o, d + 1)
    vel, velr = mac(scene.u, scene.v, scene.w), mac(scene.ur, scene.vr, scene.wr)
    for d in (1, 2, 3):
        shp = list(scene.shape)
        shp[d - 1] += 1
        launch(K.subtract_gradient_tag, tuple(shp), [vel, velr, Field(dev(p)), IntField(dev(tag_o)), d])
    for a, o in zip((vel.u.f, vel.v.f, vel.w.f), outs):
        assert np.array_equal(host(a), o)
    # fused three-axis form with the 1/h0 read scale
    ps = (p * np.float32(scene.h0)).astype(np.float32)
    vel2 = mac(scene.u, scene.v, scene.w)
    K.subtract_gradient(vel2, velr, dev(ps), dev(tag_o), p_scale=1.0 / scene.h0)
    pg = ps.copy()
    O.scale(pg, np.float32(1.0 / scene.h0))
    outs2 = [np.array(a, copy=True) for a in (scene.u, scene.v, scene.w)]
    for d, (a, ar) in enumerate(zip(outs2, (scene.ur, scene.vr, scene.wr))):
        O.subtract_gradient(a, ar, pg, tag_o, d + 1)
    for a, o in zip((vel2.u.f, vel2.v.f, vel2.w.f), outs2):
        assert np.array_equal(host(a), o)


@pytest.mark.parametrize("shape", [(12, 20, 28), (12, 20, 30), (9, 7, 4)])
def test_fused_subtract_gradient_ragged_shapes_bit_exact(shape):
    """The fused three-axis update on random tags (air, fluid and solid mixed
    everywhere) at nz % 4 == 0 (four faces per thread) and not."""
    rng = np.random.default_rng(31)
    nx, ny, nz = shape
    tag = rng.integers(0, 3, shape).astype(np.int32)
    p = rng.standard_normal(shape).astype(np.float32)
    vel = [rng.standard_normal(s).astype(np.float32) for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))]
    velr = [rng.standard_normal(a.shape).astype(np.float32) for a in vel]
    outs = [a.copy() for a in vel]
    pg = p.copy()
    O.scale(pg, np.float32(2.0))
    for d, (a, ar) in enumerate(zip(outs, velr)):
        O.subtract_gradient(a, ar, pg, tag, d + 1)
    vd = mac(*vel)
    K.subtract_gradient(vd, mac(*velr), dev(p), dev(tag), p_scale=2.0)
    for a, o in zip((vd.u.f, vd.v.f, vd.w.f), outs):
        assert np.array_equal(host(a), o)


# ---------------------------------------------------------------- multigrid

def _setup(scene):
    tag_o, _ = O.classify(scene.phi, scene.prims, scene.h, scene.h0)
    div = O.divergence(scene.u, scene.v, scene.w, scene.ur, scene.vr, scene.wr, tag_o)
    r0 = np.where(tag_o == 1, div, 0).astype(np.float32)
    mg = MGPCG(3, scene.shape, scene.levels, float)
    mg.set_tags(dev(tag_o))
    mg.init(dev(r0), 1.0)
    mg.mask_interior()
    return tag_o, r0, mg


def test_matvec_bit_exact(scene):
    tag_o, r0, mg = _setup(scene)
    p = np.random.default_rng(7).standard_normal(scene.shape).astype(np.float32)
    assert np.array_equal(host(mg.matvec(dev(p))), O.matvec(p, tag_o))


def test_vcycle_bit_exact(scene):
    tag_o, r0, mg = _setup(scene)
    z = mg.apply_preconditioner(dev(r0))
    z_o = O.vcycle(r0, O.tag_levels(tag_o, scene.levels), np.float32)
    assert np.array_equal(host(z), z_o)


@pytest.mark.parametrize("name", ["dam64", "rand32b", "box32"])
def test_vcycle_fallback_paths_bit_exact(name, monkeypatch):
    """The coarse levels run in one thread-block cluster when the GPU allows it;
    the fallback (global sweeps + one-block tail kernel) must give the same bits."""
    scene = SCENES[name]()
    tag_o, r0, mg = _setup(scene)
    z_cluster = host(mg.apply_preconditioner(dev(r0)))
    monkeypatch.setenv("FLUB_NO_CLUSTER", "1")
    tag_o, r0, mg2 = _setup(scene)
    z_plain = host(mg2.apply_preconditioner(dev(r0)))
    z_o = O.vcycle(r0, O.tag_levels(tag_o, scene.levels), np.float32)
    assert np.array_equal(z_cluster, z_o)
    assert np.array_equal(z_plain, z_o)


@pytest.mark.parametrize("case", [("dam128", "0"), ("dam64", "1")])
@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_persistent_legs_bit_exact(case, precision, monkeypatch):
    """The persistent cooperative kernels for the middle levels (FLUB_PERSIST=1)
    give the same V-cycle and the same solve as one launch per pass, with the
    reference schedule and the light one: dam128 runs its 64^3 level there
    (the 32^3 level and below in the cluster), dam64 without the cluster its
    32^3 level (16^3 and below in the one-block tail)."""
    name, no_cluster = case
    scene = TILE_SCENES[name]() if name in TILE_SCENES else SCENES[name]()
    monkeypatch.setenv("FLUB_NO_CLUSTER", no_cluster)
    out = []
    for on in ("1", "0"):
        monkeypatch.setenv("FLUB_PERSIST", on)
        tag_o, r0, _ = _setup(scene)
        mg = MGPCG(3, scene.shape, scene.levels, float, precision=precision)
        mg.set_tags(dev(tag_o))
        z = host(mg.apply_preconditioner(dev(r0)))
        mg.set_schedule("v22")
        z22 = host(mg.apply_preconditioner(dev(r0)))
        mg.init(dev(r0), 1.0)
        mg.mask_interior()
        info = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
        out.append((z, z22, info["iterations"], host(mg.x).copy()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2] and np.array_equal(out[0][3], out[1][3])
    if precision == "fp32":
        assert np.array_equal(out[0][0], O.vcycle(r0, O.tag_levels(tag_o, scene.levels), np.float32))


def test_solve_matches_oracle(scene):
    tag_o, r0, mg = _setup(scene)
    info = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    tags = O.tag_levels(tag_o, scene.levels)
    ref32 = O.pcg(r0, tags, max_iters=200, abs_tol=0.0, rel_tol=1e-12)
    ref64 = O.pcg(r0, tags, max_iters=200, abs_tol=0.0, rel_tol=1e-12, dtype=np.float64)
    assert info["converged"] and ref64["converged"]
    assert abs(info["iterations"] - ref32["iters"]) <= 1
    assert abs(info["iterations"] - ref64["iters"]) <= 1
    x = host(mg.x)
    err = np.linalg.norm(x - ref64["x"]) / np.linalg.norm(ref64["x"])
    assert err <= PRESSURE_RTOL, err
    assert info["rtr"] < info["tol"] == pytest.approx(1e-12 * ref64["rtr0"], rel=1e-9)


def test_projection_matches_oracle(scene):
    proj = Projection(scene.shape, scene.levels)
    vel, velr = mac(scene.u, scene.v, scene.w), mac(scene.ur, scene.vr, scene.wr)
    info = proj.project(vel, velr, dev(scene.phi), scene.prims)
    ref = O.project(scene, dtype=np.float64)
    assert np.array_equal(host(proj.tag.f), ref["tag"])
    assert info["converged"] and abs(info["iterations"] - ref["iters"]) <= 1
    for a, k in zip((vel.u.f, vel.v.f, vel.w.f), "uvw"):
        o = ref[k]
        assert np.linalg.norm(host(a) - o) <= 1e-5 * np.linalg.norm(o), k
    p = host(proj.p.f)
    assert np.linalg.norm(p - ref["p"]) <= PRESSURE_RTOL * np.linalg.norm(ref["p"])
    # post-projection divergence (example_fluid.py:146-147) falls by orders of magnitude
    before = np.abs(ref["div"]).max() * scene.h
    after = proj.max_abs_div(vel, velr)
    assert after < 1e-4 * max(before, 1e-30)


# ---------------------------------------------------------------- golden fixtures

@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_fixture(name):
    d = load(name)
    shape = d["phi"].shape
    h = float(d["h"])
    proj = Projection(shape, int(d["levels"]), h=h)
    vel, velr = mac(d["u"], d["v"], d["w"]), mac(d["ur"], d["vr"], d["wr"])
    info = proj.project(vel, velr, dev(d["phi"]), d["prims"])
    assert np.array_equal(host(proj.tag.f), d["tag"])
    assert np.array_equal(host(proj.div.f), d["div"])
    assert abs(info["iterations"] - int(d["iters"])) <= 1
    x = host(proj.mg.x)
    assert np.linalg.norm(x - d["x64"]) <= PRESSURE_RTOL * np.linalg.norm(d["x64"])
    z = proj.mg.apply_preconditioner(dev(d["r0"]))
    assert np.array_equal(host(z), d["vcycle_r0"])


# ---------------------------------------------------------------- edge cases and options

def test_fraction_smoother_matches_oracle():
    s = scenes.box(32, seed=30, levels=3)
    tag_o, _ = O.classify(s.phi, s.prims, s.h, s.h0)
    tag_o[tag_o == 0] = 1  # all fluid, all-Neumann walls: the singular problem "fraction" handles
    div = O.divergence(s.u, s.v, s.w, s.ur, s.vr, s.wr, tag_o)
    mg = MGPCG(3, s.shape, 3)
    mg.set_tags(dev(tag_o))
    mg.init(dev(div), 1.0)
    mg.mask_interior()
    info = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="fraction")
    ref = O.pcg(div, O.tag_levels(tag_o, 3), max_iters=200, abs_tol=0.0, rel_tol=1e-12, smoother="fraction",
                dtype=np.float64)
    assert abs(info["iterations"] - ref["iters"]) <= 1
    x = host(mg.x)
    x = x - x.mean()
    xr = ref["x"] - ref["x"].mean()
    assert np.linalg.norm(x - xr) <= 1e-4 * np.linalg.norm(xr)


def test_warm_start_reduces_iterations():
    s = scenes.dam(32, seed=31, levels=3)
    tag_o, r0, mg = _setup(s)
    cold = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    xstar = mg.x.clone()
    mg.init(dev(r0), 1.0)
    mg.mask_interior()
    warm = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases", x0=xstar)
    assert warm["converged"] and warm["iterations"] <= 1 < cold["iterations"]
    assert warm["rtr0"] == pytest.approx(cold["rtr0"])  # tolerance stays relative to the x0 = 0 residual
    mg.init(dev(r0), 1.0)
    mg.mask_interior()
    half = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases", x0=0.9 * xstar)
    assert half["iterations"] < cold["iterations"]
    assert np.linalg.norm(host(mg.x) - host(xstar)) <= 1e-3 * np.linalg.norm(host(xstar))


def test_max_iters_zero_and_one():
    s = scenes.box(32, seed=32, levels=3)
    tag_o, r0, mg = _setup(s)
    info = mg.solve(0, 1e-12, 0.0, 1e-12, smoother="phases")
    assert info["iterations"] == 0 and not info["converged"]
    assert float(mg.x.abs().max()) == 0.0
    mg.init(dev(r0), 1.0)
    mg.mask_interior()
    info = mg.solve(1, 1e-12, 0.0, 1e-12, smoother="phases")
    ref = O.pcg(r0, O.tag_levels(tag_o, 3), max_iters=1, abs_tol=0.0, rel_tol=1e-12)
    assert info["iterations"] == ref["iters"] == 1
    assert np.linalg.norm(host(mg.x) - ref["x"]) <= 1e-6 * np.linalg.norm(ref["x"])


def test_no_fluid():
    shape = (16, 16, 16)
    mg = MGPCG(3, shape, 2)
    mg.set_tags(torch.zeros(shape, dtype=torch.int32, device="cuda"))
    mg.init(torch.ones(shape, device="cuda"), 1.0)
    mg.mask_interior()
    info = mg.solve(200, 1e-12, 1e-12, 1e-12, smoother="phases")  # rTr0 = 0 < abs_tol
    assert info["converged"] and info["iterations"] == 0 and info["rtr0"] == 0.0
    assert float(mg.x.abs().max()) == 0.0
    info = mg.solve(5, 1e-12, 0.0, 1e-12, smoother="phases")      # tol 0: runs to max_iters, like the reference
    assert info["iterations"] == 5 and not info["converged"]


def test_non_cubic_grid_matches_oracle():
    """The reference's default grid is 256 x 64 x 256 (const_param.py:34-37); a
    32 x 8 x 32 version of it with 3 levels."""
    shape = (32, 8, 32)
    rng = np.random.default_rng(33)
    phi = (rng.uniform(-1, 1, shape) + 0.3).astype(np.float32)
    tag_o = O.tag_dirichlet(phi)
    tag_o[:, 0, :] = 1
    tag_o[0, 0, 0] = 0
    u, v, w = scenes.fourier_faces(shape, 33)
    zeros = [np.zeros_like(a) for a in (u, v, w)]
    div = O.divergence(u, v, w, *zeros, tag_o)
    r0 = np.where(tag_o == 1, div, 0).astype(np.float32)
    vel, velr = mac(u, v, w), mac(*zeros)
    assert np.array_equal(host(K.divergence(vel, velr, dev(tag_o))), div)
    mg = MGPCG(3, shape, 3)
    mg.set_tags(dev(tag_o))
    mg.init(dev(r0), 1.0)
    mg.mask_interior()
    tags = O.tag_levels(tag_o, 3)
    assert np.array_equal(host(mg.apply_preconditioner(dev(r0))), O.vcycle(r0, tags, np.float32))
    info = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    ref = O.pcg(r0, tags, max_iters=200, abs_tol=0.0, rel_tol=1e-12, dtype=np.float64)
    assert abs(info["iterations"] - ref["iters"]) <= 1
    assert np.linalg.norm(host(mg.x) - ref["x"]) <= PRESSURE_RTOL * np.linalg.norm(ref["x"])


def test_host_loop_equals_graph(monkeypatch):
    s = scenes.dam(32, seed=34, levels=3)
    tag_o, r0, mg = _setup(s)
    info_g = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    xg = host(mg.x)
    monkeypatch.setenv("FLUB_SOLVE_HOST_LOOP", "1")
    tag_o, r0, mg2 = _setup(s)
    info_h = mg2.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    assert info_h == info_g
    assert np.array_equal(host(mg2.x), xg)


def test_repeat_solves_are_deterministic():
    s = scenes.random_scene(32, 35, levels=3)
    tag_o, r0, mg = _setup(s)
    mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    x1 = host(mg.x)
    mg.init(dev(r0), 1.0)
    mg.mask_interior()
    mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    assert np.array_equal(host(mg.x), x1)


def test_nan_rhs_reports_breakdown():
    """A NaN in the right-hand side (made on the host) is reported as a CG
    breakdown, and the handle stays usable."""
    s = scenes.box(32, seed=36, levels=3)
    tag_o, r0, mg = _setup(s)
    bad = r0.copy()
    bad[tuple(np.argwhere(tag_o == 1)[0])] = np.nan
    mg.init(dev(bad), 1.0)
    mg.mask_interior()
    with pytest.raises(FlubError):
        mg.solve(50, 1e-12, 0.0, 1e-12, smoother="phases")
    mg.init(dev(r0), 1.0)
    mg.mask_interior()
    assert mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")["converged"]


def test_rejects_bad_arguments():
    with pytest.raises(ValueError):
        MGPCG(3, (30, 32, 32), 3)
    mg = MGPCG(3, (16, 16, 16), 2)
    with pytest.raises(NotImplementedError):
        mg.solve(1, smoother="default")
    with pytest.raises(ValueError):
        mg.set_tags(torch.zeros((8, 8, 8), dtype=torch.int32, device="cuda"))


def test_kernel_counter_advances():
    s = scenes.box(32, seed=37, levels=3)
    tag_o, r0, mg = _setup(s)
    k0 = mg.kernels_executed()
    info = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    # at least the V-cycle and the CG kernels of every iteration
    assert mg.kernels_executed() >= k0 + 4 * info["iterations"]


def test_reference_call_sequence():
    """example_fluid.py:84-147 with water_3d.py:58-68, written with launch()
    exactly as the reference writes it, against the fused Projection."""
    s = scenes.dam(32, seed=38, levels=3)
    shape = s.shape
    h = h0 = s.h
    tag = IntField(K.classify(dev(s.phi), s.prims, h, h0))
    vel, velr = mac(s.u, s.v, s.w), mac(s.ur, s.vr, s.wr)
    div = Field(torch.zeros(shape, device="cuda"))
    launch(K.divergence_tag, shape, [vel, div, velr, tag])
    launch(K.mask_with_tag, shape, [div, tag])
    launch(K.scale_by_3d, shape, [div, -1.0 / h])
    p0 = Field(torch.zeros(shape, device="cuda"))
    mg = MGPCG(3, shape, 3, float)
    mg.set_tags(tag.f)
    mg.init(div.f, -h0)
    mg.mask_interior()
    mg.solve(200, rel_tol=1e-12, abs_tol=0.0, smoother="phases")
    p0.f.copy_(mg.x)
    launch(K.scale_by_3d, shape, [p0, h0])
    launch(K.scale_by_3d, shape, [p0, 1.0 / h0])
    for d in (1, 2, 3):
        fs = list(shape)
        fs[d - 1] += 1
        launch(K.subtract_gradient_tag, tuple(fs), [vel, velr, p0, tag, d])
    proj = Projection(shape, 3)
    vel2 = mac(s.u, s.v, s.w)
    proj.project(vel2, velr, dev(s.phi), s.prims)
    for a, b in zip((vel.u.f, vel.v.f, vel.w.f), (vel2.u.f, vel2.v.f, vel2.w.f)):
        assert torch.equal(a, b)


# ---------------------------------------------------------------- mixed precision

@pytest.mark.parametrize("name", ["dam64", "sphere32", "rand32"])
def test_mixed_precision_solve(name):
    """FP16 V-cycle storage + flexible CG: same 1e-6 tolerance, true residual
    checked in FP64 on the host, error vs the FP64 oracle's solution bounded."""
    from oracle import np_oracle as N
    scene = SCENES[name]()
    tag_o, r0, mg = _setup(scene)
    info32 = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    mgm = MGPCG(3, scene.shape, scene.levels, float, precision="mixed")
    mgm.set_tags(dev(tag_o))
    mgm.init(dev(r0), 1.0)
    mgm.mask_interior()
    infom = mgm.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    assert infom["converged"] and infom["status"] == 0
    assert infom["iterations"] <= info32["iterations"] + 3
    x = host(mgm.x).astype(np.float64)
    x32 = host(mg.x).astype(np.float64)
    b = r0.astype(np.float64)
    # the true residual of an FP32 solution sits at the FP32 rounding floor (~1e-5
    # relative here) for the plain path as well; the mixed one must be as good
    true_plain = np.linalg.norm(N.matvec(x32, tag_o) - b)
    true_mixed = np.linalg.norm(N.matvec(x, tag_o) - b)
    assert true_mixed <= max(2.0 * true_plain, 2e-6 * np.linalg.norm(b)), (true_mixed, true_plain)
    # error against the FP64 oracle's solve at the same tolerance (rel. residual 1e-6)
    ref64 = O.pcg(r0, O.tag_levels(tag_o, scene.levels), max_iters=200, abs_tol=0.0, rel_tol=1e-12,
                  dtype=np.float64)
    err = np.linalg.norm(x - ref64["x"]) / np.linalg.norm(ref64["x"])
    assert err <= PRESSURE_RTOL, err


def test_mixed_precision_vcycle_close_to_fp32():
    scene = SCENES["dam64"]()
    tag_o, r0, mg = _setup(scene)
    mgm = MGPCG(3, scene.shape, scene.levels, float, precision="mixed")
    mgm.set_tags(dev(tag_o))
    z16 = host(mgm.apply_preconditioner(dev(r0)))
    z32 = O.vcycle(r0, O.tag_levels(tag_o, scene.levels), np.float32)
    assert np.isfinite(z16).all()
    assert np.linalg.norm(z16 - z32) <= 1e-2 * np.linalg.norm(z32)


# ---------------------------------------------------------------- V-cycle schedules (no reference counterpart)

@pytest.mark.parametrize("sched", [(2, 8, 0.5), (3, 4, 0.5), (1, 2, 1.0)])
@pytest.mark.parametrize("name", ["dam64", "rand32b"])
def test_vcycle_schedule_bit_exact(sched, name, monkeypatch):
    """A lighter V-cycle schedule with the scaled restriction against the FP32
    oracle run with the same schedule: bit-exact like the reference's, on the
    cluster path and on the fallback path."""
    scene = SCENES[name]()
    tags = None
    for no_cluster in ("0", "1"):
        if no_cluster == "1":
            monkeypatch.setenv("FLUB_NO_CLUSTER", "1")
        tag_o, r0, mg = _setup(scene)
        tags = O.tag_levels(tag_o, scene.levels)
        mg.set_schedule(*sched)
        z = host(mg.apply_preconditioner(dev(r0)))
        with O.schedule(*sched):
            z_o = O.vcycle(r0, tags, np.float32)
        assert np.array_equal(z, z_o), no_cluster


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_light_schedule_projection_matches_fp64_oracle(precision):
    """The "v22" schedule reaches the same tolerance in fewer CG iterations
    than the reference schedule; the pressure agrees with the FP64 oracle."""
    scene = scenes.dam(128, seed=2)
    ref = O.project(scene, dtype=np.float64)
    proj = Projection(scene.shape, scene.levels, precision=precision, schedule="v22")
    vel, velr = mac(scene.u, scene.v, scene.w), mac(scene.ur, scene.vr, scene.wr)
    info = proj.project(vel, velr, dev(scene.phi), scene.prims)
    assert info["converged"]
    assert info["iterations"] < ref["iters"], (info, ref["iters"])
    p = host(proj.p.f)
    err = np.linalg.norm(p - ref["p"]) / np.linalg.norm(ref["p"])
    assert err <= PRESSURE_RTOL, err


@pytest.mark.parametrize("no_cluster", ["0", "1"])
@pytest.mark.parametrize("sched", ["reference", "v22"])
def test_fp64_bottom_vcycle_bit_exact(sched, no_cluster, monkeypatch):
    """The bottom level smoothed in FP64 (flub_mg_set_bottom_precision(64), no
    reference counterpart) against the oracle doing the same, bit for bit, in
    the cluster kernel's tail and in the one-block tail kernel."""
    monkeypatch.setenv("FLUB_NO_CLUSTER", no_cluster)
    scene = SCENES["dam64"]()
    tag_o, r0, mg = _setup(scene)
    assert mg.bottom_precision() == 32
    mg.set_schedule(sched)
    z32 = host(mg.apply_preconditioner(dev(r0)))
    mg.set_bottom_precision(64)
    assert mg.bottom_precision() == 64
    z64 = host(mg.apply_preconditioner(dev(r0)))
    tags = O.tag_levels(tag_o, scene.levels)
    nu, nb, rs = (-1, 3, 1.0) if sched == "reference" else (2, 4, 0.5)
    with O.schedule(nu, nb, rs):
        assert np.array_equal(z32, O.vcycle(r0, tags, np.float32))
        with O.bottom_fp64():
            z64_o = O.vcycle(r0, tags, np.float32)
    assert np.array_equal(z64, z64_o)
    assert not np.array_equal(z64, z32)  # the bottom's arithmetic did change
    info = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
    assert info["converged"]


def test_mixed_handle_defaults_to_fp64_bottom():
    scene = SCENES["dam64"]()
    tag_o, r0, _ = _setup(scene)
    mgm = MGPCG(3, scene.shape, scene.levels, float, precision="mixed")
    assert mgm.bottom_precision() == 64
    mgm.set_bottom_precision(32)
    assert mgm.bottom_precision() == 32
    with pytest.raises(FlubError):
        mgm.set_bottom_precision(16)


@pytest.mark.parametrize("name", ["dam128", "rand128"])
@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_cluster_global_level_bit_exact(name, precision, monkeypatch):
    """The level above the cluster's distributed levels (64^3 at 128^3) run in
    the cluster kernel from global memory (opt-in, FLUB_CLUSTER_GLOBAL=1)
    against one launch per pass (the default): the same V-cycle and solve, bit
    for bit, with the reference schedule and the light one; FP32 also against
    the oracle."""
    scene = TILE_SCENES[name]()
    out = []
    for on in ("1", "0"):
        monkeypatch.setenv("FLUB_CLUSTER_GLOBAL", on)
        tag_o, r0, _ = _setup(scene)
        mg = MGPCG(3, scene.shape, scene.levels, float, precision=precision)
        mg.set_tags(dev(tag_o))
        z = host(mg.apply_preconditioner(dev(r0)))
        mg.set_schedule("v22")
        z22 = host(mg.apply_preconditioner(dev(r0)))
        mg.init(dev(r0), 1.0)
        mg.mask_interior()
        info = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
        out.append((z, z22, info["iterations"], host(mg.x).copy()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2] and np.array_equal(out[0][3], out[1][3])
    if precision == "fp32":
        tags = O.tag_levels(tag_o, scene.levels)
        assert np.array_equal(out[0][0], O.vcycle(r0, tags, np.float32))
        with O.schedule(2, 4, 0.5):
            assert np.array_equal(out[0][1], O.vcycle(r0, tags, np.float32))


def test_schedule_rejects_bad_values():
    mg = MGPCG(3, (32, 32, 32), 3, float)
    for bad in [(0, 8, 0.5), (2, 0, 0.5), (2, 8, 0.0), (2, 8, 2.0), (65, 8, 0.5)]:
        with pytest.raises(FlubError):
            mg.set_schedule(*bad)


# ---------------------------------------------------------------- TMA-tiled smoothing

TILE_SCENES = {
    "dam128": lambda: scenes.dam(128, seed=31, levels=5),
    "rand128": lambda: scenes.random_scene(128, 32, levels=5),
}


@pytest.mark.parametrize("name", sorted(TILE_SCENES))
def test_tiled_vcycle_bit_exact(name, monkeypatch):
    """The TMA-tiled smoother (two half-sweeps per launch, FLUB_TILE=1)
    against the oracle and against the row smoother, bit for bit, with the
    reference schedule and the light one."""
    scene = TILE_SCENES[name]()
    monkeypatch.setenv("FLUB_TILE", "1")
    tag_o, r0, mg = _setup(scene)
    tags = O.tag_levels(tag_o, scene.levels)
    z_tile = host(mg.apply_preconditioner(dev(r0)))
    assert np.array_equal(z_tile, O.vcycle(r0, tags, np.float32))
    mg.set_schedule(2, 4, 0.5)
    z_tile22 = host(mg.apply_preconditioner(dev(r0)))
    with O.schedule(2, 4, 0.5):
        assert np.array_equal(z_tile22, O.vcycle(r0, tags, np.float32))
    monkeypatch.setenv("FLUB_TILE", "0")
    _, _, mg_rows = _setup(scene)
    assert np.array_equal(host(mg_rows.apply_preconditioner(dev(r0))), z_tile)


@pytest.mark.parametrize("sched", ["reference", "v22"])
def test_tiled_solve_equals_row_solve(sched, monkeypatch):
    """A whole solve (level 0 tiled too, inside the CUDA graph) gives the same
    bits as the row smoother."""
    scene = TILE_SCENES["dam128"]()
    out = []
    for tile in ("1", "0"):
        monkeypatch.setenv("FLUB_TILE", tile)
        _, r0, mg = _setup(scene)
        mg.set_schedule(sched)
        info = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
        out.append((info["iterations"], host(mg.x).copy()))
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])


def test_tiled_vcycle_non_cubic_bit_exact(monkeypatch):
    """96 x 48 x 128 (tiles on levels 0 and 1, not on the 24 x 12 x 32 level
    below), with solid cells, air pockets and the domain walls."""
    shape = (96, 48, 128)
    rng = np.random.default_rng(34)
    phi = (rng.uniform(-1, 1, shape) + 0.6).astype(np.float32)
    tag_o = O.tag_dirichlet(phi)
    tag_o[rng.random(shape) < 0.05] = 2
    r0 = np.where(tag_o == 1, rng.standard_normal(shape), 0).astype(np.float32)
    out = []
    for tile in ("1", "0"):
        monkeypatch.setenv("FLUB_TILE", tile)
        mg = MGPCG(3, shape, 4)
        mg.set_tags(dev(tag_o))
        mg.init(dev(r0), 1.0)
        mg.mask_interior()
        out.append(host(mg.apply_preconditioner(dev(r0))))
        info = mg.solve(200, 1e-12, 0.0, 1e-12, smoother="phases")
        out.append((info["iterations"], host(mg.x).copy()))
    assert np.array_equal(out[0], O.vcycle(r0, O.tag_levels(tag_o, 4), np.float32))
    assert np.array_equal(out[0], out[2])
    assert out[1][0] == out[3][0] and np.array_equal(out[1][1], out[3][1])
