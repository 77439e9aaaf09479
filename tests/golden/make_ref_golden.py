"""Golden fixtures computed by the REFERENCE'S OWN CODE.

Imports the unmodified kernel files of Luke-Skycrawler/flub
(multigrid/mgpcg.py, divergence.py, subtract_gradient.py, geometry.py,
const_param.py, utils/util.py) with ``oracle/warp_cpu`` standing in for the
``warp`` module (Warp cannot be installed here), runs the projection exactly
as the reference's callers do, and stores every intermediate result:

* classification -- ``PrecomputeFaceFraction.tag_dirichlet``,
  ``phi_rigid.fill_(1.0)``, ``precompute_phi_with_cached_levelset`` at cell
  centres, ``tag_neumann`` (water_3d.py:55-56, example_fluid.py:96-114);
* the right-hand side -- ``divergence_tag``, ``mask_with_tag``,
  ``scale_by_3d(-1/h)`` (example_fluid.py:84-94);
* ``MGPCG(3, shape, levels)`` with ``set_tags``, ``init(div, -h0)``,
  ``mask_interior`` (water_3d.py:63-65); the tag hierarchy; one
  ``apply_preconditioner("phases")`` on r0; ``compute_Ap_mcadams`` on a seeded
  random vector;
* ``solve(200, rel_tol=1e-12, abs_tol=0, smoother="phases")`` with the
  iteration count it prints (its first ``graph_precondition`` call only
  captures, mgpcg.py:286-294, so it reports one iteration more than a solver
  without that quirk);
* the pressure and the velocity update -- ``scale_by_3d`` by h0, by 1/h0,
  ``subtract_gradient_tag`` on the three axes, ``scale_by_3d`` by h0
  (example_fluid.py:127-145, water_3d.py:66-68), and the post-projection
  divergence (example_fluid.py:146-147).

The grid-spacing constants ``h`` and ``h0`` that const_param.py derives from
its ``gridx`` (256) are set to 1/n for each fixture grid before the first
launch, as editing ``gridx`` in const_param.py would.

Inputs are the small seeded scenes of flub_gb300.scenes.  Run from the
repository root (in a process of its own per scene; seconds to a minute each):

    python tests/golden/make_ref_golden.py [--reference DIR] [names...]

Writes tests/golden/ref_<name>.npz.  The reference tree is read, never
written; it is not needed to load the fixtures.
"""
import argparse
import contextlib
import io
import multiprocessing as mp
import os
import re
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DEFAULT_REFERENCE = "/root/reference"


def _cases():
    sys.path.insert(0, ROOT)
    from flub_gb300 import scenes

    def rot16():
        """A dam-like scene with a rotated solid box and a solid sphere: every
        quaternion term of _sdf_cube is live."""
        s = scenes.dam(16, seed=54, levels=3)
        q = np.array([0.2, -0.3, 0.1, 0.9])
        q = tuple((q / np.linalg.norm(q)).astype(np.float32))
        s.prims = scenes.make_prims([
            dict(geometry=scenes.GEOM_BOX, x=(0.55, 0.3, 0.5), radius=(0.12, 0.08, 0.15), q=q),
            dict(geometry=scenes.GEOM_SPHERE, x=(0.2, 0.25, 0.7), radius=0.11),
        ])
        s.name = "rot16"
        return s

    return {
        "dam16": lambda: scenes.dam(16, seed=50, levels=3),
        "sphere16": lambda: scenes.sphere(16, seed=51, levels=3),
        "box16": lambda: scenes.box(16, seed=52, levels=2),
        "rand16": lambda: scenes.random_scene(16, 53, levels=3),
        "rot16": rot16,
        "rand8": lambda: scenes.random_scene(8, 55, levels=2),
        "dam32": lambda: scenes.dam(32, seed=56, levels=4),
        "sphere32": lambda: scenes.sphere(32, seed=57, levels=3),
    }


def import_reference(reference):
    """Import the reference modules with the CPU stand-in as ``warp``.  No
    bytecode is written: the reference tree stays as it is."""
    sys.dont_write_bytecode = True
    stand_in = os.path.join(ROOT, "oracle", "warp_cpu")
    for p in (reference, stand_in):
        if p in sys.path:
            sys.path.remove(p)
    sys.path.insert(0, reference)
    sys.path.insert(0, stand_in)
    import warp as wp
    assert os.path.dirname(os.path.abspath(wp.__file__)).startswith(stand_in), wp.__file__
    with contextlib.redirect_stdout(io.StringIO()):
        import const_param
        import divergence
        import geometry
        import subtract_gradient
        from multigrid import mgpcg
        from utils import util
    return wp, const_param, geometry, divergence, subtract_gradient, mgpcg, util


class _Pair:
    def __init__(self, cur):
        self.cur = cur


class _Bodies:
    """The attributes of RigidCoupling that precompute_phi_with_cached_levelset
    reads: positions, orientations, geometry descriptors and the (empty)
    cache of mesh level sets."""

    def __init__(self, wp, geometry, prims):
        xs, qs, gs = [], [], []
        for p in prims:
            xs.append(wp.vec3(*[float(a) for a in p["x"]]))
            qs.append(wp.quat(*[float(a) for a in p["q"]]))
            g = geometry.GeometryType3D()
            g.geometry = int(p["geometry"])
            g.radius = wp.vec3(*[float(a) for a in p["radius"]])
            g.rho = wp.float32(1.0)
            g.mesh_id = 0
            g.volume = wp.float32(0.0)
            gs.append(g)
        self.x_pair = _Pair(wp.array(xs, dtype=wp.vec3))
        self.theta_pair = _Pair(wp.array(qs, dtype=wp.quat))
        self.rigid_geometry = wp.array(gs, dtype=geometry.GeometryType3D)
        self.cached_levelset = {}


def compute_case(name, reference):
    """Every array of fixture ``name``, computed by the reference's code."""
    wp, C, G, D, S, M, U = import_reference(reference)
    scene = _cases()[name]()
    n = scene.shape[0]
    shape = scene.shape
    nx, ny, nz = shape
    assert nx == ny == nz, "divergence_tag uses tag.shape[0] on every axis"
    h = wp.constant(1.0 / n)
    h0 = h
    G.h, G.h0 = h, h0  # geometry.py reads them as module globals (from const_param import *)

    def field(arr, d, dtype=float):
        f = C.Field() if dtype is float else C.IntField()
        f.f = wp.array(np.ascontiguousarray(arr), dtype=dtype)
        f.d = d
        f.stagger = wp.vec3(0.5, 0.5, 0.5)
        return f

    def mac(u, v, w):
        g = C.MACGrid()
        g.u, g.v, g.w = field(u, 1), field(v, 2), field(w, 3)
        return g

    out = dict(phi=scene.phi, prims=scene.prims, u=scene.u, v=scene.v, w=scene.w, ur=scene.ur, vr=scene.vr,
               wr=scene.wr, levels=np.int32(scene.levels), h=np.float32(h), h0=np.float32(h0))

    # classification (water_3d.py:55-56 tag_dirichlet; example_fluid.py:111-114)
    pff = G.PrecomputeFaceFraction(use_mesh=False)
    tag = field(np.zeros(shape, np.int32), 0, int)
    phi = field(scene.phi, 0)
    pff.tag_dirichlet(tag, phi)
    out["tag_dirichlet"] = tag.f.numpy().copy()
    phi_rigid = field(np.zeros(shape, np.float32), 0)
    phi_rigid.f.fill_(1.0)
    rc = _Bodies(wp, G, scene.prims)
    # Called without ``owner`` the reference allocates a 1x1x1 owner array, and
    # precompute_grid_point_phi_prims (geometry.py:225-239) then writes
    # owner[i, j, k] out of its bounds because the stagger is non-zero (Warp
    # does not check; the values are never read).  A full-size array keeps
    # those writes in bounds and changes nothing else.
    owner = wp.zeros(shape, dtype=int)
    pff.precompute_phi_with_cached_levelset(phi_rigid.f, rc, owner=owner, stagger=wp.vec3(0.5, 0.5, 0.5))
    pff.tag_neumann(tag, phi_rigid)
    out["phi_rigid"] = phi_rigid.f.numpy().copy()
    out["tag"] = tag.f.numpy().copy()

    # divergence right-hand side (example_fluid.py:84-94)
    vel, vel_rigid = mac(scene.u, scene.v, scene.w), mac(scene.ur, scene.vr, scene.wr)
    div = field(np.zeros(shape, np.float32), 0)
    wp.launch(D.divergence_tag, dim=shape, inputs=[vel, div, vel_rigid, tag])
    out["div_raw"] = div.f.numpy().copy()
    wp.launch(D.mask_with_tag, dim=shape, inputs=[div, tag])
    wp.launch(U.scale_by_3d, dim=shape, inputs=[div, -1.0 / h])
    out["div"] = div.f.numpy().copy()

    # MGPCG set-up (water_3d.py:63-65)
    mg = M.MGPCG(3, shape, scene.levels, float)
    mg.set_tags(tag.f)
    for l in range(scene.levels):
        out[f"tag_l{l}"] = mg.tag[l].numpy().copy()
    mg.init(div.f, -h0)
    mg.mask_interior()
    out["r0"] = mg.r[0].numpy().copy()

    # one V-cycle on r0 and one matvec on a seeded vector
    mg.apply_preconditioner("phases")
    out["vcycle_z"] = mg.z[0].numpy().copy()
    assert np.array_equal(mg.r[0].numpy(), out["r0"])
    rng = np.random.default_rng(1000 + n)
    pv = wp.array(rng.standard_normal(shape).astype(np.float32), dtype=float)
    Ap = wp.zeros(shape, dtype=float)
    wp.launch(M.compute_Ap_mcadams, dim=shape, inputs=[Ap, pv, mg.tag[0]])
    out["mv_p"] = pv.numpy().copy()
    out["mv_Ap"] = Ap.numpy().copy()

    # the solve (water_3d.py:63-67 with the tolerance of the benchmark)
    mg.init(div.f, -h0)
    mg.mask_interior()
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        mg.solve(200, rel_tol=1e-12, abs_tol=0.0, smoother="phases")
    m = re.search(r"finished with\s+(\d+)\s+iterations", buf.getvalue())
    out["iters"] = np.int32(int(m.group(1)))
    out["x"] = mg.x.numpy().copy()

    # pressure and velocity update (water_3d.py:66-68, example_fluid.py:127-145)
    p0 = field(np.zeros(shape, np.float32), 0)
    wp.copy(p0.f, mg.x)
    wp.launch(U.scale_by_3d, dim=shape, inputs=[p0, h0])
    out["p"] = p0.f.numpy().copy()
    wp.launch(U.scale_by_3d, dim=shape, inputs=[p0, 1.0 / h0])
    out["p_grad"] = p0.f.numpy().copy()
    wp.launch(S.subtract_gradient_tag, dim=(nx + 1, ny, nz), inputs=[vel, vel_rigid, p0, tag, 1])
    wp.launch(S.subtract_gradient_tag, dim=(nx, ny + 1, nz), inputs=[vel, vel_rigid, p0, tag, 2])
    wp.launch(S.subtract_gradient_tag, dim=(nx, ny, nz + 1), inputs=[vel, vel_rigid, p0, tag, 3])
    out["u_out"] = vel.u.f.numpy().copy()
    out["v_out"] = vel.v.f.numpy().copy()
    out["w_out"] = vel.w.f.numpy().copy()

    # post-projection divergence (example_fluid.py:146-147)
    div2 = field(np.zeros(shape, np.float32), 0)
    wp.launch(D.divergence_tag, dim=shape, inputs=[vel, div2, vel_rigid, tag])
    wp.launch(D.mask_with_tag, dim=shape, inputs=[div2, tag])
    wp.launch(U.scale_by_3d, dim=shape, inputs=[div2, -1.0 / h])
    out["div_after"] = div2.f.numpy().copy()

    return out


def run_case(name, reference):
    t0 = time.time()
    out = compute_case(name, reference)
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
    return name, int(out["iters"]), time.time() - t0


def names():
    return sorted(_cases())


def load(name):
    d = np.load(os.path.join(HERE, f"ref_{name}.npz"))
    return {k: d[k] for k in d.files}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--reference", default=DEFAULT_REFERENCE)
    ap.add_argument("names", nargs="*")
    args = ap.parse_args()
    todo = args.names or names()
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(len(todo), os.cpu_count() or 1)) as pool:
        for name, iters, s in pool.starmap(run_case, [(n, args.reference) for n in todo]):
            print(f"{name}: reference solve {iters} iterations ({s:.0f} s for the fixture)")


if __name__ == "__main__":
    main()
