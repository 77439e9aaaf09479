"""Golden fixtures for the widening rows, computed by the reference's OWN
kernels -- test infrastructure only.

The rows on either side of the projection: velocity extrapolation
(utils/util.py set_unknown, extrapolate.py), solid face velocities and cut
cells (rigid_coupling.py precompute_solid_vel, geometry.py phi_to_fraction,
divergence.py divergence_fractional_3d, subtract_gradient.py
u/v/w_subtract_gradient_batty_3d), advection (advect.py) and level-set
redistancing (redistance.py).  Their unmodified kernels run on the CPU through
the stand-in for ``warp`` (oracle/warp_cpu, see make_ref_golden.py) on small
seeded inputs; inputs and outputs go to tests/golden/refw_<case>.npz, which
tests/test_ref_golden_widen.py compares with the oracle and
tests/test_gpu_ref_golden_widen.py with the CUDA path.

Launch sequences follow the reference's host functions.  Where those launch
over the configured grid (extrapolate_by_1 over const_param.shapeu ...), the
same kernels are launched over the fixture's arrays in the same order.  The
kernels read the module constants the reference defines for them (dt = 0.01
and h0 = 1/256 of the dam-break configuration); the fixtures record both.

redistance.py's _init_distance reads the neighbours of the cell it writes in
the same array.  That is a data race under Warp; the fixture runs it with
every read seeing the values from before the launch (all loads of the launch
ahead of its stores, one of the outcomes the race allows), which is the
reading the oracle and the CUDA kernel implement.  All other kernels here are
race-free.

Run from the repository root: python tests/golden/make_ref_widen.py
[reference_dir] (default /root/reference); minutes on one core.
"""
import contextlib
import io
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from tests.golden.make_ref_golden import DEFAULT_REFERENCE, import_reference  # noqa: E402

SHAPE = (10, 12, 14)  # non-cubic, nz not a multiple of 8
CASES = ("adv", "ext", "red", "cut")


def import_widen(reference):
    """The projection modules plus the widening rows' modules."""
    mods = import_reference(reference)
    with contextlib.redirect_stdout(io.StringIO()):
        import advect
        import extrapolate
        import redistance
        import rigid_coupling
    return mods, advect, extrapolate, redistance, rigid_coupling


class _Snapshot:
    """An array argument whose reads see the values from before the launch and
    whose writes go to the live array."""

    def __init__(self, live):
        self.live = live
        self.frozen = np.array(live, copy=True)
        self.shape = live.shape

    def __getitem__(self, idx):
        return self.frozen[idx]

    def __setitem__(self, idx, v):
        self.live[idx] = v


def _face_shapes(shape):
    nx, ny, nz = shape
    return (nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)


def compute_case(name, reference):
    (wp, C, G, D, S, M, U), A, E, R, RC = import_widen(reference)
    rng = np.random.default_rng({"adv": 71, "ext": 72, "red": 73, "cut": 74}[name])
    shape = SHAPE
    fs = _face_shapes(shape)
    stag = {0: (0.5, 0.5, 0.5), 1: (0.0, 0.5, 0.5), 2: (0.5, 0.0, 0.5), 3: (0.5, 0.5, 0.0)}
    h0 = np.float32(C.h0)
    out = {"shape": np.array(shape, np.int32), "h0": h0, "dt": np.float32(C.dt)}

    def field(arr, d, dtype=float):
        f = C.Field() if dtype is float else C.IntField()
        f.f = wp.array(np.ascontiguousarray(arr), dtype=dtype)
        f.d = d
        f.stagger = wp.vec3(*stag[d])
        return f

    def mac(arrs, dtype=float):
        g = C.MACGrid() if dtype is float else C.MACGridInt()
        g.u, g.v, g.w = (field(a, d + 1, dtype) for d, a in enumerate(arrs))
        return g

    if name == "adv":
        # velocities of up to a few cells per step (dt / h0 = 2.56): traces
        # leave the grid on every side
        vel0 = [(rng.standard_normal(s) * 1.5).astype(np.float32) for s in fs]
        phi0 = (rng.standard_normal(shape) * 0.1).astype(np.float32)
        q0 = rng.standard_normal(shape).astype(np.float32)
        out.update(u=vel0[0], v=vel0[1], w=vel0[2], phi=phi0, q=q0)
        vel = mac(vel0)
        phi, new_phi = field(phi0, 0), field(np.zeros(shape, np.float32), 0)
        wp.launch(A.advect_phi, dim=shape, inputs=[vel, phi, new_phi])
        out["advect_phi"] = new_phi.f.numpy().copy()
        vel_out = mac([np.zeros(s, np.float32) for s in fs])
        A.advect_uv_mc(vel, vel_out)
        for k, f in zip("uvw", (vel_out.u, vel_out.v, vel_out.w)):
            out["advect_mc_" + k] = f.f.numpy().copy()
        qn = wp.zeros(shape, dtype=float)
        wp.launch(A.advect_simple_3d, dim=shape,
                  inputs=[vel.u.f, vel.v.f, vel.w.f, wp.array(q0, dtype=float), qn, float(C.dt), float(h0)])
        out["advect_simple"] = qn.numpy().copy()
    elif name == "ext":
        # water below a sloped surface; velocities everywhere, flags from phi
        vel0 = [rng.standard_normal(s).astype(np.float32) for s in fs]
        x = np.arange(shape[0])[:, None, None]
        y = np.arange(shape[1])[None, :, None]
        z = np.arange(shape[2])[None, None, :]
        phi0 = ((y - 4.0 - 0.3 * x - 0.1 * z) * 0.1 + rng.standard_normal(shape) * 0.02).astype(np.float32)
        tags0 = [np.full(s, 7, np.int32) for s in fs]  # the last face layer keeps what it held
        out.update(u=vel0[0], v=vel0[1], w=vel0[2], phi=phi0, tu=tags0[0], tv=tags0[1], tw=tags0[2],
                   n_cells=np.int32(3))
        vel, tags = mac(vel0), mac(tags0, int)
        # water_3d.py:70-73 extrapolate: set_unknown, then extrapolate_by_1
        # (extrapolate.py:39-47) n_cells times
        wp.launch(U.set_unknown, dim=shape, inputs=[field(phi0, 0), tags])
        for _ in range(3):
            for d, s in zip((1, 2, 3), fs):
                wp.launch(E.extrapolate_3d, dim=s, inputs=[vel, tags, d])
            for t, s in zip((tags.u, tags.v, tags.w), fs):
                wp.launch(E.flush_1_3d, dim=s, inputs=[t.f])
        for k, f in zip("uvw", (vel.u, vel.v, vel.w)):
            out["ext_" + k] = f.f.numpy().copy()
        for k, f in zip("uvw", (tags.u, tags.v, tags.w)):
            out["ext_t" + k] = f.f.numpy().copy()
    elif name == "red":
        # a sphere of water in a box, the level set off by a random factor
        x, y, z = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
        d = np.sqrt((x - 4.5) ** 2 + (y - 6.0) ** 2 + (z - 7.0) ** 2) - 3.3
        phi0 = (d * h0 * (0.6 + 0.8 * rng.random(shape))).astype(np.float32)
        phi0[1, 1, 1] = -phi0[1, 1, 1] if phi0[1, 1, 1] > 0 else phi0[1, 1, 1]  # an isolated pocket
        out["phi"] = phi0
        for sb in (1, 0):
            phi = wp.array(phi0.copy(), dtype=float)
            snap = _Snapshot(phi)
            wp.launch(R._init_distance, dim=shape, inputs=[snap, float(h0), sb])
            out[f"init_sb{sb}"] = phi.numpy().copy()
            # redistance.py:125-136 after the init: two rounds of the eight sweeps
            for _ in range(2):
                for inc in ((1, 1, -1), (-1, 1, -1), (-1, -1, -1), (1, -1, -1),
                            (1, 1, 1), (-1, 1, 1), (-1, -1, 1), (1, -1, 1)):
                    R.sweep(phi, float(h0), *inc)
            out[f"redistance_sb{sb}"] = phi.numpy().copy()
    elif name == "cut":
        nx, ny, nz = shape
        # solid level set at the nodes and at the face centres, with faces in
        # the solid, in the fluid and cut
        xn, yn, zn = np.meshgrid(*(np.arange(n + 1) for n in shape), indexing="ij")
        phin = (np.sqrt((xn - 5.2) ** 2 + (yn - 5.7) ** 2 + (zn - 7.1) ** 2) - 3.4 +
                rng.standard_normal(xn.shape) * 0.3).astype(np.float32) * h0
        fc = [(rng.standard_normal(s) * 2.0 * h0).astype(np.float32) for s in fs]
        out.update(phin=phin, fc_u=fc[0], fc_v=fc[1], fc_w=fc[2])
        frac = mac(fc)
        # phi_to_fraction reads phi[i, j + 1, k] and phi[i, j + 1, k + 1] before
        # its branch on the axis, also for the v and w faces, whose last row
        # or column then reads one node past the array (Warp does not check;
        # the values are overwritten unused).  A node array padded by a layer
        # of NaN keeps those reads in bounds and changes nothing else.
        phin_pad = np.full((nx + 2, ny + 2, nz + 2), np.nan, np.float32)
        phin_pad[:nx + 1, :ny + 1, :nz + 1] = phin
        for d, s in zip((1, 2, 3), fs):
            wp.launch(G.phi_to_fraction, dim=s, inputs=[wp.array(phin_pad, dtype=float), frac, d])
        fr = [frac.u.f.numpy().copy(), frac.v.f.numpy().copy(), frac.w.f.numpy().copy()]
        for k, a in zip("uvw", fr):
            out["frac_" + k] = a
        # divergence with fractions and solid face velocities
        vel0 = [rng.standard_normal(s).astype(np.float32) for s in fs]
        vr0 = [rng.standard_normal(s).astype(np.float32) for s in fs]
        out.update(u=vel0[0], v=vel0[1], w=vel0[2], ur=vr0[0], vr=vr0[1], wr=vr0[2])
        div = wp.zeros(shape, dtype=float)
        wp.launch(D.divergence_fractional_3d, dim=shape,
                  inputs=[*(wp.array(a, dtype=float) for a in vel0), div,
                          *(wp.array(a, dtype=float) for a in fr), *(wp.array(a, dtype=float) for a in vr0)])
        out["div_frac"] = div.numpy().copy()
        # pressure-gradient update with cut faces (subtract_gradient.py:7-122)
        p0 = rng.standard_normal(shape).astype(np.float32)
        phic = (rng.standard_normal(shape) * 0.5).astype(np.float32)
        out.update(p=p0, phic=phic)
        kern = {1: S.u_subtract_gradient_batty_3d, 2: S.v_subtract_gradient_batty_3d,
                3: S.w_subtract_gradient_batty_3d}
        for d, k in zip((1, 2, 3), "uvw"):
            uf = wp.array(vel0[d - 1].copy(), dtype=float)
            wp.launch(kern[d], dim=fs[d - 1],
                      inputs=[uf, wp.array(p0, dtype=float), wp.array(fr[d - 1], dtype=float),
                              wp.array(phic, dtype=float), wp.array(vr0[d - 1], dtype=float), 0.0, 1.0,
                              float(1.0 / nx)])
            out["batty_" + k] = uf.numpy().copy()
        # solid face velocities of two bodies (rigid_coupling.py:51-70)
        bx = np.array([[0.3, 0.4, 0.5], [0.7, 0.2, 0.6]], np.float32)
        bv = np.array([[0.5, -0.2, 0.1], [-0.3, 0.4, 0.2]], np.float32)
        bw = np.array([[0.1, 0.7, -0.4], [-0.6, 0.2, 0.3]], np.float32)
        owners = [rng.integers(-1, 2, s).astype(np.int32) for s in fs]
        out.update(bx=bx, bv=bv, bw=bw, own_u=owners[0], own_v=owners[1], own_w=owners[2])
        xs, vs, ws = (wp.array([wp.vec3(*r) for r in a], dtype=wp.vec3) for a in (bx, bv, bw))
        vrig = mac([np.full(s, 9.0, np.float32) for s in fs])
        own = mac(owners, int)
        for d, s in zip((1, 2, 3), fs):
            wp.launch(RC.precompute_solid_vel, dim=s, inputs=[xs, vs, ws, vrig, own, d])
        for k, f in zip("uvw", (vrig.u, vrig.v, vrig.w)):
            out["solid_" + k] = f.f.numpy().copy()
    else:
        raise KeyError(name)
    return out


def _child(name, reference, q):
    try:
        q.put((name, compute_case(name, reference), None))
    except Exception as e:  # report, do not hang the parent
        import traceback
        q.put((name, None, traceback.format_exc()))


def run_case(name, reference=DEFAULT_REFERENCE):
    """compute_case in a fresh child process (the stand-in ``warp`` and the
    reference's top-level module names stay out of the caller)."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_child, args=(name, reference, q))
    p.start()
    got = q.get()
    p.join()
    if got[2]:
        raise RuntimeError(got[2])
    return got[1]


def path(name):
    return os.path.join(HERE, f"refw_{name}.npz")


def load(name):
    with np.load(path(name)) as z:
        return {k: z[k] for k in z.files}


def main():
    sys.dont_write_bytecode = True
    reference = sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REFERENCE
    for name in CASES:
        out = run_case(name, reference)
        np.savez_compressed(path(name), **out)
        print(f"{path(name)}: {len(out)} arrays")


if __name__ == "__main__":
    main()
