"""CPU oracle for flub's pressure projection -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs may
import this package.  The product library (flub_gb300) never calls it.

Two restatements of the reference algorithm live here:

* ``oracle/flub_oracle.c`` (loaded below through ctypes): FP32 and FP64
  variants.  The FP32 variant performs the same IEEE operations in the same
  order as the CUDA kernels, so single kernels match bit for bit.
* ``oracle/np_oracle.py``: an independent vectorised NumPy FP64 restatement,
  used to cross-check the C code on small grids.

Parity unpinned: the reference is Python + NVIDIA Warp, which cannot be
installed on these machines, and it ships no golden vectors for this path.
The oracle is pinned against hand-derived known-answer vectors
(tests/test_oracle_kat.py) and against the NumPy restatement.

Reference citations (paths inside the flub repository) are on each function
of flub_oracle.c.
"""
import ctypes
import os

import numpy as np

from . import build as _build

PRIM_DTYPE = np.dtype([("geometry", "<i4"), ("x", "<f4", (3,)), ("q", "<f4", (4,)),
                       ("radius", "<f4", (3,))], align=True)
assert PRIM_DTYPE.itemsize == 44

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        _declare(_lib)
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _declare(L):
    vp, i32, i64, f32, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_double
    for sfx in ("f32", "f64"):
        getattr(L, f"oracle_matvec_{sfx}").argtypes = [vp, vp, vp, i32, i32, i32]
        getattr(L, f"oracle_smooth_{sfx}").argtypes = [vp, vp, vp, i32, i32, i32, i32]
        getattr(L, f"oracle_restrict_{sfx}").argtypes = [vp, vp, vp, vp, vp, i32, i32, i32]
        getattr(L, f"oracle_prolong_{sfx}").argtypes = [vp, vp, i32, i32, i32]
        getattr(L, f"oracle_dot_{sfx}").argtypes = [vp, vp, i32, i32, i32]
        getattr(L, f"oracle_dot_{sfx}").restype = f64
        getattr(L, f"oracle_zero_centered_{sfx}").argtypes = [vp, vp, i32, i32, i32]
        getattr(L, f"oracle_vcycle_levels_{sfx}").argtypes = [vp, vp, vp, i32, i32, i32, i32]
        fn = getattr(L, f"oracle_pcg_{sfx}")
        fn.argtypes = [vp, vp, vp, i32, i32, i32, i32, i32, f64, f64, f64, i32, vp, vp, vp, vp, vp]
        fn.restype = i32
    L.oracle_restrict_tag_f32.argtypes = [vp, vp, i32, i32, i32]
    L.oracle_phi_prims.argtypes = [vp, i32, i32, i32, f32, f32, vp, vp, i32]
    L.oracle_tag_dirichlet.argtypes = [vp, vp, i64]
    L.oracle_tag_neumann.argtypes = [vp, vp, i64]
    L.oracle_divergence.argtypes = [vp] * 8 + [i32, i32, i32]
    L.oracle_mask_with_tag.argtypes = [vp, vp, i64]
    L.oracle_scale.argtypes = [vp, f32, i64]
    L.oracle_subtract_gradient.argtypes = [vp, vp, vp, vp, i32, i32, i32, i32]
    L.oracle_num_threads.restype = i32
    L.oracle_set_schedule.argtypes = [i32, i32, f64]
    L.oracle_set_schedule.restype = None
    L.oracle_set_bottom_fp64.argtypes = [i32]
    L.oracle_set_bottom_fp64.restype = None
    L.oracle_solid_vel.argtypes = [vp, vp, i32, i32, i32, i32, f32, vp, vp, vp, i32]
    L.oracle_fraction_quad.argtypes = [f32, f32, f32, f32, f32]
    L.oracle_fraction_quad.restype = f32
    L.oracle_phi_to_fraction.argtypes = [vp, vp, i32, i32, i32, i32]
    L.oracle_divergence_fractional.argtypes = [vp] * 10 + [i32, i32, i32]
    L.oracle_subtract_gradient_batty.argtypes = [vp] * 5 + [i32, i32, i32, i32, f32, f32]
    L.oracle_set_unknown.argtypes = [vp, vp, vp, vp, i32, i32, i32]
    L.oracle_extrapolate_axis.argtypes = [vp, vp, i32, i32, i32]
    L.oracle_flush_unknown.argtypes = [vp, i64]
    L.oracle_advect_mc.argtypes = [vp, vp, vp, i32, i32, i32, vp, vp, vp, i32, i32, i32, vp, f32, f32, f32, i32]
    L.oracle_advect_phi.argtypes = [vp, vp, vp, i32, i32, i32, vp, vp, i32, i32, i32, vp, f32, f32, f32]
    L.oracle_advect_simple.argtypes = [vp, vp, vp, i32, i32, i32, vp, vp, i32, i32, i32, f32, f32]
    L.oracle_sample_velocity.argtypes = [vp, vp, vp, i32, i32, i32, vp, vp]
    L.oracle_backtrace.argtypes = [vp, vp, vp, i32, i32, i32, vp, f32, f32]
    L.oracle_tricubic.argtypes = [vp, i32, i32, i32, f32, f32, f32]
    L.oracle_tricubic.restype = f32
    L.oracle_redistance_init.argtypes = [vp, vp, i32, i32, i32, f32, i32]
    L.oracle_redistance_sweep.argtypes = [vp, i32, i32, i32, i32, i32, i32, i32, f32]
    L.oracle_redistance.argtypes = [vp, i32, i32, i32, f32, i32, i32]


REFERENCE_SCHEDULE = (-1, 3, 1.0)


class schedule:
    """Context manager: run the oracle's V-cycle with another schedule
    (iterations per side at every level, or -1 for the reference's 6 << l;
    iterations of each bottom order; restriction scale), restoring the
    reference's afterwards.  No reference counterpart."""

    def __init__(self, nu=-1, bottom=3, rscale=1.0):
        self.args = (int(nu), int(bottom), float(rscale))

    def __enter__(self):
        lib().oracle_set_schedule(*self.args)
        return self

    def __exit__(self, *exc):
        lib().oracle_set_schedule(*REFERENCE_SCHEDULE)
        return False


class bottom_fp64:
    """Context manager: the FP32 V-cycle smooths its bottom level in FP64
    (the library's flub_mg_set_bottom_precision(64)); no reference
    counterpart."""

    def __enter__(self):
        lib().oracle_set_bottom_fp64(1)
        return self

    def __exit__(self, *exc):
        lib().oracle_set_bottom_fp64(0)
        return False


def num_threads() -> int:
    return lib().oracle_num_threads()


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _sfx(dtype):
    return "f32" if np.dtype(dtype) == np.float32 else "f64"


# ---------------------------------------------------------------- geometry

def tag_dirichlet(phi):
    """geometry.py:335-344 _tag_dirichlet: tag = 0 where phi > 0, else 1."""
    phi = _c(phi, np.float32)
    tag = np.empty(phi.shape, np.int32)
    lib().oracle_tag_dirichlet(_ptr(phi), _ptr(tag), phi.size)
    return tag


def phi_prims(shape, h, h0, prims, stagger=(0.5, 0.5, 0.5)):
    """geometry.py:225-239 precompute_grid_point_phi_prims (primitive SDF min)."""
    prims = np.ascontiguousarray(prims, dtype=PRIM_DTYPE)
    st = np.asarray(stagger, np.float32)
    phi = np.empty(shape, np.float32)
    lib().oracle_phi_prims(_ptr(phi), shape[0], shape[1], shape[2], h, h0, _ptr(st), _ptr(prims), len(prims))
    return phi


def tag_neumann(phi_rigid, tag):
    """geometry.py:390-397 _tag_neumann (in place): tag = 2 where phi_rigid < 0."""
    phi_rigid = _c(phi_rigid, np.float32)
    assert tag.dtype == np.int32 and tag.flags.c_contiguous
    lib().oracle_tag_neumann(_ptr(phi_rigid), _ptr(tag), tag.size)
    return tag


def classify(phi, prims, h, h0):
    """Dh(): _tag_dirichlet, phi_rigid from primitives at cell centres, _tag_neumann
    (example_fluid.py:96-114, water_3d.py:55-56).  Returns (tag, phi_rigid)."""
    tag = tag_dirichlet(phi)
    phi_rigid = phi_prims(phi.shape, h, h0, prims)
    tag_neumann(phi_rigid, tag)
    return tag, phi_rigid


# ---------------------------------------------------------------- divergence / gradient

def divergence(u, v, w, ur, vr, wr, tag):
    """divergence.py:43-99 divergence_tag (unmasked, unscaled)."""
    nx, ny, nz = tag.shape
    args = [_c(a, np.float32) for a in (u, v, w, ur, vr, wr)]
    tag = _c(tag, np.int32)
    div = np.empty(tag.shape, np.float32)
    lib().oracle_divergence(*[_ptr(a) for a in args], _ptr(tag), _ptr(div), nx, ny, nz)
    return div


def mask_with_tag(div, tag):
    """divergence.py:173-180 (in place)."""
    lib().oracle_mask_with_tag(_ptr(div), _ptr(_c(tag, np.int32)), div.size)
    return div


def scale(q, s):
    """utils/util.py:162-165 scale_by_3d (in place, FP32)."""
    assert q.dtype == np.float32 and q.flags.c_contiguous
    lib().oracle_scale(_ptr(q), s, q.size)
    return q


def subtract_gradient(uf, urf, p, tag, d):
    """subtract_gradient.py:37-68 for axis d in {1, 2, 3} (in place on uf)."""
    nx, ny, nz = tag.shape
    assert uf.dtype == np.float32 and uf.flags.c_contiguous
    lib().oracle_subtract_gradient(_ptr(uf), _ptr(_c(urf, np.float32)), _ptr(_c(p, np.float32)),
                                   _ptr(_c(tag, np.int32)), nx, ny, nz, d)
    return uf


# ---------------------------------------------------------------- rigid face velocities, cut cells

def solid_vel(ur, owner, d, h0, bx, bv, bw):
    """rigid_coupling.py:51-70 precompute_solid_vel on the face array of axis d (in place)."""
    assert ur.dtype == np.float32 and ur.flags.c_contiguous
    bx, bv, bw = (np.ascontiguousarray(a, np.float32).reshape(-1, 3) for a in (bx, bv, bw))
    lib().oracle_solid_vel(_ptr(ur), _ptr(_c(owner, np.int32)), *ur.shape, int(d), float(h0), _ptr(bx), _ptr(bv),
                           _ptr(bw), bx.shape[0])
    return ur


def fraction_quad(ya, yb, yc, yd, yctr):
    """utils/util.py:221-228 fraction_quad."""
    return float(lib().oracle_fraction_quad(ya, yb, yc, yd, yctr))


def phi_to_fraction(phi_nodes, frac, d):
    """geometry.py phi_to_fraction (in place on frac, which holds the face-centre SDF)."""
    nx, ny, nz = (s - 1 for s in phi_nodes.shape)
    assert frac.dtype == np.float32 and frac.flags.c_contiguous
    lib().oracle_phi_to_fraction(_ptr(_c(phi_nodes, np.float32)), _ptr(frac), nx, ny, nz, int(d))
    return frac


def divergence_fractional(u, v, w, fu, fv, fw, ur, vr, wr):
    """divergence.py:4-42 divergence_fractional_3d."""
    nx, ny, nz = u.shape[0] - 1, u.shape[1], u.shape[2]
    div = np.zeros((nx, ny, nz), np.float32)
    arrs = [_c(a, np.float32) for a in (u, v, w)]
    lib().oracle_divergence_fractional(*(_ptr(a) for a in arrs), _ptr(div),
                                       *(_ptr(_c(a, np.float32)) for a in (fu, fv, fw, ur, vr, wr)), nx, ny, nz)
    return div


def subtract_gradient_batty(uf, p, frac, phi, urf, d, lo, h):
    """subtract_gradient.py:7-122 u/v/w_subtract_gradient_batty_3d (in place on uf)."""
    nx, ny, nz = phi.shape
    assert uf.dtype == np.float32 and uf.flags.c_contiguous
    lib().oracle_subtract_gradient_batty(_ptr(uf), _ptr(_c(p, np.float32)), _ptr(_c(frac, np.float32)),
                                         _ptr(_c(phi, np.float32)), _ptr(_c(urf, np.float32)), nx, ny, nz, int(d),
                                         float(lo), float(h))
    return uf


# ---------------------------------------------------------------- velocity extrapolation

def set_unknown(phi, tu, tv, tw):
    """utils/util.py:423-437 set_unknown (in place on the three int32 flag arrays)."""
    nx, ny, nz = phi.shape
    for t in (tu, tv, tw):
        assert t.dtype == np.int32 and t.flags.c_contiguous
    lib().oracle_set_unknown(_ptr(_c(phi, np.float32)), _ptr(tu), _ptr(tv), _ptr(tw), nx, ny, nz)


def extrapolate_axis(q, unk):
    """extrapolate.py:8-30 extrapolate_3d on one face array (in place)."""
    assert q.dtype == np.float32 and q.flags.c_contiguous and unk.dtype == np.int32 and unk.flags.c_contiguous
    lib().oracle_extrapolate_axis(_ptr(q), _ptr(unk), *q.shape)


def flush_unknown(unk):
    """extrapolate.py:32-36 flush_1_3d (in place)."""
    lib().oracle_flush_unknown(_ptr(unk), unk.size)


def extrapolate(u, v, w, tu, tv, tw, phi, n_cells):
    """water_3d.py:70-73 extrapolate: set_unknown, then n_cells times
    extrapolate_by_1 (extrapolate.py:39-47), all in place."""
    set_unknown(phi, tu, tv, tw)
    for _ in range(n_cells):
        for q, t in ((u, tu), (v, tv), (w, tw)):
            extrapolate_axis(q, t)
        for t in (tu, tv, tw):
            flush_unknown(t)


# ---------------------------------------------------------------- advection

def _vel(u, v, w):
    u, v, w = (_c(a, np.float32) for a in (u, v, w))
    nx, ny, nz = v.shape[0], u.shape[1], u.shape[2]
    assert u.shape == (nx + 1, ny, nz) and v.shape == (nx, ny + 1, nz) and w.shape == (nx, ny, nz + 1)
    return u, v, w, (nx, ny, nz)


STAGGER = {0: (0.5, 0.5, 0.5), 1: (0.0, 0.5, 0.5), 2: (0.5, 0.0, 0.5), 3: (0.5, 0.5, 0.0)}


def advect_mc(u, v, w, q_in, stagger, dt, h, minmax_h=None, stage=0, q_out=None, q_tmp=None):
    """advect.py:57-128: _advect_mc_1/2/3 (stage 1, 2, 3; q_out and q_tmp
    updated in place and returned) or the whole advect_mc (stage 0: a new
    q_out).  minmax_h: the divisor of sample_minmax (the reference's h0, the
    default)."""
    u, v, w, (nx, ny, nz) = _vel(u, v, w)
    q_in = _c(q_in, np.float32)
    q_out = np.zeros_like(q_in) if q_out is None else q_out
    q_tmp = np.zeros_like(q_in) if q_tmp is None else q_tmp
    for a in (q_out, q_tmp):
        assert a.dtype == np.float32 and a.flags.c_contiguous and a.shape == q_in.shape
    st = np.asarray(stagger, np.float32)
    lib().oracle_advect_mc(_ptr(u), _ptr(v), _ptr(w), nx, ny, nz, _ptr(q_in), _ptr(q_out), _ptr(q_tmp), *q_in.shape,
                           _ptr(st), dt, h, h if minmax_h is None else minmax_h, int(stage))
    return q_out if stage != 2 else q_tmp


def advect_velocity_mc(u, v, w, dt, h, minmax_h=None):
    """advect.py:130-133 advect_uv_mc: the three face arrays advected by
    themselves; returns (u_out, v_out, w_out)."""
    return tuple(advect_mc(u, v, w, q, STAGGER[d], dt, h, minmax_h) for d, q in ((1, u), (2, v), (3, w)))


def advect_phi(u, v, w, phi, dt, h, outside=None, stagger=(0.5, 0.5, 0.5)):
    """advect.py:39-54 advect_phi (outside = h0 by default, as the reference)."""
    u, v, w, (nx, ny, nz) = _vel(u, v, w)
    phi = _c(phi, np.float32)
    out = np.empty_like(phi)
    st = np.asarray(stagger, np.float32)
    lib().oracle_advect_phi(_ptr(u), _ptr(v), _ptr(w), nx, ny, nz, _ptr(phi), _ptr(out), *phi.shape, _ptr(st), dt,
                            h, h if outside is None else outside)
    return out


def advect_simple(u, v, w, q, dt, h):
    """advect.py:24-37 advect_simple_3d (trilinear, cell-centred q)."""
    u, v, w, (nx, ny, nz) = _vel(u, v, w)
    q = _c(q, np.float32)
    out = np.empty_like(q)
    lib().oracle_advect_simple(_ptr(u), _ptr(v), _ptr(w), nx, ny, nz, _ptr(q), _ptr(out), *q.shape, dt, h)
    return out


def sample_velocity(u, v, w, p):
    """utils/util.py:34-88 sample_velocity_3d at one point (grid units)."""
    u, v, w, (nx, ny, nz) = _vel(u, v, w)
    pp = np.asarray(p, np.float32).copy()
    out = np.empty(3, np.float32)
    lib().oracle_sample_velocity(_ptr(u), _ptr(v), _ptr(w), nx, ny, nz, _ptr(pp), _ptr(out))
    return out


def backtrace(u, v, w, p, dt, h):
    """advect.py:10-22 backtrace of one point (grid units)."""
    u, v, w, (nx, ny, nz) = _vel(u, v, w)
    pp = np.asarray(p, np.float32).copy()
    lib().oracle_backtrace(_ptr(u), _ptr(v), _ptr(w), nx, ny, nz, _ptr(pp), dt, h)
    return pp


def tricubic(q, s, t, r):
    """utils/util.py:148-160 _tricubic at index-space point (s, t, r)."""
    q = _c(q, np.float32)
    return float(lib().oracle_tricubic(_ptr(q), *q.shape, s, t, r))


# ---------------------------------------------------------------- redistance

REDISTANCE_DIRECTIONS = ((1, 1, -1), (-1, 1, -1), (-1, -1, -1), (1, -1, -1),
                         (1, 1, 1), (-1, 1, 1), (-1, -1, 1), (1, -1, 1))


def redistance_init(phi, h, set_boundary=1):
    """redistance.py:66-119 _init_distance (every cell reads the values from
    before the launch); returns a new array."""
    phi = _c(phi, np.float32)
    out = np.empty_like(phi)
    lib().oracle_redistance_init(_ptr(phi), _ptr(out), *phi.shape, h, int(set_boundary))
    return out


def redistance_sweep(phi, incx, incy, incz, odd, h):
    """redistance.py:58-63 _sweep, in place."""
    assert phi.dtype == np.float32 and phi.flags.c_contiguous
    lib().oracle_redistance_sweep(_ptr(phi), *phi.shape, incx, incy, incz, int(odd), h)


def redistance(phi, h, set_boundary=1, n_rounds=2):
    """redistance.py:125-136 redistance; returns a new array."""
    out = _c(phi, np.float32).copy()
    lib().oracle_redistance(_ptr(out), *out.shape, h, int(set_boundary), int(n_rounds))
    return out


# ---------------------------------------------------------------- multigrid

def tag_levels(tag, levels):
    """multigrid/mgpcg.py:360-370 set_tags: the restricted tag hierarchy."""
    out = [_c(tag, np.int32)]
    for _ in range(levels - 1):
        f = out[-1]
        c = np.empty((f.shape[0] // 2, f.shape[1] // 2, f.shape[2] // 2), np.int32)
        lib().oracle_restrict_tag_f32(_ptr(f), _ptr(c), *c.shape)
        out.append(c)
    return out


def matvec(p, tag):
    """multigrid/mgpcg.py:36-39 compute_Ap_mcadams: L p."""
    p = np.ascontiguousarray(p)
    Ap = np.empty_like(p)
    getattr(lib(), f"oracle_matvec_{_sfx(p.dtype)}")(_ptr(p), _ptr(_c(tag, np.int32)), _ptr(Ap), *tag.shape)
    return Ap


def smooth(z, r, tag, phase):
    """multigrid/mgpcg.py:72-86 one red-black half-sweep (in place on z)."""
    getattr(lib(), f"oracle_smooth_{_sfx(z.dtype)}")(_ptr(z), _ptr(_c(r, z.dtype)), _ptr(_c(tag, np.int32)),
                                                     *tag.shape, phase)
    return z


def restrict(rf, zf, tagf, tagc):
    """multigrid/mgpcg.py:94-101 residual + restriction (gather form)."""
    dt = rf.dtype
    rc = np.empty(tagc.shape, dt)
    getattr(lib(), f"oracle_restrict_{_sfx(dt)}")(_ptr(_c(rf, dt)), _ptr(_c(zf, dt)), _ptr(_c(tagf, np.int32)),
                                                  _ptr(rc), _ptr(_c(tagc, np.int32)), *tagc.shape)
    return rc


def prolong(zf, zc):
    """multigrid/mgpcg.py:113-116 (in place on zf)."""
    getattr(lib(), f"oracle_prolong_{_sfx(zf.dtype)}")(_ptr(zf), _ptr(_c(zc, zf.dtype)), *zf.shape)
    return zf


def _tag_ptr_array(tags):
    arr = (ctypes.c_void_p * len(tags))(*[t.ctypes.data for t in tags])
    return arr


def vcycle(r, tags, dtype=np.float32):
    """multigrid/mgpcg.py:296-349 apply_preconditioner: z = M r."""
    r = np.array(r, dtype=dtype, copy=True, order="C")
    z = np.zeros_like(r)
    tags = [_c(t, np.int32) for t in tags]
    arr = _tag_ptr_array(tags)
    getattr(lib(), f"oracle_vcycle_levels_{_sfx(dtype)}")(_ptr(r), _ptr(z), arr, len(tags), *r.shape)
    return z


def dot(a, b):
    a = np.ascontiguousarray(a)
    return getattr(lib(), f"oracle_dot_{_sfx(a.dtype)}")(_ptr(a), _ptr(_c(b, a.dtype)), *a.shape)


def pcg(rhs, tags, max_iters=200, eps=1e-12, abs_tol=1e-12, rel_tol=1e-12, smoother="phases",
        x0=None, dtype=np.float32, history=False):
    """multigrid/mgpcg.py:378-462 MGPCG.solve.  ``rhs`` is the masked r0 (init +
    mask_interior).  Returns a dict with x, iters, rtr, rtr0, converged."""
    if smoother not in ("phases", "fraction"):
        raise ValueError("smoother must be 'phases' or 'fraction'")
    r = np.array(rhs, dtype=dtype, copy=True, order="C")
    x = np.zeros_like(r)
    tags = [_c(t, np.int32) for t in tags]
    arr = _tag_ptr_array(tags)
    rtr = ctypes.c_double()
    rtr0 = ctypes.c_double()
    conv = ctypes.c_int()
    cap = max_iters if max_iters >= 0 else 100000
    hist = np.zeros(max(cap, 1), np.float64)
    x0p = None
    if x0 is not None:
        x0 = _c(x0, dtype)
        x0p = _ptr(x0)
    it = getattr(lib(), f"oracle_pcg_{_sfx(dtype)}")(
        _ptr(x), _ptr(r), arr, len(tags), *r.shape, max_iters, eps, abs_tol, rel_tol,
        1 if smoother == "fraction" else 0, x0p, ctypes.byref(rtr), ctypes.byref(rtr0), ctypes.byref(conv),
        _ptr(hist))
    out = dict(x=x, r=r, iters=it, rtr=rtr.value, rtr0=rtr0.value, converged=bool(conv.value))
    if history:
        n = it + 1 if conv.value else it
        out["history"] = hist[:n].copy()
    return out


# ---------------------------------------------------------------- the whole projection

def project(scene, max_iters=200, rel_tol=1e-12, abs_tol=0.0, eps=1e-12, smoother="phases",
            dtype=np.float32, x0=None):
    """Example.project (example_fluid.py:120-147) with WaterExample3d.call_mgpcg
    (water_3d.py:58-68) and the classification of Dh() (example_fluid.py:96-114):

    tag <- classify(phi, prims); div <- -1/h * mask(divergence_tag(vel)); r0 <-
    mask(-h0 * div); solve; p <- x * h0; vel <- subtract_gradient(vel, p / h0 * ...).

    For power-of-two grids -1/h * -h0 == 1 exactly, so r0 is the unscaled face
    divergence and the velocity update uses x directly.  Returns a dict with the
    tags, div, pressure p (= x * h0), the projected faces and solver info."""
    tag, phi_rigid = classify(scene.phi, scene.prims, scene.h, scene.h0)
    div = divergence(scene.u, scene.v, scene.w, scene.ur, scene.vr, scene.wr, tag)
    mask_with_tag(div, tag)
    scale(div, np.float32(-1.0 / scene.h))
    r0 = div.copy()
    scale(r0, np.float32(-scene.h0))
    mask_with_tag(r0, tag)
    tags = tag_levels(tag, scene.levels)
    res = pcg(r0.astype(dtype), tags, max_iters=max_iters, eps=eps, abs_tol=abs_tol, rel_tol=rel_tol,
              smoother=smoother, x0=x0, dtype=dtype)
    x32 = res["x"].astype(np.float32)
    p = x32.copy()
    scale(p, np.float32(scene.h0))
    pg = p.copy()
    scale(pg, np.float32(1.0 / scene.h0))
    u, v, w = (np.array(a, np.float32, copy=True) for a in (scene.u, scene.v, scene.w))
    subtract_gradient(u, scene.ur, pg, tag, 1)
    subtract_gradient(v, scene.vr, pg, tag, 2)
    subtract_gradient(w, scene.wr, pg, tag, 3)
    return dict(tag=tag, phi_rigid=phi_rigid, div=div, r0=r0, tags=tags, x=res["x"], p=p, u=u, v=v, w=w,
                iters=res["iters"], rtr=res["rtr"], rtr0=res["rtr0"], converged=res["converged"])


def max_abs_div(u, v, w, ur, vr, wr, tag):
    """Post-projection check (example_fluid.py:146-147): max |div u| over fluid cells."""
    d = divergence(u, v, w, ur, vr, wr, tag)
    d = np.where(tag == 1, d, 0.0)
    return float(np.max(np.abs(d))) if d.size else 0.0
