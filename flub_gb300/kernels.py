"""The projection path's kernels under the reference's names, with a
``launch(kernel, dim, inputs)`` that mirrors ``wp.launch`` so that the call
sites in example_fluid.py / water_3d.py only change their import line:

    wp.launch(divergence_tag, dim=shape, inputs=[vel, div, vel_rigid, tag])
    wp.launch(mask_with_tag, dim=shape, inputs=[div, tag])
    wp.launch(scale_by_3d, dim=shape, inputs=[div, -1.0 / h])
    wp.launch(subtract_gradient_tag, dim=shapeu, inputs=[vel, vel_rigid, p, tag, 1])
    wp.launch(_tag_dirichlet, dim=shape, inputs=[tag, phi])
    wp.launch(_tag_neumann, dim=shape, inputs=[tag, phi_rigid])
    wp.launch(precompute_grid_point_phi_prims, dim=shape,
              inputs=[phi, owner, x, q, geometry, stagger])

Every kernel runs on the GPU through the C ABI (include/flub_gb300.h) on the
current torch stream.  Each function also exists as a plain call
(``divergence``, ``classify``, ...).
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .fields import Field, IntField, MACGrid, field_shape


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t, dtype, shape=None, name="array"):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name}: expected a torch tensor, got {type(t).__name__}")
    if not t.is_cuda:
        raise ValueError(f"{name}: tensor must be on a CUDA device")
    if t.dtype != dtype:
        raise TypeError(f"{name}: dtype {t.dtype}, expected {dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name}: tensor must be contiguous (C-order)")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name}: shape {tuple(t.shape)}, expected {tuple(shape)}")
    return ctypes.c_void_p(t.data_ptr())


def _f(x):
    return x.f if isinstance(x, (Field, IntField)) else x


# ------------------------------------------------------------------ primitives

def prims_array(prims):
    """Host array of flub_prim from a numpy structured array (fields geometry,
    x, q, radius) or a sequence of dicts."""
    n = len(prims)
    arr = (_lib.Prim * max(n, 1))()
    for o in range(n):
        p = prims[o]
        get = (lambda k: p[k]) if not isinstance(p, dict) else (lambda k: p.get(k))
        arr[o].geometry = int(get("geometry"))
        arr[o].x[:] = [float(v) for v in np.asarray(get("x"), np.float32).reshape(3)]
        q = get("q")
        arr[o].q[:] = [float(v) for v in (np.asarray(q, np.float32).reshape(4) if q is not None
                                          else np.array([0, 0, 0, 1], np.float32))]
        r = np.asarray(get("radius"), np.float32).reshape(-1)
        if r.size == 1:
            r = np.repeat(r, 3)
        arr[o].radius[:] = [float(v) for v in r]
    return arr, n


def prims_from_arrays(x, q, geometry):
    """Primitive list from the reference's rigid arrays (rigid_coupling.py:
    x_pair.cur, theta_pair.cur, rigid_geometry with fields geometry, radius)."""
    x = np.asarray(x.cpu() if isinstance(x, torch.Tensor) else x, np.float32).reshape(-1, 3)
    q = np.asarray(q.cpu() if isinstance(q, torch.Tensor) else q, np.float32).reshape(-1, 4)
    out = []
    for o, g in enumerate(geometry):
        gg = g if isinstance(g, dict) else {"geometry": g["geometry"], "radius": g["radius"]}
        out.append(dict(geometry=int(gg["geometry"]), x=x[o], q=q[o], radius=gg["radius"]))
    return out


# ------------------------------------------------------------------ plain calls

def tag_dirichlet(tag, phi):
    """geometry.py:335-344: tag = 0 where phi > 0, else 1."""
    tag, phi = _f(tag), _f(phi)
    _lib.call("flub_tag_dirichlet", _ptr(phi, torch.float32, name="phi"),
              _ptr(tag, torch.int32, phi.shape, "tag"), phi.numel(), _stream())


def tag_neumann(tag, phi_rigid):
    """geometry.py:390-397: tag = 2 where phi_rigid < 0."""
    tag, phi_rigid = _f(tag), _f(phi_rigid)
    _lib.call("flub_tag_neumann", _ptr(phi_rigid, torch.float32, name="phi_rigid"),
              _ptr(tag, torch.int32, phi_rigid.shape, "tag"), phi_rigid.numel(), _stream())


def phi_prims(phi, prims, h, h0, stagger=(0.5, 0.5, 0.5)):
    """geometry.py:225-239: phi = min primitive SDF below h0 (else 2.0)."""
    phi = _f(phi)
    arr, n = prims_array(prims)
    nx, ny, nz = phi.shape
    _lib.call("flub_phi_prims", _ptr(phi, torch.float32, name="phi"), nx, ny, nz, float(h), float(h0),
              float(stagger[0]), float(stagger[1]), float(stagger[2]), ctypes.cast(arr, ctypes.c_void_p), n,
              _stream())


def classify(phi, prims, h, h0, tag=None, phi_rigid=None):
    """Fused _tag_dirichlet + primitive phi_rigid + _tag_neumann.  Returns tag."""
    phi = _f(phi)
    if tag is None:
        tag = torch.empty(phi.shape, dtype=torch.int32, device=phi.device)
    tag = _f(tag)
    arr, n = prims_array(prims)
    nx, ny, nz = phi.shape
    pr = _ptr(_f(phi_rigid), torch.float32, phi.shape, "phi_rigid") if phi_rigid is not None else None
    _lib.call("flub_classify", _ptr(phi, torch.float32, name="phi"), ctypes.cast(arr, ctypes.c_void_p), n, nx, ny,
              nz, float(h), float(h0), _ptr(tag, torch.int32, phi.shape, "tag"), pr, _stream())
    return tag


def _faces(vel, shape):
    return [_ptr(_f(a), torch.float32, field_shape(shape, d + 1), n)
            for d, (a, n) in enumerate(zip((vel.u, vel.v, vel.w), ("u", "v", "w")))]


def divergence(vel, vel_rigid, tag, div=None, scale=None):
    """divergence.py:43-99 divergence_tag; with ``scale`` also mask_with_tag and
    scale_by_3d fused (example_fluid.py:90-93).  Returns div."""
    tag = _f(tag)
    shape = tuple(tag.shape)
    if div is None:
        div = torch.empty(shape, dtype=torch.float32, device=tag.device)
    div = _f(div)
    args = _faces(vel, shape) + _faces(vel_rigid, shape) + [_ptr(tag, torch.int32, name="tag"),
                                                            _ptr(div, torch.float32, shape, "div")]
    if scale is None:
        _lib.call("flub_divergence_tag", *args, *shape, _stream())
    else:
        _lib.call("flub_divergence_masked", *args, float(scale), *shape, _stream())
    return div


def _mask_with_tag(div, tag):
    """divergence.py:173-180: div = 0 where tag != 1."""
    div, tag = _f(div), _f(tag)
    _lib.call("flub_mask_with_tag", _ptr(div, torch.float32, name="div"), _ptr(tag, torch.int32, div.shape, "tag"),
              div.numel(), _stream())


def _scale_by_3d(q, s):
    """utils/util.py:162-165: q *= s."""
    q = _f(q)
    _lib.call("flub_scale", _ptr(q, torch.float32, name="q"), float(s), q.numel(), _stream())


def subtract_gradient(vel, vel_rigid, p, tag, d=None, p_scale=1.0):
    """subtract_gradient.py:37-68.  d in {1, 2, 3} updates one axis as the
    reference does; d=None updates all three in one fused pass."""
    p, tag = _f(p), _f(tag)
    shape = tuple(tag.shape)
    pp = _ptr(p, torch.float32, shape, "p")
    tp = _ptr(tag, torch.int32, shape, "tag")
    if d is None:
        _lib.call("flub_subtract_gradient", *_faces(vel, shape), *_faces(vel_rigid, shape), pp, float(p_scale), tp,
                  *shape, _stream())
    else:
        if float(p_scale) != 1.0:
            raise ValueError("p_scale applies to the fused update (d=None) only")
        uf = _f((vel.u, vel.v, vel.w)[d - 1])
        urf = _f((vel_rigid.u, vel_rigid.v, vel_rigid.w)[d - 1])
        fs = field_shape(shape, d)
        _lib.call("flub_subtract_gradient_tag", _ptr(uf, torch.float32, fs, "uf"), _ptr(urf, torch.float32, fs, "urf"),
                  pp, tp, *shape, int(d), _stream())


# ------------------------------------------------------------------ rigid face velocities, cut cells

def _host_vec3(a, name):
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, 3))
    return a


def solid_vel(vel_rigid, vel_owner, d, x, v, omega, h0=None):
    """rigid_coupling.py:51-70 precompute_solid_vel for axis d: the rigid
    velocity of each face's owner body (x, v, omega: one vec3 per body)."""
    ur = _f((vel_rigid.u, vel_rigid.v, vel_rigid.w)[d - 1])
    ow = _f((vel_owner.u, vel_owner.v, vel_owner.w)[d - 1])
    fs = tuple(ur.shape)
    shape = (fs[0] - (d == 1), fs[1] - (d == 2), fs[2] - (d == 3))
    bx, bv, bw = (_host_vec3(a, n) for a, n in ((x, "x"), (v, "v"), (omega, "omega")))
    hh = float(h0) if h0 is not None else 1.0 / shape[0]
    _lib.call("flub_solid_vel", _ptr(ur, torch.float32, fs, "u_rigid"), _ptr(ow, torch.int32, fs, "owner"), *shape,
              int(d), hh, bx.ctypes.data_as(ctypes.c_void_p), bv.ctypes.data_as(ctypes.c_void_p),
              bw.ctypes.data_as(ctypes.c_void_p), bx.shape[0], _stream())


def phi_to_fraction(phi_nodes, frac, d):
    """geometry.py phi_to_fraction: face fractions of axis d in place (frac
    holds the face-centre SDF on entry; phi_nodes: SDF at the grid nodes)."""
    pn = _f(phi_nodes)
    shape = tuple(s - 1 for s in pn.shape)
    fa = _f((frac.u, frac.v, frac.w)[d - 1])
    _lib.call("flub_phi_to_fraction", _ptr(pn, torch.float32, tuple(pn.shape), "phi"),
              _ptr(fa, torch.float32, field_shape(shape, d), "frac"), *shape, int(d), _stream())


def divergence_fractional(uf, vf, wf, div, fu, fv, fw, ur, vr, wr):
    """divergence.py:4-42 divergence_fractional_3d (raw face arrays)."""
    div = _f(div)
    shape = tuple(div.shape)
    faces = [(_f(a), d) for a, d in ((uf, 1), (vf, 2), (wf, 3), (fu, 1), (fv, 2), (fw, 3), (ur, 1), (vr, 2), (wr, 3))]
    ptrs = [_ptr(a, torch.float32, field_shape(shape, d), "face array") for a, d in faces]
    _lib.call("flub_divergence_fractional", *ptrs[:3], _ptr(div, torch.float32, shape, "div"), *ptrs[3:], *shape,
              _stream())
    return div


def subtract_gradient_batty(uf, pf, frac, phi, urf, d, lo, h):
    """subtract_gradient.py:7-122 u/v/w_subtract_gradient_batty_3d on axis d."""
    phi, pf = _f(phi), _f(pf)
    shape = tuple(phi.shape)
    fs = field_shape(shape, d)
    _lib.call("flub_subtract_gradient_batty", _ptr(_f(uf), torch.float32, fs, "uf"), _ptr(pf, torch.float32, shape, "p"),
              _ptr(_f(frac), torch.float32, fs, "frac"), _ptr(phi, torch.float32, shape, "phi"),
              _ptr(_f(urf), torch.float32, fs, "u_rigid"), *shape, int(d), float(lo), float(h), _stream())


# ------------------------------------------------------------------ velocity extrapolation

def _int_faces(tags, shape):
    return [_ptr(_f(t), torch.int32, field_shape(shape, d + 1), "tag." + "uvw"[d])
            for d, t in enumerate((tags.u, tags.v, tags.w))]


def set_unknown(phi, tags):
    """utils/util.py:423-437: face flags 1 where phi >= 0, else 0 (face
    index (i, j, k) < the cell grid; the last face layer keeps its flags)."""
    phi = _f(phi)
    shape = tuple(phi.shape)
    _lib.call("flub_set_unknown", _ptr(phi, torch.float32, shape, "phi"), *_int_faces(tags, shape), *shape, _stream())


def extrapolate_axis(vel, tags, d):
    """extrapolate.py:8-30 extrapolate_3d on axis d (flags of extrapolated
    faces become -1, as in the reference)."""
    q = _f((vel.u, vel.v, vel.w)[d - 1])
    t = _f((tags.u, tags.v, tags.w)[d - 1])
    fs = tuple(q.shape)
    shape = (fs[0] - (d == 1), fs[1] - (d == 2), fs[2] - (d == 3))
    _lib.call("flub_extrapolate_axis", _ptr(q, torch.float32, fs, "q"), _ptr(t, torch.int32, fs, "unknown"), *shape,
              int(d), _stream())


def flush_unknown(tag):
    """extrapolate.py:32-36 flush_1_3d: flags -1 -> 1."""
    t = _f(tag)
    _lib.call("flub_flush_unknown", _ptr(t, torch.int32, name="tag"), t.numel(), _stream())


def extrapolate_by_1(vel, tags):
    """extrapolate.py:39-47: one pass on the three axes, then the flush."""
    for d in (1, 2, 3):
        extrapolate_axis(vel, tags, d)
    for t in (tags.u, tags.v, tags.w):
        flush_unknown(t)


def extrapolate(vel, tags, phi, n_cells):
    """water_3d.py:70-73 extrapolate: set_unknown, then n_cells passes of
    extrapolate_by_1, as one sequence of fused passes (one kernel per axis per
    pass; the flush is implied, see flub_extrapolate).  phi=None skips
    set_unknown (the flags are used as they are)."""
    u = _f(vel.u)
    shape = (u.shape[0] - 1, u.shape[1], u.shape[2])
    pp = _ptr(_f(phi), torch.float32, shape, "phi") if phi is not None else None
    _lib.call("flub_extrapolate", *_faces(vel, shape), *_int_faces(tags, shape), pp, *shape, int(n_cells), _stream())


# ------------------------------------------------------------------ advection

DT = 1e-2  # const_param.py dt, the time step the reference's advection kernels read


def _vel_args(vel):
    u = _f(vel.u)
    shape = (u.shape[0] - 1, u.shape[1], u.shape[2])
    return _faces(vel, shape), shape


def _h0(shape, h0):
    return float(h0) if h0 is not None else 1.0 / shape[0]


def _stagger_of(q, default):
    st = getattr(q, "stagger", None)
    return tuple(float(x) for x in (st if st is not None else default))


def advect_mc_stage(args_common, q_in, q_out, q_tmp, stage, dt=DT, h0=None, minmax_h=None):
    """advect.py:57-101 _advect_mc_1 / _2 / _3 (stage 1, 2, 3) on the field
    q_in (a Field: its stagger is used), traced by the MACGrid args_common;
    stage 0 runs all three in one pass (q_tmp unused).  h0 defaults to 1 / nx
    (const_param.py h0), minmax_h to h0 (what sample_minmax receives)."""
    faces, shape = _vel_args(args_common)
    hh = _h0(shape, h0)
    qi, qo = _f(q_in), _f(q_out)
    qs = tuple(qi.shape)
    st = _stagger_of(q_in, (0.5, 0.5, 0.5))
    qt = _ptr(_f(q_tmp), torch.float32, qs, "q_tmp") if q_tmp is not None else None
    _lib.call("flub_advect_mc", *faces, *shape, _ptr(qi, torch.float32, qs, "q_in"), _ptr(qo, torch.float32, qs, "q_out"),
              qt, *qs, *st, float(dt), hh, hh if minmax_h is None else float(minmax_h), int(stage), _stream())


def advect_mc(args_common, q_in, q_out, dt=DT, h0=None, minmax_h=None):
    """advect.py:124-128 advect_mc: MacCormack advection of q_in into q_out,
    the three reference kernels fused into one launch (same values)."""
    advect_mc_stage(args_common, q_in, q_out, None, 0, dt, h0, minmax_h)


def advect_uv_mc(vel_in, vel_out, dt=DT, h0=None, minmax_h=None):
    """advect.py:130-133 advect_uv_mc: each face array of vel_in advected by
    vel_in into vel_out."""
    faces, shape = _vel_args(vel_in)
    hh = _h0(shape, h0)
    _lib.call("flub_advect_velocity_mc", *faces, *_faces(vel_out, shape), *shape, float(dt), hh,
              hh if minmax_h is None else float(minmax_h), _stream())


def advect_3d(vel, qf, new_vel, new_qf, dt=DT, h0=None, minmax_h=None):
    """advect.py:136-138 advect_3d: the scalar qf and the velocity itself."""
    advect_mc(vel, qf, new_qf, dt, h0, minmax_h)
    advect_uv_mc(vel, new_vel, dt, h0, minmax_h)


def advect_phi_field(vel, phi, new_phi, dt=DT, h0=None):
    """advect.py:39-54 advect_phi: the level set traced back by vel, tricubic
    where the foot of the trace lies inside the grid, else h0."""
    faces, shape = _vel_args(vel)
    hh = _h0(shape, h0)
    pi, po = _f(phi), _f(new_phi)
    ps = tuple(pi.shape)
    _lib.call("flub_advect_phi", *faces, *shape, _ptr(pi, torch.float32, ps, "phi"), _ptr(po, torch.float32, ps,
                                                                                         "new_phi"),
              *ps, *_stagger_of(phi, (0.5, 0.5, 0.5)), float(dt), hh, hh, _stream())


def advect_simple(uf, vf, wf, qf, new_qf, dt, h):
    """advect.py:24-37 advect_simple_3d (raw arrays; trilinear sample)."""
    u, v, w, q, qn = (_f(a) for a in (uf, vf, wf, qf, new_qf))
    shape = (u.shape[0] - 1, u.shape[1], u.shape[2])
    qs = tuple(q.shape)
    _lib.call("flub_advect_simple", *(_ptr(a, torch.float32, field_shape(shape, d + 1), "uvw"[d] + "f")
                                      for d, a in enumerate((u, v, w))),
              *shape, _ptr(q, torch.float32, qs, "qf"), _ptr(qn, torch.float32, qs, "new_qf"), *qs, float(dt),
              float(h), _stream())


# ------------------------------------------------------------------ level-set redistance

def init_distance(phi, h, set_boundary=1, out=None):
    """redistance.py:66-119 _init_distance.  Every cell reads the values from
    before the call; with out=None phi is updated (through a temporary)."""
    pf = _f(phi)
    shape = tuple(pf.shape)
    dst = torch.empty_like(pf) if out is None else _f(out)
    _lib.call("flub_redistance_init", _ptr(pf, torch.float32, shape, "phi"), _ptr(dst, torch.float32, shape, "out"),
              *shape, float(h), int(bool(set_boundary)), _stream())
    if out is None:
        pf.copy_(dst)


def sweep_half(phi, incx, incy, incz, odd, h):
    """redistance.py:58-63 _sweep: one red-black half of a sweep, in place."""
    pf = _f(phi)
    _lib.call("flub_redistance_sweep", _ptr(pf, torch.float32, name="phi"), *pf.shape, int(incx), int(incy),
              int(incz), int(odd), float(h), _stream())


def sweep(phi, h, incx, incy, incz):
    """redistance.py:121-123 sweep: both halves."""
    for odd in (0, 1):
        sweep_half(phi, incx, incy, incz, odd, h)


def redistance(phi, h=None, set_boundary=1, n_rounds=2):
    """redistance.py:125-136 redistance(phi, h=h0, set_boundary=1), in place
    (h defaults to 1 / nx, const_param.py h0)."""
    pf = _f(phi)
    shape = tuple(pf.shape)
    hh = float(h) if h is not None else 1.0 / shape[0]
    tmp = torch.empty_like(pf)
    _lib.call("flub_redistance", _ptr(pf, torch.float32, shape, "phi"), _ptr(tmp, torch.float32, shape, "tmp"),
              *shape, hh, int(bool(set_boundary)), int(n_rounds), _stream())
    pf.copy_(tmp)


# ------------------------------------------------------------------ wp.launch mirror

class Kernel:
    """A kernel object for ``launch``; calling it directly runs it on its inputs."""

    def __init__(self, name, fn, expect_dim):
        self.name = name
        self._fn = fn
        self._expect_dim = expect_dim

    def __call__(self, *inputs):
        return self._fn(*inputs)

    def launch(self, dim, inputs):
        expected = self._expect_dim(inputs)
        if expected is not None and tuple(dim) != tuple(expected):
            raise ValueError(f"{self.name}: launch dim {tuple(dim)} does not match the input shape {tuple(expected)}")
        self._fn(*inputs)

    def __repr__(self):
        return f"<flub_gb300 kernel {self.name}>"


def _dim_of(i):
    return lambda inputs: tuple(_f(inputs[i]).shape)


def _sg_dim(inputs):
    vel, d = inputs[0], int(inputs[4])
    return tuple(_f((vel.u, vel.v, vel.w)[d - 1]).shape)


def _phi_prims_launch(phi, owner, x, q, geometry, stagger, h=None, h0=None):
    phi = _f(phi)
    hh = h if h is not None else 1.0 / phi.shape[0]
    phi_prims(phi, prims_from_arrays(x, q, geometry), hh, h0 if h0 is not None else hh, stagger)


divergence_tag = Kernel("divergence_tag", lambda vels, div, vel_rigid, tag: divergence(vels, vel_rigid, tag, div),
                        _dim_of(1))
mask_with_tag = Kernel("mask_with_tag", _mask_with_tag, _dim_of(0))
scale_by_3d = Kernel("scale_by_3d", _scale_by_3d, _dim_of(0))
subtract_gradient_tag = Kernel("subtract_gradient_tag",
                               lambda vel, vel_rigid, pf, tag, d: subtract_gradient(vel, vel_rigid, pf, tag, int(d)),
                               _sg_dim)
_tag_dirichlet = Kernel("_tag_dirichlet", tag_dirichlet, _dim_of(1))
_tag_neumann = Kernel("_tag_neumann", tag_neumann, _dim_of(1))
precompute_grid_point_phi_prims = Kernel("precompute_grid_point_phi_prims", _phi_prims_launch, _dim_of(0))
# the reference passes the MACGrid and MACGridInt and the axis: wp.launch(extrapolate_3d, dim=shapeu, inputs=[vel, tag, 1])
extrapolate_3d = Kernel("extrapolate_3d", lambda vel, tags, d: extrapolate_axis(vel, tags, int(d)),
                        lambda inputs: tuple(_f((inputs[0].u, inputs[0].v, inputs[0].w)[int(inputs[2]) - 1]).shape))
flush_1_3d = Kernel("flush_1_3d", flush_unknown, _dim_of(0))
# rigid_coupling.py precompute_solid_vel: inputs=[x, v, omega, vel_rigid, vel_owner, d]
precompute_solid_vel = Kernel(
    "precompute_solid_vel", lambda x, v, omega, vel_rigid, vel_owner, d: solid_vel(vel_rigid, vel_owner, int(d), x, v,
                                                                                   omega),
    lambda inputs: tuple(_f((inputs[3].u, inputs[3].v, inputs[3].w)[int(inputs[5]) - 1]).shape))
# geometry.py phi_to_fraction: inputs=[phi, frac, dim]
phi_to_fraction_3d = Kernel("phi_to_fraction", lambda phi, frac, dim: phi_to_fraction(phi, frac, int(dim)),
                            lambda inputs: tuple(_f((inputs[1].u, inputs[1].v, inputs[1].w)[int(inputs[2]) - 1]).shape))
divergence_fractional_3d = Kernel("divergence_fractional_3d", divergence_fractional, _dim_of(3))
u_subtract_gradient_batty_3d = Kernel("u_subtract_gradient_batty_3d",
                                      lambda uf, pf, fu, phi, ur, l, r, h: subtract_gradient_batty(uf, pf, fu, phi, ur,
                                                                                                   1, l, h),
                                      _dim_of(0))
v_subtract_gradient_batty_3d = Kernel("v_subtract_gradient_batty_3d",
                                      lambda vf, pf, fv, phi, vr, b, t, h: subtract_gradient_batty(vf, pf, fv, phi, vr,
                                                                                                   2, b, h),
                                      _dim_of(0))
w_subtract_gradient_batty_3d = Kernel("w_subtract_gradient_batty_3d",
                                      lambda wf, pf, fw, phi, wr, far, near, h: subtract_gradient_batty(
                                          wf, pf, fw, phi, wr, 3, far, h),
                                      _dim_of(0))
set_unknown_3d = Kernel("set_unknown", set_unknown, _dim_of(0))
# advect.py kernels: inputs=[args_common, q_in, q_out, q_tmp] / [vel, phi, new_phi] / [uf, vf, wf, qf, new_qf, dt, h]
_advect_mc_1 = Kernel("_advect_mc_1", lambda vel, qi, qo, qt: advect_mc_stage(vel, qi, qo, qt, 1), _dim_of(1))
_advect_mc_2 = Kernel("_advect_mc_2", lambda vel, qi, qo, qt: advect_mc_stage(vel, qi, qo, qt, 2), _dim_of(1))
_advect_mc_3 = Kernel("_advect_mc_3", lambda vel, qi, qo, qt: advect_mc_stage(vel, qi, qo, qt, 3), _dim_of(1))
advect_phi = Kernel("advect_phi", advect_phi_field, _dim_of(1))
advect_simple_3d = Kernel("advect_simple_3d", advect_simple, _dim_of(3))
# redistance.py kernels: inputs=[phi, h, set_boundary] / [phi, incx, incy, incz, odd, h]
_init_distance = Kernel("_init_distance", lambda phi, h, sb: init_distance(phi, h, sb), _dim_of(0))
_sweep = Kernel("_sweep", sweep_half, _dim_of(0))


def launch(kernel, dim, inputs, device=None, stream=None):
    """wp.launch(kernel, dim=..., inputs=[...]) for the kernels of this module."""
    if not isinstance(kernel, Kernel):
        raise TypeError(f"{kernel!r} is not a flub_gb300 kernel")
    if stream is not None:
        with torch.cuda.stream(stream):
            kernel.launch(dim, inputs)
    else:
        kernel.launch(dim, inputs)
