"""Independent vectorised NumPy FP32 restatement of flub's advection -- TEST
INFRASTRUCTURE ONLY (small grids; used to cross-check oracle/flub_oracle.c).

Written from the reference's definitions, not from the C code:
advect.py:10-22 (backtrace), :24-37 (advect_simple_3d), :39-54 (advect_phi),
:57-101 (_advect_mc_1/2/3), :103-122 (sample_minmax), :124-138 (advect_mc,
advect_uv_mc); utils/util.py:20-28 (sample_3d), :34-88 (sample_velocity_3d),
:91-120 (trilerp, trilerp_stagger, _trilerp), :122-160 (cubic, _cubic,
_bicubic, _tricubic).  Every operation is a float32 NumPy operation (rounded
on its own; NumPy does not contract a*b+c), with wp.lerp(a, b, t) =
a*(1-t) + b*t.  Indices: floor of the position, saturating at the int32
range (NaN -> 0); fractions x - floor(x).
"""
import numpy as np

F = np.float32


def _ifloor(x):
    """floor as an integer, saturating at the int32 range, NaN -> 0."""
    f = np.floor(x).astype(np.float64)
    f = np.where(np.isnan(f), 0.0, np.clip(f, -2.0 ** 31, 2.0 ** 31 - 1))
    return f.astype(np.int64)


def _fract(x):
    return x - np.floor(x)


def _at(q, a, b, c):
    gx, gy, gz = q.shape
    return q[np.clip(a, 0, gx - 1), np.clip(b, 0, gy - 1), np.clip(c, 0, gz - 1)]


def _lerp(a, b, t):
    return a * (F(1) - t) + b * t


def _tri8(q, a, b, c, fa, fb, fc):
    v = [[[_at(q, a + da, b + db, c + dc) for dc in (0, 1)] for db in (0, 1)] for da in (0, 1)]
    # v[da][db][dc]: a..h of utils/util.py:55-62 = (000, 100, 010, 110, 001, 101, 011, 111)
    lo = _lerp(_lerp(v[0][0][0], v[1][0][0], fa), _lerp(v[0][1][0], v[1][1][0], fa), fb)
    hi = _lerp(_lerp(v[0][0][1], v[1][0][1], fa), _lerp(v[0][1][1], v[1][1][1], fa), fb)
    return _lerp(lo, hi, fc)


def sample_velocity(u, v, w, p):
    """utils/util.py:34-88 at points p = (x, y, z) (float32 arrays)."""
    x, y, z = p
    iu, iv, iw = _ifloor(x), _ifloor(y), _ifloor(z)
    fu, fv, fw = _fract(x), _fract(y), _fract(z)
    s, t, r = x - F(0.5), y - F(0.5), z - F(0.5)
    i_s, i_t, i_r = _ifloor(s), _ifloor(t), _ifloor(r)
    fs, ft, fr = _fract(s), _fract(t), _fract(r)
    return (_tri8(u, iu, i_t, i_r, fu, ft, fr), _tri8(v, i_s, iv, i_r, fs, fv, fr), _tri8(w, i_s, i_t, iw, fs, ft, fw))


def backtrace(u, v, w, p, dt, h):
    """advect.py:10-22 (dt, h: float32)."""
    dt, h = F(dt), F(h)
    v1 = sample_velocity(u, v, w, p)
    c1 = F(0.5) * dt / h
    p1 = tuple(p[a] - c1 * v1[a] for a in range(3))
    v2 = sample_velocity(u, v, w, p1)
    c2 = F(0.75) * dt / h
    p2 = tuple(p[a] - c2 * v2[a] for a in range(3))
    v3 = sample_velocity(u, v, w, p2)
    c3 = dt / h
    k1, k2, k3 = F(2) / F(9), F(1) / F(3), F(4) / F(9)
    return tuple(p[a] - c3 * ((k1 * v1[a] + k2 * v2[a]) + k3 * v3[a]) for a in range(3))


def _cubic(a, b, c, d, s):
    m13, k16, half = F(-1) / F(3), F(1) / F(6), F(0.5)
    t0 = (m13 * s + half * s * s) - k16 * s * s * s
    t1 = (F(1) - s * s) + half * (s * s * s - s)
    t2 = s + half * (s * s - s * s * s)
    t3 = k16 * (s * s * s - s)
    return ((a * t0 + b * t1) + c * t2) + d * t3


def tricubic(q, s, t, r):
    """utils/util.py:148-160 _tricubic at index-space points (s, t, r)."""
    iu, iv, iw = _ifloor(s), _ifloor(t), _ifloor(r)
    fu, fv, fw = _fract(s), _fract(t), _fract(r)
    qw = []
    for m in range(4):
        qv = []
        for n in range(4):
            b, c = iv + (n - 1), iw + (m - 1)
            qv.append(_cubic(*(_at(q, iu + (a - 1), b, c) for a in range(4)), fu))
        qw.append(_cubic(*qv, fv))
    return _cubic(*qw, fw)


def _grid_points(shape, st):
    i, j, k = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    return (i.astype(F) + F(st[0]), j.astype(F) + F(st[1]), k.astype(F) + F(st[2]))


def _sample_stagger(q, p, st):
    return tricubic(q, p[0] - F(st[0]), p[1] - F(st[1]), p[2] - F(st[2]))


def sample_minmax(q, p, h, st):
    """advect.py:103-122: min and max of the 8 values around floor(p / h - stagger)."""
    h = F(h)
    a, b, c = (_ifloor(p[x] / h - F(st[x])) for x in range(3))
    vals = [_at(q, a + da, b + db, c + dc) for dc in (0, 1) for db in (0, 1) for da in (0, 1)]
    return np.minimum.reduce(vals), np.maximum.reduce(vals)


def advect_mc(u, v, w, q, st, dt, h, minmax_h=None):
    """advect.py:124-128 advect_mc: _advect_mc_1, _advect_mc_2, _advect_mc_3 in turn."""
    mh = h if minmax_h is None else minmax_h
    p = _grid_points(q.shape, st)
    p1 = backtrace(u, v, w, p, dt, h)
    q_out = _sample_stagger(q, p1, st)                       # _advect_mc_1
    p2 = backtrace(u, v, w, p, -F(dt), h)
    q_tmp = _sample_stagger(q, p2, st)                       # _advect_mc_2
    p3 = backtrace(u, v, w, p, dt, h)                        # _advect_mc_3
    q_sl = _sample_stagger(q, p3, st)
    q_out = q_out + F(0.5) * (q - q_tmp)
    mn, mx = sample_minmax(q, p3, mh, st)
    return np.where((mn < q_out) & (q_out < mx), q_out, q_sl).astype(F)


def advect_phi(u, v, w, phi, dt, h, outside=None, st=(0.5, 0.5, 0.5)):
    """advect.py:39-54 advect_phi."""
    p = backtrace(u, v, w, _grid_points(phi.shape, st), dt, h)
    inside = np.ones(phi.shape, bool)
    for a in range(3):
        inside &= (F(0) <= p[a]) & (p[a] < F(phi.shape[a]))
    return np.where(inside, _sample_stagger(phi, p, st), F(h if outside is None else outside)).astype(F)


def advect_simple(u, v, w, q, dt, h):
    """advect.py:24-37 advect_simple_3d (trilerp, utils/util.py:91-96)."""
    p = backtrace(u, v, w, _grid_points(q.shape, (0.5, 0.5, 0.5)), dt, h)
    s, t, r = (p[a] - F(0.5) for a in range(3))
    iu, iv, iw = _ifloor(s), _ifloor(t), _ifloor(r)
    return _tri8(q, iu, iv, iw, _fract(s), _fract(t), _fract(r))
