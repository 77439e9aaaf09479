"""Independent vectorised NumPy FP64 restatement of the MGPCG path -- TEST
INFRASTRUCTURE ONLY (small grids; used to cross-check oracle/flub_oracle.c).

Written from the reference's definitions, not from the C code:
multigrid/mgpcg.py:118-142 (neighbor_dot_tag), :51-58 (_compute_divd),
:72-86 (_smooth_mcadams), :94-101 (_restrict_mcadams), :113-116 (_prolongate),
:162-174 (restrict_tag), :296-349 (apply_preconditioner), :378-462 (solve);
divergence.py:43-99; subtract_gradient.py:37-68.
"""
import numpy as np


def _shift(a, axis, d, fill):
    """b[idx] = a[idx + d along axis], fill outside the domain."""
    b = np.full_like(a, fill)
    n = a.shape[axis]
    src = [slice(None)] * 3
    dst = [slice(None)] * 3
    if d > 0:
        src[axis] = slice(d, n)
        dst[axis] = slice(0, n - d)
    else:
        src[axis] = slice(0, n + d)
        dst[axis] = slice(-d, n)
    b[tuple(dst)] = a[tuple(src)]
    return b


def matvec(x, tag):
    """L x: per axis (+ then -), neighbour in domain and non-solid contributes
    (x_nb or 0 if air) - x_c; zero at non-fluid cells."""
    x = np.asarray(x, np.float64)
    xa = np.where(tag == 0, 0.0, x)
    ret = np.zeros_like(x)
    for axis in range(3):
        t = np.zeros_like(x)
        for d in (1, -1):
            nb_tag = _shift(tag, axis, d, 2)  # outside the domain: excluded like a solid
            nb_x = _shift(xa, axis, d, 0.0)
            t = t + np.where(nb_tag < 2, nb_x - x, 0.0)
        ret = ret + t
    return np.where(tag == 1, ret, 0.0)


def divd(tag):
    cnt = np.zeros(tag.shape, np.float64)
    for axis in range(3):
        for d in (1, -1):
            cnt += _shift(tag, axis, d, 2) < 2
    return np.where(tag == 1, cnt, 0.0)


def parity_mask(shape, phase):
    i, j, k = np.indices(shape)
    return ((i + j + k) & 1) == (1 - phase)


def smooth(z, r, tag, phase, dg=None):
    if dg is None:
        dg = divd(tag)
    m = parity_mask(tag.shape, phase)
    lz = matvec(z, tag)
    with np.errstate(divide="ignore", invalid="ignore"):
        upd = np.where(dg != 0, z + (r + lz) / np.where(dg != 0, dg, 1.0), 0.0)
    return np.where(m, upd, z)


def restrict_tag(tf):
    nx, ny, nz = (s // 2 for s in tf.shape)
    c = tf.reshape(nx, 2, ny, 2, nz, 2)
    anyair = (c == 0).any(axis=(1, 3, 5))
    anyfluid = (c == 1).any(axis=(1, 3, 5))
    return np.where(anyair, 0, np.where(anyfluid, 1, 2)).astype(np.int32)


def tag_levels(tag, levels):
    out = [np.asarray(tag, np.int32)]
    for _ in range(levels - 1):
        out.append(restrict_tag(out[-1]))
    return out


def restrict(rf, zf, tagf, tagc):
    res = rf + matvec(zf, tagf)
    nx, ny, nz = tagc.shape
    s = res.reshape(nx, 2, ny, 2, nz, 2).sum(axis=(1, 3, 5))
    return np.where(tagc == 1, s, 0.0)


def prolong(zf, zc):
    return zf + np.repeat(np.repeat(np.repeat(zc, 2, 0), 2, 1), 2, 2)


def vcycle(r, tags):
    L = len(tags)
    rl = [np.asarray(r, np.float64)] + [None] * (L - 1)
    zl = [np.zeros_like(rl[0])] + [None] * (L - 1)
    dgs = [divd(t) for t in tags]
    for l in range(L - 1):
        for _ in range(6 << l):
            zl[l] = smooth(zl[l], rl[l], tags[l], 0, dgs[l])
            zl[l] = smooth(zl[l], rl[l], tags[l], 1, dgs[l])
        rl[l + 1] = restrict(rl[l], zl[l], tags[l], tags[l + 1])
        zl[l + 1] = np.zeros_like(rl[l + 1])
    l = L - 1
    for _ in range(3):
        zl[l] = smooth(zl[l], rl[l], tags[l], 0, dgs[l])
        zl[l] = smooth(zl[l], rl[l], tags[l], 1, dgs[l])
    for _ in range(3):
        zl[l] = smooth(zl[l], rl[l], tags[l], 1, dgs[l])
        zl[l] = smooth(zl[l], rl[l], tags[l], 0, dgs[l])
    for l in range(L - 2, -1, -1):
        zl[l] = prolong(zl[l], zl[l + 1])
        for _ in range(6 << l):
            zl[l] = smooth(zl[l], rl[l], tags[l], 1, dgs[l])
            zl[l] = smooth(zl[l], rl[l], tags[l], 0, dgs[l])
    return zl[0]


def pcg(rhs, tags, max_iters=200, eps=1e-12, abs_tol=1e-12, rel_tol=1e-12):
    """MGPCG.solve with smoother "phases", all FP64."""
    r = np.asarray(rhs, np.float64).copy()
    x = np.zeros_like(r)
    rTr0 = float(np.sum(r * r))
    tol = max(abs_tol, rTr0 * rel_tol)
    z = vcycle(r, tags)
    p = z.copy()
    old = float(np.sum(z * r))
    it = 0
    converged = False
    rTr = rTr0
    while it < max_iters:
        Ap = matvec(p, tags[0])
        alpha = old / (float(np.sum(p * Ap)) + eps)
        r = r - alpha * Ap
        rTr = float(np.sum(r * r))
        if rTr < tol:
            x = x + alpha * p
            converged = True
            break
        z = vcycle(r, tags)
        new = float(np.sum(z * r))
        beta = new / (old + eps)
        old = new
        x = x + alpha * p
        p = z + beta * p
        it += 1
    return dict(x=x, iters=it, rtr=rTr, rtr0=rTr0, converged=converged)


def divergence(u, v, w, ur, vr, wr, tag):
    nx, ny, nz = tag.shape
    fl, fr = u[:-1].astype(np.float64), u[1:].astype(np.float64)
    fb, ft = v[:, :-1].astype(np.float64), v[:, 1:].astype(np.float64)
    ff, fn = w[:, :, :-1].astype(np.float64), w[:, :, 1:].astype(np.float64)
    solid_m = [_shift(tag, a, -1, -1) == 2 for a in range(3)]
    solid_p = [_shift(tag, a, 1, -1) == 2 for a in range(3)]
    fl = np.where(solid_m[0], ur[:-1], fl)
    fr = np.where(solid_p[0], ur[1:], fr)
    fb = np.where(solid_m[1], vr[:, :-1], fb)
    ft = np.where(solid_p[1], vr[:, 1:], ft)
    ff = np.where(solid_m[2], wr[:, :, :-1], ff)
    fn = np.where(solid_p[2], wr[:, :, 1:], fn)
    fl[0] = 0.0
    fr[-1] = 0.0
    fb[:, 0] = 0.0
    ft[:, -1] = 0.0
    ff[:, :, 0] = 0.0
    fn[:, :, -1] = 0.0
    return (fr - fl) + (ft - fb) + (fn - ff)


def subtract_gradient(uf, urf, p, tag, d):
    a = d - 1
    uf = np.asarray(uf, np.float64).copy()
    n = tag.shape[a]
    out = np.zeros_like(uf)
    sl_face = [slice(None)] * 3
    sl_face[a] = slice(1, n)
    sl_l = [slice(None)] * 3
    sl_l[a] = slice(0, n - 1)
    sl_r = [slice(None)] * 3
    sl_r[a] = slice(1, n)
    tl, tr = tag[tuple(sl_l)], tag[tuple(sl_r)]
    pl, pr = p[tuple(sl_l)], p[tuple(sl_r)]
    inner = uf[tuple(sl_face)]
    val = np.where((tl == 2) | (tr == 2), urf[tuple(sl_face)],
                   np.where((tl == 1) | (tr == 1), inner - (pr - pl), 0.0))
    out[tuple(sl_face)] = val
    return out
