"""Independent vectorised NumPy FP32 restatement of flub's level-set
redistance -- TEST INFRASTRUCTURE ONLY (small grids; used to cross-check
oracle/flub_oracle.c).

Written from the reference's definitions, not from the C code:
redistance.py:7-55 (update), :58-63 (_sweep), :66-119 (_init_distance),
:121-136 (sweep, redistance); utils/util.py:403-412 (fraction_of_fluid).
Every operation is a float32 NumPy operation; x ** 2.0 is x * x; min / max of
two values are a < b ? a : b and a > b ? a : b.  _init_distance reads the
values from before the launch.
"""
import numpy as np

F = np.float32
DIRECTIONS = ((1, 1, -1), (-1, 1, -1), (-1, -1, -1), (1, -1, -1), (1, 1, 1), (-1, 1, 1), (-1, -1, 1), (1, -1, 1))


def _min(a, b):
    return np.where(a < b, a, b)


def _max(a, b):
    return np.where(a > b, a, b)


def _frac(p1, p2):
    """utils/util.py:403-412 fraction_of_fluid (the max as fmax: the operands are never NaN here)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        mixed = F(1) - np.fmax(p1, p2) / np.abs(p1 - p2)
    return np.where((p1 < 0) & (p2 < 0), F(1), np.where((p1 >= 0) & (p2 >= 0), F(0), mixed)).astype(F)


def _neighbour(phi, axis, d, fill):
    out = np.full_like(phi, fill)
    n = phi.shape[axis]
    src = [slice(None)] * 3
    dst = [slice(None)] * 3
    if d > 0:
        src[axis], dst[axis] = slice(1, n), slice(0, n - 1)
    else:
        src[axis], dst[axis] = slice(0, n - 1), slice(1, n)
    out[tuple(dst)] = phi[tuple(src)]
    return out


def _boundary(shape):
    i, j, k = np.meshgrid(*(np.arange(n) for n in shape), indexing="ij")
    return (i == 0) | (i == shape[0] - 1) | (j == 0) | (j == shape[1] - 1) | (k == 0) | (k == shape[2] - 1)


def init_distance(phi, h, set_boundary=1):
    h = F(h)
    hb = F(0.5) * h
    pl, pr = _neighbour(phi, 0, -1, hb), _neighbour(phi, 0, 1, hb)
    pb, pt = _neighbour(phi, 1, -1, hb), _neighbour(phi, 1, 1, hb)
    pf, pn = _neighbour(phi, 2, -1, hb), _neighbour(phi, 2, 1, hb)
    pc = phi
    bnd = _boundary(phi.shape)
    nbrs = (pl, pr, pb, pt, pf, pn)
    near_pos = (~bnd & (pl < 0)) | (pr < 0) | (pb < 0) | (pt < 0) | (pf < 0) | (pn < 0)
    near_neg = (~bnd & (pl > 0)) | (pr > 0) | (pb > 0) | (pt > 0) | (pf > 0) | (pn > 0)
    m_pos = F(1) - _frac(pc, nbrs[0])
    m_neg = _frac(pc, nbrs[0])
    for nb in nbrs[1:]:
        m_pos = _min(m_pos, F(1) - _frac(pc, nb))
        m_neg = _min(m_neg, _frac(pc, nb))
    out = pc.copy()
    pos = (pc > 0) & ~(bnd & (not set_boundary))
    neg = (pc < 0) & ~(bnd & (not set_boundary))
    out = np.where(pos, np.where(near_pos, h * m_pos, F(2)), out)
    out = np.where(neg, np.where(near_neg, (-h) * m_neg, F(-2)), out)
    return out.astype(F)


def sweep(phi, incx, incy, incz, odd, h):
    """One _sweep launch, in place."""
    h = F(h)
    nx, ny, nz = phi.shape
    a, b, c = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    sel = (a + b + c) % 2 == odd
    i = np.where(incx < 0, nx - 1 - a, a)[sel]
    j = np.where(incy < 0, ny - 1 - b, b)[sel]
    k = np.where(incz < 0, nz - 1 - c, c)[sel]
    bnd = (i == 0) | (i == nx - 1) | (j == 0) | (j == ny - 1) | (k == 0) | (k == nz - 1)
    pc = phi[i, j, k]
    upd = (np.abs(pc) > h) & ~bnd
    i, j, k, pc = i[upd], j[upd], k[upd], pc[upd]
    phii, phij, phik = phi[i - incx, j, k], phi[i, j - incy, k], phi[i, j, k - incz]
    phiii, phijj, phikk = phi[i + incx, j, k], phi[i, j + incy, k], phi[i, j, k + incz]
    neg = phii < 0
    sgn = np.where(neg, F(-1), F(1))
    phii, phij, phik = (np.where(neg, -_max(x, y), _min(x, y)) for x, y in ((phii, phiii), (phij, phijj), (phik, phikk)))
    phi0 = _min(_min(phii, phij), phik)
    phi2 = _max(_max(phii, phij), phik)
    phi1 = (((phii + phij) + phik) - phi0) - phi2
    d = phi0 + h
    e = phi0 - phi1
    with np.errstate(invalid="ignore"):
        d2 = F(0.5) * ((phi0 + phi1) + np.sqrt((F(2) * h) * h - e * e))
        s = (phi0 + phi1) + phi2
        term = s * s - F(3) * (((phi0 * phi0 + phi1 * phi1) + phi2 * phi2) - h * h)
        d3 = (F(1) / F(3)) * (((phi0 + phi1) + phi2) + np.sqrt(_max(F(0), term)))
    two = d > phi1
    d = np.where(two, np.where(d2 > phi2, d3, d2), d)
    phi[i, j, k] = sgn * _min(d, np.abs(pc))


def redistance(phi, h, set_boundary=1, n_rounds=2):
    out = init_distance(np.asarray(phi, F), h, set_boundary)
    for _ in range(n_rounds):
        for dx, dy, dz in DIRECTIONS:
            for odd in (0, 1):
                sweep(out, dx, dy, dz, odd, h)
    return out
