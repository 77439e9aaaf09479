"""Seeded synthetic scenes for the projection workloads.

No public dataset exists for this path; these generators stand in for the
reference's scenes (scenes/dam_break.json, scenes/flow_pass_sphere.json) with
the shapes and value distributions of the benchmark configurations:

* ``box64``      64^3, fluid box x < 0.4, y < 0.6, air elsewhere, walls Neumann.
* ``sphere128``  128^3 flow past a solid sphere (r = 0.15 at the centre); the
                 x = 0 inflow is a one-cell solid layer whose rigid face velocity
                 is u = 1, the x = 1 outflow a one-cell air layer (p = 0).
* ``dam256``     256^3 dam break: fluid x < 0.35, y < 0.55 plus a water sphere
                 r = 0.08 at (0.7, 0.3, 0.5); a solid box of side 0.1 centred at
                 (0.6, 0.05, 0.45); velocities get -g*dt on v (g = 9.8, dt = 1/60).
* ``dam512``     the same scene at 512^3.

Face velocities: 16 Fourier modes drawn from ``numpy.random.default_rng(seed)``
(integer wavenumbers k in [1, 8]^3, amplitude N(0,1)/|k|^2 per component,
phase U(0, 2 pi)), each component c at face position x is
sum_m a_{m,c} sin(2 pi k_m . x + phase_m), plus U(-0.01, 0.01) noise.

The level set ``phi`` (negative inside water) and the solid primitives are what
the classification kernels consume; the generator never computes tags itself.
"""
from dataclasses import dataclass, field
from typing import Tuple

import numpy as np

PRIM_DTYPE = np.dtype([("geometry", "<i4"), ("x", "<f4", (3,)), ("q", "<f4", (4,)),
                       ("radius", "<f4", (3,))], align=True)

GEOM_NONE, GEOM_BOX, GEOM_SPHERE, GEOM_RECT, GEOM_X, GEOM_MESH = 0, 1, 2, 3, 4, 5


def make_prims(objs):
    """objs: list of dicts {geometry, x, radius, q (optional, (x, y, z, w))}."""
    out = np.zeros(len(objs), PRIM_DTYPE)
    for n, o in enumerate(objs):
        out[n]["geometry"] = o["geometry"]
        out[n]["x"] = o["x"]
        r = o["radius"]
        out[n]["radius"] = (r, r, r) if np.isscalar(r) else r
        out[n]["q"] = o.get("q", (0.0, 0.0, 0.0, 1.0))
    return out


@dataclass
class Scene:
    name: str
    shape: Tuple[int, int, int]
    levels: int
    phi: np.ndarray
    prims: np.ndarray
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray
    ur: np.ndarray
    vr: np.ndarray
    wr: np.ndarray
    seed: int = 0
    meta: dict = field(default_factory=dict)

    @property
    def h(self) -> float:
        return 1.0 / self.shape[0]

    @property
    def h0(self) -> float:
        return 1.0 / self.shape[0]

    @property
    def n_cells(self) -> int:
        return int(np.prod(self.shape))


def face_shapes(shape):
    nx, ny, nz = shape
    return (nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)


def _axis(n, h, stagger, count):
    return (np.arange(count, dtype=np.float64) + stagger) * h


def fourier_faces(shape, seed, n_modes=16, kmax=8, noise=0.01):
    """Seeded sum of Fourier modes sampled at the u, v, w face centres."""
    nx, ny, nz = shape
    h = 1.0 / nx
    rng = np.random.default_rng(seed)
    ks = rng.integers(1, kmax + 1, size=(n_modes, 3))
    amps = rng.standard_normal((n_modes, 3)) / np.sum(ks.astype(np.float64) ** 2, axis=1, keepdims=True)
    phases = rng.uniform(0.0, 2.0 * np.pi, n_modes)
    out = []
    for c, fs in enumerate(face_shapes(shape)):
        st = [0.5, 0.5, 0.5]
        st[c] = 0.0
        xs = [_axis(None, h, st[a], fs[a]) for a in range(3)]
        acc = np.zeros(fs, np.float64)
        for m in range(n_modes):
            ex = np.exp(2j * np.pi * ks[m, 0] * xs[0]) * np.exp(1j * phases[m])
            ey = np.exp(2j * np.pi * ks[m, 1] * xs[1])
            ez = np.exp(2j * np.pi * ks[m, 2] * xs[2])
            exy = ex[:, None] * ey[None, :]
            # Im(exy * ez) = Im(exy) Re(ez) + Re(exy) Im(ez)
            s = exy.imag[:, :, None] * ez.real[None, None, :]
            s += exy.real[:, :, None] * ez.imag[None, None, :]
            acc += amps[m, c] * s
        out.append(acc)
    out = [(a + rng.uniform(-noise, noise, a.shape)).astype(np.float32) for a in out]
    return out


def _centres(shape):
    nx, ny, nz = shape
    h = 1.0 / nx
    x = (np.arange(nx) + 0.5) * h
    y = (np.arange(ny) + 0.5) * h
    z = (np.arange(nz) + 0.5) * h
    return x[:, None, None], y[None, :, None], z[None, None, :]


def _box_phi(shape, xmax, ymax):
    x, y, _ = _centres(shape)
    return np.maximum(x - xmax, y - ymax) + np.zeros(shape)


def _sphere_phi(shape, c, r):
    x, y, z = _centres(shape)
    return np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) - r


def box(n=64, seed=0, levels=None):
    shape = (n, n, n)
    phi = _box_phi(shape, 0.4, 0.6).astype(np.float32)
    u, v, w = fourier_faces(shape, seed)
    zeros = [np.zeros_like(a) for a in (u, v, w)]
    return Scene(f"box{n}", shape, levels or _default_levels(n), phi, make_prims([]), u, v, w, *zeros, seed=seed)


def sphere(n=128, seed=1, levels=None):
    shape = (n, n, n)
    h = 1.0 / n
    x, _, _ = _centres(shape)
    phi = (x - (1.0 - h) + np.zeros(shape)).astype(np.float32)  # air layer at i = n-1
    prims = make_prims([
        dict(geometry=GEOM_SPHERE, x=(0.5, 0.5, 0.5), radius=0.15),
        dict(geometry=GEOM_BOX, x=(0.0, 0.5, 0.5), radius=(h, 0.5 + h, 0.5 + h)),  # inflow layer i = 0
    ])
    u, v, w = fourier_faces(shape, seed)
    u += np.float32(1.0)
    ur, vr, wr = (np.zeros_like(a) for a in (u, v, w))
    ur[1] = 1.0  # face between the solid inflow layer and the first fluid cell
    return Scene(f"sphere{n}", shape, levels or _default_levels(n), phi, prims, u, v, w, ur, vr, wr, seed=seed)


def dam(n=256, seed=2, levels=None, g=9.8, dt=1.0 / 60.0):
    shape = (n, n, n)
    phi = np.minimum(_box_phi(shape, 0.35, 0.55), _sphere_phi(shape, (0.7, 0.3, 0.5), 0.08)).astype(np.float32)
    prims = make_prims([dict(geometry=GEOM_BOX, x=(0.6, 0.05, 0.45), radius=0.05)])
    u, v, w = fourier_faces(shape, seed)
    v -= np.float32(g * dt)
    zeros = [np.zeros_like(a) for a in (u, v, w)]
    return Scene(f"dam{n}", shape, levels or _default_levels(n), phi, prims, u, v, w, *zeros, seed=seed)


def _default_levels(n):
    """Coarsest level 8^3 (64 -> 4 levels, 128 -> 5, 256 -> 6, 512 -> 7)."""
    levels = 1
    while (n >> (levels - 1)) > 8 and (n >> levels) % 2 == 0:
        levels += 1
    return levels


def _random_layout(seed):
    """The random parts of a training scene: fluid boxes, water spheres and
    solid boxes, drawn in a fixed order from one seeded generator."""
    rng = np.random.default_rng(seed + 7919)
    boxes, spheres, objs = [], [], []
    for _ in range(rng.integers(1, 3)):
        xm, ym = rng.uniform(0.2, 0.6), rng.uniform(0.2, 0.7)
        zlo, zhi = sorted(rng.uniform(0.0, 1.0, 2))
        zlo, zhi = (0.0, 1.0) if rng.random() < 0.5 else (zlo * 0.5, 0.5 + zhi * 0.5)
        boxes.append((xm, ym, zlo, zhi, bool(rng.random() < 0.5)))
    for _ in range(rng.integers(0, 3)):
        c = rng.uniform(0.2, 0.8, 3)
        spheres.append((c, rng.uniform(0.05, 0.15)))
    for _ in range(rng.integers(0, 3)):
        c = rng.uniform(0.15, 0.85, 3)
        objs.append(dict(geometry=GEOM_BOX, x=tuple(c), radius=float(rng.uniform(0.03, 0.1))))
    return boxes, spheres, objs


def random_scene(n, seed, levels=None):
    """Random fluid boxes (one or two, optionally mirrored in x and cut in z),
    up to two water spheres and up to two solid boxes, with a seeded Fourier
    velocity field (training/evaluation scenes for the learned warm start)."""
    shape = (n, n, n)
    boxes, spheres, objs = _random_layout(seed)
    x, y, z = _centres(shape)
    phi = np.full(shape, 1.0)
    for xm, ym, zlo, zhi, flip in boxes:
        b = np.maximum(np.maximum(x - xm, y - ym), np.maximum(zlo - z, z - zhi)) + np.zeros(shape)
        if flip:
            b = b[::-1].copy()
        phi = np.minimum(phi, b)
    for c, r in spheres:
        phi = np.minimum(phi, _sphere_phi(shape, c, r))
    u, v, w = fourier_faces(shape, seed)
    zeros = [np.zeros_like(a) for a in (u, v, w)]
    return Scene(f"rand{n}_{seed}", shape, levels or _default_levels(n), phi.astype(np.float32),
                 make_prims(objs), u, v, w, *zeros, seed=seed)


def fourier_faces_device(shape, seed, device, n_modes=16, kmax=8, noise=0.01):
    """fourier_faces evaluated with torch on ``device`` (float64, stored FP32):
    the same modes, amplitudes and phases; the U(-noise, noise) noise comes
    from a torch generator on the device seeded with ``seed``."""
    import torch
    nx, ny, nz = shape
    h = 1.0 / nx
    rng = np.random.default_rng(seed)
    ks = rng.integers(1, kmax + 1, size=(n_modes, 3))
    amps = rng.standard_normal((n_modes, 3)) / np.sum(ks.astype(np.float64) ** 2, axis=1, keepdims=True)
    phases = rng.uniform(0.0, 2.0 * np.pi, n_modes)
    gen = torch.Generator(device=device).manual_seed(int(seed))
    out = []
    for c, fs in enumerate(face_shapes(shape)):
        st = [0.5, 0.5, 0.5]
        st[c] = 0.0
        xs = [(torch.arange(fs[a], dtype=torch.float64, device=device) + st[a]) * h for a in range(3)]
        acc = torch.zeros(fs, dtype=torch.float64, device=device)
        for m in range(n_modes):
            ax = 2 * np.pi * ks[m, 0] * xs[0] + phases[m]
            ay = 2 * np.pi * ks[m, 1] * xs[1]
            az = 2 * np.pi * ks[m, 2] * xs[2]
            sxy = torch.sin(ax)[:, None] * torch.cos(ay)[None, :] + torch.cos(ax)[:, None] * torch.sin(ay)[None, :]
            cxy = torch.cos(ax)[:, None] * torch.cos(ay)[None, :] - torch.sin(ax)[:, None] * torch.sin(ay)[None, :]
            acc += amps[m, c] * (sxy[:, :, None] * torch.cos(az)[None, None, :] +
                                 cxy[:, :, None] * torch.sin(az)[None, None, :])
        nz_ = torch.rand(fs, generator=gen, dtype=torch.float64, device=device) * (2 * noise) - noise
        out.append((acc + nz_).float())
    return out


def random_scene_device(n, seed, device, levels=None):
    """random_scene built with torch on ``device`` (the same layout; phi and
    faces are device tensors), for generating training sets quickly."""
    import torch
    shape = (n, n, n)
    boxes, spheres, objs = _random_layout(seed)
    c = (torch.arange(n, dtype=torch.float64, device=device) + 0.5) / n
    x, y, z = c[:, None, None], c[None, :, None], c[None, None, :]
    phi = torch.full(shape, 1.0, dtype=torch.float64, device=device)
    for xm, ym, zlo, zhi, flip in boxes:
        b = torch.maximum(torch.maximum(x - xm, y - ym), torch.maximum(zlo - z, z - zhi)).expand(shape)
        if flip:
            b = b.flip(0)
        phi = torch.minimum(phi, b)
    for cc, r in spheres:
        phi = torch.minimum(phi, torch.sqrt((x - cc[0]) ** 2 + (y - cc[1]) ** 2 + (z - cc[2]) ** 2) - r)
    u, v, w = fourier_faces_device(shape, seed, device)
    zeros = [torch.zeros_like(a) for a in (u, v, w)]
    return Scene(f"rand{n}_{seed}", shape, levels or _default_levels(n), phi.float().contiguous(),
                 make_prims(objs), u, v, w, *zeros, seed=seed)


def dam_device(n, seed, device, levels=None, g=9.8, dt=1.0 / 60.0):
    """dam() built with torch on ``device`` (phi and faces are device tensors;
    the faces from fourier_faces_device), for sizes whose host generation
    would take minutes (512^3)."""
    import torch
    shape = (n, n, n)
    h = 1.0 / n
    c = [((torch.arange(n, dtype=torch.float64, device=device) + 0.5) * h) for _ in range(3)]
    x, y, z = c[0][:, None, None], c[1][None, :, None], c[2][None, None, :]
    box_phi = torch.maximum(x - 0.35, y - 0.55).expand(shape)
    sph = torch.sqrt((x - 0.7) ** 2 + (y - 0.3) ** 2 + (z - 0.5) ** 2) - 0.08
    phi = torch.minimum(box_phi, sph).float().contiguous()
    del box_phi, sph
    prims = make_prims([dict(geometry=GEOM_BOX, x=(0.6, 0.05, 0.45), radius=0.05)])
    u, v, w = fourier_faces_device(shape, seed, device)
    v -= float(np.float32(g * dt))
    zeros = [torch.zeros_like(a) for a in (u, v, w)]
    return Scene(f"dam{n}", shape, levels or _default_levels(n), phi, prims, u, v, w, *zeros, seed=seed)


CONFIGS = {
    "box64": lambda seed=0: box(64, seed),
    "sphere128": lambda seed=1: sphere(128, seed),
    "dam256": lambda seed=2: dam(256, seed),
    "dam512": lambda seed=2: dam(512, seed),
}
