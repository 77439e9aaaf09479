"""MGPCG with the reference's interface (multigrid/mgpcg.py:234-490), on the
GB300 solver of the C ABI.

    mg = MGPCG(3, shape, n_mg_levels, float)
    mg.set_tags(tag)          # int32 tags: 0 air, 1 fluid, 2 solid
    mg.init(div, -h0)         # r0 = k * rhs, x = 0
    mg.mask_interior()        # r0 = 0 off the fluid
    mg.solve(200, rel_tol=1e-12, abs_tol=0, smoother="phases")
    pf.copy_(mg.x)            # MGPCG.x, a torch view of the solver's x

Differences from the reference, all deliberate:
* inner products, alpha/beta and the convergence test are FP64 (the reference
  accumulates in FP32 through warp.utils.array_inner);
* the first solve does not lose an iteration to graph capture (the reference's
  graph_precondition records the first V-cycle without running it,
  mgpcg.py:286-294);
* ``solve`` returns a dict (iterations, converged, rtr0, rtr, tol, status);
  the reference returns None and prints the iteration count (verbose=True
  prints it here, with the per-iteration residual);
* the untagged "default" smoother (mgpcg.py:41-49, 88-92) is not provided;
* ``schedule`` (default "reference", the reference's V-cycle) selects a
  lighter V-cycle with the restriction scaled by 1/2 (``set_schedule``).
"""
import ctypes

import torch

from . import _lib

SMOOTHERS = {"phases": 1, "fraction": 2}
PRECISIONS = {"fp32": 0, "mixed": 1}
# V-cycle schedules: (red-black iterations per side at every level, -1 = the
# reference's 6 << level; iterations of each bottom order; restriction scale)
SCHEDULES = {
    "reference": (-1, 3, 1.0),   # multigrid/mgpcg.py:296-349
    "v22": (2, 4, 0.5),          # 2 + 2 iterations per level, 4 + 4 at the bottom, restriction / 2
    "v33": (3, 8, 0.5),
}


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class MGPCG:
    def __init__(self, dim=3, shape=(256, 256, 256), n_mg_levels=6, real=float, precision="fp32", device=None,
                 schedule="reference"):
        if dim != 3:
            raise ValueError("only dim=3 is supported (as in the reference's kernels)")
        if real not in (float, torch.float32):
            raise ValueError("real must be float (FP32)")
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {list(PRECISIONS)}")
        self.dim = dim
        self.shape = tuple(int(s) for s in shape)
        self.n_mg_levels = int(n_mg_levels)
        self.pre_and_post_smoothing = 6
        self.bottom_smoothing = 6
        self.precision = precision
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        lib = _lib.load()
        nbytes = lib.flub_mg_workspace_bytes(*self.shape, self.n_mg_levels, PRECISIONS[precision])
        if nbytes == 0:
            raise ValueError(lib.flub_last_error().decode())
        self._lib = lib
        self._h = None
        self._ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        torch.cuda.synchronize(self.device)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(lib.flub_mg_create(*self.shape, self.n_mg_levels, PRECISIONS[precision],
                                          ctypes.c_void_p(self._ws.data_ptr()), nbytes, ctypes.byref(h)),
                       "flub_mg_create")
        self._h = h
        n = self.shape[0] * self.shape[1] * self.shape[2]
        self.x = self._view(lib.flub_mg_x(h), n)
        self.r0 = self._view(lib.flub_mg_r(h), n)
        self._tag = None
        self.last_info = None
        self.schedule = "reference"
        if schedule != "reference":
            self.set_schedule(schedule)

    def _view(self, addr, n):
        off = addr - self._ws.data_ptr()
        return self._ws[off: off + 4 * n].view(torch.float32).view(self.shape)

    def __del__(self):
        if getattr(self, "_h", None) is not None:
            try:
                self._lib.flub_mg_destroy(self._h)
            except Exception:
                pass
            self._h = None

    # ---------------------------------------------------------------- reference API
    def set_tags(self, tag=None):
        """mgpcg.py:360-370."""
        if tag is not None:
            tag = tag.f if hasattr(tag, "f") else tag
            if tag.dtype != torch.int32 or tuple(tag.shape) != self.shape or not tag.is_cuda:
                raise ValueError(f"tag must be a CUDA int32 tensor of shape {self.shape}")
            self._tag = tag.contiguous()
        if self._tag is None:
            raise ValueError("set_tags() needs a tag array on the first call")
        _lib.check(self._lib.flub_mg_set_tags(self._h, ctypes.c_void_p(self._tag.data_ptr()), _stream()),
                   "flub_mg_set_tags")

    def init(self, r, k):
        """mgpcg.py:276-284: r0 = k * r, x = 0."""
        r = r.f if hasattr(r, "f") else r
        if r.dtype != torch.float32 or tuple(r.shape) != self.shape or not r.is_cuda:
            raise ValueError(f"r must be a CUDA float32 tensor of shape {self.shape}")
        r = r.contiguous()
        _lib.check(self._lib.flub_mg_init(self._h, ctypes.c_void_p(r.data_ptr()), float(k), _stream()),
                   "flub_mg_init")

    def mask_interior(self):
        """mgpcg.py:464-465."""
        _lib.check(self._lib.flub_mg_mask_interior(self._h, _stream()), "flub_mg_mask_interior")

    def set_initial_guess(self, x0):
        """Warm start for the next solve (no reference counterpart)."""
        x0 = x0.contiguous()
        _lib.check(self._lib.flub_mg_set_x0(self._h, ctypes.c_void_p(x0.data_ptr()), _stream()), "flub_mg_set_x0")

    def set_schedule(self, schedule="reference", bottom_iters=None, restrict_scale=None):
        """V-cycle schedule (no reference counterpart).  ``schedule`` is a name
        of SCHEDULES or the red-black iterations per side at every level (-1:
        the reference's 6 << level), with ``bottom_iters`` and
        ``restrict_scale``.  See flub_mg_set_schedule."""
        if isinstance(schedule, str):
            if schedule not in SCHEDULES:
                raise ValueError(f"schedule must be one of {list(SCHEDULES)} or an iteration count")
            nu, nb, rs = SCHEDULES[schedule]
        else:
            nu, nb, rs = int(schedule), int(bottom_iters if bottom_iters is not None else 8), \
                float(restrict_scale if restrict_scale is not None else 0.5)
        _lib.check(self._lib.flub_mg_set_schedule(self._h, nu, nb, rs), "flub_mg_set_schedule")
        self.schedule = schedule if isinstance(schedule, str) else (nu, nb, rs)

    def set_bottom_precision(self, bits):
        """Bottom-level smoothing in FP32 (the reference's) or FP64 (no
        reference counterpart; the mixed-precision handle's default).  See
        flub_mg_set_bottom_precision."""
        _lib.check(self._lib.flub_mg_set_bottom_precision(self._h, int(bits)), "flub_mg_set_bottom_precision")

    def bottom_precision(self):
        b = ctypes.c_int(0)
        _lib.check(self._lib.flub_mg_get_bottom_precision(self._h, ctypes.byref(b)), "flub_mg_get_bottom_precision")
        return int(b.value)

    def set_initial_guess_scaled(self, d):
        """Warm start x0 = gamma d, gamma = (d . b) / (d . L d) computed on the
        device (no reference counterpart; the guess is never worse than 0 in
        the energy norm)."""
        d = d.contiguous()
        _lib.check(self._lib.flub_mg_set_x0_scaled(self._h, ctypes.c_void_p(d.data_ptr()), _stream()),
                   "flub_mg_set_x0_scaled")

    def level_shape(self, level):
        nx, ny, nz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(self._lib.flub_mg_level_shape(self._h, int(level), ctypes.byref(nx), ctypes.byref(ny),
                                                 ctypes.byref(nz)), "flub_mg_level_shape")
        return (nx.value, ny.value, nz.value)

    def level_tags(self, level, out=None):
        """Tags of a level of the hierarchy (0 air, 1 fluid, 2 solid)."""
        if out is None:
            out = torch.empty(self.level_shape(level), dtype=torch.int32, device=self.device)
        _lib.check(self._lib.flub_mg_level_tags(self._h, int(level), ctypes.c_void_p(out.data_ptr()), _stream()),
                   "flub_mg_level_tags")
        return out

    def restrict_vector(self, level, fine, coarse=None):
        """Level-(l-1) vector -> level l: sum of the 8 children on coarse fluid cells."""
        if coarse is None:
            coarse = torch.empty(self.level_shape(level), dtype=torch.float32, device=self.device)
        fine = fine.contiguous()
        _lib.check(self._lib.flub_mg_restrict_vector(self._h, int(level), ctypes.c_void_p(fine.data_ptr()),
                                                     ctypes.c_void_p(coarse.data_ptr()), _stream()),
                   "flub_mg_restrict_vector")
        return coarse

    def prolong_vector(self, level, coarse, fine=None):
        """Level-l vector -> level l-1 by cell-centred trilinear interpolation."""
        if fine is None:
            fine = torch.empty(self.level_shape(level - 1), dtype=torch.float32, device=self.device)
        coarse = coarse.contiguous()
        _lib.check(self._lib.flub_mg_prolong_vector(self._h, int(level), ctypes.c_void_p(coarse.data_ptr()),
                                                    ctypes.c_void_p(fine.data_ptr()), _stream()),
                   "flub_mg_prolong_vector")
        return fine

    def solve(self, max_iters=1, eps=1e-12, abs_tol=1e-12, rel_tol=1e-12, verbose=False, smoother="default",
              x0=None, sync=True):
        """mgpcg.py:378-462.  With sync=False the solve is only enqueued on the
        current stream; read the outcome later with ``info()``."""
        if smoother not in SMOOTHERS:
            raise NotImplementedError(
                f"smoother {smoother!r}: only 'phases' and 'fraction' (the tagged smoothers the reference's "
                "callers use) are provided; the untagged 'default' smoother is not")
        if x0 is not None:
            self.set_initial_guess(x0)
        info = _lib.SolveInfo()
        _lib.check(self._lib.flub_mg_solve(self._h, int(max_iters), float(eps), float(abs_tol), float(rel_tol),
                                           SMOOTHERS[smoother], _stream(),
                                           ctypes.byref(info) if (sync or verbose) else None), "flub_mg_solve")
        if not (sync or verbose):
            return None
        self.last_info = info.as_dict()
        if verbose:
            for it, rtr in enumerate(self.residual_history()):
                print(f"after iter {it + 1}, |residual|_2={rtr ** 0.5}")
            print("finished with ", info.iterations, " iterations")
        if info.status != 0:
            raise _lib.FlubError(info.status, "MGPCG.solve", "CG breakdown (non-finite alpha, beta or residual)")
        return self.last_info

    def info(self):
        info = _lib.SolveInfo()
        _lib.check(self._lib.flub_mg_get_info(self._h, _stream(), ctypes.byref(info)), "flub_mg_get_info")
        self.last_info = info.as_dict()
        return self.last_info

    def residual_history(self):
        buf = (ctypes.c_double * 4096)()
        n = ctypes.c_int()
        _lib.check(self._lib.flub_mg_residual_history(self._h, _stream(), buf, 4096, ctypes.byref(n)),
                   "flub_mg_residual_history")
        return list(buf[: n.value])

    def kernels_executed(self):
        v = ctypes.c_int64()
        _lib.check(self._lib.flub_mg_kernels_executed(self._h, _stream(), ctypes.byref(v)), "flub_mg_kernels_executed")
        return v.value

    def apply_preconditioner(self, r=None, z=None, smoother="phases"):
        """mgpcg.py:296-349: z = M r (defaults: r = the level-0 residual)."""
        r = self.r0 if r is None else r.contiguous()
        if z is None:
            z = torch.empty(self.shape, dtype=torch.float32, device=self.device)
        _lib.check(self._lib.flub_mg_apply_preconditioner(self._h, ctypes.c_void_p(r.data_ptr()),
                                                          ctypes.c_void_p(z.data_ptr()), _stream()),
                   "flub_mg_apply_preconditioner")
        return z

    def matvec(self, p, Ap=None):
        """mgpcg.py:36-39 compute_Ap_mcadams with the level-0 tags."""
        p = p.contiguous()
        if Ap is None:
            Ap = torch.empty_like(p)
        _lib.check(self._lib.flub_mg_matvec(self._h, ctypes.c_void_p(p.data_ptr()), ctypes.c_void_p(Ap.data_ptr()),
                                            _stream()), "flub_mg_matvec")
        return Ap

    def smooth(self, level=0, phase=0):
        """One red-black half-sweep (mgpcg.py:72-86) on a level of the hierarchy."""
        _lib.check(self._lib.flub_mg_smooth(self._h, int(level), int(phase), _stream()), "flub_mg_smooth")

    def smooth_iteration(self, level=0, phase=0):
        """One red-black iteration on a level; returns which kernel ran: 0 the
        natural-order row kernel (two half-sweeps), 1 the TMA-tiled kernel (one
        launch), 2 the colour-split row kernel of level 0 (two half-sweeps)."""
        t = ctypes.c_int(0)
        _lib.check(self._lib.flub_mg_smooth_iteration(self._h, int(level), int(phase), ctypes.byref(t), _stream()),
                   "flub_mg_smooth_iteration")
        return int(t.value)

    def get_x(self, out, scale=1.0):
        """x * scale into out (water_3d.py:67-68)."""
        _lib.check(self._lib.flub_mg_get_x(self._h, ctypes.c_void_p(out.data_ptr()), float(scale), _stream()),
                   "flub_mg_get_x")
        return out
