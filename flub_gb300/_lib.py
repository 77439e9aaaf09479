"""ctypes binding of libflub_gb300.so (the C ABI declared in include/flub_gb300.h).

There is no CPU fallback: if the library cannot be built or loaded, or a CUDA
call fails, the error is raised.
"""
import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None


class FlubError(RuntimeError):
    def __init__(self, status, where, detail):
        self.status = status
        super().__init__(f"{where}: {detail} (status {status})")


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("status", ctypes.c_int),
                ("reserved", ctypes.c_int), ("rtr0", ctypes.c_double), ("rtr", ctypes.c_double),
                ("tol", ctypes.c_double), ("x0_scale", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class Prim(ctypes.Structure):
    _fields_ = [("geometry", ctypes.c_int32), ("x", ctypes.c_float * 3), ("q", ctypes.c_float * 4),
                ("radius", ctypes.c_float * 3)]


assert ctypes.sizeof(Prim) == 44

_vp, _i32, _i64, _f32, _f64, _sz = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float,
                                    ctypes.c_double, ctypes.c_size_t)

# name -> (restype, argtypes); must match include/flub_gb300.h
SIGNATURES = {
    "flub_status_string": (ctypes.c_char_p, [_i32]),
    "flub_last_error": (ctypes.c_char_p, []),
    "flub_version": (_i32, []),
    "flub_tag_dirichlet": (_i32, [_vp, _vp, _i64, _vp]),
    "flub_phi_prims": (_i32, [_vp, _i32, _i32, _i32, _f32, _f32, _f32, _f32, _f32, _vp, _i32, _vp]),
    "flub_tag_neumann": (_i32, [_vp, _vp, _i64, _vp]),
    "flub_classify": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _f32, _f32, _vp, _vp, _vp]),
    "flub_divergence_tag": (_i32, [_vp] * 8 + [_i32, _i32, _i32, _vp]),
    "flub_mask_with_tag": (_i32, [_vp, _vp, _i64, _vp]),
    "flub_scale": (_i32, [_vp, _f32, _i64, _vp]),
    "flub_divergence_masked": (_i32, [_vp] * 8 + [_f32, _i32, _i32, _i32, _vp]),
    "flub_subtract_gradient_tag": (_i32, [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "flub_subtract_gradient": (_i32, [_vp] * 7 + [_f32, _vp, _i32, _i32, _i32, _vp]),
    "flub_solid_vel": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _f32, _vp, _vp, _vp, _i32, _vp]),
    "flub_phi_to_fraction": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "flub_divergence_fractional": (_i32, [_vp] * 10 + [_i32, _i32, _i32, _vp]),
    "flub_subtract_gradient_batty": (_i32, [_vp] * 5 + [_i32, _i32, _i32, _i32, _f32, _f32, _vp]),
    "flub_set_unknown": (_i32, [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp]),
    "flub_extrapolate_axis": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "flub_flush_unknown": (_i32, [_vp, _i64, _vp]),
    "flub_extrapolate": (_i32, [_vp] * 7 + [_i32, _i32, _i32, _i32, _vp]),
    "flub_advect_mc": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp, _i32, _i32, _i32, _f32, _f32, _f32,
                              _f32, _f32, _f32, _i32, _vp]),
    "flub_advect_velocity_mc": (_i32, [_vp] * 6 + [_i32, _i32, _i32, _f32, _f32, _f32, _vp]),
    "flub_advect_phi": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp, _i32, _i32, _i32, _f32, _f32, _f32, _f32,
                               _f32, _f32, _vp]),
    "flub_advect_simple": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp, _i32, _i32, _i32, _f32, _f32, _vp]),
    "flub_redistance_init": (_i32, [_vp, _vp, _i32, _i32, _i32, _f32, _i32, _vp]),
    "flub_redistance_sweep": (_i32, [_vp, _i32, _i32, _i32, _i32, _i32, _i32, _i32, _f32, _vp]),
    "flub_redistance": (_i32, [_vp, _vp, _i32, _i32, _i32, _f32, _i32, _i32, _vp]),
    "flub_mg_workspace_bytes": (_sz, [_i32, _i32, _i32, _i32, _i32]),
    "flub_mg_create": (_i32, [_i32, _i32, _i32, _i32, _i32, _vp, _sz, ctypes.POINTER(_vp)]),
    "flub_mg_destroy": (_i32, [_vp]),
    "flub_mg_set_tags": (_i32, [_vp, _vp, _vp]),
    "flub_mg_init": (_i32, [_vp, _vp, _f32, _vp]),
    "flub_mg_mask_interior": (_i32, [_vp, _vp]),
    "flub_mg_set_x0": (_i32, [_vp, _vp, _vp]),
    "flub_mg_solve": (_i32, [_vp, _i32, _f64, _f64, _f64, _i32, _vp, ctypes.POINTER(SolveInfo)]),
    "flub_mg_get_info": (_i32, [_vp, _vp, ctypes.POINTER(SolveInfo)]),
    "flub_mg_residual_history": (_i32, [_vp, _vp, ctypes.POINTER(_f64), _i32, ctypes.POINTER(_i32)]),
    "flub_mg_x": (_vp, [_vp]),
    "flub_mg_r": (_vp, [_vp]),
    "flub_mg_get_x": (_i32, [_vp, _vp, _f32, _vp]),
    "flub_mg_apply_preconditioner": (_i32, [_vp, _vp, _vp, _vp]),
    "flub_mg_matvec": (_i32, [_vp, _vp, _vp, _vp]),
    "flub_mg_kernels_executed": (_i32, [_vp, _vp, ctypes.POINTER(_i64)]),
    "flub_mg_smooth": (_i32, [_vp, _i32, _i32, _vp]),
    "flub_mg_smooth_iteration": (_i32, [_vp, _i32, _i32, ctypes.POINTER(_i32), _vp]),
    "flub_mg_set_schedule": (_i32, [_vp, _i32, _i32, _f32]),
    "flub_mg_set_bottom_precision": (_i32, [_vp, _i32]),
    "flub_mg_get_bottom_precision": (_i32, [_vp, ctypes.POINTER(_i32)]),
    "flub_mg_set_x0_scaled": (_i32, [_vp, _vp, _vp]),
    "flub_mg_level_shape": (_i32, [_vp, _i32, ctypes.POINTER(_i32), ctypes.POINTER(_i32), ctypes.POINTER(_i32)]),
    "flub_mg_level_tags": (_i32, [_vp, _i32, _vp, _vp]),
    "flub_mg_restrict_vector": (_i32, [_vp, _i32, _vp, _vp, _vp]),
    "flub_mg_prolong_vector": (_i32, [_vp, _i32, _vp, _vp, _vp]),
    "flub_vcycle_noalloc": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "flub_launch_count": (_i64, []),
    "flub_reset_launch_count": (None, []),
    "flub_conv3d_bf16": (_i32, [_vp, _i32, _vp, _vp, _i32, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp]),
    "flub_conv3d_wgrad": (_i32, [_vp, _i32, _vp, _i32, _vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "flub_conv_error": (_i32, [ctypes.POINTER(_i32), _i32]),
    "flub_unet_input": (_i32, [_vp, _vp, _i32, _i64, _vp, _vp, _vp, _vp]),
    "flub_pool2_bf16": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp]),
    "flub_pool2_bwd_bf16": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _vp]),
    "flub_up2_bf16": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp]),
    "flub_up2_bwd_bf16": (_i32, [_vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp]),
    "flub_relu_bwd_bf16": (_i32, [_vp, _vp, _vp, _i64, _vp]),
    "flub_head_fwd": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp]),
    "flub_head_bwd": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _vp]),
    "flub_unet_loss": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _f64, _vp, _vp, _vp, _vp]),
    "flub_unet_output": (_i32, [_vp, _vp, _vp, _i64, _i32, _f32, _vp, _vp]),
    "flub_adam": (_i32, [_vp, _vp, _vp, _vp, _i64, _f32, _f32, _f32, _f32, _i32, _vp, _vp, _i32, _i32, _vp]),
}


def library_path() -> str:
    return _build.LIB


def load():
    """Load (building first if needed) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            lib = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(status, where):
    if status != 0:
        lib = load()
        detail = lib.flub_last_error().decode(errors="replace") or lib.flub_status_string(status).decode()
        raise FlubError(status, where, detail)


def call(name, *args):
    fn = getattr(load(), name)
    check(fn(*args), name)
