"""flub_gb300: GB300-native (sm_103a) pressure projection for the flub fluid
simulator -- cell classification + divergence, MGPCG Poisson solve and the
pressure-gradient update -- behind the reference's own API.

    from flub_gb300 import MGPCG, launch, divergence_tag, mask_with_tag, \\
        subtract_gradient_tag, scale_by_3d, make_field, make_mac_grid

The CUDA library (flub_gb300/_build/libflub_gb300.so, C ABI in
include/flub_gb300.h) is built in-tree by ``flub_gb300.build.build()`` and
loaded on first use; there is no CPU fallback.
"""
from .fields import (DEFAULT_SHAPE, Field, IntField, MACGrid, MACGridInt, field_like, field_shape, get_uf,
                     make_field, make_mac_grid)
from .kernels import (DT, _advect_mc_1, _advect_mc_2, _advect_mc_3, _init_distance, _sweep, _tag_dirichlet, _tag_neumann, advect_3d,
                      advect_mc, advect_mc_stage, advect_phi, advect_phi_field, advect_simple, advect_simple_3d,
                      advect_uv_mc, classify, init_distance, redistance, sweep, sweep_half, divergence, divergence_fractional,
                      divergence_fractional_3d, divergence_tag, extrapolate, extrapolate_3d, extrapolate_by_1,
                      flush_1_3d, launch, mask_with_tag, phi_prims, phi_to_fraction, phi_to_fraction_3d,
                      precompute_grid_point_phi_prims, precompute_solid_vel, scale_by_3d, set_unknown, set_unknown_3d,
                      solid_vel, subtract_gradient, subtract_gradient_batty, subtract_gradient_tag, tag_dirichlet,
                      tag_neumann, u_subtract_gradient_batty_3d, v_subtract_gradient_batty_3d,
                      w_subtract_gradient_batty_3d)
from ._lib import FlubError
from .mgpcg import MGPCG
from .projection import Projection

__all__ = [
    "DEFAULT_SHAPE", "Field", "IntField", "MACGrid", "MACGridInt", "field_like", "field_shape", "get_uf",
    "make_field", "make_mac_grid", "_tag_dirichlet", "_tag_neumann", "classify", "divergence", "divergence_tag",
    "launch", "mask_with_tag", "phi_prims", "precompute_grid_point_phi_prims", "scale_by_3d", "subtract_gradient",
    "subtract_gradient_tag", "tag_dirichlet", "tag_neumann", "MGPCG", "Projection", "FlubError", "extrapolate",
    "extrapolate_3d", "extrapolate_by_1", "flush_1_3d", "set_unknown", "set_unknown_3d", "divergence_fractional",
    "divergence_fractional_3d", "phi_to_fraction", "phi_to_fraction_3d", "precompute_solid_vel", "solid_vel",
    "subtract_gradient_batty", "u_subtract_gradient_batty_3d", "v_subtract_gradient_batty_3d",
    "w_subtract_gradient_batty_3d", "DT", "_advect_mc_1", "_advect_mc_2", "_advect_mc_3", "advect_3d", "advect_mc",
    "advect_mc_stage", "advect_phi", "advect_phi_field", "advect_simple", "advect_simple_3d", "advect_uv_mc",
    "_init_distance", "_sweep", "init_distance", "redistance", "sweep", "sweep_half",
]
