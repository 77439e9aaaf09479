"""Grid containers of the projection path, as torch CUDA tensors.

Counterparts of const_param.py:80-143 (Field, IntField, MACGrid, MACGridInt,
make_field, make_mac_grid).  Arrays are C-order [i, j, k]; cell-centred fields
have ``shape``, face fields ``shape + e_d`` along their axis d (1 = u, 2 = v,
3 = w).  ``stagger`` and ``d`` carry the same meaning as in the reference.
"""
from dataclasses import dataclass
from typing import Optional, Tuple

import torch

# const_param.py:34-37: the reference's default grid (256 x 64 x 256).
DEFAULT_SHAPE = (256, 64, 256)

_STAGGER = {0: (0.5, 0.5, 0.5), 1: (0.0, 0.5, 0.5), 2: (0.5, 0.0, 0.5), 3: (0.5, 0.5, 0.0)}


@dataclass
class Field:
    """A float field; ``stagger`` defaults to the one make_field gives axis
    ``d`` (cell centres for d = 0, face centres for d = 1, 2, 3)."""
    f: torch.Tensor
    stagger: Optional[Tuple[float, float, float]] = None
    d: int = 0

    def __post_init__(self):
        if self.stagger is None:
            self.stagger = _STAGGER[self.d]


@dataclass
class IntField:
    f: torch.Tensor
    stagger: Optional[Tuple[float, float, float]] = None
    d: int = 0

    def __post_init__(self):
        if self.stagger is None:
            self.stagger = _STAGGER[self.d]


@dataclass
class MACGrid:
    u: Field
    v: Field
    w: Field


@dataclass
class MACGridInt:
    u: IntField
    v: IntField
    w: IntField


def field_shape(shape, dim):
    s = list(shape)
    if dim in (1, 2, 3):
        s[dim - 1] += 1
    return tuple(s)


def make_field(dim, dtype=float, shape=DEFAULT_SHAPE, device="cuda"):
    """const_param.py:114-133: zero field on cells (dim 0) or faces (1, 2, 3)."""
    is_float = dtype in (float, torch.float32)
    t = torch.zeros(field_shape(shape, dim), dtype=torch.float32 if is_float else torch.int32, device=device)
    cls = Field if is_float else IntField
    return cls(f=t, stagger=_STAGGER[dim], d=dim)


def make_mac_grid(dtype=float, shape=DEFAULT_SHAPE, device="cuda"):
    """const_param.py:135-143."""
    mk = MACGrid if dtype in (float, torch.float32) else MACGridInt
    return mk(*(make_field(d, dtype, shape, device) for d in (1, 2, 3)))


def field_like(field):
    """const_param.py:145-150."""
    return type(field)(f=torch.zeros_like(field.f), stagger=field.stagger, d=field.d)


def get_uf(vels, d):
    """const_param.py:104-110: the face field of axis d (1, 2, 3)."""
    return (vels.u, vels.v, vels.w)[d - 1]
