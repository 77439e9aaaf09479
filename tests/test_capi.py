"""The C ABI (include/flub_gb300.h): the library builds for sm_103a, loads,
exports every declared symbol, and validates arguments before touching the
GPU.  No compute calls: these tests run without a GPU."""
import ctypes
import os
import re

import pytest

from flub_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "flub_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(flub_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def test_library_builds_for_sm103a(lib):
    assert os.path.exists(build.LIB)
    assert "arch=compute_103a,code=sm_103a" in build.ARCH


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n


def test_binding_table_matches_header():
    assert sorted(_lib.SIGNATURES) == declared_functions()


def test_status_strings(lib):
    assert lib.flub_status_string(0) == b"ok"
    assert lib.flub_status_string(1) == b"invalid argument"
    assert lib.flub_status_string(999) == b"unknown status"
    assert lib.flub_version() >= 100


def test_workspace_size_and_shape_validation(lib):
    assert lib.flub_mg_workspace_bytes(64, 64, 64, 4, 0) > 3 * 64 ** 3 * 4
    assert lib.flub_mg_workspace_bytes(64, 64, 60, 4, 0) == 0           # 60 not divisible by 8
    assert lib.flub_mg_workspace_bytes(16, 16, 8, 4, 0) == 0            # nz >> 3 = 1 is odd
    assert lib.flub_mg_workspace_bytes(64, 64, 64, 0, 0) == 0
    assert lib.flub_mg_workspace_bytes(64, 64, 64, 4, 7) == 0


def test_create_rejects_bad_shapes_without_a_gpu(lib):
    h = ctypes.c_void_p()
    st = lib.flub_mg_create(30, 32, 32, 3, 0, None, 0, ctypes.byref(h))
    assert st == 1 and h.value is None
    assert b"divisible" in lib.flub_last_error()


def test_kernel_entry_points_validate_first(lib):
    assert lib.flub_tag_dirichlet(None, None, 0, None) == 0            # empty: nothing to do
    assert lib.flub_tag_dirichlet(None, None, 5, None) == 1            # NULL with n > 0
    assert lib.flub_phi_prims(ctypes.c_void_p(16), 2, 2, 2, 0.5, 0.5, 0.5, 0.5, 0.5, None, 65, None) == 1
    assert lib.flub_subtract_gradient_tag(None, None, None, None, 4, 4, 4, 4, None) == 1
    assert lib.flub_divergence_tag(*([None] * 8), 0, 4, 4, None) == 1
    assert lib.flub_mg_solve(None, 10, 1e-12, 0.0, 1e-12, 1, None, None) == 1
