"""The C-ABI library builds, loads and exports every entry point the public
header declares; argument validation needs no GPU."""
import ctypes as C
import os
import re

import pytest

import cadise_gb300 as cg
from cadise_gb300 import abi

INCLUDE = os.path.join(os.path.dirname(__file__), "..", "include")


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if f.endswith(".h"):
            names |= set(re.findall(r"\b(cgpu_[a-z_0-9]+)\s*\(", open(os.path.join(INCLUDE, f)).read()))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    cg.build()
    return cg.load()


def test_header_declares_the_exported_list():
    assert declared_functions() == sorted(cg.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_abi_version_and_status_strings(lib):
    assert lib.cgpu_abi_version() == 5
    for code, name in abi.STATUS_NAMES.items():
        assert lib.cgpu_status_string(code).decode() == name


def test_null_arguments_are_rejected(lib):
    assert lib.cgpu_create(None, None) == 1  # CGPU_ERR_INVALID_ARGUMENT
    assert lib.cgpu_synchronize(None) == 1
    assert lib.cgpu_render(None, None) == 1
    assert lib.cgpu_scene_upload(None, None, None) == 1
    lib.cgpu_destroy(None)  # no-op


@pytest.mark.skipif(cg.gpu_available(), reason="checks the no-device path")
def test_create_without_a_device_reports_no_device(lib):
    h = C.c_void_p()
    assert lib.cgpu_create(C.byref(h), None) == 8  # CGPU_ERR_NO_DEVICE
    assert not h.value


def test_struct_layouts_match_header():
    assert C.sizeof(abi.cgpu_ray) == 32
    assert C.sizeof(abi.cgpu_hit) == 16
    assert C.sizeof(abi.cgpu_material) == 64
    assert C.sizeof(abi.cgpu_area_light) == 24
    assert C.sizeof(abi.cgpu_render_params) == 48
    assert C.sizeof(abi.cgpu_film_filter) == 40
