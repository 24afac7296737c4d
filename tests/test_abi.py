"""The C ABI library loads and exports every entry point include/vkhr_cuda.h
declares, with the structure layouts the bindings assume (no GPU call)."""
import ctypes as C
import os
import re

from vkhr_gb300 import _abi

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "vkhr_cuda.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(vkhr_\w+)\s*\(", src, flags=re.M)))


def test_every_declared_symbol_is_exported(native_lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(native_lib, n), n


def test_struct_layouts(native_lib):
    assert native_lib.vkhr_sizeof_aabb() == C.sizeof(_abi.AABB) == 32
    assert native_lib.vkhr_sizeof_raymarch_params() == C.sizeof(_abi.RaymarchParams)
    assert native_lib.vkhr_sizeof_voxel_job() == C.sizeof(_abi.VoxelJob) == 104
    assert native_lib.vkhr_sizeof_raymarch_job() == C.sizeof(_abi.RaymarchJob)
    assert native_lib.vkhr_abi_version() == 2


def test_status_strings_and_null_context(native_lib):
    native_lib.vkhr_status_string.restype = C.c_char_p
    assert native_lib.vkhr_status_string(_abi.VKHR_ERR_CAPACITY) == b"VKHR_ERR_CAPACITY"
    # a NULL context is rejected before any CUDA call
    assert native_lib.vkhr_voxelize_vertices(None, None, None, 0, None, 1, 1, 1, 0, None, None, None,
                                             None) == _abi.VKHR_ERR_INVALID_ARG
    assert native_lib.vkhr_raymarch(None, None, None, None, None, None, None, None) == _abi.VKHR_ERR_INVALID_ARG


def test_constants_match_header(native_lib):
    src = open(HEADER).read()

    def define(name):
        return int(re.search(r"#define %s (\d+)" % name, src).group(1))

    assert define("VKHR_RAYMARCH_VARIANTS") == _abi.RAYMARCH_VARIANTS
    assert define("VKHR_WALK_CHOICES") == len(_abi.WALK_CHOICES)
    assert native_lib.vkhr_set_voxelize_walk(None, 0, 4) == _abi.VKHR_ERR_INVALID_ARG
    assert native_lib.vkhr_autotune_voxelize(None, None, 1, None, None, None) == _abi.VKHR_ERR_INVALID_ARG
