"""vkhr_raymarch_static, the allocation-free raymarch.

Some callers may not allocate device memory at all: a real-time frame loop
that forbids cudaMalloc (it synchronises the device and its latency is
unbounded), or a host engine that owns the GPU memory budget and does not let
plugins allocate.  For them the library keeps the raymarch's only scratch,
its brick occupancy bitmap, in a fixed array inside the library.  This test
calls that entry point through the C ABI twice in a row on different volumes
(the second call must not see the first call's bits), for every pair of
density and tangent texel formats, and checks each image against the
regular vkhr_raymarch: the two run the same kernel, so the images must be
equal bit for bit.  The device's free memory must not change across the
second call.  It lives in a file of its own that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

from vkhr_gb300 import _abi, scene
from tests._helpers import style

pytestmark = pytest.mark.gpu

FORMATS = [(d, t) for d in (_abi.DENSITY_U8_UNORM, _abi.DENSITY_U32_COUNT, _abi.DENSITY_F32)
           for t in (_abi.TANGENT_I8_SNORM, _abi.TANGENT_F32X4)]


def _volume(O, kind, n, verts, res, seed, density_format, tangent_format):
    """Density texels in the format asked for (normalized u8, raw counts, or
    counts as floats), tangents as int8 x4 or their SNORM values as floats."""
    st, t, idx = style(kind, n, verts, seed=seed)
    b = O.bounding_box(st.vertices)
    c, d, tq, _ = O.voxelize("segments", st.vertices, t, idx, b, res)
    if density_format == _abi.DENSITY_U8_UNORM:
        dens, iso = O.normalize(d), 0.115
    elif density_format == _abi.DENSITY_U32_COUNT:
        dens, iso = c, 1.0
    else:
        dens, iso = c.astype(np.float32) * np.float32(0.5), 0.5
    if tangent_format == _abi.TANGENT_F32X4:
        tq = np.maximum(tq.astype(np.float32) / 127.0, -1.0)
    return b, dens, tq, iso


@pytest.mark.parametrize("density_format,tangent_format", FORMATS)
def test_static_raymarch_matches_context_raymarch(native_lib, oracle_lib, density_format, tangent_format):
    import torch

    from vkhr_gb300 import _native
    from tests._helpers import to_dev

    lib = native_lib
    P = C.c_void_p
    lib.vkhr_raymarch_static.argtypes = [C.POINTER(_abi.RaymarchParams), P, P, P, P, P, P]
    lib.vkhr_raymarch_static.restype = C.c_int
    ctx = _native.Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    cases = []
    for kind, n, verts, res, seed, view in (("hemi", 3000, 14, (40, 40, 40), 21, (0.0, 0.0, 1.0)),
                                            ("disk", 6000, 10, (56, 48, 36), 22, (0.5, 0.2, 1.0))):
        b, dens, tan, iso = _volume(oracle_lib, kind, n, verts, res, seed, density_format, tangent_format)
        p = scene.make_params(b, res, 160, 120, raycast_steps=256.0, shadow_steps=32.0, view_direction=view,
                              isosurface=iso, density_format=density_format, tangent_format=tangent_format)
        cases.append((p, to_dev(dens, torch), to_dev(tan, torch)))
    outs = [(torch.full((p.height, p.width, 4), -1.0, device="cuda"), torch.full((p.height, p.width), -1.0, device="cuda"))
            for p, _, _ in cases]
    torch.cuda.synchronize()
    free = []
    for (p, dd, dt), (rgba, depth) in zip(cases, outs):  # two calls in a row; the array keeps the first call's bits
        free.append(torch.cuda.mem_get_info()[0])
        rc = lib.vkhr_raymarch_static(C.byref(p), dd.data_ptr(), dt.data_ptr(), None, rgba.data_ptr(),
                                      depth.data_ptr(), stream)
        assert rc == _abi.VKHR_OK
        torch.cuda.synchronize()
    free.append(torch.cuda.mem_get_info()[0])
    assert free[2] == free[1], "device memory changed across a call: %d -> %d bytes free" % (free[1], free[2])
    for (p, dd, dt), (rgba, depth) in zip(cases, outs):
        ref = torch.empty_like(rgba)
        ref_depth = torch.empty_like(depth)
        ctx.raymarch(p, dd.data_ptr(), dt.data_ptr(), None, ref.data_ptr(), ref_depth.data_ptr(), stream)
        torch.cuda.synchronize()
        assert (ref[..., 3] > 0).sum().item() > 100
        assert torch.equal(rgba, ref), "images differ in %d pixels" % int((rgba != ref).any(dim=2).sum().item())
        assert torch.equal(depth, ref_depth)
    ctx.close()


def test_static_raymarch_rejects_grids_above_its_scratch(native_lib, oracle_lib):
    import torch

    lib = native_lib
    P = C.c_void_p
    lib.vkhr_raymarch_static.argtypes = [C.POINTER(_abi.RaymarchParams), P, P, P, P, P, P]
    lib.vkhr_raymarch_static.restype = C.c_int
    b = _abi.aabb_from((0, 0, 0), (1, 1, 1))
    p = scene.make_params(b, (1024, 1024, 1024), 32, 24, raycast_steps=64.0)
    small = torch.zeros(64, dtype=torch.uint8, device="cuda")
    rgba = torch.zeros((24, 32, 4), device="cuda")
    rc = lib.vkhr_raymarch_static(C.byref(p), small.data_ptr(), small.data_ptr(), None, rgba.data_ptr(), None,
                                  torch.cuda.current_stream().cuda_stream)
    assert rc == _abi.VKHR_ERR_CAPACITY
