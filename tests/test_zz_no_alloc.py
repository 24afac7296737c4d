"""vkhr_raymarch_static, the allocation-free raymarch.

Some callers may not allocate device memory at all: a real-time frame loop
that forbids cudaMalloc (it synchronises the device and its latency is
unbounded), or a host engine that owns the GPU memory budget and does not let
plugins allocate.  For them the library keeps the raymarch's only scratch,
its brick occupancy bitmap, in a fixed array inside the library.  This test
calls that entry point through the C ABI twice in a row on different volumes
(the second call must not see the first call's bits) and checks each image
against the regular vkhr_raymarch with the raymarch tolerance of the suite
(per channel RMS <= 1e-3, max <= 2e-2).  It lives in a file of its own that
pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

from vkhr_gb300 import _abi, scene
from tests._helpers import style

pytestmark = pytest.mark.gpu

RMS_TOL = 1e-3
MAX_TOL = 2e-2


def _volume(O, kind, n, verts, res, seed):
    st, t, idx = style(kind, n, verts, seed=seed)
    b = O.bounding_box(st.vertices)
    c, d, tq, _ = O.voxelize("segments", st.vertices, t, idx, b, res)
    return b, O.normalize(d), tq


def test_static_raymarch_matches_context_raymarch(native_lib, oracle_lib):
    import torch

    from vkhr_gb300 import _native

    lib = native_lib
    P = C.c_void_p
    lib.vkhr_raymarch_static.argtypes = [C.POINTER(_abi.RaymarchParams), P, P, P, P, P, P]
    lib.vkhr_raymarch_static.restype = C.c_int
    ctx = _native.Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    cases = []
    for kind, n, verts, res, seed, view in (("hemi", 3000, 14, (40, 40, 40), 21, (0.0, 0.0, 1.0)),
                                            ("disk", 6000, 10, (56, 48, 36), 22, (0.5, 0.2, 1.0))):
        b, dn, tq = _volume(oracle_lib, kind, n, verts, res, seed)
        p = scene.make_params(b, res, 160, 120, raycast_steps=256.0, shadow_steps=32.0, view_direction=view)
        cases.append((p, torch.from_numpy(dn).cuda(), torch.from_numpy(tq).cuda()))
    outs = []
    for p, dd, dt in cases:  # two calls in a row; the array keeps the first call's bits
        rgba = torch.full((p.height, p.width, 4), -1.0, device="cuda")
        depth = torch.full((p.height, p.width), -1.0, device="cuda")
        rc = lib.vkhr_raymarch_static(C.byref(p), dd.data_ptr(), dt.data_ptr(), None, rgba.data_ptr(),
                                      depth.data_ptr(), stream)
        assert rc == _abi.VKHR_OK
        outs.append((rgba, depth))
    torch.cuda.synchronize()
    for (p, dd, dt), (rgba, depth) in zip(cases, outs):
        ref = torch.empty_like(rgba)
        ref_depth = torch.empty_like(depth)
        ctx.raymarch(p, dd.data_ptr(), dt.data_ptr(), None, ref.data_ptr(), ref_depth.data_ptr(), stream)
        torch.cuda.synchronize()
        a, r = rgba.cpu().numpy().astype(np.float64), ref.cpu().numpy().astype(np.float64)
        assert (r[..., 3] > 0).sum() > 100
        d = np.abs(a - r)
        assert np.all(np.sqrt((d ** 2).mean(axis=(0, 1))) <= RMS_TOL)
        assert d.max() <= MAX_TOL
        assert np.abs(depth.cpu().numpy() - ref_depth.cpu().numpy()).max() <= 1e-4
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
