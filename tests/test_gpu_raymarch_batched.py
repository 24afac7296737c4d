"""Batched raymarch (vkhr_raymarch_batched): views of several styles, each
rendering its screen footprint into an atlas, in one persistent launch.
Every pixel must equal the single-view vkhr_raymarch's (same kernel body);
one view is also checked against the FP64 oracle (volume.frag:31-103), and a
CUDA-graph replay must reproduce the uncaptured result."""
import numpy as np
import pytest

from vkhr_gb300 import _abi, _native, scene
from vkhr_gb300._native import VkhrError
from tests._helpers import image_errors, style, to_dev

pytestmark = pytest.mark.gpu

VIEWS = [  # (kind, strands, vertices/strand, resolution, width, height, distance, direction, steps)
    ("hemi", 4096, 16, (64, 64, 64), 640, 480, 4.0, (0.0, 0.0, 1.0), 256.0),
    ("disk", 3000, 13, (48, 48, 48), 800, 600, 9.0, (1.0, 0.4, 0.2), 128.0),
    ("hemi", 1500, 24, (32, 32, 32), 512, 512, 15.0, (0.0, 1.0, 0.3), 100.0),
    ("disk", 800, 8, (64, 64, 64), 320, 240, 6.0, (-0.5, 0.2, 1.0), 512.0),
    ("hemi", 6000, 10, (37, 50, 29), 1024, 768, 25.0, (0.3, -0.2, 1.0), 64.0),
]


def _views(O, density_format=_abi.DENSITY_U8_UNORM):
    out = []
    for k, (kind, n, verts, res, w, h, dist, vd, steps) in enumerate(VIEWS):
        st, t, idx = style(kind, n, verts, seed=k)
        b = O.bounding_box(st.vertices)
        c, d, tq, _ = O.voxelize("segments", st.vertices, t, idx, b, res)
        if density_format == _abi.DENSITY_U8_UNORM:
            dens, iso = O.normalize(d), 0.115
        else:
            dens, iso = c, 1.0
        p = scene.make_params(b, res, w, h, camera_distance=dist, view_direction=vd, raycast_steps=steps,
                              shadow_steps=32.0, isosurface=iso, density_format=density_format)
        out.append((p, dens, tq))
    return out


def _atlas(torch, views, with_depth_in=False):
    """Device volumes, one atlas (rows of regions side by side) and the job table."""
    rects = [_native.raymarch_footprint(p) for p, _, _ in views]
    pitch = sum(r[2] for r in rects) + 3  # an odd pitch: regions start anywhere in a row
    rows = max(r[3] for r in rects)
    rgba = torch.full((rows, pitch, 4), -7.0, dtype=torch.float32, device="cuda")
    depth = torch.full((rows, pitch), -7.0, dtype=torch.float32, device="cuda")
    depth_in = torch.full((rows, pitch), 0.9995, dtype=torch.float32, device="cuda") if with_depth_in else None
    keep, jobs, at = [], [], 0
    for (p, dens, tq), (x0, y0, w, h) in zip(views, rects):
        dd, dt = to_dev(dens, torch), to_dev(tq, torch)
        keep += [dd, dt]
        j = _abi.RaymarchJob()
        j.params = p
        j.d_density, j.d_tangent = dd.data_ptr(), dt.data_ptr()
        j.d_rgba = rgba[0, at].data_ptr()
        j.d_depth_out = depth[0, at].data_ptr()
        j.d_depth_in = depth_in[0, at].data_ptr() if with_depth_in else None
        j.x0, j.y0, j.w, j.h, j.pitch = x0, y0, w, h, pitch
        jobs.append(j)
        at += w
    return rects, rgba, depth, depth_in, jobs, keep


def _single(ctx, torch, p, dens, tq, depth_in=None):
    rgba = torch.full((p.height, p.width, 4), -7.0, dtype=torch.float32, device="cuda")
    depth = torch.full((p.height, p.width), -7.0, dtype=torch.float32, device="cuda")
    dd, dt = to_dev(dens, torch), to_dev(tq, torch)
    di = None if depth_in is None else torch.full((p.height, p.width), depth_in, dtype=torch.float32, device="cuda")
    ctx.raymarch(p, dd.data_ptr(), dt.data_ptr(), None if di is None else di.data_ptr(), rgba.data_ptr(),
                 depth.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rgba.cpu().numpy(), depth.cpu().numpy()


def _check_against_single(ctx, torch, views, rects, rgba, depth, depth_in_value=None):
    A, D = rgba.cpu().numpy(), depth.cpu().numpy()
    at = 0
    for (p, dens, tq), (x0, y0, w, h) in zip(views, rects):
        full, fdepth = _single(ctx, torch, p, dens, tq, depth_in_value)
        outside = np.ones((p.height, p.width), dtype=bool)
        outside[y0:y0 + h, x0:x0 + w] = False
        assert not full[outside].any() and np.all(fdepth[outside] == 1.0), "footprint misses a fragment"
        assert np.array_equal(A[:h, at:at + w], full[y0:y0 + h, x0:x0 + w])
        assert np.array_equal(D[:h, at:at + w], fdepth[y0:y0 + h, x0:x0 + w])
        assert (full[..., 3] > 0).any()
        at += w


@pytest.mark.parametrize("fmt", [_abi.DENSITY_U8_UNORM, _abi.DENSITY_U32_COUNT])
def test_batched_equals_single_view(ctx, oracle_lib, fmt):
    import torch

    views = _views(oracle_lib, fmt)
    rects, rgba, depth, _, jobs, keep = _atlas(torch, views)
    ctx.raymarch_batched(jobs, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    _check_against_single(ctx, torch, views, rects, rgba, depth)


def test_batched_depth_buffer(ctx, oracle_lib):
    import torch

    views = _views(oracle_lib)
    rects, rgba, depth, _, jobs, keep = _atlas(torch, views, with_depth_in=True)
    ctx.raymarch_batched(jobs, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    _check_against_single(ctx, torch, views, rects, rgba, depth, depth_in_value=0.9995)


def test_batched_view_against_oracle(ctx, oracle_lib):
    """The first view's region against the FP64 oracle, within the tolerance
    of the single-view parity tests (RMS 1e-3, max 2e-2 per channel)."""
    import torch

    views = _views(oracle_lib)
    rects, rgba, depth, _, jobs, keep = _atlas(torch, views)
    ctx.raymarch_batched(jobs, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    p, dens, tq = views[0]
    x0, y0, w, h = rects[0]
    ref, rdepth, diag = oracle_lib.raymarch(p, dens, tq, diag=True)
    gpu = rgba.cpu().numpy()[:h, :w]
    rms, mx, excluded, emitted = image_errors(gpu, ref[y0:y0 + h, x0:x0 + w], diag[y0:y0 + h, x0:x0 + w])
    assert emitted > 0 and excluded <= max(2, 0.01 * emitted)
    assert np.all(rms <= 1e-3) and np.all(mx <= 2e-2), (rms, mx)


def test_batched_graph_replay(ctx, oracle_lib):
    import torch

    views = _views(oracle_lib)
    rects, rgba, depth, _, jobs, keep = _atlas(torch, views)
    s = torch.cuda.current_stream().cuda_stream
    ctx.raymarch_batched(jobs, s)  # sizes the scratch
    torch.cuda.synchronize()
    first = rgba.cpu().numpy().copy(), depth.cpu().numpy().copy()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        ctx.raymarch_batched(jobs, torch.cuda.current_stream().cuda_stream)
    for _ in range(3):
        rgba.fill_(-7.0)
        depth.fill_(-7.0)
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        assert np.array_equal(rgba.cpu().numpy(), first[0])
        assert np.array_equal(depth.cpu().numpy(), first[1])


def test_batched_rejects_bad_jobs(ctx, oracle_lib):
    import torch

    views = _views(oracle_lib)[:2]
    rects, rgba, depth, _, jobs, keep = _atlas(torch, views)
    s = torch.cuda.current_stream().cuda_stream
    with pytest.raises(VkhrError):
        ctx.raymarch_batched([], s)
    bad = _abi.RaymarchJob.from_buffer_copy(jobs[1])
    bad.params.density_format = _abi.DENSITY_U32_COUNT
    with pytest.raises(VkhrError) as e:
        ctx.raymarch_batched([jobs[0], bad], s)
    assert e.value.status == _abi.VKHR_ERR_INVALID_ARG
    bad = _abi.RaymarchJob.from_buffer_copy(jobs[1])
    bad.x0 = bad.params.width - bad.w + 1  # region leaves the view
    with pytest.raises(VkhrError) as e:
        ctx.raymarch_batched([jobs[0], bad], s)
    assert e.value.status == _abi.VKHR_ERR_INVALID_ARG
