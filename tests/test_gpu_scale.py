"""The scale workload: 1,048,576 strands x 32 vertices (33,554,432 vertices,
32,505,856 segments) grown on a radius-1.2 hemisphere with step 0.04,
segment-voxelized into 512^3 and raymarched at 3840x2160 with 1024 steps,
128-step shadows, 16-direction AO and the workloads' dual-lobe Kajiya-Kay,
plus four 3840x2160 views of the volume in one batched launch.

The voxelization is checked bit for bit against the oracle over the whole
grid (counts, u8 densities, int8 tangents) in the reference's FP32 index
mode, which at 512^3 (> 2^24 voxels) reproduces the reference's rounded
indices (hair_style.cc:321).  The frame is checked against the FP64 oracle
on row bands; the four batched views equal their single-view renders, and
each is checked against the FP64 oracle on a row band."""
import numpy as np
import pytest

from vkhr_gb300 import _abi, _native, scene, strands
from tests._helpers import compare_images, to_dev

pytestmark = pytest.mark.gpu

RES = (512, 512, 512)


@pytest.fixture(scope="module")
def scale_style():
    st = strands.hemisphere_style(1_048_576, 32, radius=1.2, step_length=0.04, seed=4)
    t = strands.generate_tangents(st.vertices, st.segments)
    idx = strands.generate_indices(st.segments)
    return st, t, idx


@pytest.fixture(scope="module")
def scale_volume(ctx, oracle_lib, scale_style):
    """GPU voxelization (checked against the oracle) and its normalized densities."""
    import torch

    st, t, idx = scale_style
    assert st.vertex_count == 33_554_432 and st.segment_count == 32_505_856
    b = oracle_lib.bounding_box(st.vertices)
    n = RES[0] * RES[1] * RES[2]
    dv, dt, di = to_dev(st.vertices, torch), to_dev(t, torch), to_dev(idx, torch)
    counts = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    dens = torch.full((n,), 77, dtype=torch.uint8, device="cuda")
    tq = torch.full((n, 4), 55, dtype=torch.int8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    ctx.voxelize_segments(dv.data_ptr(), dt.data_ptr(), di.data_ptr(), int(idx.shape[0]), b, RES,
                          _abi.INDEX_REF_FP32, counts.data_ptr(), dens.data_ptr(), tq.data_ptr(), s)
    ctx.check_status(s)
    torch.cuda.synchronize()
    del dv, dt, di
    c_ref, d_ref, t_ref, _ = oracle_lib.voxelize("segments", st.vertices, t, idx, b, RES, _abi.INDEX_REF_FP32)
    c = counts.cpu().numpy().view(np.uint32)
    assert np.array_equal(c, c_ref), "counts differ in %d voxels" % int((c != c_ref).sum())
    del c, c_ref
    d = dens.cpu().numpy()
    assert np.array_equal(d, d_ref), "u8 densities differ in %d voxels" % int((d != d_ref).sum())
    g = tq.cpu().numpy()
    bad = np.any(g != t_ref, axis=1)
    assert not bad.any(), "tangents differ in %d voxels" % int(bad.sum())
    del d_ref, t_ref, g
    ctx.normalize_densities(dens.data_ptr(), n, s)
    torch.cuda.synchronize()
    return b, dens, tq


def test_scale_voxelization_bit_exact(scale_volume):
    b, dens, tq = scale_volume
    assert int(dens.max().item()) == 255


def _params(b, w, h, **kw):
    return scene.make_params(b, RES, w, h, camera_distance=5.0, raycast_steps=1024.0, shadow_steps=128.0,
                             ao_directions=16, **scene.CONFIG_SHADING, **kw)


def test_scale_frame_rows(ctx, oracle_lib, scale_volume):
    import torch

    b, dens, tq = scale_volume
    p = _params(b, 3840, 2160)
    rgba = torch.full((2160, 3840, 4), -7.0, dtype=torch.float32, device="cuda")
    depth = torch.full((2160, 3840), -7.0, dtype=torch.float32, device="cuda")
    ctx.raymarch(p, dens.data_ptr(), tq.data_ptr(), None, rgba.data_ptr(), depth.data_ptr(),
                 torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    gpu, gdepth = rgba.cpu().numpy(), depth.cpu().numpy()
    lit = np.nonzero((gpu[..., 3] > 0).any(axis=1))[0]
    assert lit.size > 200
    lo, hi = int(lit.min()), int(lit.max())
    dn, tqn = dens.cpu().numpy(), tq.cpu().numpy()
    excluded = emitted = 0
    for f in (0.2, 0.35, 0.5, 0.65, 0.8):  # inside the lit span: grazing rows at its edges are mostly ill-conditioned
        r0 = int(lo + f * (hi - lo))
        rows = (r0, r0 + 16)
        ref, rdepth, diag = oracle_lib.raymarch(p, dn, tqn, diag=True, rows=rows)
        _, _, ex, em = compare_images(gpu[r0:r0 + 16], gdepth[r0:r0 + 16], ref[r0:r0 + 16], rdepth[r0:r0 + 16],
                                      diag[r0:r0 + 16], label="scale frame rows %d..%d" % rows, max_excluded=0.03)
        excluded += ex
        emitted += em
    assert excluded <= 0.01 * emitted, (excluded, emitted)


def test_scale_four_views_batched(ctx, oracle_lib, scale_volume):
    """Four 3840x2160 views of the 512^3 volume in one batched launch equal
    the four single-view renders, pixel for pixel, and each matches the FP64
    oracle on a band of rows through its middle."""
    import torch

    b, dens, tq = scale_volume
    s = torch.cuda.current_stream().cuda_stream
    views = [_params(b, 3840, 2160, view_direction=vd) for vd in
             ((0.0, 0.0, 1.0), (1.0, 0.3, 0.0), (0.0, 1.0, 0.2), (-0.7, 0.2, -0.7))]
    rects = [_native.raymarch_footprint(p) for p in views]
    pitch = sum(r[2] for r in rects)
    rows = max(r[3] for r in rects)
    atlas = torch.zeros((rows, pitch, 4), dtype=torch.float32, device="cuda")
    jobs, at = [], 0
    for p, (x0, y0, w, h) in zip(views, rects):
        j = _abi.RaymarchJob()
        j.params = p
        j.d_density, j.d_tangent = dens.data_ptr(), tq.data_ptr()
        j.d_rgba = atlas[0, at].data_ptr()
        j.x0, j.y0, j.w, j.h, j.pitch = x0, y0, w, h, pitch
        jobs.append(j)
        at += w
    ctx.raymarch_batched(jobs, s)
    torch.cuda.synchronize()
    A = atlas.cpu().numpy()
    full = torch.empty((2160, 3840, 4), dtype=torch.float32, device="cuda")
    full_d = torch.empty((2160, 3840), dtype=torch.float32, device="cuda")
    dn, tqn = dens.cpu().numpy(), tq.cpu().numpy()
    at = excluded = emitted = 0
    for k, (p, (x0, y0, w, h)) in enumerate(zip(views, rects)):
        ctx.raymarch(p, dens.data_ptr(), tq.data_ptr(), None, full.data_ptr(), full_d.data_ptr(), s)
        torch.cuda.synchronize()
        F, FD = full.cpu().numpy(), full_d.cpu().numpy()
        assert np.array_equal(A[:h, at:at + w], F[y0:y0 + h, x0:x0 + w])
        assert (F[..., 3] > 0).any()
        r0 = y0 + h // 2 - 8
        ref, rdepth, diag = oracle_lib.raymarch(p, dn, tqn, diag=True, rows=(r0, r0 + 16))
        sl = slice(r0, r0 + 16)
        _, _, ex, em = compare_images(F[sl], FD[sl], ref[sl], rdepth[sl], diag[sl],
                                      label="scale view %d rows %d..%d" % (k, r0, r0 + 16), max_excluded=0.03)
        excluded += ex
        emitted += em
        at += w
    assert excluded <= 0.01 * emitted, (excluded, emitted)
