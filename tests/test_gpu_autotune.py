"""The raymarch autotuner: every ray-packet variant it tunes renders the same
image (same per-pixel device code), and vkhr_autotune_raymarch keeps a
variant that later calls use.  The TMA-staged variant equals the L2 march
bit for bit; the texture-unit variant is measured against the FP64 oracle."""
import numpy as np
import pytest

from vkhr_gb300 import _abi, scene
from vkhr_gb300._native import VkhrError
from tests._helpers import style, to_dev

pytestmark = pytest.mark.gpu


def test_variants_render_the_same_image(ctx, oracle_lib):
    import torch

    st, t, idx = style("hemi", 4096, 16)
    b = oracle_lib.bounding_box(st.vertices)
    res = (64, 64, 64)
    _, d, tq, _ = oracle_lib.voxelize("segments", st.vertices, t, idx, b, res)
    dn = oracle_lib.normalize(d)
    p = scene.make_params(b, res, 333, 251, raycast_steps=256.0, shadow_steps=32.0)
    dd, dt = to_dev(dn, torch), to_dev(tq, torch)
    imgs = []
    for v in _abi.TUNED_RAYMARCH_VARIANTS:
        ctx.set_raymarch_variant(p.density_format, p.tangent_format, v)
        rgba = torch.full((p.height, p.width, 4), -7.0, dtype=torch.float32, device="cuda")
        ctx.raymarch(p, dd.data_ptr(), dt.data_ptr(), None, rgba.data_ptr(), None)
        torch.cuda.synchronize()
        imgs.append(rgba.cpu().numpy())
    for img in imgs[1:]:
        assert np.array_equal(img, imgs[0])
    assert (imgs[0][..., 3] > 0).sum() > 1000
    rgba = torch.empty((p.height, p.width, 4), dtype=torch.float32, device="cuda")
    chosen, ms = ctx.autotune_raymarch(p, dd.data_ptr(), dt.data_ptr(), rgba.data_ptr())
    tuned = [ms[v] for v in _abi.TUNED_RAYMARCH_VARIANTS]
    assert chosen in _abi.TUNED_RAYMARCH_VARIANTS and min(tuned) > 0 and ms[chosen] == min(tuned)
    assert ms[_abi.RAYMARCH_TEXTURE_VARIANT] == 0.0 and ms[_abi.RAYMARCH_SHADE_TEXTURE_VARIANT] == 0.0  # not candidates
    assert np.array_equal(rgba.cpu().numpy(), imgs[0])
    with pytest.raises(VkhrError):
        ctx.set_raymarch_variant(p.density_format, p.tangent_format, _abi.RAYMARCH_VARIANTS)
    ctx.set_raymarch_variant(p.density_format, p.tangent_format, 0)


@pytest.mark.parametrize("fmt,tfmt,res,view,depth", [
    (_abi.DENSITY_U8_UNORM, _abi.TANGENT_I8_SNORM, (64, 64, 64), (0.0, 0.0, 1.0), False),
    (_abi.DENSITY_U8_UNORM, _abi.TANGENT_F32X4, (48, 32, 40), (0.6, 0.3, 1.0), True),
    (_abi.DENSITY_U32_COUNT, _abi.TANGENT_I8_SNORM, (40, 44, 36), (-0.4, 0.8, 0.5), False),
    (_abi.DENSITY_F32, _abi.TANGENT_F32X4, (36, 28, 52), (0.2, -0.5, -1.0), True),
    (_abi.DENSITY_U8_UNORM, _abi.TANGENT_I8_SNORM, (37, 50, 29), (0.3, 0.2, 1.0), False),  # pitch: no TMA
])
def test_staged_and_gather_variants_equal_l2_march(ctx, oracle_lib, fmt, tfmt, res, view, depth):
    """Variant 4 (each occupied brick a warp's rays need staged into shared
    memory by one TMA copy), variant 7 (texels through the texture unit's
    2x2 gathers from the tiled, zero-framed slices) and variants 8-10 (ray
    groups of 4, 2 and 8 lanes) against variant 0
    (texels from L2): the same pixels bit for bit, with and without a depth
    buffer, for every density format, for grids whose depth is not a power
    of two (a partly filled last row of tiles), for a view whose volume
    straddles the image's edge, and for a grid whose row pitch TMA cannot
    address (variant 4 falls back to variant 0); and against the FP64
    oracle."""
    import torch

    from tests._helpers import compare_images

    st, t, idx = style("hemi", 3000, 14, seed=17)
    b = oracle_lib.bounding_box(st.vertices)
    c, d, tq, _ = oracle_lib.voxelize("segments", st.vertices, t, idx, b, res)
    if fmt == _abi.DENSITY_U8_UNORM:
        dens, iso = oracle_lib.normalize(d), 0.115
    elif fmt == _abi.DENSITY_U32_COUNT:
        dens, iso = c, 1.0
    else:
        dens, iso = c.astype(np.float32) * np.float32(0.25), 0.25
    tan = tq if tfmt == _abi.TANGENT_I8_SNORM else np.maximum(tq.astype(np.float32) / 127.0, -1.0)
    o, sz = np.asarray(b.origin, dtype=np.float64), np.asarray(b.size, dtype=np.float64)
    p = scene.make_params(b, res, 300, 220, raycast_steps=256.0, shadow_steps=32.0, isosurface=iso,
                          view_direction=view, target=o + 0.5 * sz + np.array([0.45, 0.1, 0.0]) * sz,
                          density_format=fmt, tangent_format=tfmt, **scene.CONFIG_SHADING)
    dd, dt = to_dev(dens, torch), to_dev(tan, torch)
    din = None
    depth_np = None
    if depth:
        base = torch.full((p.height, p.width, 4), -7.0, dtype=torch.float32, device="cuda")
        bd = torch.empty((p.height, p.width), dtype=torch.float32, device="cuda")
        ctx.raymarch(p, dd.data_ptr(), dt.data_ptr(), None, base.data_ptr(), bd.data_ptr())
        torch.cuda.synchronize()
        depth_np = np.where(bd.cpu().numpy() < 1.0, bd.cpu().numpy() + 1e-3, 0.5).astype(np.float32)
        depth_np[:, : p.width // 2] = 1.0
        din = torch.from_numpy(depth_np).cuda()
    imgs = []
    for v in (0, 4, _abi.RAYMARCH_GATHER_VARIANT) + _abi.RAYMARCH_GROUP_VARIANTS:
        ctx.set_raymarch_variant(fmt, tfmt, v)
        rgba = torch.full((p.height, p.width, 4), -7.0, dtype=torch.float32, device="cuda")
        dep = torch.full((p.height, p.width), -7.0, dtype=torch.float32, device="cuda")
        ctx.raymarch(p, dd.data_ptr(), dt.data_ptr(), None if din is None else din.data_ptr(), rgba.data_ptr(),
                     dep.data_ptr())
        ctx.check_status(None)
        torch.cuda.synchronize()
        imgs.append((rgba.cpu().numpy(), dep.cpu().numpy()))
    ctx.set_raymarch_variant(fmt, tfmt, 0)
    for k, name in ((1, "staged"), (2, "gather"), (3, "groups of 4"), (4, "groups of 2"), (5, "groups of 8")):
        assert np.array_equal(imgs[0][0], imgs[k][0]), (name, int((imgs[0][0] != imgs[k][0]).any(axis=2).sum()))
        assert np.array_equal(imgs[0][1], imgs[k][1]), name
    assert (imgs[1][0][..., 3] > 0).sum() > 200
    ref, rdepth, diag = oracle_lib.raymarch(p, dens, tan, depth_in=depth_np, diag=True)
    # small views (300x220) whose depth buffer cuts rays mid-volume: up to 2% excluded
    compare_images(imgs[1][0], imgs[1][1], ref, rdepth, diag, label="staged variant", max_excluded=0.02)


@pytest.mark.parametrize("steps,shadow_steps,ao_kernel,ao_dirs,distance", [
    (256.0, 32.0, 2.0, 0, 4.0),   # power-of-two steps: empty-space jumps in both marches
    (200.0, 40.0, 3.0, 0, 4.0),   # no jumps; a 27-tap cube
    (512.0, 48.0, 2.0, 16, 12.0),  # jumps in the primary march only; 16 directions; a distant view
    (384.0, 64.0, 2.6, 5, 4.0),   # a cube of a non-integer size; directions not a multiple of a group
])
def test_ray_group_variants_equal_one_lane_march(ctx, oracle_lib, steps, shadow_steps, ao_kernel, ao_dirs, distance):
    """Ray groups (variants 8-10: 4, 2 or 8 lanes take consecutive samples
    of one ray at once and replay them in order) against the one-lane march
    of variant 0, bit for bit, with and without the empty-space jumps, for
    ambient-occlusion cubes and directions whose tap counts are not
    multiples of the group."""
    import torch

    st, t, idx = style("hemi", 3000, 14, seed=23)
    res = (48, 40, 44)
    b = oracle_lib.bounding_box(st.vertices)
    c, d, tq, _ = oracle_lib.voxelize("segments", st.vertices, t, idx, b, res)
    dens = oracle_lib.normalize(d)
    o, sz = np.asarray(b.origin, dtype=np.float64), np.asarray(b.size, dtype=np.float64)
    p = scene.make_params(b, res, 256, 192, camera_distance=distance, raycast_steps=steps, shadow_steps=shadow_steps,
                          isosurface=0.115, view_direction=(0.3, 0.4, 1.0), target=o + 0.5 * sz,
                          ao_directions=ao_dirs, **scene.CONFIG_SHADING)
    p.ao_kernel_size = ao_kernel
    dd, dt = to_dev(dens, torch), to_dev(tq, torch)
    imgs = []
    for v in (0,) + _abi.RAYMARCH_GROUP_VARIANTS:
        ctx.set_raymarch_variant(p.density_format, p.tangent_format, v)
        rgba = torch.full((p.height, p.width, 4), -7.0, dtype=torch.float32, device="cuda")
        dep = torch.full((p.height, p.width), -7.0, dtype=torch.float32, device="cuda")
        ctx.raymarch(p, dd.data_ptr(), dt.data_ptr(), None, rgba.data_ptr(), dep.data_ptr())
        ctx.check_status(None)
        torch.cuda.synchronize()
        imgs.append((rgba.cpu().numpy(), dep.cpu().numpy()))
    ctx.set_raymarch_variant(p.density_format, p.tangent_format, 0)
    assert (imgs[0][0][..., 3] > 0).sum() > 100
    for k, v in enumerate(_abi.RAYMARCH_GROUP_VARIANTS, start=1):
        assert np.array_equal(imgs[0][0], imgs[k][0]), (v, int((imgs[0][0] != imgs[k][0]).any(axis=2).sum()))
        assert np.array_equal(imgs[0][1], imgs[k][1]), v


@pytest.mark.parametrize("variant", [_abi.RAYMARCH_TEXTURE_VARIANT, _abi.RAYMARCH_SHADE_TEXTURE_VARIANT])
@pytest.mark.parametrize("fmt", [_abi.DENSITY_U8_UNORM, _abi.DENSITY_F32])
def test_texture_unit_variant(ctx, oracle_lib, fmt, variant):
    """Variant 5 samples the density through the texture unit (a 3D array with
    hardware LINEAR filtering and border 0), variant 6 only the shading's
    (deep-shadow and AO) samples.  The filter's weights have 8 fractional
    bits, which moves isosurface hits by a step here and there: variant 5
    does not meet the raymarch bar (measured on a GB300: colour RMS 9e-3,
    max 0.70) and neither is autotuned.  The errors against the FP64 oracle
    and the share of pixels past the bar are printed and bounded loosely
    (coverage within 0.05, colour RMS within 0.02).  Counts fall back to the
    memory path, bit for bit."""
    import torch

    st, t, idx = style("hemi", 4096, 16)
    b = oracle_lib.bounding_box(st.vertices)
    res = (64, 64, 64)
    c, d, tq, _ = oracle_lib.voxelize("segments", st.vertices, t, idx, b, res)
    if fmt == _abi.DENSITY_U8_UNORM:
        dens, iso = oracle_lib.normalize(d), 0.115
    else:
        dens, iso = (oracle_lib.normalize(d).astype(np.float32) / 255.0), 0.115
    p = scene.make_params(b, res, 320, 240, raycast_steps=256.0, shadow_steps=32.0, isosurface=iso,
                          density_format=fmt)
    dd, dt = to_dev(dens, torch), to_dev(tq, torch)
    ctx.set_raymarch_variant(fmt, p.tangent_format, variant)
    rgba = torch.full((p.height, p.width, 4), -7.0, dtype=torch.float32, device="cuda")
    ctx.raymarch(p, dd.data_ptr(), dt.data_ptr(), None, rgba.data_ptr(), None)
    torch.cuda.synchronize()
    ctx.set_raymarch_variant(fmt, p.tangent_format, 0)
    img = rgba.cpu().numpy()
    ref, rdepth, diag = oracle_lib.raymarch(p, dens, tq, diag=True)
    from tests._helpers import image_errors
    rms, mx, excluded, emitted = image_errors(img, ref, diag)
    past = (np.abs(img.astype(np.float64) - ref)[..., :3].max(axis=2) > 2e-2) & (ref[..., 3] > 0)
    print("texture-unit variant %d, density format %d: rms %s max %s, %d of %d fragments past 2e-2 "
          "(memory path bar: rms 1e-3, max 2e-2)"
          % (variant, fmt, np.round(rms, 5).tolist(), np.round(mx, 4).tolist(), int(past.sum()), emitted))
    assert (img != -7.0).all() and emitted > 1000
    assert np.all(rms[:3] <= 0.02) and mx[3] <= 0.05
    # the texture unit's filter is not the exact trilinear: the images differ
    ctx.set_raymarch_variant(fmt, p.tangent_format, 0)
    mem = torch.empty_like(rgba)
    ctx.raymarch(p, dd.data_ptr(), dt.data_ptr(), None, mem.data_ptr(), None)
    torch.cuda.synchronize()
    assert (mem.cpu().numpy() != img).any(), "variant %d rendered the memory path's image" % variant
    # counts cannot be filtered by the texture unit: the variant runs the memory path
    pc = scene.make_params(b, res, 320, 240, raycast_steps=256.0, isosurface=1.0, density_format=_abi.DENSITY_U32_COUNT)
    dc = to_dev(c, torch)
    outs = []
    for v in (0, variant):
        ctx.set_raymarch_variant(_abi.DENSITY_U32_COUNT, pc.tangent_format, v)
        o = torch.empty((pc.height, pc.width, 4), dtype=torch.float32, device="cuda")
        ctx.raymarch(pc, dc.data_ptr(), dt.data_ptr(), None, o.data_ptr(), None)
        torch.cuda.synchronize()
        outs.append(o.cpu().numpy())
    ctx.set_raymarch_variant(_abi.DENSITY_U32_COUNT, pc.tangent_format, 0)
    assert np.array_equal(outs[0], outs[1])


def test_voxelize_walk_residency(oracle_lib):
    """The one-walk kernel's resident-CTA limit changes the timing only: every
    choice gives the oracle's voxels bit for bit, for a one-style call and for
    a batch; vkhr_autotune_voxelize times each and keeps the fastest."""
    import torch

    from vkhr_gb300 import _native
    from tests.test_gpu_batched import _Batch, _styles
    from tests.test_gpu_voxelize import _check

    c = _native.Context(0)
    try:
        st, t, idx = style("disk", 3000, 14, seed=5)
        res = (64, 64, 64)
        b = oracle_lib.bounding_box(st.vertices)
        _check(c, oracle_lib, "segments", st.vertices, t, idx, b, res)  # counted: learns a slice capacity
        for k in (0, 1, 2, 4, 6, 8):
            c.set_voxelize_walk(0, k)
            _check(c, oracle_lib, "segments", st.vertices, t, idx, b, res)
        with pytest.raises(VkhrError):
            c.set_voxelize_walk(0, 9)
        with pytest.raises(VkhrError):
            c.set_voxelize_walk(2, 4)

        batch = _Batch(torch, oracle_lib, _styles(8, 6), True)
        s = torch.cuda.current_stream().cuda_stream
        c.voxelize_batched(True, batch.jobs, s)  # counted: learns the layout
        c.check_status(s)
        for k in (0, 3, 8):
            c.set_voxelize_walk(1, k)
            batch.poison()
            c.voxelize_batched(True, batch.jobs, s)
            c.check_status(s)
            batch.check(oracle_lib)

        for jobs in ([batch.jobs[0]], batch.jobs):
            batch.poison()
            chosen, ms = c.autotune_voxelize(jobs, s)
            torch.cuda.synchronize()
            assert chosen in _abi.WALK_CHOICES and min(ms) > 0
            assert ms[_abi.WALK_CHOICES.index(chosen)] == min(ms)
            print("walk residency %s: %s ms, chose %d" % (list(_abi.WALK_CHOICES), np.round(ms, 4).tolist(), chosen))
        batch.check(oracle_lib)  # the autotuner's runs leave the voxelization in the outputs
    finally:
        c.close()
