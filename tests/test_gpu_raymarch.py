"""GPU raymarch parity: vkhr_raymarch (C ABI) against the FP64 oracle
transcription of volume.frag.

Tolerance (per channel, over well-conditioned pixels): RMS <= 1e-3 and
max |diff| <= 2e-2.  A pixel is excluded only when its result hinges on a
decision FP32 cannot resolve (tests/_helpers.py ill_conditioned): the
isosurface test within 1e-4 (relative) of the threshold, a `density != 0`
test within 2e-4 texel of flipping, or a surface tangent shorter than 1e-4.
Excluded pixels are counted and must stay below 1% of the emitted fragments.
"""
import numpy as np
import pytest

from vkhr_gb300 import _abi, scene
from tests._helpers import compare_images, style, to_dev

pytestmark = pytest.mark.gpu


def _volume(O, kind, n, verts, res, mode="segments", **kw):
    st, t, idx = style(kind, n, verts, **kw)
    b = O.bounding_box(st.vertices)
    c, d, tq, _ = O.voxelize(mode, st.vertices, t, idx, b, res)
    return b, c, O.normalize(d), tq


def _gpu_raymarch(ctx, p, dens, tan, depth_in=None):
    import torch

    dd = to_dev(dens, torch)
    dt = to_dev(tan, torch)
    di = None if depth_in is None else to_dev(depth_in.astype(np.float32), torch)
    rgba = torch.full((p.height, p.width, 4), -7.0, dtype=torch.float32, device="cuda")
    depth = torch.full((p.height, p.width), -7.0, dtype=torch.float32, device="cuda")
    ctx.raymarch(p, dd.data_ptr(), dt.data_ptr(), None if di is None else di.data_ptr(), rgba.data_ptr(),
                 depth.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rgba.cpu().numpy(), depth.cpu().numpy()


def _compare(gpu, gdepth, ref, rdepth, diag, rows=None, label=""):
    if rows is not None:
        gpu, gdepth = gpu[rows[0]:rows[1]], gdepth[rows[0]:rows[1]]
        ref, rdepth, diag = ref[rows[0]:rows[1]], rdepth[rows[0]:rows[1]], diag[rows[0]:rows[1]]
    rms, mx, _, _ = compare_images(gpu, gdepth, ref, rdepth, diag, label=label)
    return rms, mx


def test_small_reference_semantics(ctx, oracle_lib):
    """4,096 x 16 hemisphere style, 64^3, 640x480, 256 steps (shadows reuse them)."""
    b, c, dn, tq = _volume(oracle_lib, "hemi", 4096, 16, (64, 64, 64))
    p = scene.make_params(b, (64, 64, 64), 640, 480, raycast_steps=256.0)
    ref, rdepth, diag = oracle_lib.raymarch(p, dn, tq, diag=True)
    gpu, gdepth = _gpu_raymarch(ctx, p, dn, tq)
    _compare(gpu, gdepth, ref, rdepth, diag)


def test_extension_knobs(ctx, oracle_lib):
    """kd 0.4, 32-step shadows, a hybrid-renderer LoD blend and non-power-of-two steps."""
    b, c, dn, tq = _volume(oracle_lib, "hemi", 4096, 16, (64, 64, 64))
    p = scene.make_params(b, (64, 64, 64), 320, 240, raycast_steps=201.0, shadow_steps=32.0, kd=0.4,
                          renderer=_abi.RENDERER_HYBRID_LOD, hair_alpha=0.8)
    p.magnified_distance, p.minified_distance = 2.0, 6.0
    ref, rdepth, diag = oracle_lib.raymarch(p, dn, tq, diag=True)
    gpu, gdepth = _gpu_raymarch(ctx, p, dn, tq)
    _compare(gpu, gdepth, ref, rdepth, diag)


@pytest.mark.parametrize("model", [_abi.SHADING_ADSM, _abi.SHADING_LAO, 1])
def test_shading_models(ctx, oracle_lib, model):
    b, c, dn, tq = _volume(oracle_lib, "hemi", 2048, 16, (48, 48, 48))
    p = scene.make_params(b, (48, 48, 48), 200, 150, raycast_steps=128.0, shading_model=model)
    ref, rdepth, diag = oracle_lib.raymarch(p, dn, tq, diag=True)
    gpu, gdepth = _gpu_raymarch(ctx, p, dn, tq)
    _compare(gpu, gdepth, ref, rdepth, diag)


def test_raw_counts_iso_one(ctx, oracle_lib):
    """uint32 count texels with an isosurface of 1 count/voxel."""
    b, c, dn, tq = _volume(oracle_lib, "hemi", 4096, 16, (64, 64, 64))
    p = scene.make_params(b, (64, 64, 64), 320, 240, raycast_steps=256.0, isosurface=1.0, shadow_steps=32.0,
                          density_format=_abi.DENSITY_U32_COUNT)
    ref, rdepth, diag = oracle_lib.raymarch(p, c, tq, diag=True)
    gpu, gdepth = _gpu_raymarch(ctx, p, c, tq)
    _compare(gpu, gdepth, ref, rdepth, diag)


def test_float_texels(ctx, oracle_lib):
    rng = np.random.default_rng(4)
    b, c, dn, tq = _volume(oracle_lib, "hemi", 2048, 16, (40, 40, 40))
    dens = (dn.astype(np.float32) / 255.0) * rng.lognormal(0.0, 0.2, dn.shape).astype(np.float32)
    tan = np.concatenate([tq[:, :3].astype(np.float32) / 127.0, np.zeros((tq.shape[0], 1), np.float32)], axis=1)
    p = scene.make_params(b, (40, 40, 40), 160, 120, raycast_steps=128.0, density_format=_abi.DENSITY_F32,
                          tangent_format=_abi.TANGENT_F32X4)
    ref, rdepth, diag = oracle_lib.raymarch(p, dens, tan, diag=True)
    gpu, gdepth = _gpu_raymarch(ctx, p, dens, tan)
    _compare(gpu, gdepth, ref, rdepth, diag)


def test_depth_buffer_breaks_rays(ctx, oracle_lib):
    b, c, dn, tq = _volume(oracle_lib, "hemi", 2048, 16, (48, 48, 48))
    p = scene.make_params(b, (48, 48, 48), 160, 120, raycast_steps=128.0)
    _, rdepth0 = oracle_lib.raymarch(p, dn, tq)
    depth_in = np.ones((120, 160), np.float32)
    depth_in[:, :80] = np.where(rdepth0[:, :80] < 1.0, rdepth0[:, :80] + 2e-3, 0.5)  # occluder mid-volume
    ref, rdepth, diag = oracle_lib.raymarch(p, dn, tq, depth_in=depth_in, diag=True)
    gpu, gdepth = _gpu_raymarch(ctx, p, dn, tq, depth_in)
    _compare(gpu, gdepth, ref, rdepth, diag)


@pytest.mark.parametrize("shift", [(0.0, 0.0, 0.0), (0.9, 0.4, 0.0)])
def test_footprint_launch_every_pixel(ctx, oracle_lib, shift):
    """The march kernel covers only the volume's screen footprint and a
    background kernel writes the other pixels: every pixel is written, those
    outside the footprint are background (RGBA 0, depth 1), and the whole
    image matches the oracle, which marches every pixel -- also for a view
    whose volume straddles the image's edge (shifted look-at point)."""
    from vkhr_gb300 import _native

    res = (48, 48, 48)
    b, c, dn, tq = _volume(oracle_lib, "hemi", 3000, 12, res)
    o, sz = np.asarray(b.origin, dtype=np.float64), np.asarray(b.size, dtype=np.float64)
    target = o + 0.5 * sz + np.asarray(shift) * sz
    p = scene.make_params(b, res, 160, 120, raycast_steps=128.0, shadow_steps=32.0, view_direction=(0.3, 0.2, 1.0),
                          target=target)
    x0, y0, w, h = _native.raymarch_footprint(p)
    assert 0 < w * h < 160 * 120  # a proper part of the view
    gpu, gdepth = _gpu_raymarch(ctx, p, dn, tq)
    assert (gpu != -7.0).all() and (gdepth != -7.0).all()
    outside = np.ones((120, 160), dtype=bool)
    outside[y0:y0 + h, x0:x0 + w] = False
    assert not gpu[outside].any() and np.all(gdepth[outside] == 1.0)
    ref, rdepth, diag = oracle_lib.raymarch(p, dn, tq, diag=True)
    assert not ref[outside].any()
    _compare(gpu, gdepth, ref, rdepth, diag)


def test_camera_inside_volume_covers_nothing(ctx, oracle_lib):
    b, c, dn, tq = _volume(oracle_lib, "hemi", 1024, 8, (32, 32, 32))
    p = scene.make_params(b, (32, 32, 32), 64, 48, camera_distance=0.1, raycast_steps=64.0)
    gpu, gdepth = _gpu_raymarch(ctx, p, dn, tq)
    assert not gpu.any() and np.all(gdepth == 1.0)


def test_production_view_full_lit_span(ctx, oracle_lib):
    """136,320 x 13 style, 256^3, 1920x1080, 512 steps, 64-step shadows:
    the full frame on the GPU against the FP64 oracle over every row the
    volume's screen footprint spans (every ray that enters the box)."""
    from vkhr_gb300 import _native

    b, c, dn, tq = _volume(oracle_lib, "disk", 136_320, 13, (256, 256, 256))
    p = scene.make_params(b, (256, 256, 256), 1920, 1080, raycast_steps=512.0, shadow_steps=64.0)
    gpu, gdepth = _gpu_raymarch(ctx, p, dn, tq)
    x0, y0, w, h = _native.raymarch_footprint(p)
    lit = np.nonzero((gpu[..., 3] > 0).any(axis=1))[0]
    assert lit.size > 100 and lit.min() >= y0 and lit.max() < y0 + h
    ref, rdepth, diag = oracle_lib.raymarch(p, dn, tq, diag=True, rows=(y0, y0 + h))
    # outside the footprint rows both images are background
    assert not gpu[:y0].any() and not gpu[y0 + h:].any()
    _compare(gpu, gdepth, ref, rdepth, diag, rows=(y0, y0 + h), label="production frame rows %d..%d" % (y0, y0 + h))


def test_config0_small_as_written(ctx, oracle_lib):
    """The small workload with its own shading: 4,096 x 16 hemisphere strands
    vertex-count voxelized into uint32 64^3, 640x480 from distance 4 (fov 45),
    256 steps, isosurface 1 count per voxel, Kajiya-Kay with kd 0.4,
    exponents 80 / 8 and shifts +-0.1, 32-step shadows."""
    b, c, dn, tq = _volume(oracle_lib, "hemi", 4096, 16, (64, 64, 64), mode="vertices")
    p = scene.make_params(b, (64, 64, 64), 640, 480, camera_distance=4.0, raycast_steps=256.0, shadow_steps=32.0,
                          isosurface=1.0, density_format=_abi.DENSITY_U32_COUNT, **scene.CONFIG_SHADING)
    ref, rdepth, diag = oracle_lib.raymarch(p, c, tq, diag=True)
    gpu, gdepth = _gpu_raymarch(ctx, p, c, tq)
    _compare(gpu, gdepth, ref, rdepth, diag, label="config 0")


@pytest.mark.parametrize("mode,fmt", [("segments", _abi.DENSITY_U8_UNORM), ("vertices", _abi.DENSITY_U32_COUNT)])
def test_config1_production_as_written(ctx, oracle_lib, mode, fmt):
    """The production style (136,320 x 13) voxelized into 256^3 by segments
    (normalized u8 texels, the reference's, isosurface 0.115) or by vertex
    counts (uint32 texels, isosurface 1 count), raymarched at 1920x1080 with
    512 steps, 64-step shadows, 8-direction AO and the workloads' dual-lobe
    Kajiya-Kay, against the FP64 oracle over every row of the footprint."""
    from vkhr_gb300 import _native

    b, c, dn, tq = _volume(oracle_lib, "disk", 136_320, 13, (256, 256, 256), mode=mode)
    u8 = fmt == _abi.DENSITY_U8_UNORM
    p = scene.make_params(b, (256, 256, 256), 1920, 1080, raycast_steps=512.0, shadow_steps=64.0,
                          isosurface=0.115 if u8 else 1.0, density_format=fmt, **scene.CONFIG_SHADING)
    dens = dn if u8 else c
    gpu, gdepth = _gpu_raymarch(ctx, p, dens, tq)
    x0, y0, w, h = _native.raymarch_footprint(p)
    ref, rdepth, diag = oracle_lib.raymarch(p, dens, tq, diag=True, rows=(y0, y0 + h))
    assert not gpu[:y0].any() and not gpu[y0 + h:].any()
    _compare(gpu, gdepth, ref, rdepth, diag, rows=(y0, y0 + h), label="config 1 %s" % mode)


@pytest.mark.parametrize("directions", [1, 7, 8, 16, 32])
def test_directional_ao(ctx, oracle_lib, directions):
    """The directional ambient occlusion (Fibonacci-sphere taps at the reach
    of the reference's 8-tap cube), alone and under Kajiya-Kay."""
    b, c, dn, tq = _volume(oracle_lib, "hemi", 2048, 16, (48, 48, 48))
    for model in (_abi.SHADING_LAO, _abi.SHADING_KAJIYA_KAY):
        p = scene.make_params(b, (48, 48, 48), 200, 150, raycast_steps=128.0, shading_model=model,
                              ao_directions=directions)
        ref, rdepth, diag = oracle_lib.raymarch(p, dn, tq, diag=True)
        gpu, gdepth = _gpu_raymarch(ctx, p, dn, tq)
        _compare(gpu, gdepth, ref, rdepth, diag, label="%d AO directions, model %d" % (directions, model))


def test_errors(ctx, oracle_lib):
    from vkhr_gb300._native import VkhrError

    b, c, dn, tq = _volume(oracle_lib, "hemi", 256, 8, (16, 16, 16))
    for field, value in (("raycast_steps", 0.0), ("raycast_steps", -3.0), ("raycast_steps", 1e9),
                         ("width", 0), ("isosurface", 0.0), ("ao_directions", 33), ("ao_directions", -1),
                         ("spec_exponent2", float("nan")), ("spec_exponent2", float("inf"))):
        p = scene.make_params(b, (16, 16, 16), 32, 24, raycast_steps=64.0)
        setattr(p, field, value)
        with pytest.raises(VkhrError) as e:
            _gpu_raymarch(ctx, p, dn, tq)
        assert e.value.status == _abi.VKHR_ERR_INVALID_ARG


@pytest.mark.parametrize("seed", range(12))
def test_seeded_random_views(ctx, oracle_lib, seed):
    """Seeded random views against the FP64 oracle at the raymarch bar:
    hemisphere or disk styles in non-cubic grids, any view direction and
    distance, power-of-two and other step counts, separate shadow steps or
    none, every shading model with or without shadows, both lobes and
    shifts, cube or directional occlusion, u8 / count / float densities, an
    isosurface drawn per case, and each of the variants the autotuner picks
    from (all give the same pixels)."""
    import torch

    rng = np.random.default_rng(2000 + seed)
    kind = ("hemi", "disk")[int(rng.integers(0, 2))]
    res = tuple(int(x) for x in rng.integers(24, 65, 3))
    b, c, dn, tq = _volume(oracle_lib, kind, int(rng.integers(500, 4001)), int(rng.integers(8, 17)), res, seed=seed)
    fmt = (_abi.DENSITY_U8_UNORM, _abi.DENSITY_U32_COUNT, _abi.DENSITY_F32)[int(rng.integers(0, 3))]
    if fmt == _abi.DENSITY_U8_UNORM:
        dens, iso = dn, float(rng.uniform(0.05, 0.3))
    elif fmt == _abi.DENSITY_U32_COUNT:
        dens, iso = c, float(rng.integers(1, 4))
    else:
        dens, iso = c.astype(np.float32) * np.float32(0.25), float(rng.uniform(0.2, 0.8))
    vd = rng.normal(size=3)
    model = (_abi.SHADING_KAJIYA_KAY, _abi.SHADING_ADSM, _abi.SHADING_LAO)[int(rng.integers(0, 3))]
    p = scene.make_params(b, res, int(rng.integers(96, 201)), int(rng.integers(72, 161)),
                          camera_distance=float(rng.uniform(2.5, 8.0)), view_direction=tuple(vd),
                          raycast_steps=float(rng.choice([64.0, 128.0, 200.0, 256.0, 300.0, 512.0])),
                          shadow_steps=float(rng.choice([0.0, 16.0, 32.0, 48.0])), isosurface=iso,
                          shading_model=model, deep_shadows_on=int(rng.integers(0, 2)),
                          kd=float(rng.uniform(0.3, 1.0)), spec_exponent2=float(rng.choice([0.0, 8.0])),
                          spec_shift=(float(rng.uniform(-0.15, 0.15)), float(rng.uniform(-0.15, 0.15))),
                          ao_directions=int(rng.choice([0, 0, 5, 16])), density_format=fmt)
    p.ao_kernel_size = float(rng.choice([2.0, 3.0]))
    variant = int(rng.choice(_abi.TUNED_RAYMARCH_VARIANTS))
    ctx.set_raymarch_variant(fmt, p.tangent_format, variant)
    try:
        gpu, gdepth = _gpu_raymarch(ctx, p, dens, tq)
    finally:
        ctx.set_raymarch_variant(fmt, p.tangent_format, 0)
    ref, rdepth, diag = oracle_lib.raymarch(p, dens, tq, diag=True)
    label = "seed %d: %s %s, format %d, model %d, steps %g, variant %d" % (seed, kind, res, fmt, model,
                                                                         p.raycast_steps, variant)
    if (ref[..., 3] > 0).sum() == 0:  # the view missed the volume: background everywhere
        assert np.array_equal(gpu, ref) and np.array_equal(gdepth, rdepth), label
        return
    compare_images(gpu, gdepth, ref, rdepth, diag, label=label, max_excluded=0.03)
