"""vkhr_composite (the PPLL-free resolve) and vkhr_resolve_ppll through the C
ABI against the oracle (oracle/resolve.c, pinned to the reference's own
resolve.comp and ppll.glsl by tests/test_oracle_composite.py) and the
reference-made fixture tests/golden/composite_tiers.npz: bit-exact RGBA8."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests._helpers import TIER_COUNTS, background_case, build_ppll, fragment_case, to_dev, volume_case
from vkhr_gb300 import _abi

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _dev_u32(a, torch):
    return to_dev(np.ascontiguousarray(a).view(np.uint32), torch)


def _composite(ctx, f, bg, vr=None, vd=None, check=True):
    import torch

    H, W = bg.shape
    df = _dev_u32(f, torch) if len(f) else None
    dc = _dev_u32(bg, torch)
    dvr = to_dev(vr, torch) if vr is not None else None
    dvd = to_dev(vd, torch) if vd is not None else None
    ctx.composite(None if df is None else df.data_ptr(), len(f), W, H, dc.data_ptr(),
                  None if dvr is None else dvr.data_ptr(), None if dvd is None else dvd.data_ptr(),
                  stream=torch.cuda.current_stream().cuda_stream)
    if check:
        ctx.check_status(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return dc.cpu().numpy().view(np.uint32).reshape(H, W)


def _resolve_ppll(ctx, heads, nodes, bg):
    import torch

    H, W = bg.shape
    dh, dn, dc = _dev_u32(heads, torch), _dev_u32(nodes, torch), _dev_u32(bg, torch)
    ctx.resolve_ppll(dh.data_ptr(), dn.data_ptr(), len(nodes), W, H, dc.data_ptr(),
                     stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return dc.cpu().numpy().view(np.uint32).reshape(H, W)


def test_golden_fixture(ctx):
    g = np.load(os.path.join(GOLDEN, "composite_tiers.npz"))
    got = _composite(ctx, g["fragments"], g["background"], g["volume_rgba"], g["volume_depth"])
    assert np.array_equal(got, g["color"])
    got = _resolve_ppll(ctx, g["heads"], g["nodes"], g["background"])
    assert np.array_equal(got, g["color"])


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_every_slice_tier(ctx, seed):
    """Pixels with 0..3000 fragments (every sort tier, the 1040-node cut),
    depths with ties and special values, with and without a volume."""
    W, H = 11, 2
    f = fragment_case(W, H, TIER_COUNTS, seed, tie_levels=16 if seed == 2 else None)
    bg = background_case(W, H, seed)
    vr, vd = volume_case(W, H, seed, coverage=0.7)
    assert np.array_equal(_composite(ctx, f, bg, vr, vd), O.composite(f, bg, vr, vd))
    assert np.array_equal(_composite(ctx, f, bg), O.composite(f, bg))


@pytest.mark.parametrize("W,H", [(1, 1), (3, 5), (97, 61), (301, 157)])
def test_image_sizes(ctx, W, H):
    """Sizes below one scan block, across blocks (4096 pixels each) and not
    multiples of 4."""
    rng = np.random.default_rng(W * H)
    counts = rng.choice([0, 0, 1, 2, 3, 9, 17, 40], W * H)
    f = fragment_case(W, H, counts, W + H)
    bg = background_case(W, H, 5)
    vr, vd = volume_case(W, H, 6)
    assert np.array_equal(_composite(ctx, f, bg, vr, vd), O.composite(f, bg, vr, vd))


def test_deep_pixels(ctx):
    """A few pixels with 5,000 to 40,000 fragments (radix-selected) among
    shallow ones; repeated calls give the same image."""
    W, H = 64, 32
    rng = np.random.default_rng(7)
    counts = rng.integers(0, 30, W * H)
    counts[[0, 100, 1000, 2047]] = [5000, 12345, 40000, 2600]
    f = fragment_case(W, H, counts, 8, tie_levels=1024)
    bg = background_case(W, H, 9)
    want = O.composite(f, bg)
    a = _composite(ctx, f, bg)
    b = _composite(ctx, f, bg)
    assert np.array_equal(a, want) and np.array_equal(b, want)


def test_volume_only_and_empty(ctx):
    W, H = 40, 30
    bg = background_case(W, H, 10)
    vr, vd = volume_case(W, H, 11)
    empty = np.zeros(0, dtype=_abi.FRAGMENT_DTYPE)
    assert np.array_equal(_composite(ctx, empty, bg, vr, vd), O.composite(empty, bg, vr, vd))
    assert np.array_equal(_composite(ctx, empty, bg), bg)


def test_ppll_resolve_matches_oracle(ctx):
    """The reference's data structure: lists linked in buffer order with the
    nodes stored in a shuffled order."""
    W, H = 53, 29
    rng = np.random.default_rng(12)
    counts = rng.choice([0, 1, 2, 5, 16, 17, 33, 200, 1100], W * H, p=[.3, .2, .1, .1, .1, .1, .05, .04, .01])
    f = fragment_case(W, H, counts, 13, tie_levels=128)
    heads, nodes = build_ppll(f, W, H, seed=14)
    bg = background_case(W, H, 15)
    rc, want = O.resolve_ppll(heads, nodes, bg)
    assert rc == 0
    assert np.array_equal(_resolve_ppll(ctx, heads, nodes, bg), want)
    # and it equals the PPLL-free composite of the same fragments
    assert np.array_equal(_composite(ctx, f, bg), want)


def test_bad_indices_are_reported(ctx):
    from vkhr_gb300 import _native

    import torch

    W, H = 16, 8
    f = fragment_case(W, H, [3] * (W * H), 16)
    bg = background_case(W, H, 17)
    ok = f[f["pixel"] != 5]
    f["pixel"][f["pixel"] == 5] = W * H + 7  # outside the image: skipped and reported
    got = _composite(ctx, f, bg, check=False)
    with pytest.raises(_native.VkhrError):
        ctx.check_status(torch.cuda.current_stream().cuda_stream)
    assert np.array_equal(got, O.composite(ok, bg))
    heads, nodes = build_ppll(fragment_case(W, H, [2] * (W * H), 18), W, H)
    nodes["prev"][nodes["prev"] != _abi.PPLL_NULL] = 1 << 30  # every list ends after its head
    got = _resolve_ppll(ctx, heads, nodes, bg)
    with pytest.raises(_native.VkhrError):
        ctx.check_status(torch.cuda.current_stream().cuda_stream)
    rc, want = O.resolve_ppll(heads, nodes, bg)
    assert rc == -1 and np.array_equal(got, want)


def test_invalid_arguments(ctx):
    from vkhr_gb300 import _native

    import torch

    dc = torch.zeros(16, dtype=torch.int32, device="cuda")
    with pytest.raises(_native.VkhrError):
        ctx.composite(None, 0, 0, 4, dc.data_ptr())
    with pytest.raises(_native.VkhrError):
        ctx.composite(None, 5, 4, 4, dc.data_ptr())
    with pytest.raises(_native.VkhrError):  # rgba without depth
        ctx.composite(None, 0, 4, 4, dc.data_ptr(), d_volume_rgba=dc.data_ptr())
    with pytest.raises(_native.VkhrError):
        ctx.resolve_ppll(None, None, 0, 4, 4, dc.data_ptr())


@pytest.mark.parametrize("distance", [226.0, 600.0])
def test_production_hybrid_frame(ctx, distance):
    """Full size: the production style (136,320 x 13) at 1280x720 under the
    hybrid renderer, strand fragments from workloads.strand_fragments (7.8M
    to 19.7M, hundreds per covered pixel) and, in the LoD band, the
    raymarched volume's fragments; bit-exact against the oracle."""
    import torch

    from vkhr_gb300 import _native, scene, strands, workloads

    st = strands.disk_style(136_320, 13, seed=0)
    t = strands.generate_tangents(st.vertices, st.segments)
    idx = strands.generate_indices(st.segments)
    b = O.bounding_box(st.vertices)
    W, H, res, scale = 1280, 720, (256, 256, 256), 4.0 / 226.0
    p = scene.make_params(b, res, W, H, camera_distance=distance * scale, raycast_steps=256.0,
                          renderer=_abi.RENDERER_HYBRID_LOD)
    p.magnified_distance, p.minified_distance = 400.0 * scale, 800.0 * scale
    lod = _native.level_of_detail(p.magnified_distance, p.minified_distance, p.look_at_distance)
    frags = workloads.strand_fragments(st.vertices, t, idx, p, lod, "cuda")
    f = frags.cpu().numpy().view(_abi.FRAGMENT_DTYPE).reshape(-1)
    vr = vd = None
    if _native.raymarcher_enabled(_abi.RENDERER_HYBRID_LOD, lod):
        s = torch.cuda.current_stream().cuda_stream
        n = 256 ** 3
        dv, dt = to_dev(st.vertices, torch), to_dev(t, torch)
        di = to_dev(idx, torch)
        counts = torch.empty(n, dtype=torch.int32, device="cuda")
        dens = torch.empty(n, dtype=torch.uint8, device="cuda")
        tq = torch.empty((n, 4), dtype=torch.int8, device="cuda")
        ctx.voxelize_segments(dv.data_ptr(), dt.data_ptr(), di.data_ptr(), idx.shape[0], b, res,
                              _abi.INDEX_REF_FP32, counts.data_ptr(), dens.data_ptr(), tq.data_ptr(), s)
        ctx.normalize_densities(dens.data_ptr(), n, s)
        rgba = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        depth = torch.empty((H, W), dtype=torch.float32, device="cuda")
        ctx.raymarch(p, dens.data_ptr(), tq.data_ptr(), None, rgba.data_ptr(), depth.data_ptr(), s)
        torch.cuda.synchronize()
        vr, vd = rgba.cpu().numpy(), depth.cpu().numpy()
        assert (vd < 1).sum() > 1000
    bg = np.full((H, W), 0xFFFFFFFF, dtype=np.uint32)
    assert len(f) > 5_000_000
    got = _composite(ctx, f, bg, vr, vd)
    want = O.composite(f, bg, vr, vd)
    assert np.array_equal(got, want)
    assert (got != bg).sum() > 3000


def test_composite_in_a_cuda_graph(ctx):
    """After one call at the same sizes the composite allocates nothing and
    can be captured; the replayed graph gives the oracle's image."""
    import torch

    W, H = 97, 61
    rng = np.random.default_rng(19)
    f = fragment_case(W, H, rng.choice([0, 1, 4, 17, 60], W * H), 20)
    bg = background_case(W, H, 21)
    vr, vd = volume_case(W, H, 22)
    df, dbg = _dev_u32(f, torch), _dev_u32(bg, torch)
    dc = dbg.clone()
    dvr, dvd = to_dev(vr, torch), to_dev(vd, torch)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx.composite(df.data_ptr(), len(f), W, H, dc.data_ptr(), dvr.data_ptr(), dvd.data_ptr(), stream=s.cuda_stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        ctx.composite(df.data_ptr(), len(f), W, H, dc.data_ptr(), dvr.data_ptr(), dvd.data_ptr(),
                      stream=torch.cuda.current_stream().cuda_stream)
    want = O.composite(f, bg, vr, vd)
    for _ in range(2):
        dc.copy_(dbg)
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(dc.cpu().numpy().view(np.uint32).reshape(H, W), want)


def test_three_radix_passes(ctx):
    """1920x1080 has 2,073,600 pixels: 21-bit keys, three 7-bit radix passes
    (every other case here takes one or two)."""
    W, H = 1920, 1080
    rng = np.random.default_rng(25)
    counts = np.zeros(W * H, dtype=np.int64)
    hit = rng.choice(W * H, 40_000, replace=False)
    counts[hit] = rng.choice([1, 2, 5, 17, 40], len(hit))
    counts[[0, W * H - 1, 1 << 20, (1 << 20) - 1]] = [3, 30, 20, 1100]
    f = fragment_case(W, H, counts, 26, tie_levels=512)
    bg = background_case(W, H, 27)
    vr, vd = volume_case(W, H, 28, coverage=0.05)
    assert np.array_equal(_composite(ctx, f, bg, vr, vd), O.composite(f, bg, vr, vd))
