"""The compositing oracle (oracle/resolve.c) pinned to the reference's own PPLL
code: share/shaders/transparency/resolve.comp and ppll.glsl compiled as C++
into oracle/_ref (oracle/ref_resolve.cc), and the fixtures that
tests/golden/make_golden.py made from it.  Also the library's host-side
level-of-detail helpers (no CUDA call)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests._helpers import (SPECIAL_DEPTHS, TIER_COUNTS, background_case, build_ppll, fragment_case,
                            volume_case)
from vkhr_gb300 import _abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _ref():
    try:
        O.ref()
    except OSError:
        pytest.skip("the reference's compiled code (oracle/_ref) is not built here")
    return O


def test_pack_unorm8x4_rounds_to_nearest_even():
    x = np.float32([0.5 / 255, 1.5 / 255, 254.5 / 255, 0.0])
    for v in list(np.linspace(-0.5, 1.5, 101, dtype=np.float32)) + list(x):
        want = int(np.rint(np.float32(np.clip(v, 0, 1)) * np.float32(255.0)))
        got = O.pack_unorm8x4(np.float32([v, 0, 1, np.nan]))
        assert got == want | (255 << 16)
    # c / 255 packs back to c for every code
    for c in range(256):
        assert O.pack_unorm8x4(np.float32([c / np.float32(255.0)] * 4)) == c * 0x01010101


@pytest.mark.parametrize("seed", [1, 2])
def test_resolve_ppll_matches_reference(seed):
    R = _ref()
    W, H = 11, 2
    counts = np.array(TIER_COUNTS, dtype=np.int64)
    f = fragment_case(W, H, counts, seed, tie_levels=64 if seed == 2 else None)
    bg = background_case(W, H, seed)
    heads, nodes, used = R.ref_build_ppll(f, W, H)
    assert used == len(f)
    want = R.ref_resolve_ppll(heads, nodes, bg)
    rc, got = O.resolve_ppll(heads, nodes, bg)
    assert rc == 0 and np.array_equal(got, want)
    # the numpy PPLL builder of the GPU tests links the same lists
    h2, n2 = build_ppll(f, W, H, seed=seed)
    rc, got2 = O.resolve_ppll(h2, n2, bg)
    assert rc == 0 and np.array_equal(got2, want)


@pytest.mark.parametrize("seed", [3, 4, 5])
def test_composite_matches_reference_ppll(seed):
    """The PPLL-free composite equals the reference's resolve of the PPLL its
    own appends build from the strand fragments (in buffer order) and then
    the volume fragments."""
    R = _ref()
    W, H = 23, 17
    rng = np.random.default_rng(seed)
    counts = rng.choice([0, 0, 1, 2, 3, 7, 12, 16, 17, 20, 40], W * H)
    counts[5], counts[77], counts[200] = 1500, 2600, 1041
    f = fragment_case(W, H, counts, seed, tie_levels=32 if seed == 4 else None)
    bg = background_case(W, H, seed)
    vr, vd = volume_case(W, H, seed)
    heads, nodes, _ = R.ref_build_ppll(f, W, H, vr, vd)
    want = R.ref_resolve_ppll(heads, nodes, bg)
    got = O.composite(f, bg, vr, vd)
    assert np.array_equal(got, want)
    # without a volume
    heads, nodes, _ = R.ref_build_ppll(f, W, H)
    assert np.array_equal(O.composite(f, bg), R.ref_resolve_ppll(heads, nodes, bg))


def test_k_buffer_special_depths():
    """Lists of up to 20 nodes drawn from the depths the k-buffer treats
    specially (0, negative, NaN, +inf, the empty slots' 3e38, above it)."""
    R = _ref()
    rng = np.random.default_rng(6)
    W, H = 40, 20
    counts = rng.integers(0, 21, W * H)
    f = fragment_case(W, H, counts, 7, special_rate=0)
    f["depth"] = rng.choice(SPECIAL_DEPTHS, len(f))
    bg = background_case(W, H, 8)
    heads, nodes, _ = R.ref_build_ppll(f, W, H)
    want = R.ref_resolve_ppll(heads, nodes, bg)
    assert np.array_equal(O.composite(f, bg), want)
    assert np.array_equal(O.resolve_ppll(heads, nodes, bg)[1], want)


def test_empty_inputs_leave_the_image():
    bg = background_case(7, 5, 9)
    assert np.array_equal(O.composite(np.zeros(0, dtype=_abi.FRAGMENT_DTYPE), bg), bg)
    heads = np.full((5, 7), _abi.PPLL_NULL, dtype=np.uint32)
    rc, out = O.resolve_ppll(heads, np.zeros(1, dtype=_abi.PPLL_NODE_DTYPE), bg)
    assert rc == 0 and np.array_equal(out, bg)


def test_bad_indices_are_reported():
    bg = background_case(4, 4, 10)
    f = fragment_case(4, 4, [1] * 16, 11)
    f["pixel"][3] = 16
    with pytest.raises(ValueError):
        O.composite(f, bg)
    heads, nodes = build_ppll(fragment_case(4, 4, [2] * 16, 12), 4, 4)
    nodes["prev"][nodes["prev"] != _abi.PPLL_NULL] = 10_000
    rc, _ = O.resolve_ppll(heads, nodes, bg)
    assert rc == -1


def test_reference_node_pool_keeps_one_node_past_its_size():
    """ppll_next_node hands out indices up to ppll_size inclusive
    (ppll.glsl:24-26), so a pool of C nodes links C + 1 fragments; the
    PPLL-free composite has no pool and drops none."""
    R = _ref()
    W, H = 8, 8
    f = fragment_case(W, H, [3] * 64, 13, special_rate=0)
    heads, nodes, used = R.ref_build_ppll(f, W, H, capacity=100)
    assert used == len(f)
    linked = 0
    for h in heads.ravel():
        while h != _abi.PPLL_NULL:
            linked += 1
            h = nodes["prev"][h]
    assert linked == 101


def test_golden_composite_fixture():
    g = np.load(os.path.join(GOLDEN, "composite_tiers.npz"))
    got = O.composite(g["fragments"], g["background"], g["volume_rgba"], g["volume_depth"])
    assert np.array_equal(got, g["color"])
    rc, got = O.resolve_ppll(g["heads"], g["nodes"], g["background"])
    assert rc == 0 and np.array_equal(got, g["color"])


def test_level_of_detail_helpers(native_lib):
    from vkhr_gb300 import _native as N

    f32 = np.float32
    for mag, mn, d in [(400, 800, 0), (400, 800, 400), (400, 800, 500), (400, 800, 799.5), (400, 800, 1e4),
                       (1, 3, 2.2)]:
        t = np.clip((f32(d) - f32(mag)) / (f32(mn) - f32(mag)), f32(0), f32(1))
        want = t * t * (f32(3) - f32(2) * t)
        assert N.level_of_detail(mag, mn, d) == want
        assert N.lod(_abi.RENDERER_HYBRID_LOD, mag, mn, d) == want
        assert N.lod(_abi.RENDERER_RAY_TRACER, mag, mn, d) == want
        assert N.lod(_abi.RENDERER_RASTERIZER, mag, mn, d) == 0.0
        assert N.lod(_abi.RENDERER_RAYMARCHER, mag, mn, d) == 1.0
    # interface.cc:534-540
    for r in range(4):
        for lv in (0.0, 0.5, 1.0):
            assert N.rasterizer_enabled(r, lv) == (r == 0 or (r == 3 and lv != 1.0))
            assert N.raymarcher_enabled(r, lv) == (r == 2 or (r == 3 and lv != 0.0))


def test_rasterized_strands_match_reference():
    """Fragments as a strand rasterizer emits them: the synthetic one-pixel
    lines of workloads.strand_fragments (primitive order, tens of fragments
    on a pixel), composited over a raymarch-like volume image; the oracle's
    PPLL-free composite equals the reference's own appends and resolve."""
    R = _ref()
    from vkhr_gb300 import scene, workloads
    from tests._helpers import style

    st, t, idx = style("hemi", 1500, 10, seed=23)
    b = O.bounding_box(st.vertices)
    W, H = 96, 64
    p = scene.make_params(b, (32, 32, 32), W, H, camera_distance=6.0, renderer=_abi.RENDERER_HYBRID_LOD)
    f = workloads.strand_fragments(st.vertices, t, idx, p, 0.25, "cpu").numpy().view(_abi.FRAGMENT_DTYPE).reshape(-1)
    assert len(f) > 2000
    assert f["pixel"].max() < W * H and np.all((f["depth"] >= 0) & (f["depth"] <= 1))
    # alpha = hair_alpha * (1 - lod) = 0.375, packed
    assert np.all(f["color"] >> 24 == round(0.5 * 0.75 * 255))
    counts = np.bincount(f["pixel"], minlength=W * H)
    assert counts.max() > 16  # some pixels reach the k-buffer's tail
    vr, vd = volume_case(W, H, 24, coverage=0.3)
    bg = np.full((H, W), 0xFFFFFFFF, dtype=np.uint32)
    heads, nodes, _ = R.ref_build_ppll(f, W, H, vr, vd)
    want = R.ref_resolve_ppll(heads, nodes, bg)
    assert np.array_equal(O.composite(f, bg, vr, vd), want)
    assert (want != bg).sum() > 500


def test_random_lists_match_reference():
    """Property: for random images (1..6 x 1..6 pixels), list lengths 0..40,
    depths mixing ties, specials and uniform values, colours and volume
    images, the oracle's composite and PPLL resolve equal the reference's."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    R = _ref()

    @hyp.settings(max_examples=150, deadline=None)
    @hyp.given(w=st.integers(1, 6), h=st.integers(1, 6), seed=st.integers(0, 2**31 - 1),
               ties=st.sampled_from([None, 4, 64]), special=st.sampled_from([0.0, 0.1, 0.5]),
               volume=st.booleans(), deep=st.integers(0, 40))
    def check(w, h, seed, ties, special, volume, deep):
        rng = np.random.default_rng(seed)
        counts = rng.integers(0, deep + 1, w * h)
        f = fragment_case(w, h, counts, seed, tie_levels=ties, special_rate=special)
        bg = background_case(w, h, seed + 1)
        vr, vd = volume_case(w, h, seed + 2) if volume else (None, None)
        heads, nodes, _ = R.ref_build_ppll(f, w, h, vr, vd)
        want = R.ref_resolve_ppll(heads, nodes, bg)
        assert np.array_equal(O.composite(f, bg, vr, vd), want)
        rc, got = O.resolve_ppll(heads, nodes, bg)
        assert rc == 0 and np.array_equal(got, want)

    check()
