"""The `.hair` format and strand reduction restated in oracle/hair.py, pinned
to the reference's own code (HairStyle::load / save / reduce of
src/vkhr/scene_graph/hair_style.cc, compiled unmodified into oracle/_ref) and
to the fixtures tests/golden/make_golden.py made from it; and the library's
header reader (no CUDA call).

HairStyle::reduce copies the strands' segment counts into an offset array
starting at its second element (hair_style.cc:392), one element past the
array's end; with an even strand count that write stays inside the
allocation's slack, so the reference runs here use even counts."""
import os

import numpy as np
import pytest

from oracle import hair as H
from tests._helpers import style

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _ref():
    from oracle import oracle as O

    try:
        O.ref()
    except OSError:
        pytest.skip("the reference's compiled code (oracle/_ref) is not built here")
    return O


@pytest.mark.parametrize("ratio", [1.0, 0.5, 0.984375, 0.25, 0.015625, 0.0])
@pytest.mark.parametrize("seed", [1, 0x9E3779B97F4A7C15, 987654321])
def test_reduce_matches_reference(ratio, seed):
    O = _ref()
    st, t, _ = style("disk", 1000, 9)
    segs = st.segments.astype(np.uint16)
    vr, tr, sr, sdr = O.ref_reduce(st.vertices, t, segs, len(segs), ratio, seed)
    vo, to, so, sdo = H.reduce(st.vertices, t, len(segs), ratio, seed, segs)
    assert sdo == sdr
    assert np.array_equal(so, sr) and np.array_equal(vo, vr) and np.array_equal(to, tr)


def test_reduce_beyond_65536_vertices():
    """Vertex offsets past the u16 range of the segment counts (84K vertices)."""
    O = _ref()
    st, t, _ = style("disk", 6000, 13)
    segs = st.segments.astype(np.uint16)
    r = O.ref_reduce(st.vertices, t, segs, len(segs), 0.6, 99)
    o = H.reduce(st.vertices, t, len(segs), 0.6, 99, segs)
    assert r[3] == o[3] and all(np.array_equal(a, b) for a, b in zip(r[:3], o[:3]))


def test_reduce_ragged_and_default_segment_count():
    O = _ref()
    st, t, _ = style("hemi", 64, 6)
    segs = np.random.default_rng(3).integers(0, 12, size=64).astype(np.uint16)  # ragged, empty strands too
    verts = np.random.default_rng(4).standard_normal((int(segs.sum()) + 64, 3)).astype(np.float32)
    tans = np.random.default_rng(5).standard_normal(verts.shape).astype(np.float32)
    for ratio in (1.0, 0.3):
        r = O.ref_reduce(verts, tans, segs, 64, ratio, 77)
        o = H.reduce(verts, tans, 64, ratio, 77, segs)
        assert r[3] == o[3] and all(np.array_equal(a, b) for a, b in zip(r[:3], o[:3]))
    # no segments array: every strand has the header's default segment count
    r = O.ref_reduce(st.vertices, t, None, 64, 0.5, 11, default_segment_count=5)
    o = H.reduce(st.vertices, t, 64, 0.5, 11, None, 5)
    assert r[3] == o[3] and all(np.array_equal(a, b) for a, b in zip(r[:3], o[:3]))


def test_reduce_golden_fixture():
    g = np.load(os.path.join(GOLDEN, "reduce_hemisphere.npz"))
    for k, ratio in enumerate(g["ratios"]):
        v, t, s, sd = H.reduce(g["vertices"], g["tangents"], len(g["segments"]), float(ratio), int(g["seed"]),
                               g["segments"])
        assert sd == int(g["r%d_seed" % k])
        assert np.array_equal(s, g["r%d_segments" % k]) and np.array_equal(v, g["r%d_vertices" % k])
        assert np.array_equal(t, g["r%d_tangents" % k])


def test_hair_files_match_reference(tmp_path):
    O = _ref()
    st, t, idx = style("hemi", 500, 10)
    segs = st.segments.astype(np.uint16)
    # the reference's saver, read by the oracle
    a = str(tmp_path / "ref.hair")
    assert O.ref_hair_save(a, segs, st.vertices, t) == 0
    o = H.read_hair(a)
    assert o["header"]["fields"] == (1 | 2 | 32)
    assert np.array_equal(o["segments"], segs) and np.array_equal(o["vertices"], st.vertices)
    assert np.array_equal(o["tangents"], t)
    # the oracle's writer (with every optional field), read by the reference's loader
    b = str(tmp_path / "ours.hair")
    thick = np.linspace(0, 1, len(st.vertices), dtype=np.float32)
    col = np.tile(np.float32([0.1, 0.2, 0.3]), (len(st.vertices), 1))
    H.write_hair(b, st.vertices, segs, tangents=t, indices=idx, thickness=thick, transparency=thick, color=col)
    err, r = O.ref_hair_load(b)
    assert err == 0 and r["fields"] == 0x7F
    assert np.array_equal(r["segments"], segs) and np.array_equal(r["vertices"], st.vertices)
    assert np.array_equal(r["tangents"], t) and np.array_equal(r["indices"], idx)


def test_hair_header_reader_of_the_library(tmp_path, native_lib):
    from vkhr_gb300 import _native

    g = os.path.join(GOLDEN, "reduce_hemisphere.hair")  # saved by the reference
    hdr = _native.hair_read_header(g)
    ref = H.read_header(g)
    assert hdr.signature == b"HAIR"
    assert (hdr.strand_count, hdr.vertex_count, hdr.fields) == (ref["strand_count"], ref["vertex_count"],
                                                               ref["fields"])
    bad = tmp_path / "bad.hair"
    bad.write_bytes(b"HAIX" + bytes(124))
    with pytest.raises(_native.VkhrError):
        _native.hair_read_header(str(bad))
    short = tmp_path / "short.hair"
    short.write_bytes(b"HAIR" + bytes(20))
    with pytest.raises(_native.VkhrError):
        _native.hair_read_header(str(short))
    with pytest.raises(_native.VkhrError):
        _native.hair_read_header(str(tmp_path / "missing.hair"))
