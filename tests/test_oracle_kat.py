"""Known-answer tests of the oracle's voxelizer, built by hand from the
reference's semantics (hair_style.cc:215-342)."""
import numpy as np

from vkhr_gb300 import _abi


def _one(v):
    return np.asarray(v, dtype=np.float32).reshape(-1, 3)


def test_aabb_contains_origin(oracle_lib):
    # min/max start at (0,0,0) (hair_style.cc:216-217)
    b = oracle_lib.bounding_box(_one([[1, 2, 3], [2, 5, 4]]))
    assert tuple(b.origin) == (0.0, 0.0, 0.0) and tuple(b.size) == (2.0, 5.0, 4.0)
    assert b.volume == 40.0 and abs(b.radius - np.sqrt(45.0)) < 1e-6


def test_vertex_at_max_clamps_to_last_voxel(oracle_lib):
    v = _one([[2, 2, 2], [0, 0, 0]])
    b = oracle_lib.bounding_box(v)
    c, d, tq, _ = oracle_lib.voxelize("vertices", v, np.zeros_like(v), None, b, (4, 4, 4))
    assert c[0] == 1 and c[63] == 1 and c.sum() == 2


def test_zero_length_segment_visits_nothing(oracle_lib):
    v = _one([[1, 1, 1], [1, 1, 1], [0, 0, 0]])
    b = oracle_lib.bounding_box(v)
    c, d, tq, _ = oracle_lib.voxelize("segments", v, np.zeros_like(v), np.array([0, 1], np.uint32), b, (4, 4, 4))
    assert c.sum() == 0


def test_fractional_steps_visit_ceil(oracle_lib):
    # root 0.5, tip 2.8 along x in voxel units: steps = 2.3 -> 3 visits at x = 0, 1, 2
    b = _abi.aabb_from((0, 0, 0), (8, 8, 8))
    v = _one([[0.5, 0.5, 0.5], [2.8, 0.5, 0.5]])
    idx = np.array([0, 1], np.uint32)
    assert oracle_lib.segment_visits(v, idx, b, (8, 8, 8))[0] == 3
    c, d, tq, _ = oracle_lib.voxelize("segments", v, np.zeros_like(v), idx, b, (8, 8, 8))
    assert list(np.nonzero(c)[0]) == [0, 1, 2]


def test_saturation_stops_tangent_sum_at_255(oracle_lib):
    # 300 vertices in one voxel: count 300, u8 density 255, tangent = mean of the first 255
    v = np.full((300, 3), 0.25, np.float32)
    t = np.zeros_like(v)
    t[:255, 0] = 1.0          # the first 255 point along +x
    t[255:, 1] = 1.0          # later ones along +y must not count
    b = _abi.aabb_from((0, 0, 0), (1, 1, 1))
    c, d, tq, _ = oracle_lib.voxelize("vertices", v, t, None, b, (2, 2, 2))
    assert c[0] == 300 and d[0] == 255
    assert tuple(tq[0]) == (127, 0, 0, 0)


def test_ref_fp32_index_rounding_above_2_24(oracle_lib):
    # voxel (511, 511, 511) of 512^3: the FP32 index rounds to 2^27 (out of range)
    b = _abi.aabb_from((0, 0, 0), (1, 1, 1))
    v = _one([[0.9999, 0.9999, 0.9999]])
    res = (512, 512, 512)
    c_ref, _, _, dropped_ref = oracle_lib.voxelize("vertices", v, np.zeros_like(v), None, b, res,
                                                   _abi.INDEX_REF_FP32)
    c_ex, _, _, dropped_ex = oracle_lib.voxelize("vertices", v, np.zeros_like(v), None, b, res, _abi.INDEX_EXACT)
    assert dropped_ref == 1 and c_ref.sum() == 0
    assert dropped_ex == 0 and c_ex[512 ** 3 - 1] == 1
    # voxel (1, 1, 64): exact index 16,777,729 is odd; FP32 rounds it to 16,777,728
    v = _one([[1.5 / 512, 1.5 / 512, 64.5 / 512]])
    c_ref, _, _, _ = oracle_lib.voxelize("vertices", v, np.zeros_like(v), None, b, res, _abi.INDEX_REF_FP32)
    assert np.nonzero(c_ref)[0].tolist() == [16_777_728]


def test_tangent_quantisation_truncates(oracle_lib):
    t = np.array([[0.6, -0.8, 0.0]], np.float32)
    v = np.full((1, 3), 0.1, np.float32)
    b = _abi.aabb_from((0, 0, 0), (1, 1, 1))
    _, _, tq, _ = oracle_lib.voxelize("vertices", v, t, None, b, (2, 2, 2))
    assert tuple(tq[0]) == (int(0.6 * 127.0), int(-0.8 * 127.0), 0, 0) == (76, -101, 0, 0)


def test_normalize(oracle_lib):
    d = np.array([0, 10, 20, 40], np.uint8)
    assert list(oracle_lib.normalize(d)) == [0, 63, 127, 255]
    assert list(oracle_lib.normalize(np.array([7, 7], np.uint8))) == [0, 0]
