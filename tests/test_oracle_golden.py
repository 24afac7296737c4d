"""The oracle against golden fixtures produced by the reference's own code
(tests/golden/make_golden.py: hair_style.cc compiled unmodified, and
volume.frag compiled as C++).  Bit-exact for the voxelizer; the FP64 raymarch
oracle within 1e-4 of the reference shader run in FP32."""
import ctypes as C
import os

import numpy as np
import pytest

from vkhr_gb300 import _abi

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _aabb(a):
    b = _abi.AABB()
    for c in range(3):
        b.origin[c] = float(a[c])
        b.size[c] = float(a[4 + c])
    b.radius = float(a[3])
    b.volume = float(a[7])
    return b


@pytest.mark.parametrize("name", ["voxel_hemisphere", "voxel_ragged", "voxel_crowded"])
def test_voxelizer_matches_reference_fixtures(oracle_lib, name):
    O = oracle_lib
    z = np.load(os.path.join(GOLD, name + ".npz"))
    v, segs = z["vertices"], z["segments"]
    t = O.generate_tangents(v, segs)
    assert np.array_equal(t.view(np.uint32), z["tangents"].view(np.uint32))
    idx = O.generate_indices(segs)
    assert np.array_equal(idx, z["indices"])
    b = O.bounding_box(v)
    got = np.array(list(b.origin) + [b.radius] + list(b.size) + [b.volume], dtype=np.float32)
    assert np.array_equal(got, z["aabb"])  # == treats -0 and +0 alike, as the voxelizer does
    k = 0
    while "res%d" % k in z:
        res = tuple(int(x) for x in z["res%d" % k])
        for mode in ("vertices", "segments"):
            c, d, tq, dropped = O.voxelize(mode, v, t, idx, _aabb(z["aabb"]), res)
            assert dropped == 0
            assert np.array_equal(d, z["%s%d_densities" % (mode, k)])
            assert np.array_equal(tq, z["%s%d_tangents" % (mode, k)])
            assert np.array_equal(O.normalize(d), z["%s%d_normalized" % (mode, k)])
            assert np.array_equal(np.minimum(c, 255).astype(np.uint8), d)
        k += 1


@pytest.mark.parametrize("name", ["raymarch_hemisphere", "raymarch_disk"])
def test_raymarch_oracle_matches_reference_shader(oracle_lib, name):
    O = oracle_lib
    z = np.load(os.path.join(GOLD, name + ".npz"))
    # the fixtures hold the parameter block as raw bytes; fields added to its
    # end since they were written are extension knobs whose zero is the
    # reference's shading
    raw = z["params"].tobytes()
    p = _abi.RaymarchParams.from_buffer_copy(raw + bytes(C.sizeof(_abi.RaymarchParams) - len(raw)))
    rgba, depth, diag = O.raymarch(p, z["densities"], z["tangents"], diag=True)
    ref = z["rgba"]
    assert (ref[..., 3] > 0).sum() > 50
    assert np.abs(rgba - ref).max() <= 1e-4
    assert np.abs(depth - z["depth"]).max() <= 1e-5
    r32, d32 = O.raymarch(p, z["densities"], z["tangents"], precision="f32")
    assert np.abs(r32 - ref).max() <= 1e-4
