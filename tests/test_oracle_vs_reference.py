"""The oracle against the reference's own code compiled here (oracle/_ref),
on fresh seeded inputs.  Skipped where the reference sources are absent."""
import numpy as np
import pytest

from vkhr_gb300 import scene, strands

try:
    from oracle import oracle as _O

    HAVE_REF = _O.has_reference()
except Exception:
    HAVE_REF = False

pytestmark = pytest.mark.skipif(not HAVE_REF, reason="oracle/_ref not built (reference sources absent)")


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_voxelizer_bit_exact(oracle_lib, seed):
    O = oracle_lib
    st = strands.hemisphere_style(3000, 14, seed=seed) if seed != 2 else strands.disk_style(5000, 10, seed=seed)
    t, idx, b = O.ref_prepare(st.vertices, st.segments)
    assert np.array_equal(t.view(np.uint32), O.generate_tangents(st.vertices, st.segments).view(np.uint32))
    assert np.array_equal(t.view(np.uint32), strands.generate_tangents(st.vertices, st.segments).view(np.uint32))
    assert np.array_equal(idx, O.generate_indices(st.segments))
    for res in ((48, 48, 48), (33, 17, 61)):
        for mode in ("vertices", "segments"):
            d_ref, t_ref = O.ref_voxelize(mode, st.vertices, t, idx, res)
            c, d, tq, _ = O.voxelize(mode, st.vertices, t, idx, b, res)
            assert np.array_equal(d, d_ref) and np.array_equal(tq, t_ref)


def test_raymarch_against_reference_shader(oracle_lib):
    O = oracle_lib
    st = strands.hemisphere_style(2048, 16, seed=5)
    t, idx, b = O.ref_prepare(st.vertices, st.segments)
    dn, tq = O.ref_voxelize("segments", st.vertices, t, idx, (40, 40, 40), normalize=True)
    p = scene.make_params(b, (40, 40, 40), 120, 90, raycast_steps=160.0)
    ref, rdepth = O.ref_raymarch(p, dn, tq)
    rgba, depth, diag = O.raymarch(p, dn, tq, diag=True)
    assert (ref[..., 3] > 0).sum() > 100
    assert np.abs(rgba - ref).max() <= 1e-4


@pytest.mark.parametrize("filt", [0, 1, 2, 3])
def test_downsample_against_reference(oracle_lib, filt):
    """Volume::downsample (hair_style.hh:228-257) with each filter the ABI offers."""
    O = oracle_lib
    st = strands.hemisphere_style(2500, 12, seed=7)
    t, idx, b = O.ref_prepare(st.vertices, st.segments)
    d_ref, _ = O.ref_voxelize("segments", st.vertices, t, idx, (32, 18, 40))
    assert np.array_equal(O.downsample(d_ref, (32, 18, 40), filt), O.ref_downsample(d_ref, (32, 18, 40), filt))
