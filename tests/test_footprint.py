"""vkhr_raymarch_footprint (host-only): the pixel rectangle outside which the
raymarch writes only background.  Checked against the oracle's FP64
raymarch (volume.frag:31-103 semantics) on small views."""
import numpy as np

from vkhr_gb300 import _abi, _native, scene
from tests._helpers import style


def _volume(O, res=(32, 32, 32)):
    st, t, idx = style("hemi", 512, 8)
    b = O.bounding_box(st.vertices)
    c, d, tq, _ = O.voxelize("segments", st.vertices, t, idx, b, res)
    return b, O.normalize(d), tq


def test_outside_is_background(oracle_lib):
    b, dn, tq = _volume(oracle_lib)
    for dist, vd in [(6.0, (0.0, 0.0, 1.0)), (12.0, (1.0, 0.5, 0.3)), (9.0, (-0.2, 1.0, 0.1))]:
        p = scene.make_params(b, (32, 32, 32), 160, 120, camera_distance=dist, view_direction=vd,
                              raycast_steps=64.0)
        x0, y0, w, h = _native.raymarch_footprint(p)
        assert 0 <= x0 and 0 <= y0 and w > 0 and h > 0 and x0 + w <= 160 and y0 + h <= 120
        assert w * h < 160 * 120, "a style seen from a distance covers part of the view"
        rgba, depth = oracle_lib.raymarch(p, dn, tq, precision="f64")
        inside = np.zeros((120, 160), dtype=bool)
        inside[y0:y0 + h, x0:x0 + w] = True
        assert not rgba[~inside].any()
        assert np.all(depth[~inside] == 1.0)
        assert (rgba[inside][:, 3] > 0).any()


def test_degenerate_views(oracle_lib):
    b, dn, tq = _volume(oracle_lib)
    c = np.array(b.origin) + 0.5 * np.array(b.size)
    # camera inside the box: some corner is behind it, the whole view is kept
    p = scene.make_params(b, (32, 32, 32), 64, 48, camera_distance=0.05)
    assert _native.raymarch_footprint(p) == (0, 0, 64, 48)
    # looking away from the box: corners behind the camera, the whole view again
    p = scene.make_params(b, (32, 32, 32), 64, 48, camera_distance=5.0, target=c + np.array([0.0, 0.0, 10.0]),
                          view_direction=(0.0, 0.0, -1.0))
    assert _native.raymarch_footprint(p) == (0, 0, 64, 48)
    rgba, depth = oracle_lib.raymarch(p, dn, tq, precision="f64")
    assert not rgba.any()
    # box in front of the camera but far outside the frustum: nothing
    p = scene.make_params(b, (32, 32, 32), 64, 48, camera_distance=5.0, target=c + np.array([40.0, 0.0, 0.0]))
    x0, y0, w, h = _native.raymarch_footprint(p)
    assert w * h == 0
    rgba, depth = oracle_lib.raymarch(p, dn, tq, precision="f64")
    assert not rgba.any()


def test_invalid_arguments():
    p = _abi.RaymarchParams()
    lib = _native.load()
    r = (__import__("ctypes").c_int32 * 4)()
    assert lib.vkhr_raymarch_footprint(None, r) == _abi.VKHR_ERR_INVALID_ARG
    assert lib.vkhr_raymarch_footprint(__import__("ctypes").byref(p), r) == _abi.VKHR_ERR_INVALID_ARG  # 0 x 0 view
