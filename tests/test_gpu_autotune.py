"""The raymarch autotuner: every ray-packet variant renders the same image
(same per-pixel device code), and vkhr_autotune_raymarch keeps a variant
that later calls use."""
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
    for v in range(_abi.RAYMARCH_VARIANTS):
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
    assert 0 <= chosen < _abi.RAYMARCH_VARIANTS and min(ms) > 0 and ms[chosen] == min(ms)
    assert np.array_equal(rgba.cpu().numpy(), imgs[0])
    with pytest.raises(VkhrError):
        ctx.set_raymarch_variant(p.density_format, p.tangent_format, _abi.RAYMARCH_VARIANTS)
    ctx.set_raymarch_variant(p.density_format, p.tangent_format, 0)
