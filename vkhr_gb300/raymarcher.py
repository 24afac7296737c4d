"""vkhr::Raymarcher: the headless volume renderer of the level-of-detail path.

The reference has no class of this name (Raymarcher is a Renderer::Type,
include/vkhr/renderer.hh:14); its raymarch is vulkan::Volume::draw
(src/vkhr/rasterizer/volume.cc:104-112) running volume.frag.  This class is
that draw call without a graphics API: `draw(volume, params)` renders into
device buffers (RGBA float4 + depth) through vkhr_raymarch in libvkhr_cuda.so.
"""
import torch

from . import _abi, _native


class Raymarcher:
    def __init__(self, device=0, ctx=None):
        self.device = torch.device("cuda", device)
        self.ctx = ctx or _native.Context(device)

    def draw(self, density, tangent, params, depth_in=None, rgba=None, depth=None):
        """Raymarch one view.  density/tangent are CUDA tensors in the formats
        named by params.density_format / params.tangent_format."""
        W, H = params.width, params.height
        if rgba is None:
            rgba = torch.empty((H, W, 4), dtype=torch.float32, device=self.device)
        if depth is None:
            depth = torch.empty((H, W), dtype=torch.float32, device=self.device)
        self.ctx.raymarch(params, density.data_ptr(), tangent.data_ptr(),
                          None if depth_in is None else depth_in.data_ptr(), rgba.data_ptr(), depth.data_ptr(),
                          torch.cuda.current_stream().cuda_stream)
        return rgba, depth

    def draw_volume(self, volume, params):
        """Raymarch a HairStyle Volume (u8 densities after normalize(), i8x4 tangents)."""
        params.density_format = _abi.DENSITY_U8_UNORM
        params.tangent_format = _abi.TANGENT_I8_SNORM
        return self.draw(volume.densities, volume.tangents, params)
