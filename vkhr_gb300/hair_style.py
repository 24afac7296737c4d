"""Host-side mirror of vkhr::HairStyle's voxelization interface over the C ABI.

Names, arguments and results follow include/vkhr/scene_graph/hair_style.hh:
`HairStyle.voxelize_vertices(width, height, depth)` and
`voxelize_segments(width, height, depth)` return a `Volume` whose
`densities` (u8, saturating at 255), `tangents` (int8 x4) and `bounds`
match `HairStyle::Volume`; `Volume.normalize()` is Volume::normalize.  The
volume additionally carries the exact uint32 `counts`.  All arrays are CUDA
tensors; every computation runs in libvkhr_cuda.so.
"""
import numpy as np
import torch

from . import _abi, _native, strands as _strands


def _ptr(t):
    return None if t is None else t.data_ptr()


def _stream():
    return torch.cuda.current_stream().cuda_stream


class Volume:
    """HairStyle::Volume (hair_style.hh:89-101) plus the uint32 counts."""

    def __init__(self, resolution, bounds, counts, densities, tangents, ctx):
        self.resolution = tuple(int(r) for r in resolution)
        self.bounds = bounds
        self.counts = counts          # torch.int32 storage of uint32 counts, (d, h, w)
        self.densities = densities    # torch.uint8, (d, h, w)
        self.tangents = tangents      # torch.int8, (d, h, w, 4)
        self._ctx = ctx

    def normalize(self):
        """Volume::normalize (hair_style.cc:344-357), in place."""
        self._ctx.normalize_densities(_ptr(self.densities), self.densities.numel(), _stream())
        return self

    def counts_numpy(self):
        return self.counts.cpu().numpy().view(np.uint32).reshape(-1)


class HairStyle:
    """The strand arrays of vkhr::HairStyle (hair_style.hh:126-139) on a CUDA device.

    vertices: (V, 3) float32; segments: (S,) uint16 segments per strand;
    tangents / indices are generated on the device when not given.
    """

    def __init__(self, vertices, segments, tangents=None, indices=None, device=0, ctx=None):
        self.device = torch.device("cuda", device)
        self.ctx = ctx or _native.Context(device)
        self.vertices = torch.as_tensor(np.ascontiguousarray(vertices, dtype=np.float32)).to(self.device)
        self.segments = np.ascontiguousarray(segments, dtype=np.uint16)
        self.tangents = None if tangents is None else torch.as_tensor(
            np.ascontiguousarray(tangents, dtype=np.float32)).to(self.device)
        self.indices = None if indices is None else torch.as_tensor(
            np.ascontiguousarray(indices, dtype=np.uint32).view(np.int32)).to(self.device)
        self._bounds = None

    @classmethod
    def from_strands(cls, strand_set, device=0, ctx=None):
        return cls(strand_set.vertices, strand_set.segments, device=device, ctx=ctx)

    def get_vertex_count(self):
        return int(self.vertices.shape[0])

    def get_strand_count(self):
        return int(self.segments.shape[0])

    def get_segment_count(self):
        return int(self.segments.astype(np.int64).sum())

    def generate_tangents(self):
        """HairStyle::generate_tangents (hair_style.cc:171-194)."""
        self.tangents = torch.empty_like(self.vertices)
        self.ctx.generate_tangents(_ptr(self.vertices), self.segments, _ptr(self.tangents), _stream())
        return self.tangents

    def generate_indices(self):
        """HairStyle::generate_indices (hair_style.cc:196-213)."""
        self.indices = torch.empty(2 * self.get_segment_count(), dtype=torch.int32, device=self.device)
        self.ctx.generate_indices(self.segments, _ptr(self.indices), _stream())
        return self.indices

    def generate_bounding_box(self):
        """HairStyle::generate_bounding_box (hair_style.cc:215-234)."""
        self._bounds = self.ctx.bounding_box(_ptr(self.vertices), self.get_vertex_count(), _stream())
        return self._bounds

    def get_bounding_box(self):
        """HairStyle::get_bounding_box (hair_style.cc:236-255)."""
        if self._bounds is None:
            self.generate_bounding_box()
        return self._bounds

    def set_bounding_box(self, bounds):
        self._bounds = bounds

    def _outputs(self, res):
        w, h, d = res
        counts = torch.empty((d, h, w), dtype=torch.int32, device=self.device)
        dens = torch.empty((d, h, w), dtype=torch.uint8, device=self.device)
        tq = torch.empty((d, h, w, 4), dtype=torch.int8, device=self.device)
        return counts, dens, tq

    def voxelize_vertices(self, width, height, depth, index_mode=_abi.INDEX_REF_FP32):
        """HairStyle::voxelize_vertices (hair_style.cc:257-294)."""
        if self.tangents is None:
            self.generate_tangents()
        res = (int(width), int(height), int(depth))
        b = self.get_bounding_box()
        counts, dens, tq = self._outputs(res)
        self.ctx.voxelize_vertices(_ptr(self.vertices), _ptr(self.tangents), self.get_vertex_count(), b, res,
                                   index_mode, _ptr(counts), _ptr(dens), _ptr(tq), _stream())
        return Volume(res, b, counts, dens, tq, self.ctx)

    def voxelize_segments(self, width, height, depth, index_mode=_abi.INDEX_REF_FP32):
        """HairStyle::voxelize_segments (hair_style.cc:296-342)."""
        if self.tangents is None:
            self.generate_tangents()
        if self.indices is None:
            self.generate_indices()
        res = (int(width), int(height), int(depth))
        b = self.get_bounding_box()
        counts, dens, tq = self._outputs(res)
        self.ctx.voxelize_segments(_ptr(self.vertices), _ptr(self.tangents), _ptr(self.indices),
                                   int(self.indices.numel()), b, res, index_mode, _ptr(counts), _ptr(dens),
                                   _ptr(tq), _stream())
        return Volume(res, b, counts, dens, tq, self.ctx)


def synthetic(kind="disk", **kw):
    """Convenience: a grown style as a HairStyle (see vkhr_gb300.strands)."""
    gen = _strands.disk_style if kind == "disk" else _strands.hemisphere_style
    return HairStyle.from_strands(gen(**kw))
