"""ctypes binding of libvkhr_cuda.so (the C ABI in include/vkhr_cuda.h).

There is no fallback: importing this module without the built library, or
using it without a CUDA device, raises.
"""
import ctypes as C
import os

from . import _abi

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libvkhr_cuda.so")

EXPORTS = [
    "vkhr_abi_version", "vkhr_create", "vkhr_destroy", "vkhr_status_string", "vkhr_last_error",
    "vkhr_bounding_box", "vkhr_generate_tangents", "vkhr_generate_indices",
    "vkhr_voxelize_vertices", "vkhr_voxelize_segments", "vkhr_normalize_densities", "vkhr_raymarch",
    "vkhr_launch_count", "vkhr_sizeof_aabb", "vkhr_sizeof_raymarch_params",
    "vkhr_set_profiling", "vkhr_profile_count", "vkhr_profile_read",
    "vkhr_malloc", "vkhr_free", "vkhr_upload", "vkhr_download", "vkhr_sync", "vkhr_check_status",
    "vkhr_voxelize_batched", "vkhr_set_visit_budget", "vkhr_sizeof_voxel_job",
    "vkhr_raymarch_batched", "vkhr_raymarch_footprint", "vkhr_sizeof_raymarch_job",
    "vkhr_downsample_densities", "vkhr_raymarch_tape_bytes", "vkhr_raymarch_train", "vkhr_raymarch_adjoint",
    "vkhr_splat_vertices", "vkhr_splat_vertices_adjoint", "vkhr_autotune_raymarch", "vkhr_set_raymarch_variant",
    "vkhr_frame_graph_create", "vkhr_frame_graph_launch", "vkhr_frame_graph_destroy",
    "vkhr_hair_read_header", "vkhr_hair_load", "vkhr_reduce_strands",
    "vkhr_resolve_ppll", "vkhr_composite", "vkhr_level_of_detail", "vkhr_lod", "vkhr_rasterizer_enabled",
    "vkhr_raymarcher_enabled",
]

_lib = None


class VkhrError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (_abi.STATUS_NAMES.get(status, status), message))
        self.status = status


def load():
    """Load the library (no CUDA call is made)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libvkhr_cuda.so is not built (run __graft_entry__.build() or "
                          "python vkhr_gb300/build.py): the GB300 path has no CPU fallback")
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    lib.vkhr_abi_version.restype = C.c_int
    lib.vkhr_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
    lib.vkhr_destroy.argtypes = [P]
    lib.vkhr_status_string.argtypes = [C.c_int]
    lib.vkhr_status_string.restype = C.c_char_p
    lib.vkhr_last_error.argtypes = [P]
    lib.vkhr_last_error.restype = C.c_char_p
    lib.vkhr_bounding_box.argtypes = [P, P, C.c_uint32, C.POINTER(_abi.AABB), P]
    lib.vkhr_generate_tangents.argtypes = [P, P, P, C.c_uint32, P, P]
    lib.vkhr_generate_indices.argtypes = [P, P, C.c_uint32, P, P]
    lib.vkhr_voxelize_vertices.argtypes = [P, P, P, C.c_uint32, C.POINTER(_abi.AABB), C.c_int32, C.c_int32,
                                           C.c_int32, C.c_int32, P, P, P, P]
    lib.vkhr_voxelize_segments.argtypes = [P, P, P, P, C.c_uint64, C.POINTER(_abi.AABB), C.c_int32, C.c_int32,
                                           C.c_int32, C.c_int32, P, P, P, P]
    lib.vkhr_voxelize_batched.argtypes = [P, C.c_int32, C.POINTER(_abi.VoxelJob), C.c_int32, P]
    lib.vkhr_set_visit_budget.argtypes = [P, C.c_uint64]
    lib.vkhr_set_voxelize_walk.argtypes = [P, C.c_int32, C.c_int32]
    lib.vkhr_autotune_voxelize.argtypes = [P, C.POINTER(_abi.VoxelJob), C.c_int32, C.POINTER(C.c_int32),
                                           C.POINTER(C.c_float), P]
    lib.vkhr_raymarch_batched.argtypes = [P, C.POINTER(_abi.RaymarchJob), C.c_int32, P]
    lib.vkhr_raymarch_footprint.argtypes = [C.POINTER(_abi.RaymarchParams), C.POINTER(C.c_int32)]
    lib.vkhr_normalize_densities.argtypes = [P, P, C.c_uint64, P]
    lib.vkhr_downsample_densities.argtypes = [P, P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P]
    lib.vkhr_autotune_raymarch.argtypes = [P, C.POINTER(_abi.RaymarchParams), P, P, P, C.POINTER(C.c_int32),
                                           C.POINTER(C.c_float), P]
    lib.vkhr_set_raymarch_variant.argtypes = [P, C.c_int32, C.c_int32, C.c_int32]
    lib.vkhr_raymarch_tape_bytes.argtypes = [C.POINTER(_abi.RaymarchParams), C.c_int32]
    lib.vkhr_raymarch_tape_bytes.restype = C.c_size_t
    lib.vkhr_raymarch_train.argtypes = [P, C.POINTER(_abi.RaymarchParams), P, P, P, P, P, C.c_size_t, C.c_int32, P]
    lib.vkhr_raymarch_adjoint.argtypes = [P, C.POINTER(_abi.RaymarchParams), P, P, P, C.c_int32, P, P, P, P, P]
    lib.vkhr_splat_vertices.argtypes = [P, P, C.c_uint32, C.POINTER(_abi.AABB), C.c_int32, C.c_int32, C.c_int32, P,
                                        P]
    lib.vkhr_splat_vertices_adjoint.argtypes = [P, P, C.c_uint32, C.POINTER(_abi.AABB), C.c_int32, C.c_int32,
                                                C.c_int32, P, P, P]
    lib.vkhr_check_status.argtypes = [P, P]
    lib.vkhr_frame_graph_create.argtypes = [P, C.c_int32, C.POINTER(_abi.VoxelJob), C.c_int32, C.c_uint64,
                                            C.POINTER(_abi.RaymarchParams), P, P, P, P, C.POINTER(C.c_void_p)]
    lib.vkhr_frame_graph_launch.argtypes = [P, P]
    lib.vkhr_hair_read_header.argtypes = [C.c_char_p, C.POINTER(_abi.HairHeader)]
    lib.vkhr_hair_load.argtypes = [P, C.c_char_p, C.POINTER(_abi.HairHeader), P, P, P, P, P]
    U32P = C.POINTER(C.c_uint32)
    lib.vkhr_reduce_strands.argtypes = [P, C.c_float, C.POINTER(C.c_uint64), P, C.c_uint32, C.c_uint32, P, P, P, U32P,
                                        U32P, P, P, P]
    lib.vkhr_frame_graph_destroy.argtypes = [P]
    lib.vkhr_resolve_ppll.argtypes = [P, P, P, C.c_uint32, C.c_int32, C.c_int32, P, P]
    lib.vkhr_composite.argtypes = [P, P, C.c_uint32, P, P, C.c_int32, C.c_int32, P, P]
    lib.vkhr_level_of_detail.argtypes = [C.c_float, C.c_float, C.c_float]
    lib.vkhr_level_of_detail.restype = C.c_float
    lib.vkhr_lod.argtypes = [C.c_int32, C.c_float, C.c_float, C.c_float]
    lib.vkhr_lod.restype = C.c_float
    lib.vkhr_rasterizer_enabled.argtypes = [C.c_int32, C.c_float]
    lib.vkhr_raymarcher_enabled.argtypes = [C.c_int32, C.c_float]
    lib.vkhr_raymarch.argtypes = [P, C.POINTER(_abi.RaymarchParams), P, P, P, P, P, P]
    lib.vkhr_malloc.argtypes = [P, C.c_size_t, C.POINTER(C.c_void_p)]
    lib.vkhr_free.argtypes = [P, P]
    lib.vkhr_upload.argtypes = [P, P, P, C.c_size_t, P]
    lib.vkhr_download.argtypes = [P, P, P, C.c_size_t, P]
    lib.vkhr_sync.argtypes = [P, P]
    lib.vkhr_set_profiling.argtypes = [P, C.c_int]
    lib.vkhr_profile_count.argtypes = [P]
    lib.vkhr_profile_read.argtypes = [P, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_float)]
    lib.vkhr_launch_count.argtypes = [P]
    lib.vkhr_launch_count.restype = C.c_uint64
    lib.vkhr_sizeof_aabb.restype = C.c_size_t
    lib.vkhr_sizeof_raymarch_params.restype = C.c_size_t
    lib.vkhr_sizeof_voxel_job.restype = C.c_size_t
    lib.vkhr_sizeof_raymarch_job.restype = C.c_size_t
    for name in EXPORTS:
        if getattr(lib, name).restype is C.c_int or getattr(lib, name).restype is None:
            getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


class FrameGraph:
    """A captured frame (vkhr_frame_graph_*): launch() replays it on a stream."""

    def __init__(self, ctx, handle):
        self.ctx, self.handle = ctx, handle

    def launch(self, stream=None):
        self.ctx.check(self.ctx.lib.vkhr_frame_graph_launch(self.handle, stream))

    def close(self):
        if self.handle:
            self.ctx.lib.vkhr_frame_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """Owns one vkhr_ctx (device pinned at creation, scratch grows on demand)."""

    def __init__(self, device=0):
        self.lib = load()
        h = C.c_void_p()
        s = self.lib.vkhr_create(int(device), C.byref(h))
        if s != _abi.VKHR_OK:
            raise VkhrError(s, "vkhr_create(%d) failed" % device)
        self.handle = h
        self.device = device

    def check(self, status):
        if status != _abi.VKHR_OK:
            raise VkhrError(status, self.lib.vkhr_last_error(self.handle).decode())

    def set_profiling(self, enable):
        self.check(self.lib.vkhr_set_profiling(self.handle, 1 if enable else 0))

    def profile(self):
        """[(kernel name, ms)] for every launch since profiling was enabled."""
        out = []
        for i in range(self.lib.vkhr_profile_count(self.handle)):
            name = C.c_char_p()
            ms = C.c_float()
            self.check(self.lib.vkhr_profile_read(self.handle, i, C.byref(name), C.byref(ms)))
            out.append((name.value.decode(), float(ms.value)))
        return out

    def launch_count(self):
        return int(self.lib.vkhr_launch_count(self.handle))

    def close(self):
        if getattr(self, "handle", None):
            self.lib.vkhr_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # thin wrappers: every pointer argument is a raw device address (int) or None
    def bounding_box(self, d_vertices, vertex_count, stream=None):
        b = _abi.AABB()
        self.check(self.lib.vkhr_bounding_box(self.handle, d_vertices, vertex_count, C.byref(b), stream))
        return b

    def generate_tangents(self, d_vertices, segments_u16, d_tangents, stream=None):
        self.check(self.lib.vkhr_generate_tangents(self.handle, d_vertices, segments_u16.ctypes.data,
                                                   segments_u16.shape[0], d_tangents, stream))

    def generate_indices(self, segments_u16, d_indices, stream=None):
        self.check(self.lib.vkhr_generate_indices(self.handle, segments_u16.ctypes.data, segments_u16.shape[0],
                                                  d_indices, stream))

    def voxelize_vertices(self, d_vertices, d_tangent_in, vertex_count, bounds, res, index_mode, d_counts,
                          d_densities, d_tangents, stream=None):
        w, h, d = res
        self.check(self.lib.vkhr_voxelize_vertices(self.handle, d_vertices, d_tangent_in, vertex_count,
                                                   C.byref(bounds), w, h, d, index_mode, d_counts, d_densities,
                                                   d_tangents, stream))

    def voxelize_segments(self, d_vertices, d_tangent_in, d_indices, index_count, bounds, res, index_mode, d_counts,
                          d_densities, d_tangents, stream=None):
        w, h, d = res
        self.check(self.lib.vkhr_voxelize_segments(self.handle, d_vertices, d_tangent_in, d_indices, index_count,
                                                   C.byref(bounds), w, h, d, index_mode, d_counts, d_densities,
                                                   d_tangents, stream))

    def voxelize_batched(self, segments, jobs, stream=None):
        """jobs: a sequence of _abi.VoxelJob (item_count = vertex or index count)."""
        arr = (_abi.VoxelJob * len(jobs))(*jobs)
        self.check(self.lib.vkhr_voxelize_batched(self.handle, 1 if segments else 0, arr, len(jobs), stream))

    def frame_graph(self, segments, job, params, d_rgba, d_depth_out=None, d_depth_in=None, normalize=True,
                    visit_budget=0, stream=None):
        """vkhr_frame_graph_create: one CUDA graph of the job's voxelization,
        Volume::normalize and the view's raymarch; FrameGraph.launch replays it."""
        h = C.c_void_p()
        self.check(self.lib.vkhr_frame_graph_create(self.handle, 1 if segments else 0, C.byref(job),
                                                    1 if normalize else 0, int(visit_budget), C.byref(params),
                                                    d_depth_in, d_rgba, d_depth_out, stream, C.byref(h)))
        return FrameGraph(self, h)

    def hair_load(self, path, d_vertices, d_tangents=None, d_indices=None, want_segments=True, stream=None):
        """vkhr_hair_load: (header, host segment counts or None)."""
        import numpy as np

        hdr = hair_read_header(path)
        segs = np.zeros(hdr.strand_count, dtype=np.uint16) if want_segments else None
        out = _abi.HairHeader()
        self.check(self.lib.vkhr_hair_load(self.handle, path.encode(), C.byref(out),
                                           None if segs is None else segs.ctypes.data_as(C.c_void_p), d_vertices,
                                           d_tangents, d_indices, stream))
        return out, segs

    def reduce_strands(self, ratio, seed, segments, strand_count, d_vertices, d_tangents, d_vertices_out,
                       d_tangents_out=None, default_segment_count=0, stream=None):
        """vkhr_reduce_strands: (kept segment counts, kept vertex count, seed after)."""
        import numpy as np

        segs = None if segments is None else np.ascontiguousarray(segments, dtype=np.uint16)
        out = np.zeros(max(strand_count, 1), dtype=np.uint16)
        sd = C.c_uint64(seed)
        ns, nv = C.c_uint32(), C.c_uint32()
        self.check(self.lib.vkhr_reduce_strands(self.handle, ratio, C.byref(sd),
                                                None if segs is None else segs.ctypes.data_as(C.c_void_p),
                                                strand_count, default_segment_count, d_vertices, d_tangents,
                                                out.ctypes.data_as(C.c_void_p), C.byref(ns), C.byref(nv),
                                                d_vertices_out, d_tangents_out, stream))
        return out[:ns.value], nv.value, sd.value

    def resolve_ppll(self, d_heads, d_nodes, node_count, width, height, d_color, stream=None):
        """vkhr_resolve_ppll: resolve.comp over the reference's PPLL onto d_color."""
        self.check(self.lib.vkhr_resolve_ppll(self.handle, d_heads, d_nodes, node_count, width, height, d_color,
                                              stream))

    def composite(self, d_fragments, fragment_count, width, height, d_color, d_volume_rgba=None,
                  d_volume_depth=None, stream=None):
        """vkhr_composite: the PPLL-free resolve of strand fragments (and the
        raymarched volume's fragments) onto d_color."""
        self.check(self.lib.vkhr_composite(self.handle, d_fragments, fragment_count, d_volume_rgba, d_volume_depth,
                                           width, height, d_color, stream))

    def raymarch_batched(self, jobs, stream=None):
        """jobs: a sequence of _abi.RaymarchJob."""
        arr = (_abi.RaymarchJob * len(jobs))(*jobs)
        self.check(self.lib.vkhr_raymarch_batched(self.handle, arr, len(jobs), stream))

    def set_visit_budget(self, max_visits):
        self.check(self.lib.vkhr_set_visit_budget(self.handle, int(max_visits)))

    def check_status(self, stream=None):
        self.check(self.lib.vkhr_check_status(self.handle, stream))

    def set_voxelize_walk(self, which, ctas_per_sm):
        """Resident CTAs per SM of the one-walk kernel (which: 0 one style, 1 batch; 0 = no limit)."""
        self.check(self.lib.vkhr_set_voxelize_walk(self.handle, which, ctas_per_sm))

    def autotune_voxelize(self, jobs, stream=None):
        """Segment jobs: (chosen residency, [median ms of each of WALK_CHOICES])."""
        arr = (_abi.VoxelJob * len(jobs))(*jobs)
        chosen = C.c_int32(-1)
        ms = (C.c_float * len(_abi.WALK_CHOICES))()
        self.check(self.lib.vkhr_autotune_voxelize(self.handle, arr, len(jobs), C.byref(chosen), ms, stream))
        return int(chosen.value), [float(x) for x in ms]

    def normalize_densities(self, d_densities, n, stream=None):
        self.check(self.lib.vkhr_normalize_densities(self.handle, d_densities, n, stream))

    def downsample_densities(self, d_in, res, filt, d_out, stream=None):
        w, h, d = res
        self.check(self.lib.vkhr_downsample_densities(self.handle, d_in, w, h, d, filt, d_out, stream))

    def autotune_raymarch(self, params, d_density, d_tangent, d_rgba, stream=None):
        """(chosen variant, [median ms of each variant])."""
        chosen = C.c_int32(-1)
        ms = (C.c_float * _abi.RAYMARCH_VARIANTS)()
        self.check(self.lib.vkhr_autotune_raymarch(self.handle, C.byref(params), d_density, d_tangent, d_rgba,
                                                   C.byref(chosen), ms, stream))
        return int(chosen.value), [float(x) for x in ms]

    def set_raymarch_variant(self, density_format, tangent_format, variant):
        self.check(self.lib.vkhr_set_raymarch_variant(self.handle, density_format, tangent_format, variant))

    # differentiable path
    def tape_bytes(self, params, checkpoint_interval):
        return int(self.lib.vkhr_raymarch_tape_bytes(C.byref(params), checkpoint_interval))

    def raymarch_train(self, params, d_density, d_tangent, d_rgba, d_depth_out, d_tape, tape_bytes,
                       checkpoint_interval, stream=None):
        self.check(self.lib.vkhr_raymarch_train(self.handle, C.byref(params), d_density, d_tangent, d_rgba,
                                                d_depth_out, d_tape, tape_bytes, checkpoint_interval, stream))

    def raymarch_adjoint(self, params, d_density, d_tangent, d_tape, checkpoint_interval, d_grad_rgba,
                         d_grad_density, d_grad_tangent, d_grad_params, stream=None):
        self.check(self.lib.vkhr_raymarch_adjoint(self.handle, C.byref(params), d_density, d_tangent, d_tape,
                                                  checkpoint_interval, d_grad_rgba, d_grad_density, d_grad_tangent,
                                                  d_grad_params, stream))

    def splat_vertices(self, d_vertices, vertex_count, bounds, res, d_density, stream=None):
        w, h, d = res
        self.check(self.lib.vkhr_splat_vertices(self.handle, d_vertices, vertex_count, C.byref(bounds), w, h, d,
                                                d_density, stream))

    def splat_vertices_adjoint(self, d_vertices, vertex_count, bounds, res, d_grad_density, d_grad_vertices,
                               stream=None):
        w, h, d = res
        self.check(self.lib.vkhr_splat_vertices_adjoint(self.handle, d_vertices, vertex_count, C.byref(bounds), w,
                                                        h, d, d_grad_density, d_grad_vertices, stream))

    def raymarch(self, params, d_density, d_tangent, d_depth_in, d_rgba, d_depth_out, stream=None):
        self.check(self.lib.vkhr_raymarch(self.handle, C.byref(params), d_density, d_tangent, d_depth_in, d_rgba,
                                          d_depth_out, stream))


def hair_read_header(path):
    """vkhr_hair_read_header (no CUDA call)."""
    lib = load()
    h = _abi.HairHeader()
    st = lib.vkhr_hair_read_header(path.encode(), C.byref(h))
    if st != 0:
        raise VkhrError(st, "vkhr_hair_read_header(%s)" % path)
    return h


def level_of_detail(magnified_distance, minified_distance, distance):
    """vkhr_level_of_detail: Rasterizer::update's smoothstep (no CUDA call)."""
    return load().vkhr_level_of_detail(magnified_distance, minified_distance, distance)


def lod(renderer, magnified_distance, minified_distance, distance):
    """vkhr_lod: scheme.glsl's lod() (no CUDA call)."""
    return load().vkhr_lod(renderer, magnified_distance, minified_distance, distance)


def rasterizer_enabled(renderer, level):
    return bool(load().vkhr_rasterizer_enabled(renderer, level))


def raymarcher_enabled(renderer, level):
    return bool(load().vkhr_raymarcher_enabled(renderer, level))


def raymarch_footprint(params):
    """(x0, y0, w, h): pixels outside it are background in vkhr_raymarch."""
    lib = load()
    r = (C.c_int32 * 4)()
    st = lib.vkhr_raymarch_footprint(C.byref(params), r)
    if st != 0:
        raise VkhrError(st, "vkhr_raymarch_footprint")
    return tuple(int(x) for x in r)
