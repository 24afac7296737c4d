"""ctypes mirror of the C ABI declared in include/vkhr_cuda.h.

The structures here must stay layout-identical to the header; the native
library exports ``vkhr_sizeof_*`` helpers and the tests compare them.
"""
import ctypes as C

import numpy as np

VKHR_OK = 0
VKHR_ERR_INVALID_ARG = 1
VKHR_ERR_DEGENERATE_AABB = 2
VKHR_ERR_OOM = 3
VKHR_ERR_CUDA = 4
VKHR_ERR_TIMEOUT = 5
VKHR_ERR_NAN_INPUT = 6
VKHR_ERR_CAPACITY = 7
VKHR_ERR_NOT_SUPPORTED = 8

STATUS_NAMES = {
    0: "VKHR_OK",
    1: "VKHR_ERR_INVALID_ARG",
    2: "VKHR_ERR_DEGENERATE_AABB",
    3: "VKHR_ERR_OOM",
    4: "VKHR_ERR_CUDA",
    5: "VKHR_ERR_TIMEOUT",
    6: "VKHR_ERR_NAN_INPUT",
    7: "VKHR_ERR_CAPACITY",
    8: "VKHR_ERR_NOT_SUPPORTED",
}

INDEX_REF_FP32 = 0
INDEX_EXACT = 1

RAYMARCH_VARIANTS = 11
TUNED_RAYMARCH_VARIANTS = (0, 1, 2, 3, 4, 7, 8, 9, 10)  # the variants that compute the same pixels (autotuned)
RAYMARCH_TEXTURE_VARIANT = 5
RAYMARCH_SHADE_TEXTURE_VARIANT = 6  # the texture unit for the shadow and AO samples only
RAYMARCH_GATHER_VARIANT = 7  # exact texels through the texture unit's gathers
RAYMARCH_GROUP_VARIANTS = (8, 9, 10)  # ray groups of 4, 2 and 8 lanes per pixel
MAX_AO_DIRECTIONS = 32
WALK_CHOICES = (0, 2, 3, 4, 5, 6)  # vkhr_autotune_voxelize: resident one-walk CTAs per SM (0: no limit)

FILTER_MAX = 0
FILTER_MIN = 1
FILTER_MEAN = 2
FILTER_SUM = 3

DENSITY_U8_UNORM = 0
DENSITY_U32_COUNT = 1
DENSITY_F32 = 2

TANGENT_I8_SNORM = 0
TANGENT_F32X4 = 1

SHADING_KAJIYA_KAY = 0
SHADING_ADSM = 2
SHADING_LAO = 3

RENDERER_RASTERIZER = 0
RENDERER_RAY_TRACER = 1
RENDERER_RAYMARCHER = 2
RENDERER_HYBRID_LOD = 3


# vkhr_ppll_node (ppll.glsl:7-11) and vkhr_fragment: 12 bytes each
PPLL_NULL = 0xFFFFFFFF
K_BUFFER_SIZE = 16
MAX_FRAGMENTS = 1024
PPLL_NODE_DTYPE = np.dtype([("color", "<u4"), ("depth", "<f4"), ("prev", "<u4")])
FRAGMENT_DTYPE = np.dtype([("color", "<u4"), ("depth", "<f4"), ("pixel", "<u4")])


class AABB(C.Structure):
    """vkhr::AABB (include/vkhr/scene_graph/hair_style.hh:16-21)."""

    _fields_ = [
        ("origin", C.c_float * 3),
        ("radius", C.c_float),
        ("size", C.c_float * 3),
        ("volume", C.c_float),
    ]

    def as_dict(self):
        return {
            "origin": tuple(self.origin),
            "radius": self.radius,
            "size": tuple(self.size),
            "volume": self.volume,
        }


class HairHeader(C.Structure):
    """vkhr_hair_header: a `.hair` file's 128-byte header (hair_style.hh:147-174)."""

    _fields_ = [
        ("signature", C.c_char * 4),
        ("strand_count", C.c_uint32),
        ("vertex_count", C.c_uint32),
        ("fields", C.c_uint32),
        ("default_segment_count", C.c_uint32),
        ("default_thickness", C.c_float),
        ("default_transparency", C.c_float),
        ("default_color", C.c_float * 3),
        ("information", C.c_char * 64),
        ("bounding_box_min", C.c_float * 3),
        ("bounding_box_max", C.c_float * 3),
    ]


HAIR_SEGMENTS, HAIR_VERTICES, HAIR_THICKNESS, HAIR_TRANSPARENCY = 1, 2, 4, 8
HAIR_COLOR, HAIR_TANGENTS, HAIR_INDICES, HAIR_BOUNDING_BOX = 16, 32, 64, 128


class VoxelJob(C.Structure):
    """vkhr_voxel_job: one style of a batched voxelization."""

    _fields_ = [
        ("d_vertices", C.c_void_p),
        ("d_tangent_in", C.c_void_p),
        ("d_indices", C.c_void_p),
        ("item_count", C.c_uint64),
        ("bounds", AABB),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("depth", C.c_int32),
        ("index_mode", C.c_int32),
        ("d_counts", C.c_void_p),
        ("d_densities", C.c_void_p),
        ("d_tangents", C.c_void_p),
    ]


class RaymarchParams(C.Structure):
    """vkhr_raymarch_params: the camera, light, strand and params UBOs."""

    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("view", C.c_float * 16),
        ("projection", C.c_float * 16),
        ("camera_position", C.c_float * 3),
        ("look_at_distance", C.c_float),
        ("light_origin", C.c_float * 3),
        ("light_intensity", C.c_float * 3),
        ("volume_bounds", AABB),
        ("volume_resolution", C.c_int32 * 3),
        ("hair_color", C.c_float * 3),
        ("hair_alpha", C.c_float),
        ("hair_exponent", C.c_float),
        ("shading_model", C.c_int32),
        ("deep_shadows_on", C.c_int32),
        ("isosurface", C.c_float),
        ("raycast_steps", C.c_float),
        ("occlusion_radius", C.c_float),
        ("ao_exponent", C.c_float),
        ("ao_max", C.c_float),
        ("magnified_distance", C.c_float),
        ("renderer", C.c_int32),
        ("minified_distance", C.c_float),
        ("shadow_thickness", C.c_float),
        ("ao_kernel_size", C.c_float),
        ("shadow_steps", C.c_float),
        ("kd", C.c_float),
        ("density_format", C.c_int32),
        ("tangent_format", C.c_int32),
        ("spec_exponent2", C.c_float),
        ("spec_shift", C.c_float * 2),
        ("ao_directions", C.c_int32),
    ]


def aabb_from(origin, size):
    """AABB with radius/volume derived exactly as get_bounding_box does (FP32)."""
    import numpy as np

    o = np.asarray(origin, dtype=np.float32)
    s = np.asarray(size, dtype=np.float32)
    b = AABB()
    for c in range(3):
        b.origin[c] = float(o[c])
        b.size[c] = float(s[c])
    dot = np.float32(np.float32(s[0] * s[0]) + np.float32(s[1] * s[1])) + np.float32(s[2] * s[2])
    b.radius = float(np.sqrt(np.float32(dot)))
    b.volume = float(np.float32(np.float32(s[0] * s[1]) * s[2]))
    return b


class RaymarchJob(C.Structure):
    """vkhr_raymarch_job: one view of a batched raymarch and its region."""

    _fields_ = [
        ("params", RaymarchParams),
        ("d_density", C.c_void_p),
        ("d_tangent", C.c_void_p),
        ("d_depth_in", C.c_void_p),
        ("d_rgba", C.c_void_p),
        ("d_depth_out", C.c_void_p),
        ("x0", C.c_int32),
        ("y0", C.c_int32),
        ("w", C.c_int32),
        ("h", C.c_int32),
        ("pitch", C.c_int32),
        ("reserved", C.c_int32),
    ]
