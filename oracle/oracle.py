"""Python bindings of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/liboracle.so (the C restatement) and, when it was built here,
oracle/_ref/libvkhr_ref.so (the reference's own voxelizer and raymarch shader
compiled from its sources).  Only tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py import this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from vkhr_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libvkhr_ref.so")
REFERENCE_ROOT = os.environ.get("VKHR_REFERENCE_ROOT", "/root/reference")

_lib = None
_ref = None


def build(with_reference=None):
    """Compile liboracle.so (always) and _ref (when the reference sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if with_reference is None:
        with_reference = os.path.isfile(os.path.join(REFERENCE_ROOT, "src/vkhr/scene_graph/hair_style.cc"))
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


DIAG_DTYPE = np.dtype([("iso_margin", np.float64), ("support_margin", np.float64), ("tangent_len", np.float64),
                       ("iso_shift", np.float64), ("fp32_res", np.float64), ("steps_taken", np.int32),
                       ("covered", np.int32)])

P = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(with_reference=False)
        _lib = C.CDLL(LIB)
        _lib.oracle_bounding_box.argtypes = [P, C.c_uint32, C.POINTER(_abi.AABB)]
        _lib.oracle_generate_tangents.argtypes = [P, P, C.c_uint32, P]
        _lib.oracle_generate_indices.argtypes = [P, C.c_uint32, P]
        _lib.oracle_voxelize_vertices.argtypes = [P, P, C.c_uint32, C.POINTER(_abi.AABB), C.c_int, C.c_int, C.c_int,
                                                  C.c_int, P, P, P]
        _lib.oracle_voxelize_vertices.restype = C.c_uint64
        _lib.oracle_voxelize_segments.argtypes = [P, P, P, C.c_uint64, C.POINTER(_abi.AABB), C.c_int, C.c_int,
                                                  C.c_int, C.c_int, P, P, P]
        _lib.oracle_voxelize_segments.restype = C.c_uint64
        _lib.oracle_segment_visits.argtypes = [P, P, C.c_uint64, C.POINTER(_abi.AABB), C.c_int, C.c_int, C.c_int]
        _lib.oracle_segment_visits.restype = C.c_uint32
        _lib.oracle_normalize.argtypes = [P, C.c_uint64]
        _lib.oracle_downsample.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P]
        _lib.oracle_diff_loss.argtypes = [C.POINTER(_abi.RaymarchParams), P, P, P, P, P, P, P, C.c_int]
        _lib.oracle_diff_loss.restype = C.c_double
        _lib.oracle_splat.argtypes = [P, C.c_uint32, C.POINTER(_abi.AABB), C.c_int, C.c_int, C.c_int, P]
        _lib.oracle_splat_adjoint.argtypes = [P, C.c_uint32, C.POINTER(_abi.AABB), C.c_int, C.c_int, C.c_int, P, P]
        _lib.oracle_pixel_entry.argtypes = [C.POINTER(_abi.RaymarchParams), C.c_int, C.c_int, P]
        _lib.oracle_raymarch_f64.argtypes = [C.POINTER(_abi.RaymarchParams), P, P, P, P, P, P, C.c_int, C.c_int,
                                             C.c_int]
        _lib.oracle_raymarch_f32.argtypes = [C.POINTER(_abi.RaymarchParams), P, P, P, P, P, C.c_int, C.c_int,
                                             C.c_int]
        _lib.oracle_max_threads.restype = C.c_int
        _lib.oracle_pack_unorm8x4.argtypes = [P]
        _lib.oracle_pack_unorm8x4.restype = C.c_uint32
        _lib.oracle_resolve_ppll.argtypes = [P, P, C.c_uint32, C.c_int, C.c_int, P, C.c_int]
        _lib.oracle_resolve_ppll.restype = C.c_int
        _lib.oracle_composite.argtypes = [P, C.c_uint32, P, P, C.c_int, C.c_int, P, C.c_int]
        _lib.oracle_composite.restype = C.c_int
    return _lib


def has_reference():
    return os.path.exists(REF_LIB)


def ref():
    global _ref
    if _ref is None:
        lib()
        _ref = C.CDLL(REF_LIB)
        _ref.ref_prepare.argtypes = [P, C.c_uint32, P, C.c_uint32, P, P, C.POINTER(_abi.AABB)]
        _ref.ref_voxelize.argtypes = [C.c_int, P, C.c_uint32, P, P, C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int,
                                      P, P]
        _ref.ref_raymarch.argtypes = [C.POINTER(_abi.RaymarchParams), P, P, P, P, P, C.c_int, C.c_int, C.c_int]
        _ref.ref_raymarch.restype = C.c_int
        _ref.ref_downsample.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, P]
        U32P = C.POINTER(C.c_uint32)
        _ref.ref_hair_load.argtypes = [C.c_char_p, U32P, U32P, U32P, U32P, P, C.c_uint32, P, P, C.c_uint32, P, C.c_uint32]
        _ref.ref_hair_load.restype = C.c_int
        _ref.ref_hair_save.argtypes = [C.c_char_p, P, C.c_uint32, P, P, C.c_uint32]
        _ref.ref_hair_save.restype = C.c_int
        _ref.ref_reduce.argtypes = [P, P, C.c_uint32, P, C.c_uint32, C.c_uint32, C.c_float, C.POINTER(C.c_uint64), P,
                                    P, P, U32P, U32P]
        _ref.ref_resolve_ppll.argtypes = [P, P, C.c_uint32, C.c_int, C.c_int, P, C.c_int]
        _ref.ref_resolve_ppll.restype = C.c_int
        _ref.ref_build_ppll.argtypes = [P, C.c_uint32, P, P, C.c_int, C.c_int, C.c_uint32, P, P]
        _ref.ref_build_ppll.restype = C.c_uint32
    return _ref


def ref_hair_load(path):
    """The reference's HairStyle::load of `path`: (error state, dict of arrays)."""
    r = ref()
    n, v, bits, ni = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_uint32()
    err = r.ref_hair_load(path.encode(), C.byref(n), C.byref(v), C.byref(bits), C.byref(ni), None, 0, None, None, 0,
                          None, 0)
    segs = np.zeros(n.value, dtype=np.uint16)
    verts = np.zeros((v.value, 3), dtype=np.float32)
    tans = np.zeros((v.value, 3), dtype=np.float32)
    idx = np.zeros(ni.value, dtype=np.uint32)
    err = r.ref_hair_load(path.encode(), C.byref(n), C.byref(v), C.byref(bits), C.byref(ni), _p(segs), n.value,
                          _p(verts), _p(tans), v.value, _p(idx), ni.value)
    return err, {"fields": bits.value, "segments": segs, "vertices": verts, "tangents": tans, "indices": idx}


def ref_hair_save(path, segments, vertices, tangents=None):
    """The reference's HairStyle::save of the given arrays; 0 on success."""
    segs = np.ascontiguousarray(segments, dtype=np.uint16)
    v = _f32(vertices)
    t = None if tangents is None else _f32(tangents)
    return ref().ref_hair_save(path.encode(), _p(segs), len(segs), _p(v), _p(t), len(v))


def ref_reduce(vertices, tangents, segments, strand_count, ratio, seed, default_segment_count=0):
    """The reference's HairStyle::reduce(ratio) with the seed fixed: (kept
    vertices, kept tangents, kept segment counts, seed after)."""
    v = _f32(vertices)
    t = None if tangents is None else _f32(tangents)
    segs = None if segments is None else np.ascontiguousarray(segments, dtype=np.uint16)
    vo = np.zeros_like(v)
    to = None if t is None else np.zeros_like(t)
    so = np.zeros(max(strand_count, 1), dtype=np.uint16)
    sd = C.c_uint64(seed)
    ns, nv = C.c_uint32(), C.c_uint32()
    ref().ref_reduce(_p(v), _p(t), len(v), _p(segs), strand_count, default_segment_count, ratio, C.byref(sd), _p(vo),
                     _p(to), _p(so), C.byref(ns), C.byref(nv))
    return vo[:nv.value], None if to is None else to[:nv.value], so[:ns.value], sd.value


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


# ---- voxelizer ---------------------------------------------------------------

def bounding_box(vertices):
    v = _f32(vertices)
    b = _abi.AABB()
    lib().oracle_bounding_box(_p(v), v.shape[0], C.byref(b))
    return b


def generate_tangents(vertices, segments):
    v = _f32(vertices)
    s = np.ascontiguousarray(segments, dtype=np.uint16)
    t = np.zeros_like(v)
    lib().oracle_generate_tangents(_p(v), _p(s), s.shape[0], _p(t))
    return t


def generate_indices(segments):
    s = np.ascontiguousarray(segments, dtype=np.uint16)
    out = np.zeros(2 * int(s.astype(np.int64).sum()), dtype=np.uint32)
    lib().oracle_generate_indices(_p(s), s.shape[0], _p(out))
    return out


def voxelize(mode, vertices, tangents, indices, bounds, res, index_mode=_abi.INDEX_REF_FP32):
    """mode 'vertices' or 'segments'; returns (counts u32, densities u8, tangents i8x4, dropped)."""
    w, h, d = (int(x) for x in res)
    n = w * h * d
    v = _f32(vertices)
    t = None if tangents is None else _f32(tangents)
    counts = np.zeros(n, dtype=np.uint32)
    dens = np.zeros(n, dtype=np.uint8)
    tq = np.zeros((n, 4), dtype=np.int8)
    if mode == "vertices":
        dropped = lib().oracle_voxelize_vertices(_p(v), _p(t), v.shape[0], C.byref(bounds), w, h, d, index_mode,
                                                 _p(counts), _p(dens), _p(tq))
    else:
        idx = np.ascontiguousarray(indices, dtype=np.uint32)
        dropped = lib().oracle_voxelize_segments(_p(v), _p(t), _p(idx), idx.shape[0], C.byref(bounds), w, h, d,
                                                 index_mode, _p(counts), _p(dens), _p(tq))
    return counts, dens, tq, int(dropped)


def segment_visits(vertices, indices, bounds, res):
    v = _f32(vertices)
    idx = np.ascontiguousarray(indices, dtype=np.uint32)
    w, h, d = (int(x) for x in res)
    return np.array([lib().oracle_segment_visits(_p(v), _p(idx), p, C.byref(bounds), w, h, d)
                     for p in range(idx.shape[0] // 2)], dtype=np.int64)


def normalize(densities):
    d = np.ascontiguousarray(densities, dtype=np.uint8).copy()
    lib().oracle_normalize(_p(d), d.size)
    return d


def downsample(densities, res, filt):
    w, h, d = (int(x) for x in res)
    src = np.ascontiguousarray(densities, dtype=np.uint8)
    out = np.zeros((w // 2) * (h // 2) * (d // 2), dtype=np.uint8)
    lib().oracle_downsample(_p(src), w, h, d, int(filt), _p(out))
    return out


# ---- raymarch ----------------------------------------------------------------

def raymarch(params, density, tangent, depth_in=None, precision="f64", rows=None, threads=0, diag=False):
    """Returns (rgba (H, W, 4) f32, depth (H, W) f32[, diag]) for rows [r0, r1)."""
    W, H = params.width, params.height
    r0, r1 = (0, H) if rows is None else rows
    rgba = np.zeros((H, W, 4), dtype=np.float32)
    depth = np.ones((H, W), dtype=np.float32)
    dens = np.ascontiguousarray(density)
    tan = np.ascontiguousarray(tangent)
    din = None if depth_in is None else _f32(depth_in)
    if precision == "f64":
        dg = np.zeros((H, W), dtype=DIAG_DTYPE) if diag else None
        lib().oracle_raymarch_f64(C.byref(params), _p(dens), _p(tan), _p(din), _p(rgba), _p(depth), _p(dg), r0, r1,
                                  threads)
        return (rgba, depth, dg) if diag else (rgba, depth)
    lib().oracle_raymarch_f32(C.byref(params), _p(dens), _p(tan), _p(din), _p(rgba), _p(depth), r0, r1, threads)
    return rgba, depth


# ---- differentiable path (FP64) ------------------------------------------------

def diff_loss(params, density, tangent, target, grads=False, threads=0, mask=None):
    """Loss sum((rgba - target)^2) of the FP64 differentiable raymarch over
    the pixels where mask (H, W) is true (None: all); with grads=True also
    (g_density, g_tangent (n, 4), g_params [kd, exponent, exponent2]).  density (n,)
    and tangent (n, 4) are converted to float64."""
    d = np.ascontiguousarray(density, dtype=np.float64).reshape(-1)
    t = np.ascontiguousarray(tangent, dtype=np.float64).reshape(-1, 4)
    tg = _f32(target)
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    if not grads:
        return float(lib().oracle_diff_loss(C.byref(params), _p(d), _p(t), _p(tg), _p(m), None, None, None, threads))
    gd = np.zeros_like(d)
    gt = np.zeros_like(t)
    gp = np.zeros(3, dtype=np.float64)
    loss = lib().oracle_diff_loss(C.byref(params), _p(d), _p(t), _p(tg), _p(m), _p(gd), _p(gt), _p(gp), threads)
    return float(loss), gd, gt, gp


def splat(vertices, bounds, res):
    v = _f32(vertices)
    w, h, d = (int(x) for x in res)
    out = np.zeros(w * h * d, dtype=np.float64)
    lib().oracle_splat(_p(v), v.shape[0], C.byref(bounds), w, h, d, _p(out))
    return out


def splat_adjoint(vertices, bounds, res, g_density):
    v = _f32(vertices)
    w, h, d = (int(x) for x in res)
    g = np.ascontiguousarray(g_density, dtype=np.float64)
    out = np.zeros((v.shape[0], 3), dtype=np.float64)
    lib().oracle_splat_adjoint(_p(v), v.shape[0], C.byref(bounds), w, h, d, _p(g), _p(out))
    return out


def max_threads():
    return int(lib().oracle_max_threads())


# ---- the reference's own code (built here only) -----------------------------

def ref_prepare(vertices, segments):
    v = _f32(vertices)
    s = np.ascontiguousarray(segments, dtype=np.uint16)
    t = np.zeros_like(v)
    idx = np.zeros(2 * int(s.astype(np.int64).sum()), dtype=np.uint32)
    b = _abi.AABB()
    ref().ref_prepare(_p(v), v.shape[0], _p(s), s.shape[0], _p(t), _p(idx), C.byref(b))
    return t, idx, b


def ref_voxelize(mode, vertices, tangents, indices, res, normalize=False):
    w, h, d = (int(x) for x in res)
    n = w * h * d
    v = _f32(vertices)
    t = _f32(tangents)
    idx = np.ascontiguousarray(indices if indices is not None else np.zeros(0), dtype=np.uint32)
    dens = np.zeros(n, dtype=np.uint8)
    tq = np.zeros((n, 4), dtype=np.int8)
    ref().ref_voxelize(1 if mode == "segments" else 0, _p(v), v.shape[0], _p(t), _p(idx), idx.shape[0], w, h, d,
                       1 if normalize else 0, _p(dens), _p(tq))
    return dens, tq


def ref_downsample(densities, res, filt):
    w, h, d = (int(x) for x in res)
    src = np.ascontiguousarray(densities, dtype=np.uint8)
    out = np.zeros((w // 2) * (h // 2) * (d // 2), dtype=np.uint8)
    ref().ref_downsample(_p(src), w, h, d, int(filt), _p(out))
    return out


def ref_raymarch(params, density, tangent, depth_in=None, rows=None, threads=0):
    W, H = params.width, params.height
    r0, r1 = (0, H) if rows is None else rows
    rgba = np.zeros((H, W, 4), dtype=np.float32)
    depth = np.ones((H, W), dtype=np.float32)
    dens = np.ascontiguousarray(density)
    tan = np.ascontiguousarray(tangent)
    din = None if depth_in is None else _f32(depth_in)
    rc = ref().ref_raymarch(C.byref(params), _p(dens), _p(tan), _p(din), _p(rgba), _p(depth), r0, r1, threads)
    if rc != 0:
        raise ValueError("the reference shader supports reference semantics only (shadow_steps <= 0, kd == 1)")
    return rgba, depth


# ---- compositing -------------------------------------------------------------

def _frags(fragments):
    return np.ascontiguousarray(fragments, dtype=_abi.FRAGMENT_DTYPE)


def _volume(volume_rgba, volume_depth):
    if volume_rgba is None:
        return None, None
    return _f32(volume_rgba), _f32(volume_depth)


def pack_unorm8x4(rgba):
    v = _f32(rgba)
    return int(lib().oracle_pack_unorm8x4(_p(v)))


def resolve_ppll(heads, nodes, color, threads=0):
    """resolve.comp over a PPLL (restatement): returns (status, new colour image)."""
    out = np.array(color, dtype=np.uint32, copy=True)
    h = np.ascontiguousarray(heads, dtype=np.uint32)
    n = np.ascontiguousarray(nodes, dtype=_abi.PPLL_NODE_DTYPE)
    H, W = out.shape
    rc = lib().oracle_resolve_ppll(_p(h), _p(n), len(n), W, H, _p(out), threads)
    return rc, out


def composite(fragments, color, volume_rgba=None, volume_depth=None, threads=0):
    """The PPLL-free composite (restatement): the new colour image; ValueError
    when a fragment's pixel is outside the image."""
    out = np.array(color, dtype=np.uint32, copy=True)
    f = _frags(fragments)
    vr, vd = _volume(volume_rgba, volume_depth)
    H, W = out.shape
    rc = lib().oracle_composite(_p(f), len(f), _p(vr), _p(vd), W, H, _p(out), threads)
    if rc != 0:
        raise ValueError("fragment pixel outside the image" if rc == -1 else "out of memory")
    return out


def ref_build_ppll(fragments, width, height, volume_rgba=None, volume_depth=None, capacity=None):
    """The reference's ppll.glsl appends (strand fragments in buffer order, then
    the volume fragments): (heads, nodes, node counter)."""
    f = _frags(fragments)
    vr, vd = _volume(volume_rgba, volume_depth)
    if capacity is None:
        capacity = len(f) + width * height
    heads = np.zeros((height, width), dtype=np.uint32)
    nodes = np.zeros(capacity + 1, dtype=_abi.PPLL_NODE_DTYPE)
    used = ref().ref_build_ppll(_p(f), len(f), _p(vr), _p(vd), width, height, capacity, _p(heads), _p(nodes))
    return heads, nodes, int(used)


def ref_resolve_ppll(heads, nodes, color, threads=0):
    """The reference's resolve.comp (compiled as C++) over a PPLL: the new colour image."""
    out = np.array(color, dtype=np.uint32, copy=True)
    h = np.ascontiguousarray(heads, dtype=np.uint32)
    n = np.ascontiguousarray(nodes, dtype=_abi.PPLL_NODE_DTYPE)
    H, W = out.shape
    ref().ref_resolve_ppll(_p(h), _p(n), len(n), W, H, _p(out), threads)
    return out
