"""Procedurally grown synthetic hair styles (seeded, deterministic per platform).

The reference's TressFX styles (ponytail: 136,320 strands, 1,772,160
vertices; bear: 961,280 strands) are Git-LFS objects that are not available,
so every workload here is grown from these generators instead.  A style is
returned in the reference's in-memory layout (vkhr::HairStyle,
include/vkhr/scene_graph/hair_style.hh:126-139): `segments` (uint16 per
strand), `vertices` (float32 x3 per vertex, strands back to back).

Growth model: a strand starts at its root with direction = the surface normal
n; each step adds (0, -gravity, 0) and isotropic Gaussian "curl" noise of
standard deviation `curl` to the direction, renormalises it, and advances the
point by `step_length`.
"""
from dataclasses import dataclass

import numpy as np


@dataclass
class StrandSet:
    vertices: np.ndarray  # (V, 3) float32
    segments: np.ndarray  # (S,) uint16, segments per strand

    @property
    def strand_count(self):
        return int(self.segments.shape[0])

    @property
    def vertex_count(self):
        return int(self.vertices.shape[0])

    @property
    def segment_count(self):
        return int(self.segments.astype(np.int64).sum())


def _grow(roots, normals, steps, step_length, gravity, curl, rng):
    s = roots.shape[0]
    pts = np.empty((s, steps + 1, 3), dtype=np.float64)
    pts[:, 0] = roots
    d = normals.copy()
    g = np.array([0.0, -gravity, 0.0])
    for k in range(steps):
        d = d + g + rng.normal(0.0, curl, size=(s, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        pts[:, k + 1] = pts[:, k] + step_length * d
    return pts


def hemisphere_style(strands, vertices_per_strand, radius=1.0, step_length=0.05, gravity=0.3, curl=0.02, seed=0):
    """Roots uniform on the upper (+y) hemisphere of a sphere, grown outward.

    Default arguments give the 4,096 x 16 small case when called with
    (4096, 16); (1_048_576, 32, radius=1.2, step_length=0.04) gives the
    33.5M-vertex scale case.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    y = rng.uniform(0.0, 1.0, strands)
    phi = rng.uniform(0.0, 2.0 * np.pi, strands)
    r = np.sqrt(np.maximum(0.0, 1.0 - y * y))
    n = np.stack([r * np.cos(phi), y, r * np.sin(phi)], axis=1)
    pts = _grow(radius * n, n, vertices_per_strand - 1, step_length, gravity, curl, rng)
    return StrandSet(
        vertices=pts.reshape(-1, 3).astype(np.float32),
        segments=np.full(strands, vertices_per_strand - 1, dtype=np.uint16),
    )


def disk_style(strands, vertices_per_strand, disk_radius=0.3, tilt_degrees=30.0, step_length=0.08, gravity=0.3,
               curl=0.02, seed=0):
    """Roots uniform on a disk tilted about the x axis (a ponytail-like bundle).

    (136_320, 13) gives the production case: 1,772,160 vertices and
    1,635,840 segments, the sizes of the reference's ponytail.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    t = np.deg2rad(tilt_degrees)
    m = np.array([0.0, np.cos(t), np.sin(t)])
    e1 = np.array([1.0, 0.0, 0.0])
    e2 = np.cross(m, e1)
    rr = disk_radius * np.sqrt(rng.uniform(0.0, 1.0, strands))
    phi = rng.uniform(0.0, 2.0 * np.pi, strands)
    roots = (rr * np.cos(phi))[:, None] * e1 + (rr * np.sin(phi))[:, None] * e2
    normals = np.broadcast_to(m, roots.shape).copy()
    pts = _grow(roots, normals, vertices_per_strand - 1, step_length, gravity, curl, rng)
    return StrandSet(
        vertices=pts.reshape(-1, 3).astype(np.float32),
        segments=np.full(strands, vertices_per_strand - 1, dtype=np.uint16),
    )


def ragged_style(strand_counts_segments, seed=0, radius=1.0, step_length=0.05, gravity=0.3, curl=0.02):
    """Strands of uneven length (one entry of `strand_counts_segments` per
    strand, >= 0 segments each), roots on the upper hemisphere."""
    rng = np.random.Generator(np.random.PCG64(seed))
    segs = np.asarray(strand_counts_segments, dtype=np.int64)
    verts = []
    for k in segs:
        y = rng.uniform(0.0, 1.0)
        phi = rng.uniform(0.0, 2.0 * np.pi)
        r = np.sqrt(max(0.0, 1.0 - y * y))
        n = np.array([[r * np.cos(phi), y, r * np.sin(phi)]])
        verts.append(_grow(radius * n, n, int(k), step_length, gravity, curl, rng)[0])
    v = np.concatenate(verts, axis=0) if verts else np.zeros((0, 3))
    return StrandSet(vertices=v.astype(np.float32), segments=segs.astype(np.uint16))


def generate_indices(segments):
    """HairStyle::generate_indices (hair_style.cc:196-213), vectorised."""
    segs = np.asarray(segments, dtype=np.int64)
    starts = np.concatenate([[0], np.cumsum(segs + 1)[:-1]]) if segs.size else np.zeros(0, np.int64)
    total = int(segs.sum())
    if total == 0:
        return np.zeros(0, dtype=np.uint32)
    strand_of = np.repeat(np.arange(segs.size), segs)
    within = np.arange(total) - np.repeat(np.cumsum(segs) - segs, segs)
    first = starts[strand_of] + within
    out = np.empty(2 * total, dtype=np.uint32)
    out[0::2] = first
    out[1::2] = first + 1
    return out


def generate_tangents(vertices, segments):
    """HairStyle::generate_tangents (hair_style.cc:171-194) in FP32, with
    glm::normalize(v) = v * (1 / sqrt(dot(v, v))), dot = (x*x + y*y) + z*z."""
    v = np.asarray(vertices, dtype=np.float32)
    segs = np.asarray(segments, dtype=np.int64)
    out = np.zeros_like(v)
    starts = np.concatenate([[0], np.cumsum(segs + 1)[:-1]]) if segs.size else np.zeros(0, np.int64)
    idx = generate_indices(segs).astype(np.int64)
    a = idx[0::2]
    d = (v[a + 1] - v[a]).astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        dot = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(np.float32) + (d[:, 2] * d[:, 2]).astype(np.float32)
        inv = (np.float32(1.0) / np.sqrt(dot.astype(np.float32))).astype(np.float32)
        out[a] = d * inv[:, None]
    # the strand's last vertex repeats the previous tangent (or the previous
    # strand's last tangent for a strand without segments)
    last = starts + segs
    has = segs > 0
    out[last[has]] = out[last[has] - 1]
    for s in np.nonzero(~has)[0]:
        out[last[s]] = out[last[s] - 1] if last[s] > 0 else 0.0
    return out
