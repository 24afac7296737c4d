"""Synthetic workloads of the path, grown procedurally (the reference's TressFX
assets are not available).

`batched_specs` draws the multi-style batch: 16 independent styles whose
strand counts are log-uniform in [5k, 136k], vertices per strand uniform in
8..32, grid resolution from {64, 128, 192, 256}^3, each seen in its own
3840x2160 view from the distance that gives it a screen footprint between
64 and 1024 pixels across (log-uniform).
"""
import numpy as np

from . import strands

BATCH_TARGET = (3840, 2160)


def batched_specs(n=16, seed=2, strand_range=(5_000, 136_000), vertex_range=(8, 32),
                  resolutions=(64, 128, 192, 256), footprint_range=(64.0, 1024.0)):
    rng = np.random.default_rng(seed)
    specs = []
    for j in range(n):
        s = int(round(np.exp(rng.uniform(np.log(strand_range[0]), np.log(strand_range[1])))))
        v = int(rng.integers(vertex_range[0], vertex_range[1] + 1))
        r = int(resolutions[int(rng.integers(len(resolutions)))])
        f = float(np.exp(rng.uniform(np.log(footprint_range[0]), np.log(footprint_range[1]))))
        az, el = rng.uniform(0.0, 2.0 * np.pi), rng.uniform(-0.3, 1.0)
        vd = (float(np.cos(az) * np.cos(el)), float(np.sin(el)), float(np.sin(az) * np.cos(el)))
        specs.append({"kind": "hemisphere" if j % 2 == 0 else "disk", "strands": s, "vertices_per_strand": v,
                      "resolution": r, "footprint": f, "view_direction": vd, "seed": 100 + j})
    return specs


def grow(spec):
    """(StrandSet, tangents, indices) of one spec: hemisphere styles grow as
    the 4,096 x 16 small case (step 0.05), disk styles as the ponytail
    bundle (0.3-radius disk tilted 30 degrees, step 0.08)."""
    gen = strands.hemisphere_style if spec["kind"] == "hemisphere" else strands.disk_style
    st = gen(spec["strands"], spec["vertices_per_strand"], seed=spec["seed"])
    return st, strands.generate_tangents(st.vertices, st.segments), strands.generate_indices(st.segments)


def camera_distance(bounds, footprint_px, height, fov_degrees=45.0):
    """Distance at which the AABB's bounding sphere spans `footprint_px`
    pixels of a `height`-pixel view (perspective, vertical fov)."""
    r = 0.5 * float(bounds.radius)  # vkhr::AABB radius is the full diagonal
    a = np.arctan(footprint_px / float(height) * np.tan(np.deg2rad(fov_degrees) * 0.5))
    return float(r / np.sin(a))


def shelf_pack(rects, width):
    """Atlas positions (x, y) for regions of sizes (w, h), packed in rows of
    `width` pixels tallest first; returns (positions, atlas height)."""
    order = sorted(range(len(rects)), key=lambda i: -rects[i][1])
    pos = [None] * len(rects)
    x = y = row_h = 0
    for i in order:
        w, h = rects[i]
        if x + w > width:
            x, y, row_h = 0, y + row_h, 0
        pos[i] = (x, y)
        x += w
        row_h = max(row_h, h)
    return pos, y + row_h


def sway(vertices, amount):
    """One step of simulated motion: the strands swayed along x by `amount`
    (world units) times the square of each vertex's relative height."""
    import numpy as np

    v = np.asarray(vertices, dtype=np.float64)
    y = v[:, 1]
    h = (y - y.min()) / max(float(y.max() - y.min()), 1e-6)
    out = v.copy()
    out[:, 0] += amount * h * h
    return out.astype(np.float32)
