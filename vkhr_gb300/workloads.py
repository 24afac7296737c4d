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


def strand_fragments(vertices, tangents, indices, params, lod, device):
    """Synthetic strand-rasterizer output for the compositing step, on the
    device: each segment projected with params' camera and sampled once per
    pixel step along its major screen axis (at most 64 samples), in segment
    order, like one-pixel lines rasterized in primitive order.  Colour: the
    hair colour lit by |tangent . light| (a stand-in for strand.frag's shading),
    coverage hair_alpha * (1 - lod) (strand.frag:39-42); depth is the clip-space
    z / w the rasterizer interpolates.  Samples outside the image or the depth
    range are dropped.  Returns a (fragment_count, 3) int32 tensor laid out as
    vkhr_fragment {color, depth bits, pixel}."""
    import torch

    W, H = params.width, params.height
    view = np.asarray(params.view, dtype=np.float64).reshape(4, 4).T
    proj = np.asarray(params.projection, dtype=np.float64).reshape(4, 4).T
    m = torch.as_tensor((proj @ view).astype(np.float32), device=device)
    v = torch.as_tensor(np.ascontiguousarray(vertices, dtype=np.float32), device=device)
    clip = v @ m[:3, :3].T + m[:3, 3]
    w = v @ m[3, :3] + m[3, 3]
    sx = (clip[:, 0] / w * 0.5 + 0.5) * W
    sy = (clip[:, 1] / w * 0.5 + 0.5) * H
    sz = clip[:, 2] / w
    idx = torch.as_tensor(np.ascontiguousarray(indices).view(np.int32).astype(np.int64), device=device)
    a, b = idx[0::2], idx[1::2]
    length = torch.maximum((sx[b] - sx[a]).abs(), (sy[b] - sy[a]).abs())
    n = torch.clamp(torch.ceil(length), 1, 64).to(torch.int64)
    seg = torch.repeat_interleave(torch.arange(len(a), device=device), n)
    first = torch.cumsum(n, 0) - n
    k = torch.arange(len(seg), device=device) - first[seg]
    t = (k.to(torch.float32) + 0.5) / n[seg].to(torch.float32)
    x = sx[a[seg]] + t * (sx[b[seg]] - sx[a[seg]])
    y = sy[a[seg]] + t * (sy[b[seg]] - sy[a[seg]])
    z = sz[a[seg]] + t * (sz[b[seg]] - sz[a[seg]])
    keep = (x >= 0) & (x < W) & (y >= 0) & (y < H) & (z >= 0) & (z <= 1)
    seg, x, y, z = seg[keep], x[keep], y[keep], z[keep]
    tan = torch.as_tensor(np.ascontiguousarray(tangents, dtype=np.float32), device=device)[a[seg]]
    ld = np.asarray(params.light_origin, dtype=np.float64) - np.asarray(params.camera_position, dtype=np.float64)
    ld = torch.as_tensor((ld / np.linalg.norm(ld)).astype(np.float32), device=device)
    shade = 0.35 + 0.65 * (tan @ ld).abs()
    hc = torch.as_tensor(np.asarray(params.hair_color, dtype=np.float32), device=device)
    rgb = torch.clamp(hc[None, :] * shade[:, None] * 2.0, 0, 1)
    alpha = torch.full_like(shade, float(params.hair_alpha) * (1.0 - float(lod)))
    q = torch.round(torch.cat([rgb, alpha[:, None]], 1) * 255.0).to(torch.int64)
    color = q[:, 0] | (q[:, 1] << 8) | (q[:, 2] << 16) | (q[:, 3] << 24)
    out = torch.empty((len(seg), 3), dtype=torch.int32, device=device)
    out[:, 0] = (color - ((color >> 31) << 32)).to(torch.int32)
    out[:, 1] = z.contiguous().view(torch.int32)
    out[:, 2] = (y.to(torch.int64) * W + x.to(torch.int64)).to(torch.int32)
    return out
