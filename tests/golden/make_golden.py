"""Generates the golden fixtures of tests/golden from the reference's own code.

Runs the reference's voxelizer (src/vkhr/scene_graph/hair_style.cc, compiled
unmodified into oracle/_ref by `make -C oracle ref`) and its raymarch shader
(share/shaders/volumes/volume.frag and includes, compiled as C++) on small
seeded synthetic styles, and its PPLL appends and resolve (ppll.glsl,
resolve.comp, compiled as C++) on seeded fragments, and stores inputs and
outputs as .npz files.
Needs the reference sources; run from the repository root:

    make -C oracle ref && python tests/golden/make_golden.py
    python tests/golden/make_golden.py reduce     # the strand-reduction fixtures only
    python tests/golden/make_golden.py composite  # the PPLL resolve fixture only
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from vkhr_gb300 import scene, strands  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def aabb_arr(b):
    return np.array(list(b.origin) + [b.radius] + list(b.size) + [b.volume], dtype=np.float32)


def voxel_case(name, st, resolutions):
    t, idx, b = O.ref_prepare(st.vertices, st.segments)
    out = {"vertices": st.vertices, "segments": st.segments, "tangents": t, "indices": idx, "aabb": aabb_arr(b)}
    for k, res in enumerate(resolutions):
        out["res%d" % k] = np.array(res, dtype=np.int32)
        for mode in ("vertices", "segments"):
            d, tq = O.ref_voxelize(mode, st.vertices, t, idx, res)
            dn, _ = O.ref_voxelize(mode, st.vertices, t, idx, res, normalize=True)
            out["%s%d_densities" % (mode, k)] = d
            out["%s%d_tangents" % (mode, k)] = tq
            out["%s%d_normalized" % (mode, k)] = dn
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)


def raymarch_case(name, st, res, W, H, **kw):
    t, idx, b = O.ref_prepare(st.vertices, st.segments)
    dn, tq = O.ref_voxelize("segments", st.vertices, t, idx, res, normalize=True)
    p = scene.make_params(b, res, W, H, **kw)
    rgba, depth = O.ref_raymarch(p, dn, tq)
    params = np.frombuffer(bytes(p), dtype=np.uint8)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), params=params, densities=dn, tangents=tq, rgba=rgba,
                        depth=depth)


def reduce_case(name, st, seed, ratios):
    """HairStyle::reduce (and its .hair saver) of the reference on a style
    with an even strand count: reduce's offset array copy writes one element
    past its end (hair_style.cc:392), which stays inside the allocation's
    slack for an even count."""
    assert len(st.segments) % 2 == 0
    t, idx, b = O.ref_prepare(st.vertices, st.segments)
    out = {"vertices": st.vertices, "segments": st.segments.astype(np.uint16), "tangents": t, "seed": np.uint64(seed),
           "ratios": np.array(ratios, dtype=np.float32)}
    for k, r in enumerate(ratios):
        v, tt, sg, sd = O.ref_reduce(st.vertices, t, st.segments, len(st.segments), float(r), seed)
        out["r%d_vertices" % k], out["r%d_tangents" % k], out["r%d_segments" % k] = v, tt, sg
        out["r%d_seed" % k] = np.uint64(sd)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)
    assert O.ref_hair_save(os.path.join(OUT, name + ".hair"), st.segments, st.vertices, t) == 0


def composite_case(name, width, height, counts, seed):
    """The reference's PPLL appends (ppll.glsl's ppll_next_node / node_data /
    link_node, strand fragments in buffer order, then the volume fragments)
    and its resolve.comp on that PPLL, both compiled as C++."""
    from tests._helpers import background_case, fragment_case, volume_case

    f = fragment_case(width, height, counts, seed, tie_levels=256)
    bg = background_case(width, height, seed + 1)
    vr, vd = volume_case(width, height, seed + 2)
    heads, nodes, used = O.ref_build_ppll(f, width, height, vr, vd)
    nodes = nodes[:used]
    color = O.ref_resolve_ppll(heads, nodes, bg)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), fragments=f, background=bg, volume_rgba=vr,
                        volume_depth=vd, heads=heads, nodes=nodes, color=color)


def main():
    if sys.argv[1:] == ["composite"]:  # only the compositing fixture
        from tests._helpers import TIER_COUNTS

        composite_case("composite_tiers", 11, 2, TIER_COUNTS, 21)
        return
    if sys.argv[1:] == ["reduce"]:  # only the strand-reduction fixtures
        reduce_case("reduce_hemisphere", strands.hemisphere_style(256, 8, seed=16), 0x9E3779B97F4A7C15,
                    [1.0, 0.5, 0.984375, 0.015625])
        return
    voxel_case("voxel_hemisphere", strands.hemisphere_style(256, 8, seed=11), [(16, 16, 16), (13, 9, 21)])
    voxel_case("voxel_ragged", strands.ragged_style([2, 0, 3, 9, 1, 17, 0, 5, 30, 2], seed=12), [(8, 8, 8), (20, 7, 11)])
    crowded = strands.disk_style(1500, 6, disk_radius=0.02, step_length=0.01, seed=13)
    voxel_case("voxel_crowded", crowded, [(4, 4, 4)])
    raymarch_case("raymarch_hemisphere", strands.hemisphere_style(512, 12, seed=14), (24, 24, 24), 64, 48,
                  raycast_steps=96.0)
    raymarch_case("raymarch_disk", strands.disk_style(2000, 9, seed=15), (32, 28, 20), 80, 60, raycast_steps=128.0,
                  view_direction=(0.3, 0.4, 1.0))
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
