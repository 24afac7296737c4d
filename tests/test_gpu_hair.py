"""`.hair` files into device memory (vkhr_hair_load) and strand reduction on
device strands (vkhr_reduce_strands), through the C ABI, against the oracle
(oracle/hair.py, pinned to the reference's HairStyle::load / save / reduce by
tests/test_oracle_hair.py) and the reference-made fixtures of tests/golden:
bit-exact arrays, seeds and segment counts; and a reduced style voxelized on
the GPU equals the oracle's voxelization of the oracle-reduced style."""
import os

import numpy as np
import pytest

from oracle import hair as H
from vkhr_gb300 import _abi, strands
from tests._helpers import gpu_voxelize, style, to_dev

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(ctx, path, n_vertices, n_indices):
    import torch

    dv = torch.full((n_vertices, 3), -9.0, dtype=torch.float32, device="cuda")
    dt = torch.full((n_vertices, 3), -9.0, dtype=torch.float32, device="cuda")
    di = torch.zeros(max(n_indices, 1), dtype=torch.int32, device="cuda")
    hdr, segs = ctx.hair_load(path, dv.data_ptr(), dt.data_ptr(), di.data_ptr(),
                              stream=torch.cuda.current_stream().cuda_stream)
    return hdr, segs, dv.cpu().numpy(), dt.cpu().numpy(), di.cpu().numpy().view(np.uint32)[:n_indices]


def test_hair_load_every_field(ctx, tmp_path):
    st, t, idx = style("disk", 3000, 11)
    segs = st.segments.astype(np.uint16)
    nv = len(st.vertices)
    thick = np.linspace(0, 1, nv, dtype=np.float32)
    col = np.tile(np.float32([0.1, 0.2, 0.3]), (nv, 1))
    path = str(tmp_path / "style.hair")
    H.write_hair(path, st.vertices, segs, tangents=t, indices=idx, thickness=thick, transparency=thick, color=col,
                 information=b"synthetic")
    ref = H.read_hair(path)
    hdr, s, v, tt, ii = _load(ctx, path, nv, len(idx))
    assert (hdr.strand_count, hdr.vertex_count, hdr.fields) == (len(segs), nv, 0x7F)
    assert np.array_equal(s, ref["segments"]) and np.array_equal(v, ref["vertices"])
    assert np.array_equal(tt, ref["tangents"]) and np.array_equal(ii, ref["indices"])


def test_hair_load_reference_saved_file(ctx):
    """A file the reference's HairStyle::save wrote (tests/golden)."""
    g = np.load(os.path.join(GOLDEN, "reduce_hemisphere.npz"))
    path = os.path.join(GOLDEN, "reduce_hemisphere.hair")
    hdr, s, v, tt, _ = _load(ctx, path, len(g["vertices"]), 0)
    assert hdr.fields == (1 | 2 | 32)
    assert np.array_equal(s, g["segments"]) and np.array_equal(v, g["vertices"]) and np.array_equal(tt, g["tangents"])


def test_hair_load_errors(ctx, tmp_path):
    from vkhr_gb300 import _native

    st, t, _ = style("hemi", 100, 6)
    path = str(tmp_path / "cut.hair")
    H.write_hair(path, st.vertices, st.segments.astype(np.uint16), tangents=t)
    data = open(path, "rb").read()
    open(path, "wb").write(data[:128 + 2 * 100 + 12 * 50])  # cut inside the vertices
    with pytest.raises(_native.VkhrError, match="ReadingVertices"):
        _load(ctx, path, len(st.vertices), 0)
    with pytest.raises(_native.VkhrError):
        ctx.hair_load(str(tmp_path / "missing.hair"), None)


@pytest.mark.parametrize("ratio", [1.0, 0.5, 0.984375, 0.015625])
def test_reduce_strands_device(ctx, ratio):
    import torch

    st, t, _ = style("disk", 4000, 13)
    segs = st.segments.astype(np.uint16)
    dv, dt = to_dev(st.vertices, torch), to_dev(t, torch)
    ov = torch.zeros_like(dv)
    ot = torch.zeros_like(dt)
    seed = 0x2545F4914F6CDD1D
    kept, nv, sd = ctx.reduce_strands(ratio, seed, segs, len(segs), dv.data_ptr(), dt.data_ptr(), ov.data_ptr(),
                                      ot.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    v, tt, s, sdo = H.reduce(st.vertices, t, len(segs), ratio, seed, segs)
    assert sd == sdo and np.array_equal(kept, s) and nv == len(v)
    assert np.array_equal(ov.cpu().numpy()[:nv], v) and np.array_equal(ot.cpu().numpy()[:nv], tt)


def test_reduce_strands_reference_fixture(ctx):
    import torch

    g = np.load(os.path.join(GOLDEN, "reduce_hemisphere.npz"))
    dv, dt = to_dev(g["vertices"], torch), to_dev(g["tangents"], torch)
    for k, ratio in enumerate(g["ratios"]):
        ov, ot = torch.zeros_like(dv), torch.zeros_like(dt)
        kept, nv, sd = ctx.reduce_strands(float(ratio), int(g["seed"]), g["segments"], len(g["segments"]),
                                          dv.data_ptr(), dt.data_ptr(), ov.data_ptr(), ot.data_ptr())
        torch.cuda.synchronize()
        assert sd == int(g["r%d_seed" % k]) and np.array_equal(kept, g["r%d_segments" % k])
        assert np.array_equal(ov.cpu().numpy()[:nv], g["r%d_vertices" % k])
        assert np.array_equal(ot.cpu().numpy()[:nv], g["r%d_tangents" % k])


def test_reduced_style_voxelizes_like_the_oracle(ctx, oracle_lib):
    import torch

    st, t, _ = style("disk", 6000, 13)
    segs = st.segments.astype(np.uint16)
    dv, dt = to_dev(st.vertices, torch), to_dev(t, torch)
    ov, ot = torch.zeros_like(dv), torch.zeros_like(dt)
    kept, nv, _ = ctx.reduce_strands(0.6, 99, segs, len(segs), dv.data_ptr(), dt.data_ptr(), ov.data_ptr(),
                                     ot.data_ptr())
    v, tt, s, _ = H.reduce(st.vertices, t, len(segs), 0.6, 99, segs)
    idx = strands.generate_indices(s)
    b = oracle_lib.bounding_box(v)
    res = (48, 48, 48)
    c_ref, d_ref, t_ref, _ = oracle_lib.voxelize("segments", v, tt, idx, b, res)
    c, d, tq = gpu_voxelize(ctx, "segments", ov.cpu().numpy()[:nv], ot.cpu().numpy()[:nv], idx, b, res)
    assert np.array_equal(c, c_ref) and np.array_equal(d, d_ref) and np.array_equal(tq, t_ref)
