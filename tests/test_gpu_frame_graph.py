"""Per-frame voxelization feeding the raymarcher as one CUDA graph
(vkhr_frame_graph_*), the per-frame path of rasterizer.cc:216-230 +
volume.cc:104-112: after the caller rewrites the vertices and tangents in
place (a hair simulation step), each replay equals the oracle's
voxelization (bit-exact counts, u8 and int8 tangents), Volume::normalize and
raymarch (FP32 vs FP64 tolerance, as tests/test_gpu_raymarch.py) of that
frame's strands."""
import numpy as np
import pytest

from vkhr_gb300 import _abi, scene, strands
from tests._helpers import ill_conditioned, image_errors, style, to_dev

pytestmark = pytest.mark.gpu

RMS_TOL = 1e-3
MAX_TOL = 2e-2


def _sway(st, frames):
    """The strands swaying along x, more at the tips: one vertex set per frame."""
    y = st.vertices[:, 1].astype(np.float64)
    h = (y - y.min()) / max(float(y.max() - y.min()), 1e-6)
    out = []
    for f in range(frames):
        v = st.vertices.astype(np.float64).copy()
        v[:, 0] += 0.03 * f * h * h
        out.append(v.astype(np.float32))
    return out


@pytest.mark.parametrize("budget", [0, 200_000])
def test_frame_graph_follows_moving_strands(native_lib, oracle_lib, budget):
    import torch

    from vkhr_gb300 import _native

    res = (64, 64, 64)
    n = res[0] * res[1] * res[2]
    W, H = 160, 120
    st, _, idx = style("hemi", 3000, 12)
    frames = _sway(st, 3)
    lo = np.min([v.min(axis=0) for v in frames], axis=0)
    hi = np.max([v.max(axis=0) for v in frames], axis=0)
    b = _abi.aabb_from(lo, hi - lo)  # fixed bounds holding every frame

    dv = to_dev(frames[0], torch)
    dt = to_dev(strands.generate_tangents(frames[0], st.segments), torch)
    di = to_dev(np.asarray(idx, dtype=np.uint32), torch)
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    dens = torch.zeros(n, dtype=torch.uint8, device="cuda")
    tq = torch.zeros((n, 4), dtype=torch.int8, device="cuda")
    rgba = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    depth = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    job = _abi.VoxelJob()
    job.d_vertices, job.d_tangent_in, job.d_indices = dv.data_ptr(), dt.data_ptr(), di.data_ptr()
    job.item_count = len(idx)
    job.bounds = b
    job.width, job.height, job.depth = res
    job.index_mode = _abi.INDEX_REF_FP32
    job.d_counts, job.d_densities, job.d_tangents = counts.data_ptr(), dens.data_ptr(), tq.data_ptr()
    p = scene.make_params(b, res, W, H, raycast_steps=128.0, shadow_steps=32.0, view_direction=(0.3, 0.2, 1.0))

    ctx = _native.Context(0)
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    try:
        graph = ctx.frame_graph(True, job, p, rgba.data_ptr(), depth.data_ptr(), visit_budget=budget, stream=s)
        launches = ctx.launch_count()
        for f, v in enumerate(frames):
            t = strands.generate_tangents(v, st.segments)
            dv.copy_(torch.from_numpy(v))  # the simulation's step, in place
            dt.copy_(torch.from_numpy(t))
            graph.launch(s)
            torch.cuda.synchronize()
            ctx.check_status(s)
            c_ref, d_ref, t_ref, _ = oracle_lib.voxelize("segments", v, t, idx, b, res)
            assert np.array_equal(counts.cpu().numpy().view(np.uint32), c_ref), f
            dn = oracle_lib.normalize(d_ref)
            assert np.array_equal(dens.cpu().numpy(), dn), f
            assert np.array_equal(tq.cpu().numpy(), t_ref), f
            ref, rdepth, diag = oracle_lib.raymarch(p, dn, t_ref, diag=True)
            rms, mx, excluded, emitted = image_errors(rgba.cpu().numpy(), ref, diag)
            assert emitted > 0 and excluded <= max(2, 0.01 * emitted), (f, excluded, emitted)
            assert np.all(rms <= RMS_TOL) and np.all(mx <= MAX_TOL), (f, rms, mx)
            ok = ~ill_conditioned(ref, diag)
            assert np.all(np.abs(depth.cpu().numpy() - rdepth)[ok] <= 1e-4), f
        assert ctx.launch_count() == launches  # replays launch no kernel through the context
        graph.close()
    finally:
        ctx.close()


def test_live_frame_graph_keeps_scratch_in_place(native_lib, oracle_lib):
    """A frame graph holds the addresses of its context's scratch: while it
    exists, a call on that context that would have to grow a scratch buffer
    (here the raymarch's occupancy bitmap, for a larger grid) fails with
    VKHR_ERR_CAPACITY instead of moving it, and the graph still renders the
    frame it captured; once the graph is destroyed the call succeeds."""
    import torch

    from vkhr_gb300 import _native
    from vkhr_gb300._native import VkhrError

    res = (32, 32, 32)
    n = res[0] * res[1] * res[2]
    W, H = 96, 72
    st, t, idx = style("hemi", 1500, 10)
    b = oracle_lib.bounding_box(st.vertices)
    dv, dt = to_dev(st.vertices, torch), to_dev(t, torch)
    di = to_dev(np.asarray(idx, dtype=np.uint32), torch)
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    dens = torch.zeros(n, dtype=torch.uint8, device="cuda")
    tq = torch.zeros((n, 4), dtype=torch.int8, device="cuda")
    rgba = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    job = _abi.VoxelJob()
    job.d_vertices, job.d_tangent_in, job.d_indices = dv.data_ptr(), dt.data_ptr(), di.data_ptr()
    job.item_count = len(idx)
    job.bounds = b
    job.width, job.height, job.depth = res
    job.index_mode = _abi.INDEX_REF_FP32
    job.d_counts, job.d_densities, job.d_tangents = counts.data_ptr(), dens.data_ptr(), tq.data_ptr()
    p = scene.make_params(b, res, W, H, raycast_steps=128.0, shadow_steps=32.0)
    # a larger grid the context has not raymarched yet
    big = (264, 264, 264)  # more occupancy bricks than the scratch the graph holds (grown with headroom)
    pb = scene.make_params(b, big, W, H, raycast_steps=64.0)
    bd = torch.zeros(big[0] * big[1] * big[2], dtype=torch.uint8, device="cuda")
    bt = torch.zeros((big[0] * big[1] * big[2], 4), dtype=torch.int8, device="cuda")
    out = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    ctx = _native.Context(0)
    s = torch.cuda.current_stream().cuda_stream
    try:
        graph = ctx.frame_graph(True, job, p, rgba.data_ptr(), None, stream=s)
        with pytest.raises(VkhrError) as e:
            ctx.raymarch(pb, bd.data_ptr(), bt.data_ptr(), None, out.data_ptr(), None, s)
        assert e.value.status == _abi.VKHR_ERR_CAPACITY
        rgba.zero_()
        graph.launch(s)
        torch.cuda.synchronize()
        ctx.check_status(s)
        c_ref, d_ref, t_ref, _ = oracle_lib.voxelize("segments", st.vertices, t, idx, b, res)
        assert np.array_equal(counts.cpu().numpy().view(np.uint32), c_ref)
        assert (rgba[..., 3] > 0).sum().item() > 50
        graph.close()
        ctx.raymarch(pb, bd.data_ptr(), bt.data_ptr(), None, out.data_ptr(), None, s)  # may grow now
        torch.cuda.synchronize()
    finally:
        ctx.close()
