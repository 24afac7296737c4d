"""Shared helpers of the test-suite: device uploads and C-ABI calls."""
import numpy as np

from vkhr_gb300 import _abi, strands


def style(kind, strands_n, verts, seed=0, **kw):
    gen = strands.disk_style if kind == "disk" else strands.hemisphere_style
    st = gen(strands_n, verts, seed=seed, **kw)
    t = strands.generate_tangents(st.vertices, st.segments)
    idx = strands.generate_indices(st.segments)
    return st, t, idx


def to_dev(a, torch):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    return torch.from_numpy(a).cuda()


def gpu_voxelize(ctx, mode, vertices, tangents, indices, bounds, res, index_mode=_abi.INDEX_REF_FP32,
                 want_tangents=True, want_dens=True):
    import torch

    w, h, d = res
    n = w * h * d
    dv = to_dev(vertices, torch)
    dt = to_dev(tangents, torch) if tangents is not None else None
    counts = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    dens = torch.full((n,), 77, dtype=torch.uint8, device="cuda") if want_dens else None
    tq = torch.full((n, 4), 55, dtype=torch.int8, device="cuda") if want_tangents else None
    s = torch.cuda.current_stream().cuda_stream
    p = lambda t: None if t is None else t.data_ptr()
    if mode == "vertices":
        ctx.voxelize_vertices(p(dv), p(dt), int(np.asarray(vertices).shape[0]), bounds, res, index_mode, p(counts),
                              p(dens), p(tq), s)
    else:
        di = to_dev(np.asarray(indices, dtype=np.uint32), torch) if len(indices) else torch.zeros(2, dtype=torch.int32,
                                                                                                   device="cuda")
        ctx.voxelize_segments(p(dv), p(dt), p(di), int(len(indices)), bounds, res, index_mode, p(counts), p(dens),
                              p(tq), s)
    ctx.check_status(s)  # errors the kernels recorded on the device
    torch.cuda.synchronize()
    return (counts.cpu().numpy().view(np.uint32), None if dens is None else dens.cpu().numpy(),
            None if tq is None else tq.cpu().numpy())


def ill_conditioned(ref, diag, margin=1e-4, support=2e-4, tangent_floor=1e-4):
    """Pixels whose shader result hinges on a decision FP32 cannot resolve:
    the isosurface test within `margin` (relative) of the threshold, a
    `density != 0` test on a sample whose nonzero taps carry less than
    `support` trilinear weight (about FP32's position resolution in texels),
    or a surface tangent shorter than `tangent_floor` (normalisation
    amplifies rounding)."""
    emitted = ref[..., 3] > 0
    return ((diag["iso_margin"] < margin) | (diag["support_margin"] < support)
            | (emitted & (diag["tangent_len"] < tangent_floor) & (diag["tangent_len"] > 0)))


def image_errors(gpu, ref, diag, **kw):
    """Per-channel RMS and max over well-conditioned pixels, the excluded
    count and the emitted-fragment count."""
    emitted = ref[..., 3] > 0
    ill = ill_conditioned(ref, diag, **kw)
    ok = ~ill
    d = np.abs(gpu.astype(np.float64) - ref.astype(np.float64))
    rms = np.sqrt((d[ok] ** 2).mean(axis=0)) if ok.any() else np.zeros(4)
    mx = d[ok].max(axis=0) if ok.any() else np.zeros(4)
    return rms, mx, int(ill.sum()), int(emitted.sum())
