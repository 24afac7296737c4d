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


def ill_conditioned(ref, diag, margin=1e-4, support=2e-4, tangent_floor=1e-4, shift_factor=0.5):
    """Pixels whose shader result hinges on a decision FP32 cannot resolve:
    the isosurface test within `margin` (relative) of the threshold, or
    within `shift_factor` times the view's FP32 position resolution (in
    texels) of flipping when the samples move (iso_shift: the margin over
    the accumulated density slope); a `density != 0` test on a sample whose
    nonzero taps carry less than `support` trilinear weight (or less than one
    position resolution); or a surface tangent shorter than `tangent_floor`
    (normalisation amplifies rounding).  The FP32 position resolution
    (fp32_res) grows with the camera's distance and the grid's resolution."""
    emitted = ref[..., 3] > 0
    res = diag["fp32_res"]
    return ((diag["iso_margin"] < margin) | (diag["support_margin"] < np.maximum(support, res))
            | (diag["iso_shift"] < shift_factor * res)
            | (emitted & (diag["tangent_len"] < tangent_floor) & (diag["tangent_len"] > 0)))


RMS_TOL = 1e-3  # per channel, over well-conditioned pixels
MAX_TOL = 2e-2


def compare_images(gpu, gdepth, ref, rdepth, diag, label="", depth_tol=1e-4, max_excluded=0.01):
    """The raymarch parity bar: per channel RMS <= 1e-3 and max <= 2e-2 over
    well-conditioned pixels, at most `max_excluded` of the emitted fragments
    excluded (1% of a frame; a test over many views or row bands allows 3%
    in one of them and checks 1% over all of them), and every
    well-conditioned depth within `depth_tol`.  Prints the counts (pytest -s
    shows them); returns (rms, max, excluded, emitted)."""
    rms, mx, excluded, emitted = image_errors(gpu, ref, diag)
    print("%s: %d emitted fragments, %d excluded (%.3f%%), rms %s, max %s"
          % (label, emitted, excluded, 100.0 * excluded / max(emitted, 1), np.round(rms, 6).tolist(),
             np.round(mx, 5).tolist()))
    assert emitted > 0, label
    assert excluded <= max(2, max_excluded * emitted), (label, excluded, emitted)
    assert np.all(rms <= RMS_TOL), (label, rms)
    assert np.all(mx <= MAX_TOL), (label, mx)
    ok = ~ill_conditioned(ref, diag)
    dd = np.abs(gdepth - rdepth)
    bad = np.argwhere(ok & (dd > depth_tol))
    info = [(int(y), int(x), float(diag["iso_margin"][y, x]), float(diag["support_margin"][y, x]),
             float(diag["tangent_len"][y, x]), float(rdepth[y, x]), float(gdepth[y, x]), ref[y, x].tolist(),
             gpu[y, x].tolist()) for y, x in bad[:8]]
    assert len(bad) == 0, (label, len(bad), info)
    return rms, mx, excluded, emitted


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


# ---- compositing cases -----------------------------------------------------------
# Depths the k-buffer treats specially: 0 and below never count as "furthest"
# (resolve.comp:48-57 starts from 0), NaN compares false, 3e38 is the empty
# slots' depth, above it and +inf beat the empty slots.
SPECIAL_DEPTHS = np.array([0.0, -0.25, np.nan, np.inf, np.float32(3e38), np.float32(3.2e38), 0.5, 1.0],
                          dtype=np.float32)

# per-pixel fragment counts that reach every slice tier and both resolve
# phases (k-buffer only, tail, past the 1040 nodes a pixel resolves)
TIER_COUNTS = [0, 1, 2, 5, 8, 9, 16, 17, 32, 33, 100, 128, 129, 400, 512, 513, 1039, 1040, 1041, 2048, 2049, 3000]


def fragment_case(width, height, counts, seed, tie_levels=None, special_rate=0.02):
    """Strand fragments, counts[p] of them at pixel p, in a shuffled buffer
    order; random RGBA8 colours; depths in [0, 1), rounded to tie_levels
    levels when given (so that equal depths occur), a few special values."""
    rng = np.random.default_rng(seed)
    counts = np.asarray(counts, dtype=np.int64)
    assert counts.size == width * height
    pix = np.repeat(np.arange(width * height, dtype=np.uint32), counts)
    rng.shuffle(pix)
    f = np.zeros(len(pix), dtype=_abi.FRAGMENT_DTYPE)
    f["pixel"] = pix
    f["color"] = rng.integers(0, 1 << 32, len(pix), dtype=np.uint64).astype(np.uint32)
    d = rng.random(len(pix), dtype=np.float32)
    if tie_levels:
        d = (np.floor(d * tie_levels) / tie_levels).astype(np.float32)
    if special_rate and len(pix):
        sel = rng.random(len(pix)) < special_rate
        d[sel] = rng.choice(SPECIAL_DEPTHS, int(sel.sum()))
    f["depth"] = d
    return f


def volume_case(width, height, seed, coverage=0.5):
    """A raymarch-like volume image: RGBA a little outside [0, 1] (packing
    clamps), depth below 1 on about `coverage` of the pixels, 1 elsewhere,
    a few NaN depths (no fragment)."""
    rng = np.random.default_rng(seed)
    rgba = rng.uniform(-0.1, 1.1, (height, width, 4)).astype(np.float32)
    depth = rng.random((height, width), dtype=np.float32)
    depth[rng.random((height, width)) >= coverage] = 1.0
    depth[rng.random((height, width)) < 0.01] = np.nan
    return rgba, depth


def background_case(width, height, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 1 << 32, (height, width), dtype=np.uint64).astype(np.uint32)


def build_ppll(fragments, width, height, seed=None):
    """The PPLL that linking `fragments` in buffer order builds (each new node
    becomes its pixel's head, its `prev` the old head).  With a seed the nodes
    are stored in a shuffled order (node indices are arbitrary in a PPLL)."""
    n = len(fragments)
    pix = fragments["pixel"].astype(np.int64)
    slot = np.arange(n, dtype=np.int64)
    if seed is not None:
        slot = np.random.default_rng(seed).permutation(n)
    order = np.argsort(pix, kind="stable")
    prev = np.full(n, _abi.PPLL_NULL, dtype=np.uint32)
    same = pix[order][1:] == pix[order][:-1]
    prev[order[1:][same]] = slot[order[:-1][same]]
    nodes = np.zeros(n, dtype=_abi.PPLL_NODE_DTYPE)
    nodes["color"][slot] = fragments["color"]
    nodes["depth"][slot] = fragments["depth"]
    nodes["prev"][slot] = prev
    heads = np.full(width * height, _abi.PPLL_NULL, dtype=np.uint32)
    last = np.ones(n, dtype=bool)
    last[order[:-1][same]] = False
    heads[pix[last]] = slot[last]
    return heads.reshape(height, width), nodes
