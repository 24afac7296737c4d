"""GPU voxelizer parity: libvkhr_cuda.so (through the C ABI) against the oracle,
bit-exact on counts, u8 densities and int8 tangents
(hair_style.cc:257-342 semantics)."""
import numpy as np
import pytest

from vkhr_gb300 import _abi, strands
from tests._helpers import gpu_voxelize, style, to_dev

pytestmark = pytest.mark.gpu


def _check(ctx, O, mode, v, t, idx, b, res, index_mode=_abi.INDEX_REF_FP32):
    c_ref, d_ref, t_ref, dropped = O.voxelize(mode, v, t, idx, b, res, index_mode)
    c, d, tq = gpu_voxelize(ctx, mode, v, t, idx, b, res, index_mode)
    assert np.array_equal(c, c_ref), "counts differ in %d voxels" % int((c != c_ref).sum())
    assert np.array_equal(d, d_ref), "u8 densities differ in %d voxels" % int((d != d_ref).sum())
    bad = np.any(tq != t_ref, axis=1)
    assert not bad.any(), "tangents differ in %d voxels" % int(bad.sum())
    return c_ref


@pytest.mark.parametrize("mode", ["vertices", "segments"])
@pytest.mark.parametrize("res", [(64, 64, 64), (37, 50, 29)])
def test_small_style(ctx, oracle_lib, mode, res):
    st, t, idx = style("hemi", 4096, 16)
    b = oracle_lib.bounding_box(st.vertices)
    c = _check(ctx, oracle_lib, mode, st.vertices, t, idx, b, res)
    assert c.sum() > 0


def test_unbudgeted_calls_learn_their_size(native_lib, oracle_lib):
    """Segment calls without a visit budget.  The first call at a size (index
    count, grid, index mode, tangents) reads its visit total back, which a
    stream capture refuses; a later call at that size sizes its scratch from
    it, walks once into per-brick slices with the device choosing the
    layout, and waits on nothing, so it can be captured.  A call at a known
    size that needs more than twice the learned visits in its visit list
    records a capacity overflow (reported by vkhr_check_status); the next
    call at that size counts again.  Every result that is not reported as
    overflowed is bit-exact."""
    import torch

    from vkhr_gb300 import _native
    from vkhr_gb300._native import VkhrError

    c = _native.Context(0)
    try:
        sparse = style("hemi", 2048, 12)    # 56,145 visits into 96^3
        dense = style("disk", 2048, 12)     # the same index count: 177,814 visits
        big = style("disk", 40_000, 13)     # bricks far above the sparse style's largest
        res = (96, 96, 96)

        def captured(s):
            """The call under stream capture: True if it captured (no host wait)."""
            st, t, idx = s
            b = oracle_lib.bounding_box(st.vertices)
            n = res[0] * res[1] * res[2]
            dv, dt, di = to_dev(st.vertices, torch), to_dev(t, torch), to_dev(idx, torch)
            out = [torch.full((n,), -1, dtype=torch.int32, device="cuda"),
                   torch.full((n,), 77, dtype=torch.uint8, device="cuda"),
                   torch.full((n, 4), 55, dtype=torch.int8, device="cuda")]
            torch.cuda.synchronize()
            graph = torch.cuda.CUDAGraph()
            ok = True
            try:
                with torch.cuda.graph(graph):
                    c.voxelize_segments(dv.data_ptr(), dt.data_ptr(), di.data_ptr(), len(idx), b, res,
                                        _abi.INDEX_REF_FP32, out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(),
                                        torch.cuda.current_stream().cuda_stream)
            except VkhrError as e:
                assert e.status == _abi.VKHR_ERR_INVALID_ARG  # needs its visit total: not capturable
                ok = False
            if ok:
                graph.replay()
                torch.cuda.synchronize()
                c.check_status(None)
                c_ref, d_ref, t_ref, _ = oracle_lib.voxelize("segments", st.vertices, t, idx, b, res)
                assert np.array_equal(out[0].cpu().numpy().view(np.uint32), c_ref)
                assert np.array_equal(out[1].cpu().numpy(), d_ref)
                assert np.array_equal(out[2].cpu().numpy(), t_ref)
            return ok

        def run(s):
            st, t, idx = s
            _check(c, oracle_lib, "segments", st.vertices, t, idx, oracle_lib.bounding_box(st.vertices), res)

        # (a capture must not allocate either: the larger style sizes the scratch first)
        run(big)                      # counted: the context learns the size and a per-brick capacity
        run(big)                      # known size: scratch for twice its visits
        assert captured(big)          # known size: no host wait
        assert not captured(sparse)   # a new size: reads its visits back
        run(sparse)                   # counted: the context learns the size
        assert captured(sparse)
    finally:
        c.close()
    # A context that has seen only the sparse style: its per-brick slices are
    # too small for the dense style's bricks, so a dense call at the sparse
    # style's size is laid out compactly in a visit list sized for twice the
    # sparse style's visits, which is too small: a reported overflow.
    c = _native.Context(0)
    try:
        run(sparse)
        st, t, idx = dense
        b = oracle_lib.bounding_box(st.vertices)
        dv, dt, di = to_dev(st.vertices, torch), to_dev(t, torch), to_dev(idx, torch)
        n = res[0] * res[1] * res[2]
        counts = torch.empty(n, dtype=torch.int32, device="cuda")
        dens = torch.empty(n, dtype=torch.uint8, device="cuda")
        tq = torch.empty((n, 4), dtype=torch.int8, device="cuda")
        c.voxelize_segments(dv.data_ptr(), dt.data_ptr(), di.data_ptr(), len(idx), b, res, _abi.INDEX_REF_FP32,
                            counts.data_ptr(), dens.data_ptr(), tq.data_ptr(), torch.cuda.current_stream().cuda_stream)
        with pytest.raises(VkhrError) as e:
            c.check_status(None)
        assert e.value.status == _abi.VKHR_ERR_CAPACITY
        run(dense)                    # the context forgot its sizes: this call counts again, bit-exact
        run(dense)                    # and the next one sizes from that count
    finally:
        c.close()


def test_budgeted_one_walk_device_fallback(native_lib, oracle_lib):
    """Under a visit budget (no read-back; capturable) a context that knows a
    per-brick capacity still walks once, and the device picks the layout: a
    style whose largest brick fits reads the fixed slices, one whose largest
    brick outgrew them is filled compactly by the (otherwise idle) fill pass.
    Both bit-exact."""
    from vkhr_gb300 import _native

    c = _native.Context(0)
    try:
        sparse = style("hemi", 2048, 12)
        dense = style("disk", 40_000, 13)  # largest brick 30,553 visits: far above the learned capacity
        res = (96, 96, 96)

        def run(s):
            st, t, idx = s
            b = oracle_lib.bounding_box(st.vertices)
            _check(c, oracle_lib, "segments", st.vertices, t, idx, b, res)

        run(sparse)                  # no budget: learns a capacity of 384 visits per brick
        c.set_visit_budget(4_000_000)
        run(sparse)                  # budgeted, fits: the fixed slices
        run(dense)                   # budgeted, a brick outgrew its slice: the device fills compactly
        run(sparse)
    finally:
        c.close()


@pytest.mark.parametrize("mode", ["vertices", "segments"])
def test_production_style_256(ctx, oracle_lib, mode):
    """136,320 strands x 13 vertices (1,635,840 segments) into 256^3, full size."""
    st, t, idx = style("disk", 136_320, 13)
    b = oracle_lib.bounding_box(st.vertices)
    c = _check(ctx, oracle_lib, mode, st.vertices, t, idx, b, (256, 256, 256))
    if mode == "vertices":
        assert int(c.sum(dtype=np.uint64)) == st.vertex_count


def test_saturation_and_crowded_voxels(ctx, oracle_lib):
    """Thousands of visits per voxel: the stop-at-255 rule and the shared-memory
    sort path (counts > 16 and > 2048) must still match bit for bit."""
    st, t, idx = style("disk", 20_000, 8, disk_radius=0.02, step_length=0.01)
    b = oracle_lib.bounding_box(st.vertices)
    for mode in ("vertices", "segments"):
        c = _check(ctx, oracle_lib, mode, st.vertices, t, idx, b, (8, 8, 8))
        assert c.max() > 2048


def test_bricks_above_shared_capacity(ctx, oracle_lib):
    """A dense style in a small, ragged grid: many bricks with more visits
    than a brick sorts in shared memory (keys sorted in the global scratch),
    next to bricks that fit, in both modes."""
    st, t, idx = style("hemi", 30_000, 16)
    b = oracle_lib.bounding_box(st.vertices)
    for mode in ("vertices", "segments"):
        c = _check(ctx, oracle_lib, mode, st.vertices, t, idx, b, (20, 17, 23))
        bricks = np.zeros((3, 3, 3), dtype=np.int64)
        cz = c.reshape(23, 17, 20)
        for z in range(3):
            for y in range(3):
                for x in range(3):
                    bricks[z, y, x] = cz[8 * z:8 * z + 8, 8 * y:8 * y + 8, 8 * x:8 * x + 8].sum()
        if mode == "segments":
            assert bricks.max() > 22528 and (bricks[bricks > 0] <= 22528).any()


def test_exact_index_mode(ctx, oracle_lib):
    st, t, idx = style("hemi", 2048, 12)
    b = oracle_lib.bounding_box(st.vertices)
    for mode in ("vertices", "segments"):
        _check(ctx, oracle_lib, mode, st.vertices, t, idx, b, (48, 40, 56), _abi.INDEX_EXACT)


def test_ref_fp32_index_rounding_large_grid(ctx, oracle_lib):
    """Above 2^24 voxels the reference's FP32 index rounds; REF_FP32 mode
    reproduces the rounding, EXACT does not."""
    st, t, idx = style("hemi", 256, 8)
    b = oracle_lib.bounding_box(st.vertices)
    res = (512, 512, 80)  # 20.9M voxels > 2^24
    c_ref = _check(ctx, oracle_lib, "vertices", st.vertices, t, idx, b, res, _abi.INDEX_REF_FP32)
    c_ex = _check(ctx, oracle_lib, "vertices", st.vertices, t, idx, b, res, _abi.INDEX_EXACT)
    assert not np.array_equal(c_ref, c_ex)


def test_ragged_and_degenerate_strands(ctx, oracle_lib):
    """Uneven strand lengths, zero-segment strands and zero-length segments."""
    segs = [4, 0, 1, 5, 31, 2, 0, 17, 3]  # a first strand without segments is undefined in the reference
    st = strands.ragged_style(segs, seed=3)
    v = st.vertices.copy()
    v[3] = v[2]  # a zero-length segment (NaN tangent, no visit)
    t = strands.generate_tangents(v, st.segments)
    idx = strands.generate_indices(st.segments)
    b = oracle_lib.bounding_box(v)
    for mode in ("vertices", "segments"):
        _check(ctx, oracle_lib, mode, v, t, idx, b, (16, 16, 16))


def test_custom_bounds_drop_outside(ctx, oracle_lib):
    """Vertices outside caller-supplied bounds: below the box they are dropped
    (undefined behaviour in the reference), above it they clamp to res-1."""
    st, t, idx = style("hemi", 1024, 10)
    b = _abi.aabb_from((-0.5, 0.0, -0.5), (1.0, 0.8, 1.0))
    for mode in ("vertices", "segments"):
        for im in (_abi.INDEX_REF_FP32, _abi.INDEX_EXACT):
            _check(ctx, oracle_lib, mode, st.vertices, t, idx, b, (32, 32, 32), im)


def test_empty_input(ctx, oracle_lib):
    b = _abi.aabb_from((0, 0, 0), (1, 1, 1))
    v = np.zeros((0, 3), np.float32)
    c, d, tq = gpu_voxelize(ctx, "vertices", v, v, [], b, (8, 8, 8))
    assert c.sum() == 0 and d.sum() == 0 and not tq.any()
    c, d, tq = gpu_voxelize(ctx, "segments", v, v, [], b, (8, 8, 8))
    assert c.sum() == 0 and d.sum() == 0 and not tq.any()


def test_counts_only(ctx, oracle_lib):
    st, t, idx = style("hemi", 4096, 16)
    b = oracle_lib.bounding_box(st.vertices)
    c_ref, d_ref, _, _ = oracle_lib.voxelize("segments", st.vertices, t, idx, b, (64, 64, 64))
    c, d, tq = gpu_voxelize(ctx, "segments", st.vertices, None, idx, b, (64, 64, 64), want_tangents=False)
    assert np.array_equal(c, c_ref) and np.array_equal(d, d_ref)


def test_errors(ctx, oracle_lib):
    from vkhr_gb300._native import VkhrError

    st, t, idx = style("hemi", 64, 4)
    flat = _abi.aabb_from((0, 0, 0), (1, 0, 1))
    with pytest.raises(VkhrError) as e:
        gpu_voxelize(ctx, "vertices", st.vertices, t, idx, flat, (8, 8, 8))
    assert e.value.status == _abi.VKHR_ERR_DEGENERATE_AABB
    b = oracle_lib.bounding_box(st.vertices)
    with pytest.raises(VkhrError) as e:
        gpu_voxelize(ctx, "vertices", st.vertices, t, idx, b, (0, 8, 8))
    assert e.value.status == _abi.VKHR_ERR_INVALID_ARG
    far = st.vertices.copy()
    far[1] = (1e9, 0.0, 0.0)  # a segment spanning > 2^24 voxels: the reference never terminates
    with pytest.raises(VkhrError) as e:
        gpu_voxelize(ctx, "segments", far, t, idx, b, (8, 8, 8))
    assert e.value.status == _abi.VKHR_ERR_INVALID_ARG


def test_normalize(ctx, oracle_lib):
    import torch

    st, t, idx = style("hemi", 4096, 16)
    b = oracle_lib.bounding_box(st.vertices)
    _, d_ref, _, _ = oracle_lib.voxelize("segments", st.vertices, t, idx, b, (64, 64, 64))
    dd = torch.from_numpy(d_ref.copy()).cuda()
    ctx.normalize_densities(dd.data_ptr(), dd.numel(), torch.cuda.current_stream().cuda_stream)
    assert np.array_equal(dd.cpu().numpy(), oracle_lib.normalize(d_ref))
    const = torch.full((1000,), 9, dtype=torch.uint8, device="cuda")
    ctx.normalize_densities(const.data_ptr(), const.numel(), torch.cuda.current_stream().cuda_stream)
    assert int(const.sum()) == 0


def test_prepare_kernels(ctx, oracle_lib):
    import torch

    st = strands.ragged_style([3, 0, 7, 12, 1], seed=5)
    dv = torch.from_numpy(st.vertices).cuda()
    b = ctx.bounding_box(dv.data_ptr(), st.vertex_count, torch.cuda.current_stream().cuda_stream)
    bo = oracle_lib.bounding_box(st.vertices)
    assert b.as_dict() == bo.as_dict()
    dt = torch.empty_like(dv)
    ctx.generate_tangents(dv.data_ptr(), st.segments, dt.data_ptr(), torch.cuda.current_stream().cuda_stream)
    t_ref = oracle_lib.generate_tangents(st.vertices, st.segments)
    assert np.array_equal(dt.cpu().numpy().view(np.uint32), t_ref.view(np.uint32))
    di = torch.empty(2 * st.segment_count, dtype=torch.int32, device="cuda")
    ctx.generate_indices(st.segments, di.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(di.cpu().numpy().view(np.uint32), oracle_lib.generate_indices(st.segments))


@pytest.mark.parametrize("filt", [_abi.FILTER_MAX, _abi.FILTER_MIN, _abi.FILTER_MEAN, _abi.FILTER_SUM])
def test_downsample(ctx, oracle_lib, filt):
    """Volume::downsample (hair_style.hh:228-257) on the GPU against the oracle."""
    import torch

    st, t, idx = style("hemi", 4096, 16)
    b = oracle_lib.bounding_box(st.vertices)
    res = (64, 38, 50)
    _, d, _, _ = oracle_lib.voxelize("segments", st.vertices, t, idx, b, res)
    ref = oracle_lib.downsample(d, res, filt)
    din = torch.from_numpy(d).cuda()
    out = torch.full((ref.size,), 7, dtype=torch.uint8, device="cuda")
    ctx.downsample_densities(din.data_ptr(), res, filt, out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)
    with pytest.raises(Exception):
        ctx.downsample_densities(din.data_ptr(), (63, 38, 50), filt, out.data_ptr())  # odd width


def test_light_brick_rare_paths(ctx, oracle_lib):
    """Bricks of up to 512 visits are resolved by one warp each; their rare
    paths against the oracle, in both modes: a voxel of 100 visits (a crowded
    voxel's keys handed to the crowded kernels), one of 300 (past the stop at
    255), and voxels of 3..64 visits whose tangents all sit next to one
    quantization step (k / 127 per cluster, jittered by 1e-6), so that
    certification fails and the keys are sorted in place.  Each cluster is one
    voxel in its own brick of a 64^3 grid, every brick below 512 visits."""
    rng = np.random.default_rng(12)
    b = _abi.aabb_from((0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    vox = 1.0 / 64.0
    clusters = [(100, (4, 4, 4)), (300, (20, 4, 4)), (40, (36, 4, 4)), (17, (52, 4, 4)), (5, (4, 20, 4)),
                (64, (4, 36, 4)), (3, (4, 52, 4))]
    for mode in ("vertices", "segments"):
        verts, tans = [], []
        for n, (x, y, z) in clusters:  # n visits: n vertices, or n pairs of two vertices in the voxel
            centre = (np.array([x, y, z], dtype=np.float64) + 0.5) * vox
            k = int(rng.integers(20, 100))
            for _ in range(n if mode == "vertices" else 2 * n):
                verts.append(centre + rng.uniform(-0.3, 0.3, 3) * vox)
                tans.append([k / 127.0 + rng.normal(0.0, 1e-6), -(k / 127.0) + rng.normal(0.0, 1e-6),
                             0.5 + rng.normal(0.0, 1e-6)])
        v = np.asarray(verts, dtype=np.float32)
        t = np.asarray(tans, dtype=np.float32)
        idx = np.arange(v.shape[0], dtype=np.uint32)
        c = _check(ctx, oracle_lib, mode, v, t, idx, b, (64, 64, 64))
        assert sorted(c[c > 0].tolist()) == sorted(n for n, _ in clusters)


def test_uncertified_voxels_past_the_descriptor_list(native_lib, oracle_lib):
    """Voxels of up to 64 visits whose tangents all sit next to a
    quantization step (k / 127 jittered by a few ulps) cannot be certified;
    the brick kernels hand them to the crowded-warp kernel through a
    descriptor list behind the crowded voxels' (as long as theirs), and past
    its end the voxel's own thread sorts its keys in place.  A fresh context
    per call, so the list is no longer than one call sizes it: 4 bricks of
    512 voxels of 3 visits (keys in shared memory), then 24 bricks of 512
    voxels of 45 visits (552,960 visits: keys in the global scratch), each
    with more uncertified voxels than the list holds, in both modes, against
    the oracle (the sums of some of these voxels differ by order)."""
    from vkhr_gb300 import _native

    rng = np.random.default_rng(21)
    b = _abi.aabb_from((0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    vox = 1.0 / 32.0
    cases = [(4, 3, 3e-8), (24, 45, 3e-7)]  # bricks, visits per voxel, tangent jitter
    for mode in ("vertices", "segments"):
        for nb, n, jitter in cases:
            per = n if mode == "vertices" else 2 * n   # points per voxel: n vertices, or n pairs
            lx = np.arange(512) % 8
            ly = (np.arange(512) // 8) % 8
            lz = np.arange(512) // 64
            cells = np.concatenate([np.stack([8 * (j % 4) + lx, 8 * ((j // 4) % 4) + ly, 8 * (j // 16) + lz], 1)
                                    for j in range(nb)])
            centre = np.repeat((cells + 0.5) * vox, per, axis=0)
            v = (centre + rng.uniform(-0.3, 0.3, centre.shape) * vox).astype(np.float32)
            k = np.repeat(rng.integers(20, 100, len(cells)), per)
            t = np.stack([(k / 127.0).astype(np.float32) + rng.normal(0.0, jitter, len(k)),
                          np.full(len(k), 0.25), np.full(len(k), 0.5)], 1).astype(np.float32)
            idx = np.arange(v.shape[0], dtype=np.uint32)
            c = _native.Context(0)
            try:
                got = _check(c, oracle_lib, mode, v, t, idx, b, (32, 32, 32))
            finally:
                c.close()
            assert (got == n).sum() == 512 * nb and got.sum() == 512 * nb * n


@pytest.mark.parametrize("seed", range(24))
def test_seeded_random_styles(ctx, oracle_lib, seed):
    """Seeded random cases over the voxelizer's whole input space, against
    the oracle bit for bit: strand counts of 1..3000 (pair counts that are
    rarely a multiple of a block), 2..24 vertices, hemisphere or disk roots,
    segment lengths from a fraction of a voxel to many voxels, grids of 1..96
    per axis (non-cubic, down to a few voxels, so that voxels crowd past 64
    and 255 visits), the style's bounding box or a box that cuts it, both
    index modes, both voxelization modes, with and without tangents."""
    rng = np.random.default_rng(1000 + seed)
    kind = ("hemi", "disk")[int(rng.integers(0, 2))]
    n_strands = int(rng.integers(1, 3001))
    verts = int(rng.integers(2, 25))
    step = float(rng.choice([0.005, 0.02, 0.05, 0.15]))
    st, t, idx = style(kind, n_strands, verts, seed=seed, step_length=step)
    if rng.random() < 0.25:
        res = tuple(int(x) for x in rng.integers(1, 9, 3))      # a handful of voxels: crowded
    else:
        res = tuple(int(x) for x in rng.integers(8, 97, 3))
    b = oracle_lib.bounding_box(st.vertices)
    if rng.random() < 0.3:  # a box that cuts the style: visits outside it are dropped
        o = np.asarray(b.origin, dtype=np.float64)
        s = np.asarray(b.size, dtype=np.float64)
        b = _abi.aabb_from(tuple(o + s * rng.uniform(0.0, 0.3, 3)), tuple(s * rng.uniform(0.4, 0.8, 3)))
    mode = ("vertices", "segments")[int(rng.integers(0, 2))]
    index_mode = (_abi.INDEX_REF_FP32, _abi.INDEX_EXACT)[int(rng.integers(0, 2))]
    if rng.random() < 0.2:  # counts and densities only
        c_ref, d_ref, _, _ = oracle_lib.voxelize(mode, st.vertices, t, idx, b, res, index_mode)
        c, d, _ = gpu_voxelize(ctx, mode, st.vertices, t, idx, b, res, index_mode, want_tangents=False)
        assert np.array_equal(c, c_ref) and np.array_equal(d, d_ref)
    else:
        c = _check(ctx, oracle_lib, mode, st.vertices, t, idx, b, res, index_mode)
    print("seed %d: %s %d x %d, step %.3f, %s, grid %s, %s, max %d visits in a voxel"
          % (seed, kind, n_strands, verts, step, mode, res, "exact" if index_mode else "fp32", int(c.max())))
