"""Batched voxelization (vkhr_voxelize_batched): many styles of uneven size in
one launch per phase, each bit-exact against the oracle's single-style
HairStyle::voxelize_* (hair_style.cc:257-342); the visit budget that makes
the call capturable, and a CUDA-graph replay over new vertex data."""
import ctypes as C

import numpy as np
import pytest

from vkhr_gb300 import _abi
from vkhr_gb300._native import VkhrError
from tests._helpers import style, to_dev

pytestmark = pytest.mark.gpu

RES_CHOICES = [(16, 16, 16), (24, 24, 24), (32, 32, 32), (37, 50, 29), (48, 48, 48), (64, 64, 64)]


def _styles(seed, n_jobs, crowded=True):
    """Uneven styles: strand counts log-uniform in [50, 3000], 8-32 vertices
    per strand, grids from RES_CHOICES; optionally one dense style in an 8^3
    grid whose bricks exceed the shared-memory capacity (keys sorted in global scratch)."""
    rng = np.random.default_rng(seed)
    out = []
    for j in range(n_jobs):
        n = int(np.exp(rng.uniform(np.log(50), np.log(3000))))
        verts = int(rng.integers(8, 33))
        kind = "disk" if j % 2 else "hemi"
        res = RES_CHOICES[int(rng.integers(len(RES_CHOICES)))]
        mode = _abi.INDEX_EXACT if j % 5 == 3 else _abi.INDEX_REF_FP32
        out.append((style(kind, n, verts, seed=seed * 100 + j), res, mode))
    if crowded:
        out.insert(n_jobs // 2, (style("hemi", 6000, 16, seed=seed * 100 + 99), (8, 8, 8), _abi.INDEX_REF_FP32))
    return out


class _Batch:
    """Device buffers and the job table of one batch."""

    def __init__(self, torch, oracle, styles, segments, tangents=True):
        self.torch, self.styles, self.segments = torch, styles, segments
        self.keep, self.jobs, self.outs = [], [], []
        for (st, t, idx), res, mode in styles:
            b = oracle.bounding_box(st.vertices)
            n = res[0] * res[1] * res[2]
            dv, dt = to_dev(st.vertices, torch), to_dev(t, torch)
            di = to_dev(idx.astype(np.uint32), torch)
            counts = torch.full((n,), -1, dtype=torch.int32, device="cuda")
            dens = torch.full((n,), 77, dtype=torch.uint8, device="cuda")
            tq = torch.full((n, 4), 55, dtype=torch.int8, device="cuda") if tangents else None
            self.keep += [dv, dt, di]
            self.outs.append((counts, dens, tq))
            j = _abi.VoxelJob()
            j.d_vertices, j.d_tangent_in = dv.data_ptr(), dt.data_ptr()
            j.d_indices = di.data_ptr() if segments else None
            j.item_count = len(idx) if segments else st.vertex_count
            j.bounds = b
            j.width, j.height, j.depth = res
            j.index_mode = mode
            j.d_counts, j.d_densities = counts.data_ptr(), dens.data_ptr()
            j.d_tangents = tq.data_ptr() if tq is not None else None
            self.jobs.append(j)
        self.bounds = [j.bounds for j in self.jobs]

    def poison(self):
        for counts, dens, tq in self.outs:
            counts.fill_(-1)
            dens.fill_(77)
            if tq is not None:
                tq.fill_(55)

    def check(self, oracle, vertices=None):
        m = "segments" if self.segments else "vertices"
        for k, (((st, t, idx), res, mode), (counts, dens, tq)) in enumerate(zip(self.styles, self.outs)):
            v = st.vertices if vertices is None else vertices[k]
            c_ref, d_ref, t_ref, _ = oracle.voxelize(m, v, t, idx, self.bounds[k], res, mode)
            c = counts.cpu().numpy().view(np.uint32)
            assert np.array_equal(c, c_ref), "job %d: counts differ in %d voxels" % (k, int((c != c_ref).sum()))
            d = dens.cpu().numpy()
            assert np.array_equal(d, d_ref), "job %d: densities differ in %d voxels" % (k, int((d != d_ref).sum()))
            if tq is not None:
                bad = np.any(tq.cpu().numpy() != t_ref, axis=1)
                assert not bad.any(), "job %d: tangents differ in %d voxels" % (k, int(bad.sum()))


@pytest.mark.parametrize("segments", [True, False])
def test_batched_matches_single_style(ctx, oracle_lib, segments):
    import torch

    batch = _Batch(torch, oracle_lib, _styles(1, 16), segments)
    s = torch.cuda.current_stream().cuda_stream
    ctx.voxelize_batched(segments, batch.jobs, s)
    ctx.check_status(s)
    batch.check(oracle_lib)


def test_batched_counts_only(ctx, oracle_lib):
    import torch

    batch = _Batch(torch, oracle_lib, _styles(2, 6, crowded=False), True, tangents=False)
    s = torch.cuda.current_stream().cuda_stream
    ctx.voxelize_batched(True, batch.jobs, s)
    ctx.check_status(s)
    batch.check(oracle_lib)


def test_batched_rejects_bad_tables(ctx, oracle_lib):
    import torch

    batch = _Batch(torch, oracle_lib, _styles(3, 2, crowded=False), True)
    s = torch.cuda.current_stream().cuda_stream
    with pytest.raises(VkhrError) as e:
        ctx.voxelize_batched(True, [], s)
    assert e.value.status == _abi.VKHR_ERR_INVALID_ARG
    mixed = [batch.jobs[0], _abi.VoxelJob.from_buffer_copy(batch.jobs[1])]
    mixed[1].d_tangents = None
    with pytest.raises(VkhrError) as e:
        ctx.voxelize_batched(True, mixed, s)
    assert e.value.status == _abi.VKHR_ERR_INVALID_ARG
    bad = _abi.VoxelJob.from_buffer_copy(batch.jobs[0])
    bad.width = 0
    with pytest.raises(VkhrError):
        ctx.voxelize_batched(True, [batch.jobs[1], bad], s)


def test_visit_budget_overflow_is_reported(ctx, oracle_lib):
    import torch

    batch = _Batch(torch, oracle_lib, _styles(4, 4), True)
    s = torch.cuda.current_stream().cuda_stream
    ctx.set_visit_budget(1000)
    try:
        ctx.voxelize_batched(True, batch.jobs, s)
        with pytest.raises(VkhrError) as e:
            ctx.check_status(s)
        assert e.value.status == _abi.VKHR_ERR_CAPACITY
    finally:
        ctx.set_visit_budget(0)
    batch.poison()
    ctx.voxelize_batched(True, batch.jobs, s)  # the context stays usable
    ctx.check_status(s)
    batch.check(oracle_lib)


@pytest.mark.parametrize("segments", [True, False])
def test_batched_graph_replay(ctx, oracle_lib, segments):
    """Capture once with a visit budget, then replay over new vertex data in
    the same buffers: every replay equals the oracle on that data."""
    import torch

    styles = _styles(5, 16)
    batch = _Batch(torch, oracle_lib, styles, segments)
    s = torch.cuda.current_stream().cuda_stream
    ctx.voxelize_batched(segments, batch.jobs, s)  # without a budget: sized from the counted visits
    ctx.check_status(s)
    visits = sum(int(c.cpu().numpy().view(np.uint32).sum(dtype=np.uint64)) for c, _, _ in batch.outs)
    ctx.set_visit_budget(2 * visits + 4096 if segments else 0)
    try:
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            ctx.voxelize_batched(segments, batch.jobs, side.cuda_stream)  # sizes the scratch for the budget
        ctx.check_status(side.cuda_stream)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            ctx.voxelize_batched(segments, batch.jobs, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        rng = np.random.default_rng(7)
        for rep in range(2):
            moved = []
            for k, ((st, t, idx), res, mode) in enumerate(styles):
                v = (st.vertices + rng.normal(0, 0.01, st.vertices.shape)).astype(np.float32)
                batch.keep[3 * k].copy_(torch.from_numpy(v))
                moved.append(v)
            batch.poison()
            torch.cuda.synchronize()
            graph.replay()
            torch.cuda.synchronize()
            ctx.check_status(None)
            batch.check(oracle_lib, vertices=moved)
    finally:
        ctx.set_visit_budget(0)


def test_batch_learns_one_walk_layout(oracle_lib):
    """A batch without a budget counts its visits (two walks) and learns a
    layout: a slice per visited brick of its count + 25%.  The next call of
    the same shape walks once, writing every brick's entries into its slice.
    A call whose bricks outgrow their slices fills again compactly and
    learns the layout anew; under a budget (captured) the device takes that
    fallback itself.  Every result is bit-exact."""
    import torch

    from vkhr_gb300 import _native

    c = _native.Context(0)
    styles = _styles(6, 8)
    batch = _Batch(torch, oracle_lib, styles, True)
    s = torch.cuda.current_stream().cuda_stream

    def kernels():
        """Kernel names of one unbudgeted call."""
        batch.poison()
        c.set_profiling(True)
        c.voxelize_batched(True, batch.jobs, s)
        c.check_status(s)
        torch.cuda.synchronize()
        names = [n for n, _ in c.profile()]
        c.set_profiling(False)
        return names

    def walks(names):
        direct = sum(1 for n in names if n.startswith("(bin_kernel<false") and n.endswith("true>)"))
        counting = sum(1 for n in names if n.startswith("(bin_kernel<false") and not n.endswith("true>)"))
        fill = sum(1 for n in names if n.startswith("(bin_kernel<true"))
        return direct, counting, fill, sum(1 for n in names if "layout_kernel" in n)

    def move(contract):
        """Every style's vertices pulled towards its box centre (same bounds)."""
        out = []
        for k, ((st, t, idx), res, mode) in enumerate(styles):
            lo, hi = st.vertices.min(axis=0), st.vertices.max(axis=0)
            v = st.vertices if contract == 1.0 else ((st.vertices - 0.5 * (lo + hi)) * contract + 0.5 * (lo + hi))
            v = v.astype(np.float32)
            batch.keep[3 * k].copy_(torch.from_numpy(v))
            out.append(v)
        torch.cuda.synchronize()
        return out

    try:
        names = kernels()                                  # counted: two walks, learns the layout
        assert walks(names) == (0, 1, 1, 1), names
        batch.check(oracle_lib)
        names = kernels()                                  # the same shape: one walk
        assert walks(names) == (1, 0, 0, 0), names
        batch.check(oracle_lib)
        moved = move(0.4)                                  # crowded bricks outgrow their slices
        names = kernels()
        assert walks(names) == (1, 0, 1, 1), names         # compact fill, layout learned again
        batch.check(oracle_lib, vertices=moved)
        names = kernels()
        assert walks(names) == (1, 0, 0, 0), names
        batch.check(oracle_lib, vertices=moved)

        # under a budget, captured: one walk, the fill a device-side fallback
        visits = sum(int(x.cpu().numpy().view(np.uint32).sum(dtype=np.uint64)) for x, _, _ in batch.outs)
        c.set_visit_budget(4 * visits + 4096)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            c.voxelize_batched(True, batch.jobs, side.cuda_stream)  # sizes the scratch for the budget
        c.check_status(side.cuda_stream)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            c.voxelize_batched(True, batch.jobs, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        for contract in (0.4, 1.0, 0.4):                   # fits; outgrows (fallback); fits
            moved = move(contract)
            batch.poison()
            graph.replay()
            torch.cuda.synchronize()
            c.check_status(None)
            batch.check(oracle_lib, vertices=moved)
        del graph
    finally:
        c.set_visit_budget(0)
        c.close()


def test_batch_one_walk_with_wide_keys(oracle_lib):
    """A batch one of whose styles has more than 2^23 index pairs keeps
    (key, local voxel) visit entries of 8 bytes; its learned one-walk layout
    and the walk into it give the oracle's voxels bit for bit."""
    import torch

    from vkhr_gb300 import _native

    big = style("hemi", 700_000, 13, seed=21)  # 8.4M pairs: keys past 2^23
    assert big[2].shape[0] // 2 > (1 << 23)
    styles = [(big, (64, 64, 64), _abi.INDEX_REF_FP32),
              (style("disk", 2500, 14, seed=22), (48, 48, 48), _abi.INDEX_REF_FP32)]
    c = _native.Context(0)
    try:
        batch = _Batch(torch, oracle_lib, styles, True)
        s = torch.cuda.current_stream().cuda_stream
        for _ in range(2):  # counted (learns the layout), then one walk into it
            batch.poison()
            c.set_profiling(True)
            c.voxelize_batched(True, batch.jobs, s)
            c.check_status(s)
            torch.cuda.synchronize()
            names = [n for n, _ in c.profile()]
            c.set_profiling(False)
            batch.check(oracle_lib)
        assert any(n.startswith("(bin_kernel<false, true, false, false, false, true>") for n in names), names
    finally:
        c.close()
