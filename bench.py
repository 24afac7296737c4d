#!/usr/bin/env python3
"""Benchmark of the volumetric level-of-detail path on GB300.

One step = one frame of the path at production size: segment-voxelize a
136,320-strand x 13-vertex style (1,635,840 segments, grown procedurally:
roots on a 0.3-radius disk tilted 30 degrees, 12 steps of 0.08) into a
256^3 grid (uint32 counts, u8 densities, int8 tangents), normalize the
densities, then raymarch a 1920x1080 view with 512 steps, 64-step density
shadows, 8-tap ambient occlusion and the workloads' dual-lobe Kajiya-Kay
(kd 0.4, specular exponents 80 / 8, tangent shifts +0.1 / -0.1).

`value` is frame throughput in Mpixels/s (1920*1080 / step time) with the
inputs resident in HBM; the per-stage rates (Msegments/s voxelized, Mpixels/s
raymarched) are reported beside it.  L2 is flushed (a 512 MiB write) before
every timed step.  `e2e` repeats the step through the C ABI with host
buffers: the H2D copy of the strand arrays from pinned memory and the D2H
read of the frame (RGBA + depth) are inside the timed region.

--impl reference times the reference's CPU algorithm for the same frame on
the host cores (the oracle's restatement of HairStyle::voxelize_segments,
serial as in the reference, plus the FP32 raymarch of volume.frag over every
pixel row of the volume's screen footprint -- the proxy cube's fragments,
volume.vert:17-25 -- with all threads).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOAD = {
    "workload": "production frame: 136,320 strands x 13 vertices (1,635,840 segments) segment-voxelized into "
                "256^3, raymarched at 1920x1080, 512 steps, 64-step shadows, 8-tap AO, Kajiya-Kay kd 0.4, "
                "exponents 80/8, shifts +-0.1",
    "strands": 136_320,
    "vertices_per_strand": 13,
    "resolution": 256,
    "width": 1920,
    "height": 1080,
    "raycast_steps": 512,
    "shadow_steps": 64,
    "ao_taps": 8,
    "shading": "Kajiya-Kay: kd 0.4, specular exponents 80 / 8, tangent shifts +0.1 / -0.1",
    "density": "u8 unorm (normalized)",
    "l2": "flushed before every timed step (512 MiB write)",
}
# DRAM bytes (read + write) per launch from one ncu capture of the production
# frame (profiles/voxelizer_kernels_production_frame.md and
# profiles/raymarch_kernel_production_frame.md), by kernel family.
TRAFFIC = {
    "bin_kernel<false, true, true, true, false, true": 57_001_472 + 96_199_168,  # one walk
    "brick_kernel<SEG, TANG, false": 154_601_472 + 26_825_472,
    "bin_kernel<true": 55_134_208 + 72_237_312,
    "bin_kernel<false": 55_694_080 + 24_500_992,
    "raymarch_kernel": 8_215_040 + 0,
}

METRIC = "Msegments/s voxelized + Mpixels/s raymarched, 1 GB300 (frame throughput in Mpixels/s)"
UNIT = "Mpixels/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_style():
    from vkhr_gb300 import strands

    st = strands.disk_style(WORKLOAD["strands"], WORKLOAD["vertices_per_strand"], seed=0)
    t = strands.generate_tangents(st.vertices, st.segments)
    idx = strands.generate_indices(st.segments)
    return st, t, idx


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        threading.Thread(target=self._read, daemon=True).start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def frame_params(b, res):
    from vkhr_gb300 import scene

    return scene.make_params(b, res, WORKLOAD["width"], WORKLOAD["height"],
                             raycast_steps=float(WORKLOAD["raycast_steps"]), shadow_steps=float(WORKLOAD["shadow_steps"]),
                             **scene.CONFIG_SHADING)


def cpu_frame(O, st, t, idx, b):
    """One CPU frame: the serial voxelizer + normalize, then the FP32 raymarch
    of every pixel with all threads (a pixel whose ray misses the volume's
    box, which the proxy cube does not cover, costs only its box test).
    Returns the seconds of both parts."""
    res = (WORKLOAD["resolution"],) * 3
    t0 = time.perf_counter()
    _, d, tq, _ = O.voxelize("segments", st.vertices, t, idx, b, res)
    dn = O.normalize(d)
    t1 = time.perf_counter()
    p = frame_params(b, res)
    t2 = time.perf_counter()
    O.raymarch(p, dn, tq, precision="f32")
    t3 = time.perf_counter()
    return (t1 - t0), (t3 - t2)


def reference_arm(args):
    from vkhr_gb300 import replicas

    rank, _, _ = replicas.world()
    if rank != 0:  # the CPU reference runs once, on rank 0
        return 0
    from oracle import oracle as O

    if not os.path.exists(O.LIB):
        O.build(with_reference=False)
    st, t, idx = make_style()
    b = O.bounding_box(st.vertices)
    for _ in range(args.warmup):
        cpu_frame(O, st, t, idx, b)
    vox, ray = [], []
    for _ in range(args.steps):
        a, r = cpu_frame(O, st, t, idx, b)
        vox.append(a)
        ray.append(r)
    step_s = (sum(vox) + sum(ray)) / args.steps
    px = WORKLOAD["width"] * WORKLOAD["height"]
    value = px / step_s / 1e6
    cores = O.max_threads()
    sample = ("every step is the whole frame: the serial voxelization (1,635,840 segments -> 256^3) + normalize, "
              "and the FP32 raymarch of all 1920x1080 pixels (all threads)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": WORKLOAD,
        "components": {"voxelize_msegments_per_s": st.segment_count / (sum(vox) / args.steps) / 1e6,
                       "raymarch_mpixels_per_s": px / (sum(ray) / args.steps) / 1e6,
                       "voxelize_s": sum(vox) / args.steps, "raymarch_s": sum(ray) / args.steps},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


BATCH = {
    "workload": "16 styles in one batched voxelize + one persistent raymarch launch, CUDA graph: strands "
                "log-uniform 5k-136k, 8-32 vertices, grids from {64,128,192,256}^3, each in a 3840x2160 view at "
                "the distance giving a 64-1024 pixel footprint; 512 steps, 64-step shadows, 8-tap AO on uint32 "
                "counts (isosurface 1 count)",
    "plain": "per style: vkhr_voxelize_segments (sizes its visit list from a host read) + vkhr_raymarch of "
             "the whole 3840x2160 view",
}


def batched_comparison(args, dev, stream, rank, world, flush):
    """The multi-style batch three ways: plain per-style calls, the batched
    calls, and the batched calls replayed from a CUDA graph.  Returns the
    JSON object of the comparison (times are maxima over ranks; each rank
    takes its share of the styles)."""
    import torch

    from vkhr_gb300 import _abi, _native, replicas, scene, workloads

    specs = workloads.batched_specs()
    costs = [sp["strands"] * (sp["vertices_per_strand"] - 1) * sp["resolution"] for sp in specs]
    mine = replicas.shard(costs, rank, world)
    W, H = workloads.BATCH_TARGET
    s = stream.cuda_stream
    ctx_p = _native.Context(dev.index)
    ctx_b = _native.Context(dev.index)
    styles = []
    for i in mine:
        sp = specs[i]
        st, t, idx = workloads.grow(sp)
        res = (sp["resolution"],) * 3
        n = res[0] ** 3
        x = {"spec": sp, "segments": st.segment_count, "index_count": int(idx.shape[0]), "res": res,
             "dv": torch.from_numpy(st.vertices).to(dev), "dt": torch.from_numpy(t).to(dev),
             "di": torch.from_numpy(idx.view(np.int32)).to(dev),
             "counts_p": torch.empty(n, dtype=torch.int32, device=dev),
             "tq_p": torch.empty((n, 4), dtype=torch.int8, device=dev),
             "counts_b": torch.empty(n, dtype=torch.int32, device=dev),
             "tq_b": torch.empty((n, 4), dtype=torch.int8, device=dev)}
        x["b"] = ctx_p.bounding_box(x["dv"].data_ptr(), st.vertex_count, s)
        dist = workloads.camera_distance(x["b"], sp["footprint"], H)
        x["p"] = scene.make_params(x["b"], res, W, H, camera_distance=dist, view_direction=sp["view_direction"],
                                   raycast_steps=512.0, shadow_steps=64.0, isosurface=1.0,
                                   density_format=_abi.DENSITY_U32_COUNT)
        x["distance"] = dist
        x["rect"] = _native.raymarch_footprint(x["p"])
        styles.append(x)
    pos, atlas_h = workloads.shelf_pack([(x["rect"][2], x["rect"][3]) for x in styles], W)
    atlas = torch.zeros((max(atlas_h, 1), W, 4), dtype=torch.float32, device=dev)
    atlas_d = torch.ones((max(atlas_h, 1), W), dtype=torch.float32, device=dev)
    full = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    full_d = torch.empty((H, W), dtype=torch.float32, device=dev)
    vjobs, rjobs = [], []
    for x, (ax, ay) in zip(styles, pos):
        v = _abi.VoxelJob()
        v.d_vertices, v.d_tangent_in, v.d_indices = x["dv"].data_ptr(), x["dt"].data_ptr(), x["di"].data_ptr()
        v.item_count = x["index_count"]
        v.bounds = x["b"]
        v.width, v.height, v.depth = x["res"]
        v.index_mode = _abi.INDEX_REF_FP32
        v.d_counts, v.d_densities, v.d_tangents = x["counts_b"].data_ptr(), None, x["tq_b"].data_ptr()
        vjobs.append(v)
        r = _abi.RaymarchJob()
        r.params = x["p"]
        r.d_density, r.d_tangent, r.d_depth_in = x["counts_b"].data_ptr(), x["tq_b"].data_ptr(), None
        r.d_rgba, r.d_depth_out = atlas[ay, ax].data_ptr(), atlas_d[ay, ax].data_ptr()
        r.x0, r.y0, r.w, r.h = x["rect"]
        r.pitch = W
        rjobs.append(r)

    def plain():
        for x in styles:
            ctx_p.voxelize_segments(x["dv"].data_ptr(), x["dt"].data_ptr(), x["di"].data_ptr(), x["index_count"],
                                    x["b"], x["res"], _abi.INDEX_REF_FP32, x["counts_p"].data_ptr(), None,
                                    x["tq_p"].data_ptr(), s)
            ctx_p.raymarch(x["p"], x["counts_p"].data_ptr(), x["tq_p"].data_ptr(), None, full.data_ptr(),
                           full_d.data_ptr(), s)

    def batched(st_handle):
        ctx_b.voxelize_batched(True, vjobs, st_handle)
        ctx_b.raymarch_batched(rjobs, st_handle)

    # the one-walk residency for this batch (counts it, learns its layout), then the visit budget from
    # one counted run (+25%), a warm-up at that budget and the capture
    bwalk, bwalk_ms = ctx_b.autotune_voxelize(vjobs, s)
    ctx_b.voxelize_batched(True, vjobs, s)
    ctx_b.check_status(s)
    visits = int(sum(int(x["counts_b"].sum(dtype=torch.int64).item()) for x in styles))
    ctx_b.set_visit_budget(visits + visits // 4 + 4096)
    side = torch.cuda.Stream(device=dev)
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        batched(side.cuda_stream)
    ctx_b.check_status(side.cuda_stream)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        batched(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()

    variants = {"plain": plain, "batched": lambda: batched(s), "batched_graph": graph.replay}
    launches = {}
    for _ in range(max(args.warmup, 3)):
        for f in variants.values():
            flush.zero_()
            f()
    torch.cuda.synchronize()
    times = {k: [] for k in variants}
    walls = {k: [] for k in variants}
    for _ in range(args.steps):
        for k, f in variants.items():
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            l0 = ctx_p.launch_count() + ctx_b.launch_count()
            w0 = time.perf_counter()
            e0.record(stream)
            f()
            e1.record(stream)
            torch.cuda.synchronize()
            walls[k].append((time.perf_counter() - w0) * 1e3)
            times[k].append(e0.elapsed_time(e1))
            launches[k] = ctx_p.launch_count() + ctx_b.launch_count() - l0
    ctx_b.check_status(s)
    # per-kernel device time of the batched calls (event pair per launch, outside the timed runs)
    ctx_b.set_profiling(True)
    flush.zero_()
    batched(s)
    torch.cuda.synchronize()
    kern = {}
    for name, kms in ctx_b.profile():
        e = kern.setdefault(name, [0, 0.0])
        e[0] += 1
        e[1] += kms
    ctx_b.set_profiling(False)
    ms = {k: replicas.max_over_ranks(statistics.median(v), device=dev) for k, v in times.items()}
    wall_ms = {k: replicas.max_over_ranks(statistics.median(v), device=dev) for k, v in walls.items()}

    # identical results: voxels bit-exact, and every region equal to the plain full-view render
    same = all(torch.equal(x["counts_p"], x["counts_b"]) and torch.equal(x["tq_p"], x["tq_b"]) for x in styles)
    for x, (ax, ay) in zip(styles, pos):
        x0, y0, w, h = x["rect"]
        ctx_p.raymarch(x["p"], x["counts_b"].data_ptr(), x["tq_b"].data_ptr(), None, full.data_ptr(),
                       full_d.data_ptr(), s)
        torch.cuda.synchronize()
        outside = full.clone()
        outside[y0:y0 + h, x0:x0 + w] = 0.0
        same = same and torch.equal(atlas[ay:ay + h, ax:ax + w], full[y0:y0 + h, x0:x0 + w])
        same = same and torch.equal(atlas_d[ay:ay + h, ax:ax + w], full_d[y0:y0 + h, x0:x0 + w])
        same = same and not bool(outside.any())
    segs = sum(x["segments"] for x in styles)
    pixels = sum(x["rect"][2] * x["rect"][3] for x in styles)
    out = {
        "config": dict(BATCH, styles=len(specs), ranks=world),
        "styles_this_rank": [{"strands": x["spec"]["strands"], "vertices": x["spec"]["vertices_per_strand"],
                              "resolution": x["res"][0], "footprint": list(x["rect"][2:]),
                              "camera_distance": round(x["distance"], 2)} for x in styles],
        "segments": segs, "region_pixels": pixels, "visits": visits,
        "ms": ms, "wall_ms": wall_ms, "launches_per_step": launches,
        "batched_kernels_ms": {k: round(v[1], 4) for k, v in sorted(kern.items(), key=lambda kv: -kv[1][1])},
        "speedup_vs_plain": {"batched": ms["plain"] / ms["batched"], "batched_graph": ms["plain"] / ms["batched_graph"]},
        "batched_graph_msegments_per_s": world * segs / (ms["batched_graph"] / 1e3) / 1e6,
        "batched_graph_region_mpixels_per_s": world * pixels / (ms["batched_graph"] / 1e3) / 1e6,
        "identical_to_plain": bool(same),
        "autotune": {"voxelize_walk_ctas_per_sm": bwalk,
                     "walk_ms": {str(k): round(m, 4) for k, m in zip(_abi.WALK_CHOICES, bwalk_ms)}},
    }
    ctx_b.set_visit_budget(0)
    return out


SCALE = {
    "workload": "1,048,576 strands x 32 vertices (33,554,432 vertices, 32,505,856 segments; radius-1.2 hemisphere, "
                "step 0.04) segment-voxelized into 512^3 (u32 counts, u8, i8x4 tangents; 8-byte visit entries), "
                "normalized, raymarched at 3840x2160 with 1024 steps, 128-step shadows, 16-direction AO, Kajiya-Kay "
                "kd 0.4, exponents 80/8, shifts +-0.1; plus 4 views of the volume (3840x2160 each) in one batched "
                "launch",
}


def scale_section(args, dev, stream, flush):
    """The scale workload: per-stage device times (median of the steps)."""
    import torch

    from vkhr_gb300 import _abi, _native, scene, strands

    s = stream.cuda_stream
    ctx = _native.Context(dev.index)
    st = strands.hemisphere_style(1_048_576, 32, radius=1.2, step_length=0.04, seed=4)
    t = strands.generate_tangents(st.vertices, st.segments)
    idx = strands.generate_indices(st.segments)
    res = (512, 512, 512)
    n = 512 ** 3
    dv = torch.from_numpy(st.vertices).to(dev)
    dt = torch.from_numpy(t).to(dev)
    di = torch.from_numpy(idx.view(np.int32)).to(dev)
    b = ctx.bounding_box(dv.data_ptr(), st.vertex_count, s)
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    dens = torch.empty(n, dtype=torch.uint8, device=dev)
    tq = torch.empty((n, 4), dtype=torch.int8, device=dev)
    kw = dict(camera_distance=5.0, raycast_steps=1024.0, shadow_steps=128.0, ao_directions=16, **scene.CONFIG_SHADING)
    p = scene.make_params(b, res, 3840, 2160, **kw)
    rgba = torch.empty((2160, 3840, 4), dtype=torch.float32, device=dev)
    depth = torch.empty((2160, 3840), dtype=torch.float32, device=dev)
    views = [scene.make_params(b, res, 3840, 2160, view_direction=vd, **kw)
             for vd in ((0.0, 0.0, 1.0), (1.0, 0.3, 0.0), (0.0, 1.0, 0.2), (-0.7, 0.2, -0.7))]
    rects = [_native.raymarch_footprint(v) for v in views]
    atlas = torch.empty((max(r[3] for r in rects), sum(r[2] for r in rects), 4), dtype=torch.float32, device=dev)
    jobs, at = [], 0
    for v, (x0, y0, w, h) in zip(views, rects):
        j = _abi.RaymarchJob()
        j.params = v
        j.d_density, j.d_tangent = dens.data_ptr(), tq.data_ptr()
        j.d_rgba = atlas[0, at].data_ptr()
        j.x0, j.y0, j.w, j.h, j.pitch = x0, y0, w, h, atlas.shape[1]
        jobs.append(j)
        at += w

    # the ray-packet variant for the 3840x2160 view (vkhr_autotune_raymarch), after one voxelization
    ctx.voxelize_segments(dv.data_ptr(), dt.data_ptr(), di.data_ptr(), idx.shape[0], b, res, _abi.INDEX_REF_FP32,
                          counts.data_ptr(), dens.data_ptr(), tq.data_ptr(), s)
    ctx.normalize_densities(dens.data_ptr(), n, s)
    tuned, tuned_ms = ctx.autotune_raymarch(p, dens.data_ptr(), tq.data_ptr(), rgba.data_ptr(), s)
    stages = {
        "voxelize": lambda: ctx.voxelize_segments(dv.data_ptr(), dt.data_ptr(), di.data_ptr(), idx.shape[0], b, res,
                                                  _abi.INDEX_REF_FP32, counts.data_ptr(), dens.data_ptr(),
                                                  tq.data_ptr(), s),
        "normalize": lambda: ctx.normalize_densities(dens.data_ptr(), n, s),
        "raymarch": lambda: ctx.raymarch(p, dens.data_ptr(), tq.data_ptr(), None, rgba.data_ptr(),
                                         depth.data_ptr(), s),
        "raymarch_4_views_batched": lambda: ctx.raymarch_batched(jobs, s),
    }
    times = {k: [] for k in stages}
    for k in range(max(args.warmup, 3) + args.steps):
        for name, f in stages.items():
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            f()
            e1.record(stream)
            torch.cuda.synchronize()
            if k >= max(args.warmup, 3):
                times[name].append(e0.elapsed_time(e1))
    ctx.check_status(s)
    ms = {k: statistics.median(v) for k, v in times.items()}
    view_px = sum(r[2] * r[3] for r in rects)
    out = {
        "config": SCALE, "ms": ms,
        "voxelize_msegments_per_s": st.segment_count / (ms["voxelize"] / 1e3) / 1e6,
        "raymarch_mpixels_per_s": 3840 * 2160 / (ms["raymarch"] / 1e3) / 1e6,
        "batched_views_region_pixels": view_px,
        "batched_views_mpixels_per_s": view_px / (ms["raymarch_4_views_batched"] / 1e3) / 1e6,
        "visits": int(counts.sum(dtype=torch.int64).item()),
        "autotune": {"raymarch_variant": tuned, "variant_ms": tuned_ms},
    }
    ctx.close()
    return out


DIFF = {
    "workload": "differentiable view: the 136,320 x 13 style (1,772,160 vertices) trilinearly splatted into an FP32 "
                "256^3 density, FP32 tangents, 960x540 with 512 steps, 64-step shadows, 8-tap AO; L2 loss against a "
                "target from log-normally perturbed densities (sigma 0.2) with first exponent 60; Kajiya-Kay kd 0.4, "
                "exponents 80/8, shifts +-0.1; gradients with respect to density, tangents, kd, both exponents and "
                "(through the splat) the vertices",
}


def diff_section(args, dev, stream, flush):
    """Forward vs adjoint cost of the differentiable path (median device ms)."""
    import torch

    from vkhr_gb300 import _abi, _native, scene

    s = stream.cuda_stream
    ctx = _native.Context(dev.index)
    st, t, idx = make_style()
    res = (256, 256, 256)
    n = 256 ** 3
    V = torch.from_numpy(st.vertices).to(dev)
    b = ctx.bounding_box(V.data_ptr(), st.vertex_count, s)
    dens = torch.zeros(n, dtype=torch.float32, device=dev)
    ctx.splat_vertices(V.data_ptr(), st.vertex_count, b, res, dens.data_ptr(), s)
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    tq = torch.empty((n, 4), dtype=torch.int8, device=dev)
    dt = torch.from_numpy(t).to(dev)
    di = torch.from_numpy(idx.view(np.int32)).to(dev)
    ctx.voxelize_segments(V.data_ptr(), dt.data_ptr(), di.data_ptr(), idx.shape[0], b, res, _abi.INDEX_REF_FP32,
                          counts.data_ptr(), None, tq.data_ptr(), s)
    tan = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    tan[:, :3] = torch.clamp(tq[:, :3].float() / 127.0, min=-1.0)
    kw = dict(camera_distance=4.0, raycast_steps=512.0, shadow_steps=64.0, isosurface=1.0,
              density_format=_abi.DENSITY_F32, tangent_format=_abi.TANGENT_F32X4,
              **{k: v for k, v in scene.CONFIG_SHADING.items() if k != "hair_exponent"})
    p = scene.make_params(b, res, 960, 540, hair_exponent=80.0, **kw)
    pt = scene.make_params(b, res, 960, 540, hair_exponent=60.0, **kw)
    gen = torch.Generator(device=dev).manual_seed(3)
    noisy = dens * torch.exp(0.2 * torch.randn(n, generator=gen, device=dev))
    target = torch.empty((540, 960, 4), dtype=torch.float32, device=dev)
    ctx.raymarch(pt, noisy.data_ptr(), tan.data_ptr(), None, target.data_ptr(), None, s)
    rgba = torch.empty_like(target)
    out = {"config": DIFF, "ms": {}}
    for K in (16, 32, 64):
        nbytes = ctx.tape_bytes(p, K)
        tape = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        g_rgba = torch.empty_like(target)
        gd = torch.empty_like(dens)
        gt = torch.empty_like(tan)
        gp = torch.empty(3, dtype=torch.float64, device=dev)  # kd and the two exponents
        gv = torch.empty_like(V)

        def adjoint_pass():
            torch.mul(rgba - target, 2.0, out=g_rgba)  # dL/drgba of the L2 loss
            gd.zero_()
            gt.zero_()
            gp.zero_()
            ctx.raymarch_adjoint(p, dens.data_ptr(), tan.data_ptr(), tape.data_ptr(), K, g_rgba.data_ptr(),
                                 gd.data_ptr(), gt.data_ptr(), gp.data_ptr(), s)
            ctx.splat_vertices_adjoint(V.data_ptr(), st.vertex_count, b, res, gd.data_ptr(), gv.data_ptr(), s)

        stages = {
            "forward": lambda: ctx.raymarch(p, dens.data_ptr(), tan.data_ptr(), None, rgba.data_ptr(), None, s),
            "forward_train": lambda: ctx.raymarch_train(p, dens.data_ptr(), tan.data_ptr(), rgba.data_ptr(), None,
                                                        tape.data_ptr(), nbytes, K, s),
            "adjoint": adjoint_pass,
        }
        times = {k: [] for k in stages}
        for k in range(max(args.warmup, 3) + args.steps):
            for name, f in stages.items():
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                f()
                e1.record(stream)
                torch.cuda.synchronize()
                if k >= max(args.warmup, 3):
                    times[name].append(e0.elapsed_time(e1))
        ms = {k: statistics.median(v) for k, v in times.items()}
        out["ms"]["K=%d" % K] = ms
        out["adjoint_over_forward_K%d" % K] = ms["adjoint"] / ms["forward"]
        out["train_plus_adjoint_over_forward_K%d" % K] = (ms["forward_train"] + ms["adjoint"]) / ms["forward"]
        out["tape_bytes_K%d" % K] = nbytes
    ctx.close()
    return out


def frame_graph_section(args, dev, stream, flush, st, t, idx, b, res, p):
    """The per-frame path as one CUDA graph (vkhr_frame_graph_*): the
    production style voxelized under a visit budget, normalized and
    raymarched, replayed per frame.  Device time with inputs resident, and
    end to end with each frame's swayed vertices and tangents uploaded and
    the image read back (serial)."""
    import torch

    from vkhr_gb300 import _abi, _native, strands, workloads

    ctx = _native.Context(dev.index)
    s = stream.cuda_stream
    n = res[0] * res[1] * res[2]
    W, H = p.width, p.height
    dv = torch.from_numpy(st.vertices).to(dev)
    dt = torch.from_numpy(t).to(dev)
    di = torch.from_numpy(idx.view(np.int32)).to(dev)
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    dens = torch.empty(n, dtype=torch.uint8, device=dev)
    tq = torch.empty((n, 4), dtype=torch.int8, device=dev)
    rgba = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    depth = torch.empty((H, W), dtype=torch.float32, device=dev)
    job = _abi.VoxelJob()
    job.d_vertices, job.d_tangent_in, job.d_indices = dv.data_ptr(), dt.data_ptr(), di.data_ptr()
    job.item_count = idx.shape[0]
    job.bounds = b
    job.width, job.height, job.depth = res
    job.index_mode = _abi.INDEX_REF_FP32
    job.d_counts, job.d_densities, job.d_tangents = counts.data_ptr(), dens.data_ptr(), tq.data_ptr()
    graph = ctx.frame_graph(True, job, p, rgba.data_ptr(), depth.data_ptr(), stream=s)
    # two frames of motion, alternated: the style as loaded and swayed (inside the same bounds)
    v1 = workloads.sway(st.vertices, 0.02)
    v1 = np.clip(v1, np.asarray(b.origin, dtype=np.float32),
                 (np.asarray(b.origin, dtype=np.float64) + np.asarray(b.size, dtype=np.float64)).astype(np.float32))
    hv = [torch.from_numpy(st.vertices).pin_memory(), torch.from_numpy(v1).pin_memory()]
    ht = [torch.from_numpy(t).pin_memory(), torch.from_numpy(strands.generate_tangents(v1, st.segments)).pin_memory()]
    ho = torch.empty((H, W, 4), dtype=torch.float32).pin_memory()
    hd = torch.empty((H, W), dtype=torch.float32).pin_memory()
    for _ in range(max(args.warmup, 3)):
        flush.zero_()
        graph.launch(s)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        graph.launch(s)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    dev_ms = sum(a.elapsed_time(z) for a, z in ev) / args.steps
    for k in range(args.steps + 2):
        if k >= 2:
            ev[k - 2][0].record(stream)
        dv.copy_(hv[k % 2], non_blocking=True)
        dt.copy_(ht[k % 2], non_blocking=True)
        graph.launch(s)
        ho.copy_(rgba, non_blocking=True)
        hd.copy_(depth, non_blocking=True)
        if k >= 2:
            ev[k - 2][1].record(stream)
        torch.cuda.synchronize()
    e2e_ms = sum(a.elapsed_time(z) for a, z in ev) / args.steps
    ctx.check_status(s)
    graph.close()
    ctx.close()
    return {
        "config": {"workload": "the production frame as one CUDA graph per frame: voxelize (segments, visit budget = "
                               "1.25x the first frame's visits), normalize, occupancy, raymarch 1920x1080; e2e: "
                               "each frame uploads its swayed vertices and tangents and reads the image back, serial"},
        "ms": dev_ms, "mpixels_per_s": W * H / dev_ms / 1e3,
        "e2e_ms": e2e_ms, "e2e_mpixels_per_s": W * H / e2e_ms / 1e3,
        "h2d_bytes_per_step": hv[0].numel() * 4 + ht[0].numel() * 4, "d2h_bytes_per_step": ho.numel() * 4 + hd.numel() * 4,
    }


def schedule_section(args, dev, stream):
    """The reference's benchmark schedule for the raymarcher (benchmark.hh:
    12-140, run by rasterizer.cc:599-772) restated headlessly on the synthetic
    ponytail at 1280x720: distance 200..2000 (step 1800/64), raymarch samples
    512..64 (step 448/64 = 7), strand ratio 1..1/64 (step 1/64) around the
    defaults (distance 226, ratio 1, 512 samples).  Distances map to this
    scene's units by 4.0 / 226 (the default camera distance here over the
    reference's).  Distance and samples time the raymarch of the loaded
    volume; each strand ratio applies HairStyle::reduce (vkhr_reduce_strands,
    the reference's seeded choice) to the loaded style and times the
    voxelization (segments, normalized) plus the raymarch."""
    import torch

    from vkhr_gb300 import _abi, _native, scene, strands

    ctx = _native.Context(dev.index)
    s = stream.cuda_stream
    st, t, idx = make_style()
    res = (WORKLOAD["resolution"],) * 3
    n = res[0] * res[1] * res[2]
    W, H = 1280, 720
    dv = torch.from_numpy(st.vertices).to(dev)
    dt = torch.from_numpy(t).to(dev)
    b = ctx.bounding_box(dv.data_ptr(), st.vertex_count, s)
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    dens = torch.empty(n, dtype=torch.uint8, device=dev)
    tq = torch.empty((n, 4), dtype=torch.int8, device=dev)
    rgba = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    depth = torch.empty((H, W), dtype=torch.float32, device=dev)
    scale = 4.0 / 226.0
    reps = max(args.steps, 3)

    def params(distance=226.0, samples=512):
        return scene.make_params(b, res, W, H, camera_distance=distance * scale, raycast_steps=float(samples),
                                 renderer=_abi.RENDERER_RAYMARCHER)

    def voxelize(v_ptr, t_ptr, di, count):
        ctx.voxelize_segments(v_ptr, t_ptr, di.data_ptr(), count, b, res, _abi.INDEX_REF_FP32, counts.data_ptr(),
                              dens.data_ptr(), tq.data_ptr(), s)
        ctx.normalize_densities(dens.data_ptr(), n, s)

    def timed(fn):
        for _ in range(2):
            fn()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, z in ev:
            a.record(stream)
            fn()
            z.record(stream)
        torch.cuda.synchronize()
        return sorted(a.elapsed_time(z) for a, z in ev)[reps // 2]

    di_full = torch.from_numpy(idx.view(np.int32)).to(dev)
    voxelize(dv.data_ptr(), dt.data_ptr(), di_full, idx.shape[0])
    torch.cuda.synchronize()

    def march(p):
        return lambda: ctx.raymarch(p, dens.data_ptr(), tq.data_ptr(), None, rgba.data_ptr(), depth.data_ptr(), s)

    out = {"config": {"workload": "the reference's raymarcher benchmark schedule on the synthetic ponytail "
                                  "(136,320 x 13, 256^3), 1280x720; median of %d runs per point" % reps,
                      "distance_scale": scale,
                      "distance": "[distance, ms of variant 0, ms of the variant the autotuner picks for that "
                                  "view, that variant]"}}
    rows = []
    for d in (200.0 + k * (1800.0 / 64.0) for k in range(64)):
        p = params(distance=d)
        ctx.set_raymarch_variant(p.density_format, p.tangent_format, 0)
        ms0 = timed(march(p))
        chosen, _ = ctx.autotune_raymarch(p, dens.data_ptr(), tq.data_ptr(), rgba.data_ptr(), s)
        rows.append([d, ms0, timed(march(p)), chosen])
    ctx.set_raymarch_variant(_abi.DENSITY_U8_UNORM, _abi.TANGENT_I8_SNORM, 0)
    out["distance"] = rows
    out["samples"] = [[k, timed(march(params(samples=k)))] for k in range(512, 63, -(448 // 64))]
    ov, ot = torch.empty_like(dv), torch.empty_like(dt)
    segs = st.segments.astype(np.uint16)
    rows = []
    for k in range(64):
        ratio = 1.0 - k / 64.0
        kept, nv, _ = ctx.reduce_strands(ratio, 0x9E3779B97F4A7C15, segs, len(segs), dv.data_ptr(), dt.data_ptr(),
                                         ov.data_ptr(), ot.data_ptr(), stream=s)
        kidx = strands.generate_indices(kept)
        di = torch.from_numpy(kidx.view(np.int32)).to(dev)
        p = params()
        vox_ms = timed(lambda: voxelize(ov.data_ptr(), ot.data_ptr(), di, kidx.shape[0]))
        rows.append([ratio, int(len(kept)), vox_ms, timed(march(p))])
    out["strands"] = rows
    ctx.close()
    return out


def composite_section(args, dev, stream, flush, st, t, idx, b, res):
    """The colour pass's transparency without a linked list (vkhr_composite):
    the production style at 1280x720 (the reference's window) under the
    hybrid LoD renderer, at the reference's default LoD band (magnified 400,
    minified 800; distances scaled to this scene by 4.0 / 226).  Two views:
    the close-up at the reference's default distance 226 (lod 0: strands
    only) and the band's middle, 600 (lod 0.5: strands at half coverage plus
    the raymarched volume's fragments).  Strand fragments come from the
    synthetic one-pixel-line rasterizer of workloads.strand_fragments (the
    strand rasterizer is not part of this library), in primitive order.
    Device time of the composite with its inputs resident (L2 flushed, the
    white background restored before each step, outside the timed region);
    e2e: the fragments uploaded from pinned memory, the raymarch, the
    composite and the image read back, serial, per frame."""
    import torch

    from vkhr_gb300 import _abi, _native, scene, workloads

    ctx = _native.Context(dev.index)
    s = stream.cuda_stream
    W, H = 1280, 720
    npix = W * H
    scale = 4.0 / 226.0
    n = res[0] * res[1] * res[2]
    dv = torch.from_numpy(st.vertices).to(dev)
    dt = torch.from_numpy(t).to(dev)
    di = torch.from_numpy(idx.view(np.int32)).to(dev)
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    dens = torch.empty(n, dtype=torch.uint8, device=dev)
    tq = torch.empty((n, 4), dtype=torch.int8, device=dev)
    ctx.voxelize_segments(dv.data_ptr(), dt.data_ptr(), di.data_ptr(), idx.shape[0], b, res, _abi.INDEX_REF_FP32,
                          counts.data_ptr(), dens.data_ptr(), tq.data_ptr(), s)
    ctx.normalize_densities(dens.data_ptr(), n, s)
    rgba = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    depth = torch.empty((H, W), dtype=torch.float32, device=dev)
    color = torch.empty((H, W), dtype=torch.int32, device=dev)
    hbm, peak_kind = peaks()
    reps = max(args.steps, 3)
    out = {"config": {"workload": "hybrid-LoD compositing of the production style (136,320 x 13) at 1280x720: "
                                  "synthetic one-pixel strand fragments in primitive order + the raymarched "
                                  "volume's fragments, resolved per pixel (16-node k-buffer + 1024 blended)",
                      "lod_band": [400.0, 800.0], "distance_scale": scale}}
    for name, distance in (("close", 226.0), ("hybrid", 600.0)):
        p = scene.make_params(b, res, W, H, camera_distance=distance * scale, raycast_steps=512.0,
                              renderer=_abi.RENDERER_HYBRID_LOD)
        p.magnified_distance, p.minified_distance = 400.0 * scale, 800.0 * scale
        lod = _native.level_of_detail(p.magnified_distance, p.minified_distance, p.look_at_distance)
        strands_on = _native.rasterizer_enabled(_abi.RENDERER_HYBRID_LOD, lod)
        volume_on = _native.raymarcher_enabled(_abi.RENDERER_HYBRID_LOD, lod)
        frags = workloads.strand_fragments(st.vertices, t, idx, p, lod, dev) if strands_on else \
            torch.zeros((0, 3), dtype=torch.int32, device=dev)
        F = frags.shape[0]
        vr, vd = (rgba.data_ptr(), depth.data_ptr()) if volume_on else (None, None)
        if volume_on:
            ctx.raymarch(p, dens.data_ptr(), tq.data_ptr(), None, rgba.data_ptr(), depth.data_ptr(), s)

        def composite():
            ctx.composite(frags.data_ptr() if F else None, F, W, H, color.data_ptr(), vr, vd, s)

        for _ in range(3):
            color.fill_(-1)
            composite()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, z in ev:
            flush.zero_()
            color.fill_(-1)
            a.record(stream)
            composite()
            z.record(stream)
        torch.cuda.synchronize()
        ms = sorted(a.elapsed_time(z) for a, z in ev)[reps // 2]
        ctx.set_profiling(True)
        for _ in range(reps):
            flush.zero_()
            color.fill_(-1)
            composite()
        torch.cuda.synchronize()
        kern = {}
        for kname, kms in ctx.profile():
            e = kern.setdefault(kname, [0, 0.0])
            e[0] += 1
            e[1] += kms
        ctx.set_profiling(False)
        ctx.check_status(s)
        changed = int(((color != -1).sum()).item())
        # e2e: upload the fragments, raymarch (when on), composite, read the image back
        hf = frags.cpu().pin_memory()
        hc = torch.empty((H, W), dtype=torch.int32).pin_memory()
        e2e = []
        for k in range(reps + 2):
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            color.fill_(-1)
            a.record(stream)
            frags.copy_(hf, non_blocking=True)
            if volume_on:
                ctx.raymarch(p, dens.data_ptr(), tq.data_ptr(), None, rgba.data_ptr(), depth.data_ptr(), s)
            composite()
            hc.copy_(color, non_blocking=True)
            z.record(stream)
            torch.cuda.synchronize()
            if k >= 2:
                e2e.append(a.elapsed_time(z))
        e2e_ms = sorted(e2e)[len(e2e) // 2]
        alg = F * 12 + npix * 8 + (npix * 20 if volume_on else 0)
        row = {"distance": distance, "lod": lod, "strand_fragments": F, "volume": bool(volume_on),
               "pixels_changed": changed, "ms": ms, "mfragments_per_s": F / ms / 1e3,
               "algorithmic_bytes": alg, "achieved_gbs": alg / ms / 1e6, "peak_gbs": hbm, "peak": peak_kind,
               "frac": alg / ms / 1e6 / hbm,
               "kernels": {k: {"launches": v[0], "avg_ms": v[1] / v[0]} for k, v in sorted(kern.items())},
               "e2e_ms": e2e_ms, "h2d_bytes_per_step": F * 12, "d2h_bytes_per_step": npix * 4}
        if not args.no_cpu_baseline:
            from oracle import oracle as O

            if not os.path.exists(O.LIB):
                O.build(with_reference=False)
            hfr = frags.cpu().numpy().view(_abi.FRAGMENT_DTYPE).reshape(-1)
            bg = np.full((H, W), 0xFFFFFFFF, dtype=np.uint32)
            vra = rgba.cpu().numpy() if volume_on else None
            vda = depth.cpu().numpy() if volume_on else None
            t0 = time.perf_counter()
            O.composite(hfr, bg, vra, vda)
            cpu_s = time.perf_counter() - t0
            row["cpu_baseline"] = {"value": F / cpu_s / 1e6, "unit": "Mfragments/s", "cores": O.max_threads(),
                                   "kind": "port", "sample": "the whole composite once (%.2f s)" % cpu_s}
        out[name] = row
        del frags, hf
    ctx.close()
    return out


RAY_AB = {
    "workload": "raymarch variants on three views: the production frame's 1920x1080 view of its normalized 256^3 "
                "volume (512 steps, 64-step shadows, 8-tap AO), the same from 4x the camera distance (a 74x80-pixel "
                "footprint), and a 3840x2160 view of the 512^3 scale volume (1024 steps, 128-step shadows, "
                "16-direction AO); workloads' Kajiya-Kay",
    "variants": {"0-3": "ray packets reading texels from L2/HBM (8x4, 16x2, 4x8, 8x4 at 64 registers)",
                 "4": "8x4 packets, each occupied density brick a warp's rays need staged into shared memory by one "
                      "TMA tensor copy",
                 "5": "8x4 packets sampling through the texture unit (3D array copy + hardware trilinear, "
                      "8-bit weights)",
                 "6": "variant 5's texture for the deep-shadow and AO samples only; the isosurface search reads "
                      "memory",
                 "7": "8x4 packets reading exact texels through the texture unit's 2x2 gathers (slices tiled into a "
                      "2D array, copied per call); the software trilinear filters them",
                 "8-10": "ray groups: 4 / 2 / 8 lanes per pixel take as many consecutive samples of its primary "
                         "march, shadow march and AO taps at once and replay them in order (4x2 / 4x4 / 2x2 pixels "
                         "per warp)"},
    "warm": "the volume L2-resident, as right after the voxelizer wrote it; cold: L2 flushed (512 MiB write) first",
}


def raymarch_ab_section(args, dev, stream, flush):
    """Time every raymarch variant on the headline view, a distant view and a 512^3 view."""
    import torch

    from vkhr_gb300 import _abi, _native, scene, strands

    s = stream.cuda_stream
    ctx = _native.Context(dev.index)
    views = {}
    st, t, idx = make_style()
    res = (WORKLOAD["resolution"],) * 3
    dv, dt, di = (torch.from_numpy(a).to(dev) for a in (st.vertices, t, idx.view(np.int32)))
    b = ctx.bounding_box(dv.data_ptr(), st.vertex_count, s)
    n = res[0] ** 3
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    dens = torch.empty(n, dtype=torch.uint8, device=dev)
    tq = torch.empty((n, 4), dtype=torch.int8, device=dev)
    ctx.voxelize_segments(dv.data_ptr(), dt.data_ptr(), di.data_ptr(), idx.shape[0], b, res, _abi.INDEX_REF_FP32,
                          counts.data_ptr(), dens.data_ptr(), tq.data_ptr(), s)
    ctx.normalize_densities(dens.data_ptr(), n, s)
    views["production 1920x1080, 256^3"] = (frame_params(b, res), dens, tq)
    far_p = scene.make_params(b, res, WORKLOAD["width"], WORKLOAD["height"], camera_distance=16.0,
                              raycast_steps=float(WORKLOAD["raycast_steps"]),
                              shadow_steps=float(WORKLOAD["shadow_steps"]), **scene.CONFIG_SHADING)
    views["production style from 4x the distance (74x80-pixel footprint)"] = (far_p, dens, tq)
    if not args.no_scale:
        sst = strands.hemisphere_style(1_048_576, 32, radius=1.2, step_length=0.04, seed=4)
        st_t = strands.generate_tangents(sst.vertices, sst.segments)
        s_idx = strands.generate_indices(sst.segments)
        r5 = (512, 512, 512)
        n5 = 512 ** 3
        v5, t5, i5 = (torch.from_numpy(a).to(dev) for a in (sst.vertices, st_t, s_idx.view(np.int32)))
        b5 = ctx.bounding_box(v5.data_ptr(), sst.vertex_count, s)
        c5 = torch.empty(n5, dtype=torch.int32, device=dev)
        d5 = torch.empty(n5, dtype=torch.uint8, device=dev)
        q5 = torch.empty((n5, 4), dtype=torch.int8, device=dev)
        ctx.voxelize_segments(v5.data_ptr(), t5.data_ptr(), i5.data_ptr(), s_idx.shape[0], b5, r5,
                              _abi.INDEX_REF_FP32, c5.data_ptr(), d5.data_ptr(), q5.data_ptr(), s)
        ctx.normalize_densities(d5.data_ptr(), n5, s)
        del v5, t5, i5, c5
        p5 = scene.make_params(b5, r5, 3840, 2160, camera_distance=5.0, raycast_steps=1024.0, shadow_steps=128.0,
                               ao_directions=16, **scene.CONFIG_SHADING)
        views["scale 3840x2160, 512^3"] = (p5, d5, q5)
    torch.cuda.synchronize()
    out = {"config": RAY_AB, "views": {}}
    for name, (p, d, q) in views.items():
        rgba = torch.empty((p.height, p.width, 4), dtype=torch.float32, device=dev)
        base = None
        rows = {}
        for v in range(_abi.RAYMARCH_VARIANTS):
            if args.variant >= 0 and v not in (0, args.variant):
                continue
            ctx.set_raymarch_variant(p.density_format, p.tangent_format, v)
            res_v = {}
            for mode in ("warm", "cold"):
                ms = []
                for k in range(max(args.warmup, 3) + max(args.steps, 5)):
                    if mode == "cold":
                        flush.zero_()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    ctx.raymarch(p, d.data_ptr(), q.data_ptr(), None, rgba.data_ptr(), None, s)
                    e1.record(stream)
                    torch.cuda.synchronize()
                    if k >= max(args.warmup, 3):
                        ms.append(e0.elapsed_time(e1))
                res_v[mode + "_ms"] = statistics.median(ms)
            ctx.set_profiling(True)
            ctx.raymarch(p, d.data_ptr(), q.data_ptr(), None, rgba.data_ptr(), None, s)
            torch.cuda.synchronize()
            res_v["kernels_warm_ms"] = {k_: round(m_, 4) for k_, m_ in ctx.profile()}
            ctx.set_profiling(False)
            img = rgba.clone()
            if base is None:
                base = img
            diff = (img - base).abs()
            res_v["max_diff_vs_variant0"] = float(diff.max().item())
            res_v["rms_diff_vs_variant0"] = float(diff.pow(2).mean().sqrt().item())
            rows[str(v)] = res_v
        ctx.set_raymarch_variant(p.density_format, p.tangent_format, 0)
        out["views"][name] = rows
    ctx.close()
    return out


def gb300_arm(args):
    import torch

    from vkhr_gb300 import _abi, _native, replicas, scene

    rank, world, local = replicas.world()
    torch.cuda.set_device(local)
    replicas.init("nccl")  # N replicas of the frame, one per GPU; no data-path collective

    ctx = _native.Context(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    if args.section == "scale":  # the scale workload alone (profiling runs)
        flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
        if rank == 0:
            print(json.dumps({"section": "scale", "scale": scale_section(args, dev, stream, flush)}))
        return 0
    if args.section == "schedule":  # the reference's benchmark schedule (opt-in)
        if rank == 0:
            print(json.dumps({"section": "schedule", "schedule": schedule_section(args, dev, stream)}))
        return 0
    if args.section == "diff":  # the differentiable workload alone (profiling runs)
        flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
        if rank == 0:
            print(json.dumps({"section": "diff", "diff": diff_section(args, dev, stream, flush)}))
        return 0
    if args.section == "composite":  # the compositing workload alone (profiling runs)
        flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
        if rank == 0:
            st, t, idx = make_style()
            res = (WORKLOAD["resolution"],) * 3
            dv = torch.from_numpy(st.vertices).to(dev)
            b = ctx.bounding_box(dv.data_ptr(), st.vertex_count, s)
            print(json.dumps({"section": "composite",
                              "composite": composite_section(args, dev, stream, flush, st, t, idx, b, res)}))
        return 0
    if args.section == "raymarch_ab":  # the raymarch variants' A/B (opt-in)
        flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
        if rank == 0:
            print(json.dumps({"section": "raymarch_ab", "raymarch_ab": raymarch_ab_section(args, dev, stream, flush)}))
        return 0
    if args.section == "batched":  # the multi-style comparison alone (profiling runs)
        flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
        out = batched_comparison(args, dev, stream, rank, world, flush)
        if rank == 0:
            print(json.dumps({"section": "batched", "batched": out}))
        return 0

    st, t, idx = make_style()
    res = (WORKLOAD["resolution"],) * 3
    n = res[0] * res[1] * res[2]
    W, H = WORKLOAD["width"], WORKLOAD["height"]
    dv = torch.from_numpy(st.vertices).to(dev)
    dt = torch.from_numpy(t).to(dev)
    di = torch.from_numpy(idx.view(np.int32)).to(dev)
    b = ctx.bounding_box(dv.data_ptr(), st.vertex_count, s)  # load-time, as in the reference
    counts = torch.empty(n, dtype=torch.int32, device=dev)
    dens = torch.empty(n, dtype=torch.uint8, device=dev)
    tq = torch.empty((n, 4), dtype=torch.int8, device=dev)
    rgba = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    depth = torch.empty((H, W), dtype=torch.float32, device=dev)
    p = frame_params(b, res)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    # two sets of device inputs and outputs (the streamed end-to-end loop below
    # double-buffers them; every other measurement uses set 0)
    ins = [(dv, dt, di), (torch.empty_like(dv), torch.empty_like(dt), torch.empty_like(di))]
    outs = [(rgba, depth), (torch.empty_like(rgba), torch.empty_like(depth))]

    def voxelize(i=0):
        v_, t_, i_ = ins[i]
        ctx.voxelize_segments(v_.data_ptr(), t_.data_ptr(), i_.data_ptr(), idx.shape[0], b, res, _abi.INDEX_REF_FP32,
                              counts.data_ptr(), dens.data_ptr(), tq.data_ptr(), s)
        ctx.normalize_densities(dens.data_ptr(), n, s)

    def raymarch(i=0):
        ctx.raymarch(p, dens.data_ptr(), tq.data_ptr(), None, outs[i][0].data_ptr(), outs[i][1].data_ptr(), s)

    for _ in range(max(args.warmup, 3)):
        flush.zero_()
        voxelize()
        raymarch()
    torch.cuda.synchronize()
    # the ray-packet variant for this view (vkhr_autotune_raymarch), kept in the context
    tuned, tuned_ms = ctx.autotune_raymarch(p, dens.data_ptr(), tq.data_ptr(), rgba.data_ptr(), s)
    # the one-walk kernel's resident CTAs per SM for this style (vkhr_autotune_voxelize), kept in the context
    vjob = _abi.VoxelJob()
    vjob.d_vertices, vjob.d_tangent_in, vjob.d_indices = dv.data_ptr(), dt.data_ptr(), di.data_ptr()
    vjob.item_count = int(idx.shape[0])
    vjob.bounds = b
    vjob.width, vjob.height, vjob.depth = res
    vjob.index_mode = _abi.INDEX_REF_FP32
    vjob.d_counts, vjob.d_densities, vjob.d_tangents = counts.data_ptr(), dens.data_ptr(), tq.data_ptr()
    walk, walk_ms = ctx.autotune_voxelize([vjob], s)
    for _ in range(2):  # back to the timed calls' own (unbudgeted) path
        flush.zero_()
        voxelize()
        raymarch()
    torch.cuda.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    replicas.barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launch_count()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        voxelize()
        ev[k][1].record(stream)
        raymarch()
        ev[k][2].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = ctx.launch_count() - launches0
    replicas.barrier()
    clocks.stop()
    vox_ms = [e[0].elapsed_time(e[1]) for e in ev]
    ray_ms = [e[1].elapsed_time(e[2]) for e in ev]
    step_ms = replicas.max_over_ranks(sum(vox_ms + ray_ms) / args.steps, device=dev)
    px = W * H
    value = world * px / (step_ms / 1e3) / 1e6

    # ---- per-kernel durations (event pair around each launch, same workload) ----
    ctx.set_profiling(True)
    for _ in range(args.steps):
        flush.zero_()
        voxelize()
        raymarch()
    torch.cuda.synchronize()
    prof = ctx.profile()
    ctx.set_profiling(False)
    per_kernel = {}
    for name, ms in prof:
        e = per_kernel.setdefault(name, [0, 0.0])
        e[0] += 1
        e[1] += ms
    hbm, peak_kind = peaks()
    # dominant kernel and its algorithmic bytes per launch
    top = max(per_kernel.items(), key=lambda kv: kv[1][1])
    top_name, (top_n, top_ms) = top[0], top[1]
    top_avg_ms = top_ms / top_n
    S = st.segment_count
    V = st.vertex_count
    # algorithmic (compulsory) bytes, each byte once: the inputs read (index
    # pairs 8 B per segment, vertices and tangents 12 B each per vertex) and
    # the outputs written (counts 4 B, u8 1 B, i8x4 tangents 4 B per voxel);
    # the visit entries, pair records and key scratch are the design's own
    # traffic (reported as ncu-measured `traffic`), not algorithmic bytes
    visits = int(counts.sum(dtype=torch.int64).item())
    R = WORKLOAD["resolution"]
    occupied = int(counts.view(R // 8, 8, R // 8, 8, R // 8, 8).amax(dim=(1, 3, 5)).gt(0).sum().item())
    covered = int((rgba != 0).any(dim=2).sum().item())  # image.cc:259-271: pixels not the background

    def alg_bytes_of(name):
        """Algorithmic bytes per launch of a kernel of the frame, by kernel family."""
        if "brick_kernel" in name:
            return 9 * 512 * occupied              # counts, u8, i8x4 of the occupied bricks
        if "zero_empty_kernel" in name:
            return 9 * (n - 512 * occupied)        # the same outputs of the unvisited bricks
        if name.startswith("(bin_kernel<false"):
            return 8 * S + 24 * V                  # index pairs, vertices and tangents read
        if "raymarch_kernel" in name:
            return n * 1 + n * 4 + px * 20         # u8 densities + i8x4 tangents + RGBA and depth out
        return None

    alg_bytes = alg_bytes_of(top_name)
    achieved = (alg_bytes / (top_avg_ms / 1e3) / 1e9) if alg_bytes else None
    roofline = {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": (achieved / hbm) if achieved else None,
                "traffic": next((v for k, v in TRAFFIC.items() if k in top_name), None),
                "peak_kind": peak_kind, "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": top_avg_ms,
                "visits": visits, "occupied_bricks": occupied}
    # whole stages against the same peak: inputs once + outputs once
    vox_alg = 24 * V + 8 * S + 9 * n
    ray_alg = n * 1 + n * 4 + px * 20
    vms, rms_ = sum(vox_ms) / args.steps, sum(ray_ms) / args.steps
    stages = {
        "voxelize": {"alg_bytes": vox_alg, "ms": vms, "achieved_gbs": vox_alg / (vms / 1e3) / 1e9,
                     "frac": vox_alg / (vms / 1e3) / 1e9 / hbm},
        "raymarch": {"alg_bytes": ray_alg, "ms": rms_, "achieved_gbs": ray_alg / (rms_ / 1e3) / 1e9,
                     "frac": ray_alg / (rms_ / 1e3) / 1e9 / hbm},
    }
    per_kernel_roofline = {}
    for name, (cnt, kms) in per_kernel.items():
        ab = alg_bytes_of(name)
        if ab:
            per_kernel_roofline[name] = {"alg_bytes": ab, "avg_ms": kms / cnt,
                                         "frac": ab / (kms / cnt / 1e3) / 1e9 / hbm}

    # ---- vertex mode: the same style by vertex counts (HairStyle::voxelize_vertices) ----
    vtimes = []
    for k in range(max(args.warmup, 3) + args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.voxelize_vertices(dv.data_ptr(), dt.data_ptr(), V, b, res, _abi.INDEX_REF_FP32, counts.data_ptr(),
                              dens.data_ptr(), tq.data_ptr(), s)
        e1.record(stream)
        torch.cuda.synchronize()
        if k >= max(args.warmup, 3):
            vtimes.append(e0.elapsed_time(e1))
    vertex_ms = statistics.median(vtimes)

    # ---- end to end through the C ABI with host buffers ------------------------
    hv = torch.from_numpy(st.vertices).pin_memory()
    ht = torch.from_numpy(t).pin_memory()
    hi = torch.from_numpy(idx.view(np.int32)).pin_memory()
    ho = torch.empty((H, W, 4), dtype=torch.float32).pin_memory()
    hd = torch.empty((H, W), dtype=torch.float32).pin_memory()
    e2e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps + 2):
        flush.zero_()
        if k >= 2:
            e2e_ev[k - 2][0].record(stream)
        dv.copy_(hv, non_blocking=True)
        dt.copy_(ht, non_blocking=True)
        di.copy_(hi, non_blocking=True)
        voxelize()
        raymarch()
        ho.copy_(rgba, non_blocking=True)
        hd.copy_(depth, non_blocking=True)
        if k >= 2:
            e2e_ev[k - 2][1].record(stream)
        torch.cuda.synchronize()
    e2e_serial_ms = sum(a.elapsed_time(b_) for a, b_ in e2e_ev) / args.steps
    h2d = hv.numel() * 4 + ht.numel() * 4 + hi.numel() * 4
    d2h = ho.numel() * 4 + hd.numel() * 4

    # Streamed, as a frame loop runs it: step k+1's inputs go up (one copy
    # stream) and step k-1's image comes down (another) while step k computes;
    # device inputs and outputs are double-buffered and every step's copies
    # lie inside the timed region, which spans all the steps.
    hos = [ho, torch.empty_like(ho).pin_memory()]
    hds = [hd, torch.empty_like(hd).pin_memory()]
    up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def streamed(K):
        in_ready = [torch.cuda.Event() for _ in range(K)]
        computed = [torch.cuda.Event() for _ in range(K)]
        copied = [torch.cuda.Event() for _ in range(K)]
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

        def upload(k):
            if k >= 2:
                up.wait_event(computed[k - 2])  # the step that read this input set is done
            with torch.cuda.stream(up):
                for d_, h_ in zip(ins[k % 2], (hv, ht, hi)):
                    d_.copy_(h_, non_blocking=True)
            in_ready[k].record(up)

        t0.record(stream)
        up.wait_stream(stream)
        upload(0)
        for k in range(K):
            if k + 1 < K:
                upload(k + 1)
            stream.wait_event(in_ready[k])
            if k >= 2:
                stream.wait_event(copied[k - 2])  # this output set has been read back
            voxelize(k % 2)
            raymarch(k % 2)
            computed[k].record(stream)
            down.wait_event(computed[k])
            with torch.cuda.stream(down):
                hos[k % 2].copy_(outs[k % 2][0], non_blocking=True)
                hds[k % 2].copy_(outs[k % 2][1], non_blocking=True)
            copied[k].record(down)
        stream.wait_event(copied[K - 1])
        t1.record(stream)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / K

    # a frame loop's steady state: at least 40 frames, so that the pipeline's fill (the
    # first upload) and drain (the last read-back) are a small part of the time per frame
    e2e_frames = max(args.steps, 40)
    streamed(3)  # warm-up
    e2e_ms = replicas.max_over_ranks(streamed(e2e_frames), device=dev)

    batched = None if (args.no_batched or args.section == "frame") else batched_comparison(
        args, dev, stream, rank, world, flush)
    frame_graph = None if (args.section == "frame" or world > 1) else frame_graph_section(
        args, dev, stream, flush, st, t, idx, b, res, p)
    scale = None if (args.no_scale or args.section == "frame" or world > 1) else scale_section(args, dev, stream, flush)
    diff = None if (args.no_diff or args.section == "frame" or world > 1) else diff_section(args, dev, stream, flush)
    composite = None if (args.no_composite or args.section == "frame" or world > 1) else composite_section(
        args, dev, stream, flush, st, t, idx, b, res)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": WORKLOAD,
        "components": {
            "voxelize_ms": sum(vox_ms) / args.steps, "raymarch_ms": sum(ray_ms) / args.steps,
            "voxelize_msegments_per_s": S / (sum(vox_ms) / args.steps / 1e3) / 1e6,
            "raymarch_mpixels_per_s": px / (sum(ray_ms) / args.steps / 1e3) / 1e6,
            "covered_pixels": covered,
            "raymarch_covered_mpixels_per_s": covered / (sum(ray_ms) / args.steps / 1e3) / 1e6,
            "voxelize_vertices_ms": vertex_ms,
            "voxelize_vertices_mvertices_per_s": V / (vertex_ms / 1e3) / 1e6,
            "wall_ms_per_step_incl_flush": wall * 1e3 / args.steps,
        },
        "kernels": {k: {"launches": v[0], "avg_ms": v[1] / v[0]} for k, v in sorted(per_kernel.items())},
        "roofline": roofline,
        "roofline_stages": stages,
        "roofline_kernels": per_kernel_roofline,
        "e2e": {"value": world * px / (e2e_ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "copies": "streamed: step k+1's upload and step k-1's read-back overlap step k's compute "
                          "(double-buffered device inputs and outputs, one copy stream each way); the timed "
                          "region spans all the frames, from the first upload to the last read-back",
                "frames": e2e_frames,
                "serial_ms_per_step": e2e_serial_ms,
                "serial_value": world * px / (e2e_serial_ms / 1e3) / 1e6},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "autotune": {"voxelize_walk_ctas_per_sm": walk,
                     "walk_ms": {str(k): round(m, 4) for k, m in zip(_abi.WALK_CHOICES, walk_ms)},
                     "raymarch_variant": tuned, "variant_ms": tuned_ms,
                     "variants": ["8x4 tiles", "16x2 tiles", "4x8 tiles", "8x4 tiles, 64 registers",
                                  "8x4 tiles, density bricks staged in shared memory by TMA",
                                  "8x4 tiles, density through the texture unit (not tuned: 8-bit filter weights)",
                                  "8x4 tiles, shadow and AO samples through the texture unit (not tuned)",
                                  "8x4 tiles, exact texels by texture gathers"]},
    }
    if batched is not None:
        line["batched_speedup_vs_plain"] = round(batched["speedup_vs_plain"]["batched_graph"], 3)
    if diff is not None:
        line["adjoint_over_forward"] = round(diff["adjoint_over_forward_K16"], 3)
    if scale is not None:
        line["scale_frame_ms"] = round(scale["ms"]["voxelize"] + scale["ms"]["normalize"] + scale["ms"]["raymarch"], 3)
    if batched is not None:
        line["batched"] = batched
    if frame_graph is not None:
        line["frame_graph"] = frame_graph
    if scale is not None:
        line["scale"] = scale
    if diff is not None:
        line["diff"] = diff
    if composite is not None:
        line["composite"] = composite
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O

        if not os.path.exists(O.LIB):
            O.build(with_reference=False)
        a, r = cpu_frame(O, st, t, idx, b)
        line["cpu_baseline"] = {
            "value": px / (a + r) / 1e6, "unit": UNIT, "cores": O.max_threads(), "kind": "port",
            "sample": "one whole frame: the serial voxelization + normalize (%.2f s) and the FP32 raymarch of all "
                      "1920x1080 pixels, all threads (%.2f s)" % (a, r)}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 16-style batched vs plain comparison")
    ap.add_argument("--no-scale", action="store_true", help="skip the 512^3 scale workload")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiable workload")
    ap.add_argument("--no-composite", action="store_true", help="skip the hybrid-LoD compositing workload")
    ap.add_argument("--variant", type=int, default=-1,
                    help="raymarch_ab: time only variant 0 and this raymarch variant (profiling runs)")
    ap.add_argument("--section", default="all",
                    choices=["all", "frame", "batched", "scale", "diff", "schedule", "composite", "raymarch_ab"],
                    help="frame: the production frame only; batched: the multi-style comparison only; "
                         "scale: the 512^3 workload only; diff: the differentiable workload only; "
                         "composite: the hybrid-LoD compositing only; raymarch_ab: the raymarch variants' A/B")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    return gb300_arm(args)


if __name__ == "__main__":
    sys.exit(main())
