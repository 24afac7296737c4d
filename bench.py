#!/usr/bin/env python3
"""Benchmark of the volumetric level-of-detail path on GB300.

One step = one frame of the path at production size: segment-voxelize a
136,320-strand x 13-vertex style (1,635,840 segments, grown procedurally:
roots on a 0.3-radius disk tilted 30 degrees, 12 steps of 0.08) into a
256^3 grid (uint32 counts, u8 densities, int8 tangents), normalize the
densities, then raymarch a 1920x1080 view with 512 steps, 64-step density
shadows and 8-tap ambient occlusion.

`value` is frame throughput in Mpixels/s (1920*1080 / step time) with the
inputs resident in HBM; the per-stage rates (Msegments/s voxelized, Mpixels/s
raymarched) are reported beside it.  L2 is flushed (a 512 MiB write) before
every timed step.  `e2e` repeats the step through the C ABI with host
buffers: the H2D copy of the strand arrays from pinned memory and the D2H
read of the frame (RGBA + depth) are inside the timed region.

--impl reference times the reference's CPU algorithm for the same frame on
the host cores (the oracle's restatement of HairStyle::voxelize_segments,
serial as in the reference, plus the FP32 raymarch of volume.frag on a
sample of rows, all threads).
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
                "256^3, raymarched at 1920x1080, 512 steps, 64-step shadows, 8-tap AO",
    "strands": 136_320,
    "vertices_per_strand": 13,
    "resolution": 256,
    "width": 1920,
    "height": 1080,
    "raycast_steps": 512,
    "shadow_steps": 64,
    "ao_taps": 8,
    "density": "u8 unorm (normalized)",
    "l2": "flushed before every timed step (512 MiB write)",
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


def cpu_frame(O, st, t, idx, b, rows_sample):
    """One CPU frame: the serial voxelizer + normalize, then the FP32 raymarch
    on `rows_sample` evenly spread rows (all threads); returns seconds for a
    full frame (raymarch time scaled by H / rows)."""
    from vkhr_gb300 import scene

    res = (WORKLOAD["resolution"],) * 3
    t0 = time.perf_counter()
    _, d, tq, _ = O.voxelize("segments", st.vertices, t, idx, b, res)
    dn = O.normalize(d)
    t1 = time.perf_counter()
    p = scene.make_params(b, res, WORKLOAD["width"], WORKLOAD["height"], raycast_steps=float(WORKLOAD["raycast_steps"]),
                          shadow_steps=float(WORKLOAD["shadow_steps"]))
    H = WORKLOAD["height"]
    rows = np.linspace(0, H - 1, rows_sample).astype(int)
    t2 = time.perf_counter()
    for r in rows:
        O.raymarch(p, dn, tq, precision="f32", rows=(int(r), int(r) + 1))
    t3 = time.perf_counter()
    return (t1 - t0), (t3 - t2) * H / len(rows)


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
    rows = 36
    for _ in range(args.warmup):
        cpu_frame(O, st, t, idx, b, rows)
    vox, ray = [], []
    for _ in range(args.steps):
        a, r = cpu_frame(O, st, t, idx, b, rows)
        vox.append(a)
        ray.append(r)
    step_s = (sum(vox) + sum(ray)) / args.steps
    px = WORKLOAD["width"] * WORKLOAD["height"]
    value = px / step_s / 1e6
    cores = O.max_threads()
    sample = ("per step: the full serial voxelization (1,635,840 segments -> 256^3) + normalize, and the FP32 "
              "raymarch of %d of 1080 evenly spread rows, scaled to the frame" % rows)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": WORKLOAD,
        "components": {"voxelize_msegments_per_s": st.segment_count / (sum(vox) / args.steps) / 1e6,
                       "raymarch_mpixels_per_s": px / (sum(ray) / args.steps) / 1e6},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


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
    p = scene.make_params(b, res, W, H, raycast_steps=float(WORKLOAD["raycast_steps"]),
                          shadow_steps=float(WORKLOAD["shadow_steps"]))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def voxelize():
        ctx.voxelize_segments(dv.data_ptr(), dt.data_ptr(), di.data_ptr(), idx.shape[0], b, res, _abi.INDEX_REF_FP32,
                              counts.data_ptr(), dens.data_ptr(), tq.data_ptr(), s)
        ctx.normalize_densities(dens.data_ptr(), n, s)

    def raymarch():
        ctx.raymarch(p, dens.data_ptr(), tq.data_ptr(), None, rgba.data_ptr(), depth.data_ptr(), s)

    for _ in range(max(args.warmup, 3)):
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
    visits = None
    alg = {
        # read voxel-space stepping inputs once (index pairs + both vertices per pair), update counts
        "count_segments_kernel": 8 * S + 24 * S + 4 * n,
        "fill_segments_kernel": 8 * S + 24 * S + 4 * n,
        "resolve_kernel": 4 * n + 4 * n + n + 4 * n,
        "(raymarch_kernel<DF, TF>)": n * 1 + n * 4 + px * 20,
        "alloc_ranges_kernel": 8 * n,
    }
    alg_bytes = alg.get(top_name)
    achieved = (alg_bytes / (top_avg_ms / 1e3) / 1e9) if alg_bytes else None
    roofline = {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": (achieved / hbm) if achieved else None, "traffic": None, "peak_kind": peak_kind,
                "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": top_avg_ms}

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
    e2e_ms = sum(a.elapsed_time(b_) for a, b_ in e2e_ev) / args.steps
    h2d = hv.numel() * 4 + ht.numel() * 4 + hi.numel() * 4
    d2h = ho.numel() * 4 + hd.numel() * 4

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": dict(WORKLOAD, parallelism="replicas" if world > 1 else "single"),
        "components": {
            "voxelize_ms": sum(vox_ms) / args.steps, "raymarch_ms": sum(ray_ms) / args.steps,
            "voxelize_msegments_per_s": S / (sum(vox_ms) / args.steps / 1e3) / 1e6,
            "raymarch_mpixels_per_s": px / (sum(ray_ms) / args.steps / 1e3) / 1e6,
            "wall_ms_per_step_incl_flush": wall * 1e3 / args.steps,
        },
        "kernels": {k: {"launches": v[0], "avg_ms": v[1] / v[0]} for k, v in sorted(per_kernel.items())},
        "roofline": roofline,
        "e2e": {"value": world * px / (e2e_ms / 1e3) / 1e6, "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O

        if not os.path.exists(O.LIB):
            O.build(with_reference=False)
        rows = 36
        a, r = cpu_frame(O, st, t, idx, b, rows)
        line["cpu_baseline"] = {
            "value": px / (a + r) / 1e6, "unit": UNIT, "cores": O.max_threads(), "kind": "port",
            "sample": "one frame: the full serial voxelization + normalize (%.2f s) and the FP32 raymarch of %d of "
                      "1080 rows scaled to the frame (%.2f s)" % (a, rows, r)}
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
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    return gb300_arm(args)


if __name__ == "__main__":
    sys.exit(main())
