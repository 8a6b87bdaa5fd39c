#!/usr/bin/env python
"""Benchmark of the batched adaptive-precision point rasterizer on GB300.

Workload (default): 1,000,000,000 synthetic terrain points over 10 x 10 km in
the LAS-derived batched layout, one 1920x1080 view from the reference's
zoom-to-cloud pose (src/main.cpp:251-270).  One step = one frame: cull +
raster + resolve (+ re-clear), the dispatch sequence of
compute_loop_las.h:117-304.  `value` is Gpoints/s with the cloud resident in
HBM; `e2e` is the same frame through the C ABI with the cloud in pinned host
memory (the kernels read each visible batch's words across the link) and the
RGBA8 image copied back every step; `e2e.upload` uploads every stream first.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = dict(name="terrain_1b_1080p", points=1_000_000_000, extent=10_000.0, seed=1,
                width=1920, height=1080)
CPU_SAMPLE_POINTS = 32_000_000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--points", type=int, default=WORKLOAD["points"])
    ap.add_argument("--payload", default="color", choices=["color", "index"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--cpu-table", action="store_true",
                    help="time the oracle per workload on this host's cores and exit")
    ap.add_argument("--serving", default="quick", choices=["quick", "full", "off"])
    ap.add_argument("--extras", default="payloads,multiview,configs,serving,ingest,potree",
                    help="comma list of extra workloads after the headline frame")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def camera(box_min, box_max, width, height):
    from compute_rasterizer_gb300 import synth
    yaw, pitch, radius, target = synth.zoom_to_cloud(box_min, box_max)
    view = synth.orbit_view(yaw, pitch, radius, target)
    proj = synth.perspective(60.0, width / height, 0.1, 200000.0)
    return view, proj


class Clocks:
    """nvidia-smi samples (SM clock, throttle reasons) while the timed region runs."""

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.1)
        self.p.terminate()
        self.p.wait()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_sample(points_full: int, extent_full: float, seed: int, sample: int):
    """A bounded sample of the workload for the CPU: the central square of the
    same terrain (same seed, noise wavelength and point density), Morton-sorted
    and encoded on the host, viewed by the full cloud's camera."""
    from compute_rasterizer_gb300 import _lib as L
    from compute_rasterizer_gb300 import synth
    ext = extent_full * (sample / points_full) ** 0.5
    p = synth.synth_params(L.SYNTH_TERRAIN, ext, seed, wavelength=extent_full / 4.0)
    p.origin[0] = p.origin[1] = 0.5 * (extent_full - ext)
    rec, hdr = synth.las_records_host(p, sample)
    enc = encode_parallel(rec, sample, hdr)
    return p, hdr, enc, ext


def encode_parallel(rec, n, hdr, threads=None):
    """The oracle's loadLas restatement (or_encode_las) over batch-aligned
    chunks on host threads (ctypes drops the GIL): the CPU legs encode with the
    oracle, not with the product's host encoder."""
    import concurrent.futures as cf

    from compute_rasterizer_gb300 import _lib as L
    from oracle import oracle as O
    lib = O.lib()
    nb = -(-n // 10240)
    batches = np.zeros(nb, L.BATCH_DTYPE)
    st = [np.zeros(n, np.uint32) for _ in range(4)]
    sc, of, mn = (np.ascontiguousarray(x[:], np.float64) for x in (hdr.scale, hdr.offset, hdr.min))
    threads = threads or os.cpu_count() or 1
    per = max(1, -(-nb // threads))

    def job(k):
        b0, b1 = k * per, min(nb, (k + 1) * per)
        if b0 >= b1:
            return 0
        p0, p1 = b0 * 10240, min(n, b1 * 10240)
        lib.or_encode_las(rec.ctypes.data + p0 * 26, p1 - p0, 26, 2, sc.ctypes.data,
                          of.ctypes.data, mn.ctypes.data, p0, 0, batches.ctypes.data + b0 * 64,
                          *(s.ctypes.data + p0 * 4 for s in st))
        return 0
    with cf.ThreadPoolExecutor(threads) as ex:
        assert all(r == 0 for r in ex.map(job, range(threads)))
    return (batches, *st)


def time_oracle(frame, enc, n, threads, min_seconds=0.0, steps=1, warmup=0):
    from oracle import oracle as O
    batches, lo, md, hi, rgba = enc
    lo, md, hi, rgba = (O.pad_stream(x) for x in (lo, md, hi, rgba))
    fb = np.empty(O.fb_words(frame.width, frame.height), np.uint64)
    lib = O.lib()
    b = np.ascontiguousarray(batches)

    def one():
        fb.fill(0xFF800000FF800000)
        lib.or_raster_batched_mt(C.byref(frame), b.ctypes.data, len(b), n, lo.ctypes.data,
                                 md.ctypes.data, hi.ctypes.data, rgba.ctypes.data, fb.ctypes.data,
                                 threads)
    for _ in range(warmup):
        one()
    t0 = time.perf_counter()
    frames = 0
    while frames < steps or time.perf_counter() - t0 < min_seconds:
        one()
        frames += 1
    dt = time.perf_counter() - t0
    return dt / frames, frames


def reference_arm(args, world, rank):
    """--impl reference: the oracle (the reference's CPU restatement) on the host cores,
    in its literal arithmetic mode: the shader math evaluated as the GLSL
    source writes it, the mode pinned bit for bit to the reference's shaders
    compiled as C++ (tests/test_cpu_shader_pin.py)."""
    if rank != 0:
        return
    from oracle import oracle as O
    O.lib().or_set_arith(O.ARITH_LITERAL)
    n_full = args.points
    s = min(CPU_SAMPLE_POINTS, n_full)
    p, hdr, enc, ext = cpu_sample(n_full, WORKLOAD["extent"], WORKLOAD["seed"], s)
    full_min = np.array([0.0, 0.0, hdr.min[2]])
    full_max = np.array([WORKLOAD["extent"], WORKLOAD["extent"], hdr.max[2]])
    view, proj = camera(full_min, full_max, WORKLOAD["width"], WORKLOAD["height"])
    payload = O.PAYLOAD_COLOR if args.payload == "color" else O.PAYLOAD_INDEX
    fr = O.make_frame(view, proj, WORKLOAD["width"], WORKLOAD["height"], np.array(hdr.min[:])[None],
                      1, O.L0_X12, payload)
    cores = os.cpu_count() or 1
    per_frame, frames = time_oracle(fr, enc, s, cores, steps=args.steps, warmup=min(args.warmup, 3))
    v = s / per_frame / 1e9
    sample = (f"{s:,} points: the central {ext:.0f} m square of the same 10 km terrain at the "
              f"same density, same camera; oracle (literal arithmetic) {args.steps} frames")
    out = {"impl": "reference", "metric": metric_name(), "value": round(v, 4),
           "unit": "Gpoints/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(per_frame * 1e3, 3), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+u64", "data": "synthetic",
           "config": config_dict(args),
           "cpu_baseline": {"value": round(v, 4), "unit": "Gpoints/s", "cores": cores,
                            "kind": "port", "sample": sample},
           "e2e": {"value": round(v, 4), "unit": "Gpoints/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def cpu_table(args):
    """--cpu-table: the oracle (the reference's CPU restatement) per workload on
    this host's cores, 1 thread and all threads where the oracle has both, on
    bounded samples of each workload; one JSON line.  A host-only run."""
    from compute_rasterizer_gb300 import _lib as L
    from compute_rasterizer_gb300 import synth, workloads
    from oracle import oracle as O
    cores = os.cpu_count() or 1

    def rate(fn, points, min_s=3.0):
        fn()
        t0, k = time.perf_counter(), 0
        while k < 1 or time.perf_counter() - t0 < min_s:
            fn()
            k += 1
        return round(points * k / (time.perf_counter() - t0) / 1e9, 4)

    out = {}
    # plain 16 B path, 4,194,304 points at 1920x1080 (single-threaded oracle)
    n1, W1, H1 = 4_194_304, 1920, 1080
    v = synth.uniform_vertices_host(1, n1, 100.0)
    cam1 = synth.look_at([150.0, 150.0, 150.0], [50.0, 50.0, 50.0], [0.0, 0.0, 1.0])
    proj1 = synth.perspective(60.0, W1 / H1, 0.1, 1000.0)
    out["plain_4m_1080p"] = {"threads_1": rate(lambda: O.plain(cam1, proj1, W1, H1, v), n1),
                             "sample": "the full workload"}

    def batched(points_full, extent, seed, sample, cams, own_bounds=False):
        p, hdr, enc, ext = cpu_sample(points_full, extent, seed, sample)
        # streams padded once (the oracle's calls copy unpadded streams every frame)
        enc = (enc[0], *(O.pad_stream(x, n=sample) for x in enc[1:]))
        fmin = np.array(hdr.min[:]) if own_bounds else np.array([0.0, 0.0, hdr.min[2]])
        fmax = np.array(hdr.max[:]) if own_bounds else np.array([extent, extent, hdr.max[2]])
        r1, rn = [], []
        for view, proj, w, h in cams(fmin, fmax):
            fr = O.make_frame(view, proj, w, h, np.array(hdr.min[:])[None], 1, O.L0_X12,
                              O.PAYLOAD_COLOR)
            r1.append(rate(lambda: O.raster_batched(fr, enc[0], sample, *enc[1:]), sample, 1.0))
            rn.append(rate(lambda: O.raster_batched(fr, enc[0], sample, *enc[1:], threads=cores),
                           sample, 1.0))
        return r1, rn, ext, enc, hdr, fmin, fmax

    def main_cam(fmin, fmax):
        view, proj = camera(fmin, fmax, WORKLOAD["width"], WORKLOAD["height"])
        return [(view, proj, WORKLOAD["width"], WORKLOAD["height"])]

    s2 = 8_000_000
    r1, rn, ext, _, _, _, _ = batched(100_000_000, 1000.0, 2, s2, workloads.flight_path, True)
    out["flight_100m_1440p"] = {"threads_1": round(float(np.mean(r1)), 4),
                                f"threads_{cores}": round(float(np.mean(rn)), 4),
                                "sample": f"{s2:,} points, the central {ext:.0f} m square at the "
                                          "same density, the 5 flight poses laid over the sample"}
    s3 = CPU_SAMPLE_POINTS
    r1, rn, ext, enc, hdr, fmin, fmax = batched(WORKLOAD["points"], WORKLOAD["extent"],
                                                WORKLOAD["seed"], s3, main_cam)
    out["terrain_1b_1080p"] = {"threads_1": r1[0], f"threads_{cores}": rn[0],
                               "sample": f"{s3:,} points, the central {ext:.0f} m square at the "
                                         "same density, the same camera"}
    (view, proj, w, h), = main_cam(fmin, fmax)
    fr = O.make_frame(view, proj, w, h, np.array(hdr.min[:])[None], 1, O.L0_X12, O.PAYLOAD_INDEX)
    out["terrain_1b_1080p_hqs"] = {"threads_1": rate(lambda: O.hqs(fr, enc[0], s3, *enc[1:]), s3),
                                   "sample": out["terrain_1b_1080p"]["sample"]}
    print(json.dumps({"cpu_table": out, "cores": cores, "unit": "Gpoints/s",
                      "kind": "port (the oracle)"}), flush=True)


def max_over_ranks(value: float, device: str = "cuda") -> float:
    """The slowest rank's value: every rank passes its own, all get the max."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def metric_name():
    return "Gpoints/s at 1B points (frame = cull + raster + resolve)"


def config_dict(args):
    return {"workload": WORKLOAD["name"], "points": args.points, "extent_m": WORKLOAD["extent"],
            "width": WORKLOAD["width"], "height": WORKLOAD["height"], "method": "loop_las",
            "payload": args.payload, "view": "zoom-to-cloud orbit pose (yaw 0.53, pitch -0.68)",
            "l2": "no flush: inputs (8-16 GB) exceed the 129 MB L2",
            "parallelism": f"replicas x{args.gpus}"}


def main():
    args = parse()
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.cpu_table:
        cpu_table(args)
        return
    if args.impl == "reference":
        reference_arm(args, world, rank)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    import torch

    import compute_rasterizer_gb300 as cr
    from compute_rasterizer_gb300 import _lib as L
    from compute_rasterizer_gb300 import synth

    torch.cuda.set_device(local)
    ctx = cr.Context(local)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    n = args.points
    W, H = WORKLOAD["width"], WORKLOAD["height"]
    sp = synth.synth_params(L.SYNTH_TERRAIN, WORKLOAD["extent"], WORKLOAD["seed"] + rank)
    cloud, hdr, build_ms = synth.build_cloud_device_timed(ctx, sp, n, sh)
    bmin, bmax = np.array(hdr.min[:]), np.array(hdr.max[:])
    view, proj = camera(bmin, bmax, W, H)
    cv = cr.make_view(view, proj, W, H)
    payload = L.PAYLOAD_COLOR if args.payload == "color" else L.PAYLOAD_INDEX
    params = cr.default_params(L.METHOD_LOOP_LAS, payload=payload)
    fb = ctx.framebuffer(W, H)
    fb.clear(stream=sh)

    def frames(k):
        for _ in range(k):
            ctx.render(cloud, cv, params, fb, sh)

    frames(max(3, args.warmup))
    ctx.sync(sh)
    stats = ctx.frame_stats(cloud, params)
    clocks = Clocks(local)
    frames(20)  # keep the GPU loaded while the sampler starts
    ctx.timing_enable(args.steps)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    frames(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    elapsed = e0.elapsed_time(e1) / 1e3
    clk = clocks.stop()
    if world > 1:
        elapsed = max_over_ranks(elapsed, "cuda")
        dist.barrier()
    ctx.sync(sh)
    raster_ms = ctx.timing_read(L.STAGE_RASTER, args.steps)
    cull_ms = ctx.timing_read(L.STAGE_CULL, args.steps)
    resolve_ms = ctx.timing_read(L.STAGE_RESOLVE, args.steps)
    ctx.timing_enable(0)
    frame_s = elapsed / args.steps
    value = world * n / frame_s / 1e9
    peak, peak_kind = measured_peaks()
    raster_s = float(np.mean(raster_ms)) / 1e3
    achieved = stats.stream_bytes / raster_s / 1e9
    # DRAM bytes per launch: the ncu traffic / algorithmic ratio of the color
    # raster (profiles/raster_terrain_1b_traffic.json) times this launch's
    # algorithmic bytes (the traffic grows with the bytes streamed)
    prof = ROOT / "profiles" / "raster_terrain_1b_traffic.json"
    ratio = json.loads(prof.read_text()).get("traffic_over_algorithmic") if prof.exists() else None
    traffic = (int(round(ratio * stats.stream_bytes))
               if ratio and args.payload == "color" else None)

    out = {"metric": metric_name(), "value": round(value, 3), "unit": "Gpoints/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(frame_s * 1e3, 4), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+u64", "data": "synthetic",
           "config": config_dict(args),
           "roofline": {"bound": "hbm", "kernel": "k_batched (raster)",
                        "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                        "traffic": traffic,
                        "algorithmic_bytes_per_launch": int(stats.stream_bytes),
                        "raster_ms": round(raster_s * 1e3, 4)},
           "stages_ms": {"cull": round(float(np.mean(cull_ms)), 4),
                         "raster": round(raster_s * 1e3, 4),
                         "resolve": round(float(np.mean(resolve_ms)), 4)},
           "frame_stats": {"batches_visible": int(stats.batches_visible),
                           "batches_dispatched": int(stats.batches_dispatched),
                           "points_per_level": list(stats.points_per_level)},
           "gpu_launches": 4 * args.steps,  # cull, raster list 1, raster list 0, resolve
           "clocks": clk}

    if not args.no_extras:
        out["extras"] = {"cloud_build": {
            "points": n, "ms": build_ms,
            "what": "GPU generator (LAS records) -> Morton sort (radix sort + gather) -> "
                    "LAS-derived layout encoder, CUDA events per stage; outside the timed frames"}}
        want = set(args.extras.split(","))
        runs = [("payloads", lambda: extras(ctx, cloud, cv, fb, sh, n, args)),
                ("multiview", lambda: {"multiview_64": multiview_64(ctx, sh, args.steps, payload)}),
                ("configs", lambda: small_configs(ctx, sh, args, payload)),
                ("ingest", lambda: {"ingest": ingest(ctx, sh)}),
                ("potree", lambda: {"potree_loop_nodes": potree_nodes(ctx, sh, args.steps)})]
        if args.serving != "off":
            runs.append(("serving", lambda: {"serving": serving(ctx, sh, args, payload)}))
        for name, fn in runs:
            if name not in want:
                continue
            try:
                out["extras"].update(fn())
            except Exception as exc:  # the headline line is printed regardless
                out["extras"][name] = {"error": repr(exc)}
    if not args.no_e2e:
        out["e2e"] = e2e(ctx, cloud, cv, params, fb, sh, n, args, bmin)
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args, view, proj)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def extras(ctx, cloud, cv, fb, sh, n, args):
    """The same frame with the index payload (loop_las as registered), HQS,
    and the color payload under CR_QUIRK_LITERAL_ARITH, timed with CUDA
    events; HQS also per pass, with its roofline fraction."""
    import torch

    import compute_rasterizer_gb300 as cr
    from compute_rasterizer_gb300 import _lib as L
    stream = torch.cuda.ExternalStream(sh)
    peak, _ = measured_peaks()
    res = {}
    k = max(5, min(args.steps, 50))
    for name, method, payload, kind in (("index_payload", L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX, L.FB_U64),
                                        ("hqs", L.METHOD_LOOP_LAS_HQS, L.PAYLOAD_INDEX, L.FB_HQS)):
        f = ctx.framebuffer(fb.W, fb.H, kind)
        f.clear(0xFF800000 if kind == L.FB_HQS else L.DEFAULT_CLEAR, stream=sh)
        p = cr.default_params(method, payload=payload)
        for _ in range(3):
            ctx.render(cloud, cv, p, f, sh)
        ctx.sync(sh)
        ctx.timing_enable(k)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            ctx.render(cloud, cv, p, f, sh)
        e1.record(stream)
        ctx.sync(sh)
        ms = e0.elapsed_time(e1) / k
        r = {"ms_per_frame": round(ms, 4), "gpoints_per_s": round(n / ms / 1e6, 3)}
        stages = {"cull": L.STAGE_CULL, "raster": L.STAGE_RASTER, "resolve": L.STAGE_RESOLVE}
        if kind == L.FB_HQS:
            stages = {"cull": L.STAGE_CULL, "depth_pass": L.STAGE_RASTER,
                      "color_pass": L.STAGE_HQS_COLOR, "resolve": L.STAGE_RESOLVE}
        r["stages_ms"] = {s: round(float(np.mean(ctx.timing_read(v, k))), 4) for s, v in stages.items()}
        ctx.timing_enable(0)
        st = ctx.frame_stats(cloud, p)
        P = fb.W * fb.H
        # stream words of both passes + depth/accumulator clear, resolve read, image write
        fbytes = int(st.stream_bytes) + (20 * P + 20 * P + 4 * P if kind == L.FB_HQS else 20 * P + 4 * P)
        r["algorithmic_bytes"] = fbytes
        r["frac_of_measured_hbm"] = round(fbytes / ms / 1e6 / peak, 4)
        res[name] = r
        f.close()
    # the same color frame with CR_QUIRK_LITERAL_ARITH (the shader math as the
    # GLSL source writes it: no fused decode / projection, two correctly
    # rounded divisions per point), identical to the reference's shaders
    # compiled as C++
    f = ctx.framebuffer(fb.W, fb.H, L.FB_U64)
    f.clear(L.DEFAULT_CLEAR, stream=sh)
    p = cr.default_params(L.METHOD_LOOP_LAS, payload=L.PAYLOAD_COLOR,
                          quirks=L.QUIRK_L0_X12 | L.QUIRK_LITERAL_ARITH)
    for _ in range(3):
        ctx.render(cloud, cv, p, f, sh)
    ctx.sync(sh)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(k):
        ctx.render(cloud, cv, p, f, sh)
    e1.record(stream)
    ctx.sync(sh)
    ms = e0.elapsed_time(e1) / k
    res["literal_arith"] = {"ms_per_frame": round(ms, 4), "gpoints_per_s": round(n / ms / 1e6, 3),
                            "what": "the headline frame (color payload) with CR_QUIRK_LITERAL_ARITH"}
    f.close()
    return res


def ingest(ctx, sh, points=50_000_000):
    """File ingest (LasLoaderSparse.cpp:477-713 with loadLas / loadLaz): a
    Morton-sorted terrain of `points` format-2 records (generated and sorted on
    the GPU, read back) written as LAS bytes in host memory and as LAZ by the
    product's writer; each loaded into a cloud through the C ABI (host
    records -> load tasks -> GPU encoder; LAZ: parallel chunk decode on all host
    threads overlapping upload and encode).  Wall-clock, one run each after a
    warm-up on a small file; the two clouds are compared word for word."""
    import ctypes as C
    import os
    import time

    import torch

    from compute_rasterizer_gb300 import _lib as L
    from compute_rasterizer_gb300 import las, synth
    lib = L.load()
    n, bpp = points, L.LAS_FORMAT2_BYTES
    p = synth.synth_params(L.SYNTH_TERRAIN, 3000.0, 77)
    hdr = L.LasHeader()
    rec_d = torch.empty(n * bpp, dtype=torch.uint8, device="cuda")
    ctx.check(lib.cr_synth_points_device(ctx.handle, C.byref(p), n, rec_d.data_ptr(), C.byref(hdr), sh), "gen")
    ctx.check(lib.cr_morton_sort_device(ctx.handle, rec_d.data_ptr(), n, bpp, C.byref(hdr), sh), "sort")
    ctx.sync(sh)
    rec = rec_d.cpu().numpy()
    del rec_d
    torch.cuda.empty_cache()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    laz = las.laz_bytes(rec, n, hdr.scale, hdr.offset, hdr.min, hdr.max, threads=0)
    write_s = time.perf_counter() - t0
    info = las.parse_header(las._header(n, hdr.scale, hdr.offset, hdr.min, hdr.max, 2, bpp, (1, 2)))
    nb = int(lib.cr_las_num_batches(n))
    lz = las.LazFile(laz)

    def load_las():
        c = ctx.cloud(n, nb, 1)
        t = time.perf_counter()
        ctx.check(lib.cr_cloud_load_las(ctx.handle, c.handle, rec.ctypes.data, n, C.byref(info), 0, 0, 0, sh),
                  "load las")
        return c, time.perf_counter() - t

    def load_laz():
        c = ctx.cloud(n, nb, 1)
        t = time.perf_counter()
        ctx.check(lib.cr_cloud_load_laz(ctx.handle, c.handle, lz.handle, 0, 0, 0, 0, sh), "load laz")
        return c, time.perf_counter() - t

    small = las.LazFile(las.laz_bytes(rec[:2_000_000 * bpp], 2_000_000, hdr.scale, hdr.offset, hdr.min,
                                      hdr.max))
    warm = ctx.cloud(2_000_000, int(lib.cr_las_num_batches(2_000_000)), 1)
    ctx.check(lib.cr_cloud_load_laz(ctx.handle, warm.handle, small.handle, 0, 0, 0, 0, sh), "warm-up")
    warm.close()
    c_las, las_s = load_las()
    c_laz, laz_s = load_laz()
    same = all(np.array_equal(c_las.read(w), c_laz.read(w)) for w in
               (0, L.STREAM_LOW, L.STREAM_MED, L.STREAM_HIG, L.STREAM_RGBA))
    c_las.close()
    c_laz.close()
    sub = 5_000_000
    t = time.perf_counter()
    lz.decode(0, sub, threads=1)
    one_s = time.perf_counter() - t
    t = time.perf_counter()
    lz.decode(threads=0)
    dec_s = time.perf_counter() - t
    return {"points": n, "host_threads": threads, "laz_bytes": len(laz),
            "laz_bytes_per_point": round(len(laz) / n, 3),
            "las_load_mpts_per_s": round(n / las_s / 1e6, 1),
            "laz_load_mpts_per_s": round(n / laz_s / 1e6, 1),
            "laz_decode_mpts_per_s": round(n / dec_s / 1e6, 1),
            "laz_decode_1thread_mpts_per_s": round(sub / one_s / 1e6, 2),
            "laz_write_mpts_per_s": round(n / write_s / 1e6, 1),
            "laz_equals_las_cloud": bool(same),
            "what": "cr_cloud_load_las / cr_cloud_load_laz wall clock from host memory; decode-only "
                    "cr_laz_decode on all threads and on one (5M points)"}


def potree_nodes(ctx, sh, steps, points=50_000_000):
    """loop_nodes ("render Potree nodes", compute_loop_nodes) on a Potree 2.0
    dataset: a Morton-sorted terrain of `points` records (generated and sorted
    on the GPU) written by potree.write_octree (hashed 1/8 samples in inner
    nodes, leaves of at most 20,000 points, hierarchy chunks of 2 levels),
    opened and loaded through the C ABI (metadata.json, hierarchy.bin,
    octree.bin encoded one batch record per node) and rendered at 1920x1080
    from the zoom-to-cloud pose with the method's defaults (level-4 cut, node
    loop, float uniforms, tiled resolve); CUDA events over the frames."""
    import ctypes as C
    import shutil
    import tempfile
    import time

    import torch

    import compute_rasterizer_gb300 as cr
    from compute_rasterizer_gb300 import _lib as L
    from compute_rasterizer_gb300 import potree, synth
    lib = L.load()
    n, bpp = points, L.LAS_FORMAT2_BYTES
    p = synth.synth_params(L.SYNTH_TERRAIN, 1500.0, 31)
    hdr = L.LasHeader()
    rec_d = torch.empty(n * bpp, dtype=torch.uint8, device="cuda")
    ctx.check(lib.cr_synth_points_device(ctx.handle, C.byref(p), n, rec_d.data_ptr(), C.byref(hdr), sh), "gen")
    ctx.check(lib.cr_morton_sort_device(ctx.handle, rec_d.data_ptr(), n, bpp, C.byref(hdr), sh), "sort")
    ctx.sync(sh)
    rec = rec_d.cpu().numpy()
    del rec_d
    d = tempfile.mkdtemp(prefix="cr_potree_")
    try:
        t0 = time.perf_counter()
        nodes = potree.write_octree(d, rec, n, hdr.scale[:], hdr.offset[:], hdr.min[:], hdr.max[:],
                                    max_leaf=20000, chunk_levels=2)
        write_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        o = potree.open_octree(d)
        cloud = o.load(ctx, stream=sh)
        ctx.sync(sh)
        load_s = time.perf_counter() - t0
        extent = np.array(hdr.max[:]) - np.array(hdr.min[:])
        yaw, pitch, radius, target = synth.zoom_to_cloud(np.zeros(3), extent)
        W, H = 1920, 1080
        view = synth.orbit_view(yaw, pitch, radius, target)
        cv = cr.make_view(view, synth.perspective(60.0, W / H, 0.1, 200000.0), W, H)
        params = cr.default_params(L.METHOD_LOOP_NODES)
        fb = ctx.framebuffer(W, H)
        fb.clear(stream=sh)
        stream = torch.cuda.ExternalStream(sh)
        for _ in range(3):
            ctx.render(cloud, cv, params, fb, sh)
        ctx.sync(sh)
        k = max(5, min(steps, 50))
        ctx.timing_enable(k)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            ctx.render(cloud, cv, params, fb, sh)
        e1.record(stream)
        ctx.sync(sh)
        ms = e0.elapsed_time(e1) / k
        stages = {name: round(float(np.mean(ctx.timing_read(v, k))), 4) for name, v in
                  (("cull", L.STAGE_CULL), ("raster", L.STAGE_RASTER), ("resolve", L.STAGE_RESOLVE))}
        ctx.timing_enable(0)
        st = ctx.frame_stats(cloud, params)
        peak, _ = measured_peaks()
        out = {"points": n, "nodes": len(nodes), "levels": int(max(nd["level"] for nd in nodes)) + 1,
               "max_node_points": int(max(nd["num_points"] for nd in nodes)),
               "ms_per_frame": round(ms, 4), "gpoints_per_s": round(n / ms / 1e6, 2),
               "stages_ms": stages,
               "points_per_level": list(st.points_per_level),
               "batches_visible": int(st.batches_visible),
               "stream_bytes": int(st.stream_bytes),
               "raster_frac_of_measured_hbm": round(int(st.stream_bytes) / stages["raster"] / 1e6 / peak, 4),
               "octree_write_s": round(write_s, 2), "open_load_s": round(load_s, 3),
               "what": "cr_potree_open + cr_potree_load (host encode, upload) then loop_nodes frames; "
                       "the level-4 cut drops nodes that project below 80 px"}
        fb.close()
        cloud.close()
        o.close()
        return out
    finally:
        shutil.rmtree(d, ignore_errors=True)


def multiview_64(ctx, sh, steps, payload):
    """200M points (terrain + 2000 boxes), 64 views: the multi-view plan
    (autotuned, CUDA graph) against one cr_render per view, images compared."""
    import torch

    import compute_rasterizer_gb300 as cr
    from compute_rasterizer_gb300 import _lib as L
    from compute_rasterizer_gb300 import synth, workloads
    from compute_rasterizer_gb300.multiview import MultiView
    n = 200_000_000
    cloud, hdr = synth.build_cloud_device(ctx, workloads.multiview_cloud_params(), n, sh)
    cams = workloads.multiview_64(np.array(hdr.min[:]), np.array(hdr.max[:]))
    views = [cr.make_view(*c) for c in cams]
    params = cr.default_params(L.METHOD_LOOP_LAS, payload=payload)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views(views)
    mv.clear(stream=sh)
    best, report = mv.autotune(frames=3, stream=sh)
    k = max(3, min(steps, 20))
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    stream = torch.cuda.ExternalStream(sh)
    for _ in range(3):
        mv.render(True, sh)
    ctx.sync(sh)
    ev[0].record(stream)
    for _ in range(k):
        mv.render(True, sh)
    ev[1].record(stream)
    ctx.sync(sh)
    mv_ms = ev[0].elapsed_time(ev[1]) / k
    fbs = [ctx.framebuffer(c[2], c[3]) for c in cams]
    for f in fbs:
        f.clear(stream=sh)
    for v, f in zip(views, fbs):
        ctx.render(cloud, v, params, f, sh)
    ctx.sync(sh)
    ev[2].record(stream)
    for _ in range(k):
        for v, f in zip(views, fbs):
            ctx.render(cloud, v, params, f, sh)
    ev[3].record(stream)
    ctx.sync(sh)
    plain_ms = ev[2].elapsed_time(ev[3]) / k
    same = all(np.array_equal(mv.read(i, L.FB_IMAGE, sh), f.read(L.FB_IMAGE, sh))
               for i, f in enumerate(fbs))
    pairs = mv.shared_pairs()
    # A/B of the stereo sharing: the eyes built by look_at from their own
    # positions (same cameras up to rounding, rows not bitwise equal)
    mv.set_views([cr.make_view(*c) for c in workloads.multiview_64(np.array(hdr.min[:]), np.array(hdr.max[:]),
                                                                    compose_eyes=False)])
    unshared_pairs = mv.shared_pairs()
    for _ in range(3):
        mv.render(True, sh)
    ctx.sync(sh)
    ev[0].record(stream)
    for _ in range(k):
        mv.render(True, sh)
    ev[1].record(stream)
    ctx.sync(sh)
    unshared_ms = ev[0].elapsed_time(ev[1]) / k
    mv.close()

    def timed(plan):
        for _ in range(3):
            plan.render(True, sh)
        ctx.sync(sh)
        ev[0].record(stream)
        for _ in range(k):
            plan.render(True, sh)
        ev[1].record(stream)
        ctx.sync(sh)
        return ev[0].elapsed_time(ev[1]) / k

    # the 16 stereo pairs alone (a headset's frames), shared and by look_at
    eyes = cams[:32]
    st_mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in eyes], params)
    st_mv.set_views([cr.make_view(*c) for c in eyes])
    st_mv.clear(stream=sh)
    st_best, _ = st_mv.autotune(frames=3, stream=sh)
    st_pairs = st_mv.shared_pairs()
    st_ms = timed(st_mv)
    st_mv.set_views([cr.make_view(*c) for c in workloads.multiview_64(np.array(hdr.min[:]), np.array(hdr.max[:]),
                                                                      compose_eyes=False)[:32]])
    st_unshared = st_mv.shared_pairs()
    st_unshared_ms = timed(st_mv)
    st_mv.close()
    out = {"points": n, "views": len(cams), "payload": "color" if payload else "index",
           "batched_ms_per_frame": round(mv_ms, 3), "plain_ms_per_frame": round(plain_ms, 3),
           "batched_frames_per_s": round(1e3 / mv_ms, 2), "plain_frames_per_s": round(1e3 / plain_ms, 2),
           "speedup_vs_plain": round(plain_ms / mv_ms, 3), "bit_exact_images": bool(same),
           "shared_stereo_pairs": pairs,
           "eyes_by_look_at": {"shared_stereo_pairs": unshared_pairs,
                               "batched_ms_per_frame": round(unshared_ms, 3)},
           "stereo_32_views": {"shared_stereo_pairs": st_pairs, "batched_ms_per_frame": round(st_ms, 3),
                               "eyes_by_look_at_pairs": st_unshared,
                               "eyes_by_look_at_ms_per_frame": round(st_unshared_ms, 3),
                               "views_per_group": st_best.views_per_group,
                               "block_threads": st_best.block_threads},
           "autotuned": {"block_threads": best.block_threads, "views_per_group": best.views_per_group,
                         "points_per_thread": 10240 // max(1, best.block_threads)},
           "autotune_ms": report,
           "plain": "64 x cr_render (cull + raster + resolve per view), same stream",
           "batched": "one multi-view plan frame (one cull, one persistent raster, one resolve), CUDA graph"}
    for f in fbs:
        f.close()
    cloud.close()
    return out


def small_configs(ctx, sh, args, payload):
    """The plain 16 B path at 4,194,304 points and 1920x1080 (early-z, the
    reference's uniform-cube scene), and the 100M-point terrain seen from 5
    flight-path poses at 2560x1440 (batched adaptive path, culling on).
    Roofline: algorithmic bytes per frame / frame time, against the measured
    copy bandwidth."""
    import torch

    import compute_rasterizer_gb300 as cr
    from compute_rasterizer_gb300 import _lib as L
    from compute_rasterizer_gb300 import synth, workloads
    stream = torch.cuda.ExternalStream(sh)
    peak, _ = measured_peaks()
    k = max(10, min(args.steps, 100))

    def timed(fn, frames):
        for _ in range(3):
            fn()
        ctx.sync(sh)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(frames):
            fn()
        e1.record(stream)
        ctx.sync(sh)
        return e0.elapsed_time(e1) / frames

    out = {}
    n1, W1, H1 = 4_194_304, 1920, 1080
    cloud = synth.uniform_cloud_device(ctx, 1, n1, 100.0, sh)
    view = synth.look_at([150.0, 150.0, 150.0], [50.0, 50.0, 50.0], [0.0, 0.0, 1.0])
    cv = cr.make_view(view, synth.perspective(60.0, W1 / H1, 0.1, 1000.0), W1, H1)
    fb = ctx.framebuffer(W1, H1)
    fb.clear(0xFFFFFFFFFFFFFFFF, stream=sh)
    p = cr.default_params(L.METHOD_EARLYZ)  # resolve + re-clear, as the reference's frame
    ms = timed(lambda: ctx.render(cloud, cv, p, fb, sh), k)
    P = W1 * H1
    bytes1 = 16 * n1 + 8 * P + 4 * P + 8 * P
    out["plain_4m_1080p"] = {
        "points": n1, "ms_per_frame": round(ms, 4), "gpoints_per_s": round(n1 / ms / 1e6, 2),
        "algorithmic_bytes": bytes1, "achieved_gbs": round(bytes1 / ms / 1e6, 1),
        "frac_of_measured_hbm": round(bytes1 / ms / 1e6 / peak, 4),
        "frame": "early-z raster (16 B/point) + resolve + re-clear"}
    # the reference's warp-reduction variants of the same frame (2021 dedup,
    # early-z & reduce): same bytes, different per-point atomics
    for key, m in (("plain_4m_1080p_dedup", L.METHOD_DEDUP),
                   ("plain_4m_1080p_earlyz_reduce", L.METHOD_EARLYZ_REDUCE)):
        pm = cr.default_params(m)
        ms = timed(lambda: ctx.render(cloud, cv, pm, fb, sh), k)
        out[key] = {"ms_per_frame": round(ms, 4), "gpoints_per_s": round(n1 / ms / 1e6, 2),
                    "frac_of_measured_hbm": round(bytes1 / ms / 1e6 / peak, 4)}
    fb.close()
    cloud.close()

    n2 = 100_000_000
    cloud, hdr = synth.build_cloud_device(ctx, synth.synth_params(L.SYNTH_TERRAIN, 1000.0, 2), n2, sh)
    cams = workloads.flight_path(np.array(hdr.min[:]), np.array(hdr.max[:]))
    p = cr.default_params(L.METHOD_LOOP_LAS, payload=payload)
    poses = []
    for view, proj, W, H in cams:
        cv = cr.make_view(view, proj, W, H)
        fb = ctx.framebuffer(W, H)
        fb.clear(stream=sh)
        ms = timed(lambda: ctx.render(cloud, cv, p, fb, sh), k)
        st = ctx.frame_stats(cloud, p)
        P = W * H
        gather = 4 * P if payload == L.PAYLOAD_INDEX else 0
        fbytes = int(st.stream_bytes) + 20 * P + gather
        poses.append({"ms_per_frame": round(ms, 4), "gpoints_per_s": round(n2 / ms / 1e6, 2),
                      "batches_visible": int(st.batches_visible),
                      "points_per_level": list(st.points_per_level),
                      "algorithmic_bytes": fbytes,
                      "frac_of_measured_hbm": round(fbytes / ms / 1e6 / peak, 4)})
        fb.close()
    total = sum(q["ms_per_frame"] for q in poses)
    out["flight_100m_1440p"] = {
        "points": n2, "poses": poses, "mean_ms_per_frame": round(total / len(poses), 4),
        "gpoints_per_s": round(n2 * len(poses) / total / 1e6, 2),
        "payload": "color" if payload == L.PAYLOAD_COLOR else "index",
        "frame": "cull + raster + resolve + re-clear; bytes = coordinate/color words of visible "
                 "batches at their levels + 64 B per visible batch + 20 B per pixel"}
    cloud.close()
    return out


def serving(ctx, sh, args, payload):
    """8 resident terrains (10-500 M points), requests with Poisson arrivals,
    clouds drawn Zipf(1.1), random orbit cameras at five resolutions, an 8 GiB
    framebuffer pool.  Both arms run the same replay through the frame server:
    batched (continuous batching into multi-view launches) and plain (one
    single-view render per request).  Every request's image is copied back to
    pinned host memory inside its latency."""
    import torch

    import compute_rasterizer_gb300 as cr
    from compute_rasterizer_gb300 import _lib as L
    from compute_rasterizer_gb300 import synth, workloads
    from compute_rasterizer_gb300.serve import Server, latency_summary

    clouds, boxes = [], []
    for i, m in enumerate(workloads.SERVING_CLOUD_MPOINTS):
        n = m * 1_000_000
        c, hdr = synth.build_cloud_device(ctx, workloads.serving_cloud_params(i, n), n, sh)
        clouds.append(c)
        boxes.append((np.array(hdr.min[:]), np.array(hdr.max[:])))
    ctx.sync(sh)
    # a ring of pinned host memory for the returned images; the pool bounds the
    # bytes in flight (images are a third of each request's pool bytes)
    ring_bytes = 4 << 30
    ring = torch.empty(ring_bytes // 4, dtype=torch.int32, pin_memory=True)
    ring_np = ring.numpy().view(np.uint32)
    cursor = [0]

    def host_slot(words):
        if cursor[0] + words > ring_np.size:
            cursor[0] = 0
        a = ring_np[cursor[0]:cursor[0] + words]
        cursor[0] += words
        return a

    def make_requests(cams):
        return [Server.request(c, cr.make_view(v, p, w, h), host_slot(w * h), user_tag=i)
                for i, (c, v, p, w, h) in enumerate(cams)]

    # each arm at its best measured setting on this workload: batched launches
    # of up to 16 views, 4 in flight; plain launches, 8 in flight
    def server(plain):
        srv = Server(ctx, pool_bytes=8 << 30, max_batch_views=1 if plain else 16,
                     max_inflight=8 if plain else 4, plain_launches=plain, payload=payload)
        for c in clouds:
            srv.add_cloud(c)
        return srv

    arms = {"batched": server(False), "plain": server(True)}
    out = {"clouds_mpoints": list(workloads.SERVING_CLOUD_MPOINTS),
           "resolutions": [f"{w}x{h}" for w, h in workloads.SERVING_RESOLUTIONS],
           "zipf_s": 1.1, "pool_bytes": 8 << 30, "max_batch_views": 16,
           "max_inflight": {"batched": 4, "plain": 8},
           "payload": "color" if payload == L.PAYLOAD_COLOR else "index",
           "latency": "arrival -> image in pinned host memory (server clock)"}
    # warm-up
    arr, cams = workloads.serving_requests(boxes, 64, 1e5, seed=99)
    for srv in arms.values():
        srv.replay(make_requests(cams), arr)

    # capacity: a burst of requests all arriving at t = 0
    nb = 2000  # about 0.4 s per arm at capacity; shorter bursts varied more from run to run
    arr, cams = workloads.serving_requests(boxes, nb, 1e9, seed=7)
    cap = {}
    for name, srv in arms.items():
        done = srv.replay(make_requests(cams), np.zeros(nb))
        cap[name] = latency_summary(done)
    out["capacity_req_per_s"] = {k: round(v["served_req_per_s"], 1) for k, v in cap.items()}
    out["capacity_speedup_vs_plain"] = round(cap["batched"]["served_req_per_s"]
                                             / cap["plain"]["served_req_per_s"], 3)
    out["capacity_mean_batch_views"] = round(cap["batched"]["mean_batch_views"], 2)

    rates = ([100, 250, 500, 1000, 2000, 3000, 4000, 5000] if args.serving == "full"
             else [100, 500, 1000, 2000, 5000])
    seconds = 2.0 if args.serving == "full" else 1.0
    sweep = []
    for k, rate in enumerate(rates):
        n = int(max(200, min(rate * seconds, 10000)))
        arr, cams = workloads.serving_requests(boxes, n, float(rate), seed=20 + k)
        row = {"rate_req_per_s": rate, "requests": n}
        for name, srv in arms.items():
            s = latency_summary(srv.replay(make_requests(cams), arr))
            row[name] = {key: (round(v, 3) if isinstance(v, float) else v) for key, v in s.items()}
        row["p99_ratio_plain_over_batched"] = round(row["plain"]["p99_ms"] / row["batched"]["p99_ms"], 3)
        sweep.append(row)
    out["sweep"] = sweep
    for name, srv in arms.items():
        st = srv.stats()
        out[f"{name}_stats"] = {k: st[k] for k in ("launches", "views_launched", "max_views_in_launch",
                                                   "rejected", "failed", "pool_peak_bytes")}

    # bit-exact: a mixed burst against each request rendered alone
    arr, cams = workloads.serving_requests(boxes, 64, 1e9, seed=123)
    imgs = [np.zeros(w * h, np.uint32) for (_, _, _, w, h) in cams]
    reqs = [Server.request(c, cr.make_view(v, p, w, h), imgs[i], user_tag=i)
            for i, (c, v, p, w, h) in enumerate(cams)]
    done = arms["batched"].replay(reqs, np.zeros(len(reqs)))
    params = cr.default_params(L.METHOD_LOOP_LAS, payload=payload, resolve=1, clear_after=0)
    same = bool((done["status"] == L.OK).all())
    for i, (c, v, p, w, h) in enumerate(cams):
        fb = ctx.framebuffer(w, h)
        fb.clear(stream=sh)
        ctx.render(clouds[c], cr.make_view(v, p, w, h), params, fb, sh)
        same = same and np.array_equal(fb.read(L.FB_IMAGE, sh), imgs[i])
        fb.close()
    out["bit_exact_alone_vs_mix"] = same
    out["bit_exact_checked"] = {"requests": len(cams),
                                "mean_batch_views": round(float(done["batch_views"].mean()), 2)}
    for srv in arms.values():
        srv.close()
    for c in clouds:
        c.close()
    return out


def e2e(ctx, cloud, cv, params, fb, sh, n, args, box_min):
    """The frame with the cloud in pinned host memory, through the C ABI, every
    step ending with the RGBA8 image in pinned host memory.  Main path: a cloud
    over the host arrays (cr_cloud_wrap); the kernels read the words each
    visible batch needs across the NVLink-C2C link, so those bytes are the
    step's host-to-device traffic.  Second path (`upload`): the loader's way,
    every stream and the batch records copied to device memory
    (cr_cloud_upload), then rendered."""
    import torch

    from compute_rasterizer_gb300 import _lib as L
    lib = L.load()
    words = n + 64
    host = {}
    for which, key in ((0, "batches"), (L.STREAM_LOW, "low"), (L.STREAM_MED, "med"),
                       (L.STREAM_HIG, "hig"), (L.STREAM_RGBA, "rgba")):
        nbytes = cloud.nb * 64 if which == 0 else n * 4
        t = torch.zeros(nbytes if which == 0 else words * 4, dtype=torch.uint8, pin_memory=True)
        ctx.check(lib.cr_cloud_read(ctx.handle, cloud.handle, which, t.data_ptr(), nbytes, sh), "read")
        host[key] = t
    img = torch.empty(fb.W * fb.H * 4, dtype=torch.uint8, pin_memory=True)
    box = np.ascontiguousarray(box_min, np.float64)
    ctx.sync(sh)
    wrapped = ctx.cloud_wrap(n, cloud.nb, host["batches"], host["low"], host["med"], host["hig"],
                             host["rgba"], box_min=box, stream_words=words)

    def read_image():
        ctx.check(lib.cr_fb_read(ctx.handle, fb.handle, L.FB_IMAGE, img.data_ptr(), img.numel(), sh),
                  "image read")

    def step_wrapped():
        ctx.render(wrapped, cv, params, fb, sh)
        read_image()

    def step_upload():
        ctx.check(lib.cr_cloud_upload(ctx.handle, cloud.handle, host["batches"].data_ptr(),
                                      host["low"].data_ptr(), host["med"].data_ptr(),
                                      host["hig"].data_ptr(), host["rgba"].data_ptr(),
                                      box.ctypes.data, sh), "upload")
        ctx.render(cloud, cv, params, fb, sh)
        read_image()

    def timed(step, k):
        step()
        ctx.sync(sh)
        t0 = time.perf_counter()
        for _ in range(k):
            step()
        ctx.sync(sh)
        return (time.perf_counter() - t0) / k

    k = max(3, min(args.steps, 20))
    dt = timed(step_wrapped, k)
    link_bytes = int(ctx.frame_stats(wrapped, params).stream_bytes)
    ku = max(2, min(args.steps, 5))
    dtu = timed(step_upload, ku)
    wrapped.close()
    return {"value": round(n / dt / 1e9, 4), "unit": "Gpoints/s", "h2d_bytes_per_step": link_bytes,
            "d2h_bytes_per_step": fb.W * fb.H * 4, "ms_per_step": round(dt * 1e3, 3), "steps": k,
            "path": "cr_cloud_wrap over pinned host streams + cr_render + cr_fb_read: the kernels "
                    "read each visible batch's words from host memory (h2d = those bytes)",
            "upload": {"value": round(n / dtu / 1e9, 4), "unit": "Gpoints/s",
                       "h2d_bytes_per_step": cloud.nb * 64 + 4 * n * 4,
                       "d2h_bytes_per_step": fb.W * fb.H * 4, "ms_per_step": round(dtu * 1e3, 3),
                       "steps": ku,
                       "path": "cr_cloud_upload (all four streams + batch records) + cr_render + "
                               "cr_fb_read, pinned host buffers"}}


def cpu_baseline(args, view, proj):
    """The oracle's multi-threaded raster on a bounded sample, on this host's cores."""
    from oracle import oracle as O
    s = min(CPU_SAMPLE_POINTS, args.points)
    p, hdr, enc, ext = cpu_sample(args.points, WORKLOAD["extent"], WORKLOAD["seed"], s)
    payload = O.PAYLOAD_COLOR if args.payload == "color" else O.PAYLOAD_INDEX
    fr = O.make_frame(view, proj, WORKLOAD["width"], WORKLOAD["height"], np.array(hdr.min[:])[None],
                      1, O.L0_X12, payload)
    cores = os.cpu_count() or 1
    per_frame, frames = time_oracle(fr, enc, s, cores, min_seconds=10.0, warmup=1)
    return {"value": round(s / per_frame / 1e9, 4), "unit": "Gpoints/s", "cores": cores,
            "kind": "port",
            "sample": f"{s:,} points (the central {ext:.0f} m square of the same terrain, same "
                      f"density and camera), {frames} frames"}


if __name__ == "__main__":
    main()
