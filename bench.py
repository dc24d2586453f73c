"""Ray-tracing throughput on one GB300 (Mrays/s).

Workload (default): the 1.31M-triangle displaced icosphere (20 faces
subdivided 8 times, radius 1, radial value-noise displacement 0.05), SAH kd
tree (traversal cost 1, intersection cost 1.5), 1920x1080, one primary ray per
pixel plus one occlusion ray per light (2 point lights) where the light is in
front of the surface. det threshold 0 (the reference's absolute 1e-4 culls
every triangle of this unit sphere, whose |ab x ac| are about 2e-5). One step =
one frame rendered by the fused ray-tracing kernel with the scene resident in
HBM.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). Under torchrun every rank renders its own frames
on its own GPU (replicas; the path does not exchange data), value = all ranks'
rays / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 256 << 20  # > 129 MB L2
PARAM_BLOCK_BYTES = 1676     # kernel parameter block of one render launch (camera, lights, pointers)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["icosphere", "soup", "room", "batch", "cornell", "denoise", "denoise-infer",
                                           "denoise-train"], default="icosphere")
    ap.add_argument("--dn-steps", type=int, default=1000, help="denoise: training steps")
    ap.add_argument("--dn-train", type=int, default=96, help="denoise: training rooms")
    ap.add_argument("--dn-eval", type=int, default=16, help="denoise: held-out rooms")
    ap.add_argument("--dn-res", type=int, default=512, help="denoise: evaluation image size")
    ap.add_argument("--dn-train-res", type=int, default=512, help="denoise: training image size")
    ap.add_argument("--dn-cuda-cores", action="store_true", help="denoise-infer: CUDA-core convolutions")
    ap.add_argument("--dn-batch", type=int, default=1, help="denoise-infer: frames per denoise call")
    ap.add_argument("--dn-spp-in", type=int, default=4, help="denoise: samples per pixel of the noisy input")
    ap.add_argument("--dn-depth-in", type=int, default=0,
                    help="denoise: path depth of the noisy input (0: the full depth of the references)")
    ap.add_argument("--dn-rr-in", type=int, default=-1,
                    help="denoise: Russian roulette from this depth in the noisy input (-1: from depth 3, as the "
                         "references and plain renders)")
    ap.add_argument("--dn-ref-spp", type=int, default=1024, help="denoise: training target samples per pixel")
    ap.add_argument("--dn-eval-ref-spp", type=int, default=4096,
                    help="denoise: samples per pixel of the held-out rooms' references")
    ap.add_argument("--scheduler", choices=["pixel", "wavefront"], default="wavefront",
                    help="room workload: path-tracing scheduler")
    ap.add_argument("--spp", type=int, default=0, help="room/batch: samples per pixel (0 = workload default)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="default workload: skip the path-tracing room and the 64-scene batch")
    ap.add_argument("--leaf-refine", type=int, default=8,
                    help="device layout: sub-hierarchy inside reference leaves larger than this (0 = off)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    return ap.parse_args()


def workload(name):
    from nostrum_pray_gb300 import scenes
    if name == "icosphere":
        mesh = scenes.icosphere(8)
        setup = scenes.icosphere_setup(1920, 1080, det_eps=0.0)
        cfg = {"workload": "displaced icosphere 1,310,720 triangles, SAH kd tree (Ct 1, Ci 1.5), 1920x1080, "
                           "1 primary + up to 2 occlusion rays per pixel, det threshold 0",
               "triangles": mesh.n, "width": 1920, "height": 1080, "lights": 2, "tree": "sah",
               "det_epsilon": 0.0}
    else:
        mesh = scenes.soup(10_000, 0)
        setup = scenes.soup_setup()
        cfg = {"workload": "triangle soup 10,000 triangles, median kd tree (leaf 8, depth 24), 512x512, "
                           "1 primary + 1 occlusion ray per pixel, det threshold 1e-4",
               "triangles": mesh.n, "width": 512, "height": 512, "lights": 1, "tree": "median",
               "det_epsilon": 1e-4}
    return mesh, setup, cfg


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle samples of one GPU during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = os.path.join("/tmp", f"pray_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_bf16():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["bf16_tflops"]), "measured cuBLAS bf16 (burst)"
    return 1900.0, "fallback cuBLAS bf16 (burst)"


def committed_profile(kernel: str, workload_name: str) -> dict:
    """Per-launch figures of the committed ncu capture of a kernel on a
    workload (DRAM bytes, warp instructions, ...), or {}."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_{workload_name}.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def cpu_frames(orc, setup, budget_s: float, min_frames: int = 1):
    """Whole ray-traced frames of the oracle's restatement of the reference's
    tracer (full depth-first traversal, scalar Moeller-Trumbore, OpenMP over
    pixels on every host thread) until `budget_s` is spent. Returns (seconds,
    rays, frames, threads OpenMP ran with)."""
    from oracle import oracle as O
    elapsed, rays, frames = 0.0, 0, 0
    while frames < min_frames or elapsed < budget_s:
        t0 = time.perf_counter()
        _, nsh = orc.render_rt(setup, threads=O.default_threads())
        elapsed += time.perf_counter() - t0
        rays += setup.width * setup.height + nsh
        frames += 1
    return elapsed, rays, frames, O.last_threads()


def cpu_baseline(mesh, setup, budget_s: float):
    """The CPU port timed beside the GPU: whole frames of the same workload.
    Returns (Mrays/s, threads, sample description)."""
    from oracle import oracle as O
    O.build()
    orc = O.OracleScene.from_setup(mesh, setup)
    elapsed, rays, frames, thr = cpu_frames(orc, setup, budget_s)
    return rays / elapsed / 1e6, thr, f"{frames} whole frame(s) ({rays} rays) in {elapsed:.1f} s"


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    mesh, setup, cfg = workload(args.workload)
    from oracle import oracle as O
    O.build()
    orc = O.OracleScene.from_setup(mesh, setup)
    for _ in range(args.warmup):
        cpu_frames(orc, setup, 0.0)
    total_t, total_r, thr = 0.0, 0, 0
    for _ in range(args.steps):
        t, r, _, thr = cpu_frames(orc, setup, 0.0)
        total_t += t
        total_r += r
    v = total_r / total_t / 1e6
    sample = f"each step: one whole frame ({setup.width}x{setup.height} pixels with their occlusion rays)"
    line = {"impl": "reference", "metric": "Mrays/s", "value": round(v, 4), "unit": "Mrays/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * total_t / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": round(v, 4), "unit": "Mrays/s", "cores": thr, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(v, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "CPU restatement of the reference's scalar tracer (oracle/pray_oracle.cpp), OpenMP over pixels "
                    "on every host thread; the reference's sources are not on this host, and its own build (x86 "
                    "AVX) would not run here"}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    from nostrum_pray_gb300 import native, replicas
    try:
        native.lib()
    except native.PrayError:
        from nostrum_pray_gb300 import build
        build.build()
    mesh, setup, cfg = workload(args.workload)
    t0 = time.perf_counter()
    sc = native.Scene.from_setup(mesh, setup, device=dev, leaf_refine=args.leaf_refine)
    build_s = time.perf_counter() - t0
    h, w = setup.height, setup.width
    rgb = torch.empty((h, w, 3), dtype=torch.uint8, device="cuda")
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    counts = sc.render_rt_counts(setup)  # [primary, occlusion, pair fetches, tri fetches, shaded hits]
    rays_per_frame = int(counts[0] + counts[1])
    for _ in range(args.warmup):
        sc.render_rt(setup, rgb, counters=cnt)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(dev) if rank == 0 else None
    replicas.barrier()
    torch.cuda.synchronize()
    if sampler:
        sampler.start()
        time.sleep(0.3)
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()  # evict the scene from L2 between frames
        starts[k].record(stream)
        sc.render_rt(setup, rgb, stream=stream)
        ends[k].record(stream)
    torch.cuda.synchronize()
    replicas.barrier()
    wall = time.perf_counter() - wall0
    clocks = sampler.stop() if sampler else None
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    kernel_ms = sum(times)
    kernel_ms_max = replicas.slowest(kernel_ms, "cuda")
    value = replicas.whole_job_rate(rays_per_frame * args.steps, kernel_ms / 1e3, "cuda") / 1e6

    # end to end through the host-memory C ABI entry point (params in, image
    # out into a pinned host frame that the loop reuses)
    h_img = torch.empty((setup.height, setup.width, 3), dtype=torch.uint8).pin_memory().numpy()
    for _ in range(2):
        sc.render_rt_host(setup, out=h_img)
    e2e_times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        img, _ = sc.render_rt_host(setup, out=h_img)
        e2e_times.append(time.perf_counter() - t0)
    e2e_val = replicas.whole_job_rate(rays_per_frame, statistics.mean(e2e_times), "cuda") / 1e6

    # roofline of the render kernel. It is bound by instruction issue (ncu:
    # issue slots busy most cycles, DRAM under 1 % of peak), so the headline
    # is warp instructions per second against the issue limit of 4 warp
    # instructions per SM per cycle at the sampled SM clock; the instruction
    # count per launch is a property of the kernel and the frame, taken from
    # the committed ncu capture of this command (profiles/). DRAM traffic and
    # the logical per-ray fetch bytes are reported beside it.
    prim, occl, pairs, tris, hits = (int(x) for x in counts)
    logical_bytes = 32 * (prim + occl) + 64 * pairs + 48 * tris + 32 * hits + 3 * w * h
    mean_s = kernel_ms / args.steps / 1e3
    hbm_peak, hbm_kind = measured_peaks()
    prof = committed_profile("k_render_rt", args.workload)
    traffic = prof.get("dram_bytes_per_launch")
    inst = prof.get("inst_executed_per_launch")
    sms = torch.cuda.get_device_properties(dev).multi_processor_count

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        v, cores, sample = cpu_baseline(mesh, setup, args.cpu_seconds)
        cpu = {"value": round(v, 4), "unit": "Mrays/s", "cores": cores, "kind": "port", "sample": sample}
    cfg = dict(cfg)
    traversal = {native.TRAVERSAL_LANES: "per lane", native.TRAVERSAL_PACKETS: "warp packets",
                 native.TRAVERSAL_PRIMARY_PACKETS: "warp packets for primary rays"}.get(sc.traversal(), "auto")
    cfg.update({"parallelism": f"replicas x{world}", "l2": "flushed between steps (256 MB write)",
                "tree_build_s": round(build_s, 2), "rays_per_frame": rays_per_frame,
                "leaf_refine": args.leaf_refine, "traversal": f"{traversal} (timed on the first frame)"})
    line = {"metric": "Mrays/s", "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(kernel_ms_max / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg,
            "e2e": {"value": round(e2e_val, 2), "unit": "Mrays/s", "h2d_bytes_per_step": PARAM_BLOCK_BYTES,
                    "d2h_bytes_per_step": 3 * w * h + 16},
            "gpu_launches": args.steps,
            "roofline": issue_roofline(inst, mean_s, sms, clocks, traffic, hbm_peak, hbm_kind, prof, logical_bytes,
                                       {"primary": prim, "occlusion": occl, "node_pair_fetches": pairs,
                                        "triangle_fetches": tris, "shaded_hits": hits}),
            "wall_s_timed_loop": round(wall, 4), "clocks": clocks, "cpu_baseline": cpu}
    if world == 1 and not args.no_secondary:
        sub = argparse.Namespace(**vars(args))
        sub.steps, sub.warmup, sub.spp = max(3, min(args.steps, 10)), 3, 0
        sub.cpu_seconds = args.cpu_seconds / 2
        line["secondary"] = {}
        dn_fast = lambda a: run_denoise_secondary(a, spp_in=1, rr_in=0)
        for key, fn in (("room", run_pt), ("batch", run_batch), ("denoise", dn_fast),
                        ("denoise_4spp_input", run_denoise_secondary)):
            try:
                line["secondary"][key] = fn(sub)
            except Exception as exc:  # a secondary workload must not cost the main line
                line["secondary"][key] = {"error": f"{type(exc).__name__}: {exc}"}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def issue_roofline(inst, mean_s, sms, clocks, traffic, hbm_peak, hbm_kind, prof, logical_bytes, counts):
    """Roofline object of an issue-bound kernel: warp instructions per launch
    (committed ncu capture) over the CUDA-event time, against 4 warp
    instructions per SM per cycle at the median SM clock sampled during the
    timed region (the maximum clock when no sample was taken)."""
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
    peak = 4 * sms * mhz / 1e3  # G warp instructions / s
    achieved = inst / mean_s / 1e9 if inst else None
    return {"bound": "issue", "achieved": round(achieved, 1) if achieved else None, "peak": round(peak, 1),
            "unit": "G warp instructions/s", "frac": round(achieved / peak, 4) if achieved else None,
            "traffic": traffic,
            "peak_kind": f"4 warp instructions per SM per cycle x {sms} SMs x {mhz:.0f} MHz (sampled)",
            "inst_executed_per_launch": inst,
            "ncu_issue_active_pct": prof.get("issue_active_pct"),
            "ncu_l1tex_throughput_pct": prof.get("l1tex_throughput_pct"),
            "dram_gbs": round(traffic / mean_s / 1e9, 1) if traffic else None,
            "dram_frac": round(traffic / mean_s / 1e9 / hbm_peak, 4) if traffic else None,
            "dram_peak_kind": f"{hbm_kind} HBM copy bandwidth ({hbm_peak} GB/s)",
            "logical_fetch_bytes_per_launch": logical_bytes,
            "logical_fetch_gbs": round(logical_bytes / mean_s / 1e9, 1),
            "counts": counts,
            "note": "instruction issue binds this kernel; logical fetch bytes count 64 B per node-pair visit and "
                    "48 B per triangle test per ray, most of them served by warp-wide broadcast loads from L1, so "
                    "they are not a DRAM figure; traffic is the DRAM bytes of one launch (ncu)"}


def _timed_frames(fn, steps, warmup, flush):
    """CUDA-event time of `steps` calls of fn (L2 flushed before each)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        flush.zero_()
        starts[k].record(stream)
        fn()
        ends[k].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in zip(starts, ends))


def run_pt(args):
    """Path tracing of the closed room (next-event estimation + Russian
    roulette after depth 3), 1024x1024, 64 spp, depth 8."""
    import torch
    from nostrum_pray_gb300 import native, scenes
    torch.cuda.set_device(0)
    mesh = scenes.room()
    spp = args.spp or 64
    st = scenes.room_setup(1024, 1024, spp=spp, max_depth=8)
    sc = native.Scene.from_setup(mesh, st, leaf_refine=args.leaf_refine)
    sched = native.SCHED_WAVEFRONT if args.scheduler == "wavefront" else native.SCHED_PIXEL
    p = native.pt_params(st, seed=1, mode=native.PT_NEE, rr_depth=3, scheduler=sched)
    rgb = torch.empty((st.height, st.width, 3), dtype=torch.uint8, device="cuda")
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    sc.render_pt(p, rgb, counters=cnt)
    torch.cuda.synchronize()
    paths, segs = int(cnt[0]), int(cnt[1])
    ms = _timed_frames(lambda: sc.render_pt(p, rgb), args.steps, args.warmup, flush)
    sec = ms / 1e3
    cpu = None
    if not args.no_cpu_baseline:
        # the oracle's restatement of the same path tracer (full depth-first
        # traversal per ray) on whole central rows, until the time budget
        from oracle import oracle as O
        O.build()
        orc = O.OracleScene.from_setup(mesh, st)
        row, rows, elapsed = st.height // 2, 0, 0.0
        while elapsed < args.cpu_seconds and row < st.height:
            t0 = time.perf_counter()
            orc.render_pt(st, spp=spp, max_depth=8, seed=1, mode=native.PT_NEE, rr_depth=3, rows=(row, row + 2),
                          threads=O.default_threads())
            elapsed += time.perf_counter() - t0
            row, rows = row + 2, rows + 2
        thr = O.last_threads()
        cpu = {"value": round(rows * st.width * spp / elapsed / 1e6, 5), "unit": "Msamples/s", "cores": thr,
               "kind": "port", "sample": f"{rows} central rows of {st.height} at {spp} spp in {elapsed:.1f} s"}
    line = {"metric": "Msamples/s", "value": round(paths * args.steps / sec / 1e6, 2), "unit": "Msamples/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"closed room {mesh.n} triangles, 1024x1024, {spp} spp, depth 8, NEE + "
                                   f"Russian roulette after depth 3, {args.scheduler} scheduler",
                       "l2": "flushed between steps"},
            "mrays_per_s": round(segs * args.steps / sec / 1e6, 2), "segments_per_frame": segs, "cpu_baseline": cpu}
    sc.close()
    return line


def run_batch(args):
    """64 scenes (displaced icospheres and soups, lognormal triangle counts,
    256^2..1024^2, 16 spp, depth 6) in one persistent launch, tuned first."""
    import torch
    from nostrum_pray_gb300 import native, scenes
    torch.cuda.set_device(0)
    spp = args.spp or 16
    items = scenes.batch_workload(64, seed=0, spp=spp)
    t0 = time.perf_counter()
    scs, params, outs = [], [], []
    for i, (mesh, st) in enumerate(items):
        scs.append(native.Scene.from_setup(mesh, st, leaf_refine=args.leaf_refine))
        params.append(native.pt_params(st, seed=i, mode=native.PT_KAJIYA))
        outs.append((torch.empty((st.height, st.width, 3), dtype=torch.uint8, device="cuda"), None))
    build_s = time.perf_counter() - t0
    b = native.Batch(scs, params, outs)
    t0 = time.perf_counter()
    cfg, tune_ms = b.tune()
    tune_s = time.perf_counter() - t0
    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    b.render(cnt)
    torch.cuda.synchronize()
    paths, segs = int(cnt[0]), int(cnt[1])
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    ms = _timed_frames(lambda: b.render(), args.steps, args.warmup, flush)
    sec = ms / 1e3
    line = {"metric": "Msamples/s", "value": round(paths * args.steps / sec / 1e6, 2), "unit": "Msamples/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"64 scenes, {sum(m.n for m, _ in items)} triangles, "
                                   f"{sum(st.width * st.height for _, st in items)} pixels, {spp} spp, depth 6, "
                                   "one persistent graph-captured launch", "tuned": cfg.as_dict(),
                       "tuning_s": round(tune_s, 2), "scene_build_s": round(build_s, 2),
                       "l2": "flushed between steps"},
            "mrays_per_s": round(segs * args.steps / sec / 1e6, 2), "segments_per_frame": segs}
    del b
    for sc in scs:
        sc.close()
    return line


def cornell_scene():
    """The reference's examples/pt_cornell scene as its own loader returns it
    (triangles, camera and settings stored in tests/golden/golden_small.npz):
    800x600, fov 130, branching path tracing with max_depth 1 and 4,000 rays
    per hit, black background."""
    from nostrum_pray_gb300 import scenes
    g = np.load(os.path.join(ROOT, "tests", "golden", "golden_small.npz"))
    info = g["ex_pt_cornell_info"]
    mesh = scenes.Mesh(g["ex_pt_cornell_verts"], g["ex_pt_cornell_colors"], g["ex_pt_cornell_emit"])
    st = scenes.RenderSetup(width=int(info[0]), height=int(info[1]), fov=int(info[2]),
                            cam_pos=tuple(float(x) for x in info[6:9]), cam_look=tuple(float(x) for x in info[9:12]),
                            lights=[], background=tuple(float(x) for x in info[12:15]), tree="median",
                            method="path_tracing", max_depth_pt=int(info[4]), num_samples=int(info[5]))
    cfg = {"workload": f"reference example pt_cornell as shipped: {mesh.n} triangles, {st.width}x{st.height}, "
                       f"branching path tracing, max_depth {st.max_depth_pt}, {st.num_samples} rays per hit",
           "frame": "one whole frame per step"}
    return mesh, st, cfg


def run_cornell(args):
    """pt_cornell frames (the reference's GPU path tracer's own use case: a
    scene under 10,000 triangles) through pray_render_pt_host."""
    import torch
    from nostrum_pray_gb300 import native
    torch.cuda.set_device(0)
    mesh, st, cfg = cornell_scene()
    sc = native.Scene.from_setup(mesh, st)
    p = native.pt_params(st, seed=1, mode=native.PT_DIFFUSE)
    _, _, cnt = sc.render_pt_host(p)
    segs = int(cnt[1])
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    rgb = torch.empty((st.height, st.width, 3), dtype=torch.uint8, device="cuda")
    ms = _timed_frames(lambda: sc.render_pt(p, rgb), args.steps, args.warmup, flush)
    h_img = torch.empty((st.height, st.width, 3), dtype=torch.uint8).pin_memory().numpy()
    h_rad = torch.empty((st.height, st.width, 3), dtype=torch.float32).pin_memory().numpy()
    sc.render_pt_host(p, out=h_img, out_radiance=h_rad)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sc.render_pt_host(p, out=h_img, out_radiance=h_rad)
    e2e = time.perf_counter() - t0
    sec = ms / 1e3
    line = {"metric": "frames/s", "value": round(args.steps / sec, 3), "unit": "frames/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "reference example",
            "config": cfg, "mrays_per_s": round(segs * args.steps / sec / 1e6, 1), "segments_per_frame": segs,
            "e2e": {"value": round(args.steps / e2e, 3), "unit": "frames/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 15 * st.width * st.height}}
    sc.close()
    return line


def run_reference_cornell(args):
    """The reference's own GPU path tracer (evaluatePathKernelDiffuse of
    src/path_trace.cu, built from its sources into an sm_103a cubin) on
    pt_cornell as shipped, launched as pathTraceOnGPURecursive launches it:
    1,024 pixels per launch, 256 threads per block."""
    from oracle import ref_gpu as G
    mesh, st, cfg = cornell_scene()
    if not G.available():
        return {"impl": "reference", "unavailable": "the reference's GPU path tracer was not built here "
                                                    "(oracle/_ref/prayref_path_trace.cubin missing)"}
    G.render(mesh, st, st.max_depth_pt, st.num_samples, True, frames=args.warmup)
    t0 = time.perf_counter()
    img, ms = G.render(mesh, st, st.max_depth_pt, st.num_samples, True, frames=args.steps)
    wall = time.perf_counter() - t0
    return {"impl": "reference", "metric": "frames/s", "value": round(args.steps / (ms / 1e3), 4),
            "unit": "frames/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms / args.steps, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "reference example", "config": cfg,
            "e2e": {"value": round(args.steps / wall, 4), "unit": "frames/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 3 * st.width * st.height},
            "kernel": "reference src/path_trace.cu evaluatePathKernelDiffuse, sm_103a cubin built from its sources",
            "image_mean": round(float(img.mean()), 3)}


def run_denoise(args):
    """Learned denoiser: train on rooms rendered by the path tracer, then time
    to relMSE <= 0.01 against FP64-accumulated references, denoised vs plain."""
    import torch
    from nostrum_pray_gb300 import denoise as D, native
    torch.cuda.set_device(0)
    cfg = D.DenoiseConfig(res=args.dn_res, train_res=args.dn_train_res, spp_ref=args.dn_ref_spp,
                          train_rooms=args.dn_train, eval_rooms=args.dn_eval, steps=args.dn_steps,
                          spp_in=args.dn_spp_in, depth_in=args.dn_depth_in, rr_in=args.dn_rr_in)
    t0 = time.perf_counter()
    train_seeds = list(range(cfg.seed, cfg.seed + cfg.train_rooms))
    eval_seeds = list(range(cfg.seed + 100_000, cfg.seed + 100_000 + cfg.eval_rooms))
    _, rad, feat, ref = D.make_dataset(cfg, train_seeds, torch, cfg.train_res, keep_scenes=False)
    # held-out rooms are judged against references with more samples (the error target's yardstick),
    # rendered one at a time during the evaluation
    eval_cfg = dataclasses.replace(cfg, spp_ref=args.dn_eval_ref_spp)
    data_s = time.perf_counter() - t0
    den = native.Denoiser(seed=cfg.seed)
    t0 = time.perf_counter()
    losses = D.train(den, rad, feat, ref, cfg, torch)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    # calibration of the fallback sample count on a few training rooms
    calib_scs, _, _, calib_refs = D.make_dataset(cfg, train_seeds[:4], torch)
    calib = [D.plain_curve(cfg, sc, calib_refs[i], train_seeds[i], torch, spps=(4, 8, 16, 32, 64, 128, 256))
             for i, sc in enumerate(calib_scs)]
    fb_spp = D.fallback_spp_from(calib, cfg.target)
    t0 = time.perf_counter()
    res = D.evaluate(cfg, den, D.iter_rooms(eval_cfg, eval_seeds, torch), torch, fb_spp)
    eval_s = time.perf_counter() - t0
    rows = res["rooms"]
    tp = [r["time_plain_s"] for r in rows if r["spp_plain_to_target"] is not None]
    td = [r["time_final_s"] for r in rows]
    ok_d = sum(1 for r in rows if r["relmse_final"] <= cfg.target)
    line = {"metric": "time to relMSE<=0.01, denoised / plain", "value": round(float(np.mean(td) / np.mean(tp)), 4)
            if tp else None, "unit": "ratio", "n_gpus": 1, "higher_is_better": False, "dtype": "bf16",
            "data": "synthetic", "config": {"workload": f"procedural rooms, evaluated at {cfg.res}x{cfg.res}, {cfg.spp_in} spp input"
                                                        f"{f' (paths cut at {cfg.depth_in} bounces)' if cfg.depth_in else ''}"
                                                        f"{f' (Russian roulette from depth {cfg.rr_in})' if cfg.rr_in >= 0 else ''},"
                                                        f" path depth {cfg.depth} (RR from {cfg.rr_depth}),"
                                                        f" {cfg.spp_ref} spp FP64 training targets,"
                                                        f" {eval_cfg.spp_ref} spp FP64 evaluation references, {cfg.train_rooms} train rooms"
                                                        f" at {cfg.train_res}^2 ({cfg.crop}^2 crops, batch {cfg.batch}),"
                                                        f" {cfg.eval_rooms} held-out rooms, {cfg.steps} Adam steps"},
            "relmse_noisy_mean": float(np.mean([r["relmse_noisy"] for r in rows])),
            "relmse_denoised_mean": float(np.mean([r["relmse_denoised"] for r in rows])),
            "relmse_final_mean": float(np.mean([r["relmse_final"] for r in rows])),
            "value_with_prediction": round(float(np.mean([r["time_final_with_prediction_s"] for r in rows])
                                                 / np.mean(tp)), 4) if tp else None,
            "prediction_note": "value: denoised time = input render + features + inference, plain time = one render at "
                               "the smallest sample count that meets the target (known from the reference); neither "
                               "side pays for estimating its error. value_with_prediction adds the fallback decision "
                               "(a second input render and inference, and the relMSE between the two outputs read back)",
            "rooms_meeting_target": ok_d, "fallbacks": sum(r["fallback"] for r in rows), "fallback_spp": fb_spp,
            "time_plain_mean_s": float(np.mean(tp)) if tp else None, "time_denoised_mean_s": float(np.mean(td)),
            "render_input_mean_s": float(np.mean([r["render_s"] for r in rows])),
            "inference_mean_s": float(np.mean([r["inference_s"] for r in rows])),
            "time_with_prediction_mean_s": float(np.mean([r["time_with_prediction_s"] for r in rows])),
            "spp_plain_to_target": [r["spp_plain_to_target"] for r in rows],
            "loss_first_last": [losses[0][1], losses[-1][1]], "data_s": round(data_s, 1),
            "train_s": round(train_s, 1), "eval_s": round(eval_s, 1),
            "per_room": [{k: r[k] for k in ("seed", "relmse_noisy", "relmse_denoised", "relmse_final", "fallback",
                                            "spp_plain_to_target", "time_plain_s", "time_final_s")} for r in rows]}
    return line


def run_denoise_secondary(args, spp_in: int = 4, rr_in: int = -1):
    """The denoiser's time to relMSE <= 0.01, denoised / plain, at a reduced
    size for the default bench line: 64 training rooms with 256-spp targets,
    3,000 Adam steps, 16 held-out rooms against 1,024-spp references; the
    input at spp_in samples per pixel (the configured 4, or 1 with Russian
    roulette from the first bounce, rr_in 0). The stated size (2,000 training
    rooms, 200 held-out rooms against 4,096-spp references) is `--workload
    denoise --dn-train 2000 --dn-eval 200 --dn-steps 6000 --dn-ref-spp 256
    --dn-eval-ref-spp 4096 --dn-spp-in 1 --dn-rr-in 0`."""
    sub = argparse.Namespace(**vars(args))
    sub.dn_train, sub.dn_eval, sub.dn_steps = 64, 16, 3000
    sub.dn_ref_spp, sub.dn_eval_ref_spp, sub.dn_spp_in, sub.dn_depth_in, sub.dn_rr_in = 256, 1024, spp_in, 0, rr_in
    sub.dn_res = sub.dn_train_res = 512
    line = run_denoise(sub)
    line.pop("per_room", None)
    line.pop("spp_plain_to_target", None)
    return line


def run_denoise_infer(args):
    """Denoiser inference on --dn-batch 512x512 frames per call (copies of a
    4-spp render of a procedural room and its features), the tensor-core
    forward pass."""
    import torch
    from nostrum_pray_gb300 import denoise as D, native
    torch.cuda.set_device(0)
    res = args.dn_res
    cfg = D.DenoiseConfig(res=res, spp_ref=1, spp_in=args.dn_spp_in)
    st = D._setup(cfg)
    sc = native.Scene.from_setup(D.scenes.random_room(cfg.seed, grid=cfg.room_grid), st)
    nb = max(1, args.dn_batch)
    rad = torch.empty((nb, res, res, 3), dtype=torch.float32, device="cuda")
    feat = torch.empty((nb, res, res, 7), dtype=torch.float16, device="cuda")
    sc.render_pt(D._params(cfg, st, cfg.spp_in, seed=1), None, rad[0])
    sc.render_features(D._params(cfg, st, 1, seed=0), feat[0])
    for k in range(1, nb):
        rad[k].copy_(rad[0])
        feat[k].copy_(feat[0])
    out = torch.empty_like(rad)
    den = native.Denoiser(seed=cfg.seed)
    if args.dn_cuda_cores:
        den.set_tensor_cores(False)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    clocks = ClockSampler(0)
    clocks.start()
    ms = _timed_frames(lambda: den.denoise(rad, feat, out), args.steps, args.warmup, flush)
    clk = clocks.stop()
    den.check()
    # end to end: pinned host input -> device, inference, output -> pinned host
    h_rad, h_feat = rad.cpu().pin_memory(), feat.cpu().pin_memory()
    h_out = torch.empty(out.shape, dtype=out.dtype).pin_memory()
    stream = torch.cuda.current_stream()

    def e2e_step():
        rad.copy_(h_rad, non_blocking=True)
        feat.copy_(h_feat, non_blocking=True)
        den.denoise(rad, feat, out)
        h_out.copy_(out, non_blocking=True)

    e2e_ms = _timed_frames(e2e_step, args.steps, args.warmup, flush)
    stream.synchronize()
    flops = D.forward_flops(res, res, nb)
    nbytes = D.forward_bytes(res, res, nb)
    per = ms / args.steps / 1e3
    peak, peak_kind = measured_bf16()
    hbm, hbm_kind = measured_peaks()
    achieved = flops / per / 1e12
    # the pass's arithmetic intensity (FLOPs per algorithmic DRAM byte) is
    # below the machine's ridge point (bf16 peak / HBM bandwidth), so the
    # memory roofline binds; the tensor-core figure is reported beside it
    intensity = flops / nbytes
    ridge = peak * 1e12 / (hbm * 1e9)
    gbs = nbytes / per / 1e9
    # DRAM bytes of one pass from the committed ncu capture (the sum over the
    # pass's launches, one 512^2 frame on the tensor cores), scaled by frames
    prof = committed_profile("denoise_infer", f"{res}")  # profiles/denoise_infer_512.json
    traffic = (int(prof["dram_bytes_per_frame"] * nb) if prof.get("dram_bytes_per_frame") and not args.dn_cuda_cores
               else None)
    line = {"metric": "denoised frames/s", "value": round(nb * args.steps / (ms / 1e3), 2), "unit": "frames/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": f"U-Net denoiser inference (19 3x3 convs, {D.num_params()} parameters, random "
                                   f"initialisation), {nb} {res}x{res} frame(s) per call: {cfg.spp_in}-spp room "
                                   f"render + features",
                       "tensor_cores": not args.dn_cuda_cores, "l2": "flushed between steps",
                       "launch": "one CUDA graph per call (recorded by the first call)"},
            "e2e": {"value": round(nb * args.steps / (e2e_ms / 1e3), 2), "unit": "frames/s",
                    "h2d_bytes_per_step": rad.numel() * 4 + feat.numel() * 2, "d2h_bytes_per_step": out.numel() * 4},
            "gpu_launches": D.denoise_launches(res, res, nb, tensor_cores=not args.dn_cuda_cores,
                                               sm_count=torch.cuda.get_device_properties(0).multi_processor_count)
            * args.steps,
            "roofline": ({"bound": "hbm", "achieved": round(gbs, 1), "peak": hbm, "unit": "GB/s",
                          "frac": round(gbs / hbm, 4), "peak_kind": f"{hbm_kind} HBM copy bandwidth"}
                         if intensity < ridge else
                         {"bound": "tensor", "achieved": round(achieved, 2), "peak": peak, "unit": "TFLOP/s",
                          "frac": round(achieved / peak, 5), "peak_kind": peak_kind})
                        | {"traffic": traffic, "algorithmic_bytes_per_call": nbytes, "algorithmic_flops_per_call": flops,
                           "intensity_flop_per_byte": round(intensity, 1), "ridge_flop_per_byte": round(ridge, 1),
                           "tensor": {"achieved": round(achieved, 2), "peak": peak, "unit": "TFLOP/s",
                                      "frac": round(achieved / peak, 5), "peak_kind": peak_kind},
                         "note": "whole forward pass timed: input packing and the 19 convolutions (on the tensor"
                                 " cores the pooling, upsampling + concatenation, residual and output transform are"
                                 " stores of their epilogues; on the CUDA cores kernels of their own)"},
            "clocks": clk}
    print(json.dumps(line), flush=True)


def run_denoise_train(args):
    """Denoiser training steps (forward, L1 loss, backward, Adam) on a fixed
    random batch of 8 crops of 128 x 128, the training shape of the denoise
    workload, on the tensor cores (--dn-cuda-cores: every convolution on the
    CUDA cores)."""
    import torch
    from nostrum_pray_gb300 import denoise as D, native
    torch.cuda.set_device(0)
    n, h, w = 8, 128, 128
    rng = np.random.default_rng(0)
    rad = torch.from_numpy((rng.random((n, h, w, 3)) * 2).astype(np.float32)).cuda()
    feat = torch.from_numpy(rng.random((n, h, w, 7)).astype(np.float16)).cuda()
    tgt = torch.from_numpy(rng.random((n, h, w, 3)).astype(np.float32)).cuda()
    den = native.Denoiser(seed=1)
    if args.dn_cuda_cores:
        den.set_tensor_cores(False)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    clocks = ClockSampler(0)
    clocks.start()
    ms = _timed_frames(lambda: den.train_step(rad, feat, tgt, 1e-4), args.steps, args.warmup, flush)
    clk = clocks.stop()
    den.check()
    # forward, backward-data (every convolution but the first) and weight gradient: 2 FLOPs per MAC each
    fwd = D.forward_flops(h, w, n)
    first = 2 * 9 * D.CONVS[0][0] * D.CONVS[0][1] * h * w * n
    flops = 3 * fwd - first
    per = ms / args.steps / 1e3
    peak, peak_kind = measured_bf16()
    achieved = flops / per / 1e12
    line = {"metric": "training steps/s", "value": round(args.steps / (ms / 1e3), 2), "unit": "steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": f"U-Net denoiser training step (forward, L1 loss, backward, Adam; {D.num_params()} "
                                   f"parameters), batch {n} x {h}x{w}, random inputs",
                       "tensor_cores": not args.dn_cuda_cores, "l2": "flushed between steps"},
            "roofline": {"bound": "tensor", "achieved": round(achieved, 2), "peak": peak, "unit": "TFLOP/s",
                         "frac": round(achieved / peak, 5), "traffic": None, "peak_kind": peak_kind,
                         "algorithmic_flops_per_step": flops,
                         "note": "convolution FLOPs of the forward pass, the backward-data pass (all but the first "
                                 "convolution) and the weight gradients over the whole step's time (pooling, "
                                 "upsampling, loss, Adam and format kernels included)"},
            "clocks": clk}
    return line


def main():
    args = parse()
    if args.impl == "reference" and args.workload == "cornell":
        print(json.dumps(run_reference_cornell(args)), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "cornell":
        print(json.dumps(run_cornell(args)), flush=True)
    elif args.workload == "room":
        print(json.dumps(run_pt(args)), flush=True)
    elif args.workload == "batch":
        print(json.dumps(run_batch(args)), flush=True)
    elif args.workload == "denoise":
        print(json.dumps(run_denoise(args)), flush=True)
    elif args.workload == "denoise-infer":
        run_denoise_infer(args)
    elif args.workload == "denoise-train":
        print(json.dumps(run_denoise_train(args)), flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
