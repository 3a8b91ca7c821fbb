#!/usr/bin/env python
"""Benchmark of the PT-MIS / PLOC hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step" = one render job): the single-job plain GPU
configuration -- a procedural icosphere at subdivision 8 (1,310,720
triangles) radially displaced by 4-octave fBm of amplitude 0.15, on a
2-triangle ground plane, seeded Disney parameters on the sphere and a
Lambertian ground, a constant environment of 0.5 plus a directional light of
2.0, 1024x1024, 256 samples per pixel, depth 16 (Russian roulette after
bounce 5), PLOC search radius 16 with the tree built on the GPU.  The scene
is synthetic and seeded.

Printed on one JSON line:
  value       Msamples/s of the job with the scene resident in HBM (the
              BVH built once), timed with CUDA events on the launching
              stream; the L2 is flushed (256 MiB write) between steps
  e2e         the same metric through the C ABI with host buffers: every
              step uploads the triangles, builds the PLOC tree on the GPU,
              renders and copies the film back
  roofline    the dominant traversal kernel: algorithmic bytes (nodes
              visited x node size -- 64 B binary, 32*W B for W-wide nodes --
              + triangles tested x 48 B, counted in-kernel)
              per launch over its CUDA-event duration, against the measured
              HBM copy bandwidth
  cpu_baseline  the oracle (a C++ restatement of the reference's CPU path)
              on the host cores, on a bounded sample of the same job
With --gpus N (torchrun), every rank renders its own job (replicas: the path
shards by job with no exchange), and value is the sum over ranks over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Msamples/s + p99 job latency, 1 GB300, batched/served vs plain at equal RMSE"
WORKLOAD = ("single-job plain GPU: displaced icosphere subdiv 8 (1,310,720 tris) "
            "+ 2-tri ground, Disney, 1024x1024, 256 spp, depth 16, PLOC r=16 built on the GPU")
SPP, RES, DEPTH, MIN_B, RADIUS = 256, 1024, 16, 5, 16
TRI_BYTES = 48


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--spp", type=int, default=SPP)
    ap.add_argument("--res", type=int, default=RES)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--batch-jobs", type=int, default=48)
    ap.add_argument("--serve-jobs", type=int, default=340,
                    help="jobs per load point of the serving sweep")
    ap.add_argument("--serve-policy", choices=["fair", "fifo"], default="fair")
    ap.add_argument("--serve-capacity", type=float, default=0.0,
                    help="Msamples/s the serving loads are fractions of (0: the "
                         "plain tracer's throughput on the serving workload)")
    ap.add_argument("--only-serve", action="store_true",
                    help="run the serving sweep alone (one JSON line)")
    ap.add_argument("--serve-loads", default="0.6,0.9,1.5",
                    help="arrival rates of the serving sweep, as fractions of the "
                         "batched throughput")
    ap.add_argument("--rmse-crop", type=int, default=32)
    ap.add_argument("--rmse-spp", type=int, default=4096)
    ap.add_argument("--wave-paths", type=int, default=0,
                    help="paths in flight per wave (0: library default)")
    ap.add_argument("--batch-wave-paths", type=int, default=0,
                    help="paths per wave of the batched/served context (0: default)")
    ap.add_argument("--no-sppm", action="store_true")
    ap.add_argument("--only-sppm", action="store_true",
                    help="run the SPPM section alone (one JSON line)")
    ap.add_argument("--sppm-iters", type=int, default=32)
    ap.add_argument("--sppm-photons", type=int, default=4_000_000)
    ap.add_argument("--no-large", action="store_true",
                    help="skip the large-scene workload (26.2 M triangles, "
                         "1920x1080, 1024 spp, depth 32, FP64 crop reference)")
    ap.add_argument("--no-cornell", action="store_true",
                    help="skip the Cornell-box workload (256x256, 64 spp, depth 8)")
    ap.add_argument("--large-ref-spp", type=int, default=65536)
    ap.add_argument("--bvh-width", type=lambda v: (int(v[:-1]) | 0x100) if v.endswith("c")
                    else int(v), default=0,
                    help="traversal tree: 2 binary, 4/8 collapsed, 4c/8c collapsed with "
                         "quantised boxes, 0 library default")
    return ap.parse_args()


def workload_scene(res):
    from ajisai_render_gb300 import scenes as S
    return S.flatten(S.icosphere_scene(subdiv=8, seed=0, width=res, height=res))


def config(args):
    return {"workload": WORKLOAD, "resolution": f"{args.res}x{args.res}", "spp": args.spp,
            "max_depth": DEPTH, "min_bounces": MIN_B, "cont_prob": 0.9,
            "ploc_search_radius": RADIUS, "triangles": 1310722, "sampler": "counter (seeded)",
            "l2": "flushed between steps (256 MiB write)", "tri_test": "moller-trumbore"}


# ----------------------------------------------------------------- clocks --
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names[1:], f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_profile(kernel, scene, bvh_width):
    """The committed ncu figures of a traversal kernel (profiles/traffic.json,
    a small capture of the same kernel: per captured launch its rays, DRAM
    bytes, time, L1/L2 hit rates and throughput, threads per warp
    instruction), when they were taken on this scene and tree layout; None
    otherwise."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    k = d.get(kernel)
    if not k or d.get("scene") != scene or d.get("bvh_width") != bvh_width:
        return None
    return {**k, "source": d.get("source"), "captured": d.get("captured")}


def scaled_traffic(prof, rays_per_launch):
    """DRAM bytes per launch of this run: each launch's rays times the
    captured DRAM bytes per ray of the same bounce (later bounces take the
    last captured bounce's figure), averaged over the launches."""
    bpr = [b for b in prof["dram_bytes_per_ray"] if b is not None]
    if not bpr or not rays_per_launch:
        return None
    tot = sum(r * bpr[min(i, len(bpr) - 1)] for i, r in enumerate(rays_per_launch))
    return tot / len(rays_per_launch)


def any_hit_total(by_kind, node_bytes, peak):
    """Algorithmic bytes (node visits x node size + triangle tests x 48 B)
    of every any-hit launch of the profiled step -- the per-lane kernel and
    the packet launches -- over their summed device time, per launch kind
    and together, against the measured HBM copy rate."""
    out = {}
    for name, kinds in (("k_shadow", ("any",)), ("k_shadow_packet", ("any_packets",)),
                        ("together", ("any", "any_packets"))):
        recs = [r for k in kinds for r in by_kind.get(k, [])]
        ms = float(sum(r["ms"] for r in recs))
        rays = int(sum(r["rays"] for r in recs))
        b = float(sum(r["nodes"] * node_bytes + r["tris"] * TRI_BYTES for r in recs))
        gbs = b / (ms / 1e3) / 1e9 if ms > 0 else None
        out[name] = {"rays": rays, "ms": ms, "algorithmic_bytes": b,
                     "achieved_gbs": gbs, "frac": gbs / peak if gbs else None}
    return out


def time_weighted(prof, key):
    """A captured per-launch figure averaged with the launches' times as
    weights."""
    ms = np.asarray(prof["ms"], np.float64)
    return float(np.dot(ms, np.asarray(prof[key], np.float64)) / ms.sum())


# ------------------------------------------------------------- CPU side --
def cpu_sample(flat, seconds, threads, spp):
    """Time the oracle on a bounded sample of the job: whole image rows spread
    evenly over the film, as many as fit the time budget."""
    from oracle import pyoracle as O
    sc = O.OracleScene(flat, RADIUS)
    W = int(flat.camera[34])
    H = int(flat.camera[35])
    params = dict(spp=spp, min_bounces=MIN_B, max_bounces=DEPTH)
    # calibrate on one row through the middle, then size the sample
    t = time.perf_counter()
    sc.render(flat.camera, params, seed=1, pixel_range=((H // 2) * W, (H // 2 + 1) * W),
              threads=threads)
    per_row = time.perf_counter() - t
    nrows = int(max(1, min(H, seconds / max(per_row, 1e-6))))
    rows = np.linspace(0, H - 1, nrows).round().astype(int)
    t = time.perf_counter()
    for y in rows:
        sc.render(flat.camera, params, seed=1, pixel_range=(y * W, (y + 1) * W),
                  threads=threads)
    dt = time.perf_counter() - t
    samples = len(rows) * W * spp
    build_s = sc.build_seconds
    sc.close()
    return samples / dt / 1e6, len(rows), dt, build_s


def run_reference(args):
    """The reference's CPU path on the host cores: the oracle port (the
    reference's own build needs its x86 toolchain setup and sources, which
    the GPU host does not have), all host threads, a bounded pixel sample of
    the same job per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    flat = workload_scene(args.res)
    threads = os.cpu_count() or 1
    per_step = max(1.0, args.cpu_seconds / 2)
    for _ in range(args.warmup):
        cpu_sample(flat, 0.5, threads, args.spp)
    vals, npxs, secs = [], [], []
    for _ in range(args.steps):
        v, npx, dt, _ = cpu_sample(flat, per_step, threads, args.spp)
        vals.append(v)
        npxs.append(npx)
        secs.append(dt)
    value = float(np.sum(np.array(npxs) * args.res * args.spp) / np.sum(secs) / 1e6)
    sample = (f"{int(np.mean(npxs))} image rows spread over the film x {args.res} px x "
              f"{args.spp} spp per step (about {per_step:.0f} s of CPU work), oracle port "
              "of the reference path")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Msamples/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": float(np.mean(secs) * 1e3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scene)", "config": config(args),
        "cpu_baseline": {"value": value, "unit": "Msamples/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}))


# ----------------------------------------------------------------- ranks --
def whole_job_rate(dist, world, units_per_rank, seconds, device=None):
    """Throughput of the whole job under N replicas: every rank processed
    `units_per_rank` in its own `seconds`; the job took the slowest rank's
    time (a MAX all-reduce).  Returns (M units/s over all ranks, that
    time)."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        seconds = float(t.item())
    return world * units_per_rank / seconds / 1e6, seconds


# ------------------------------------------------------------- GPU side --
def run_ours(args):
    import torch

    from ajisai_render_gb300 import api

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    flat = workload_scene(args.res)
    W = H = args.res
    samples_per_step = W * H * args.spp
    ctx = api.Context(local, wave_paths=args.wave_paths)
    scene = api.GpuScene(ctx, flat, api.CreatePLOCAggregate(RADIUS, bvh_width=args.bvh_width))
    rend = api.PTRenderer(api.PTRendererArgs(spp=args.spp, min_bounces=MIN_B,
                                             max_bounces=DEPTH), seed=1 + rank)
    out = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        rend.render_device(scene, flat.camera, out.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize(dev)

    # timed region: exactly K steps (no per-kernel events inside it)
    ctx.stats(reset=True)
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        rend.render_device(scene, flat.camera, out.data_ptr(), stream.cuda_stream)
        b.record(stream)
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = float(np.sum(step_ms))
    launches_timed = int(ctx.stats()["kernel_launches"])
    # one more step, outside the timed region, with CUDA events around every
    # traversal and shading launch: the per-kernel breakdown and roofline
    ctx.stats(reset=True)
    ctx.set_profiling(True)
    flush.zero_()
    pa, pb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pa.record(stream)
    rend.render_device(scene, flat.camera, out.data_ptr(), stream.cuda_stream)
    pb.record(stream)
    torch.cuda.synchronize(dev)
    prof_ms = pa.elapsed_time(pb)
    st = ctx.stats()
    log = ctx.launch_log(reset=True)
    ctx.set_profiling(False)
    value, total_s = whole_job_rate(dist, world, samples_per_step * args.steps,
                                    total_ms / 1e3, dev)
    total_ms = total_s * 1e3

    # per kernel, from the per-launch log: the per-lane traversals (kinds
    # closest, any) and the packet traversals of bounce 0's camera and
    # directional-light shadow rays (closest_packets, any_packets)
    by_kind = {}
    for r in log:
        by_kind.setdefault(r["kind"], []).append(r)
    kind_ms = {k: float(sum(r["ms"] for r in v)) for k, v in by_kind.items()}

    # roofline of the dominant traversal kernel
    kinds = {"closest": "k_extend", "any": "k_shadow"}
    dom = max(kinds, key=lambda k: kind_ms.get(k, 0.0))
    kname = kinds[dom]
    launches_k = by_kind.get(dom, [])
    launches = max(1, len(launches_k))
    n_nodes = sum(r["nodes"] for r in launches_k)
    n_tris = sum(r["tris"] for r in launches_k)
    # closest-hit rays walk the binary layout kept beside a 4-wide tree
    node_bytes = scene.info()["closest_node_bytes" if dom == "closest" else "bvh_node_bytes"]
    bytes_per_launch = (n_nodes * node_bytes + n_tris * TRI_BYTES) / launches
    node_bytes_any = scene.info()["bvh_node_bytes"]
    avg_ms = kind_ms.get(dom, 0.0) / launches
    achieved = bytes_per_launch / (avg_ms / 1e3) / 1e9 if avg_ms > 0 else None
    peak, peak_kind = peaks()
    prof = committed_profile(kname, "icosphere1310k", scene.info()["bvh_width"])
    traffic = scaled_traffic(prof, [r["rays"] for r in launches_k]) if prof else None
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak if achieved else None,
                "traffic": traffic,
                "traffic_note": ("DRAM bytes per ray of a small capture of the same kernel "
                                 "on the same scene (per bounce), times this run's rays "
                                 "per launch" if prof else None),
                "traffic_source": prof["source"] if prof else None,
                # where the gathers are served: the same capture's cache figures,
                # weighted by launch time (ncu: L1TEX and L2 throughput as a
                # fraction of their peaks, hit rates, active threads per warp
                # instruction = SIMT efficiency x 32)
                "cache": None if not prof else {
                    k: time_weighted(prof, k) for k in (
                        "l1_throughput_pct", "l2_throughput_pct", "l1_hit_rate_pct",
                        "l2_hit_rate_pct", "threads_per_warp_inst")},
                "rays_per_launch": [int(r["rays"]) for r in launches_k],
                "nodes_per_ray_per_launch": [round(r["nodes"] / max(1, r["rays"]), 2)
                                             for r in launches_k],
                "other_kind_rays_per_launch": [int(r["rays"]) for r in log
                                               if r["kind"] not in (dom, "shade")],
                "ms_per_launch": [round(float(r["ms"]), 3) for r in launches_k],
                "algorithmic_bytes_per_launch": bytes_per_launch,
                # the same fraction with the nominal 80-byte 4-wide node
                # (six planes of four floats and four 32-bit references) in
                # place of this layout's 128-byte, 64-byte-aligned node
                "frac_at_80_byte_nodes": ((n_nodes * 80 + n_tris * TRI_BYTES) / launches
                                          / (avg_ms / 1e3) / 1e9 / peak)
                if avg_ms > 0 and node_bytes == 128 else None,
                # the any-hit traversal as a whole: the per-lane kernel and
                # bounce 0's packet launch together (a packet reads a node
                # once for up to 32 lanes, so the packets' algorithmic rate
                # is not bounded by the HBM copy rate)
                "any_hit_all_kernels": any_hit_total(by_kind, node_bytes_any, peak),
                "avg_launch_ms": avg_ms, "launches": len(launches_k),
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                "kernel_time_share": kind_ms.get(dom, 0.0) / max(1e-9, prof_ms),
                "rays_per_s": (st["closest_rays"] + st["any_rays"]) / (prof_ms / 1e3),
                "measured_on": "one extra step with CUDA events around each launch"}

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        h2d = (flat.tris.nbytes + flat.corner_n.nbytes + flat.tri_mat.nbytes +
               flat.tri_flags.nbytes + flat.world.nbytes + flat.materials.nbytes +
               flat.lights.nbytes)
        d2h = W * H * 16

        # the step's inputs and its result live in pinned host memory (numpy
        # views of pinned tensors, handed to the C ABI as plain pointers)
        def pinned(a):
            return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

        flat_h = dataclasses.replace(
            flat, tris=pinned(flat.tris), corner_n=pinned(flat.corner_n),
            tri_mat=pinned(flat.tri_mat), tri_flags=pinned(flat.tri_flags),
            world=pinned(flat.world), materials=pinned(flat.materials),
            lights=pinned(flat.lights))
        film = api.Film(W, H, rgbw=pinned(np.zeros((H, W, 4), np.float32)))
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s2 = api.GpuScene(ctx, flat_h, api.CreatePLOCAggregate(RADIUS,
                                                                    bvh_width=args.bvh_width))
            rend.Render(s2, flat_h.camera, film)
            s2.release()
        dt = time.perf_counter() - t0
        e2e_value, dt = whole_job_rate(dist, world, samples_per_step * args.steps,
                                       dt, dev)
        e2e = {"value": e2e_value,
               "unit": "Msamples/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": dt / args.steps * 1e3}

    cpu = None
    rays_per_sample = (st["closest_rays"] + st["any_rays"]) / samples_per_step
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, npx, dt, build_s = cpu_sample(flat, args.cpu_seconds, threads, args.spp)
        cpu = {"value": v, "unit": "Msamples/s", "cores": threads, "kind": "port",
               "sample": f"{npx} image rows spread over the film x {args.res} px x "
                         f"{args.spp} spp ({dt:.1f} s), oracle port of the reference "
                         "path, all host threads",
               "ploc_build_ms": build_s * 1e3,
               "ploc_build_note": "the oracle's PLOCAggregate::Build restatement, one "
                                  "host thread, 1,310,722 triangles",
               "mrays_s": v * rays_per_sample,
               "mrays_note": "samples/s times the rays per sample the GPU counted on "
                             "the same job (the same paths: shared counter sampler)"}

    img = out.float().cpu().numpy()
    nonfinite = int((~np.isfinite(img)).any(-1).sum())

    batched = served = large = sppm = cornell = None
    if rank == 0 and world == 1 and not args.no_cornell:
        cornell = run_cornell(args, local)
    if rank == 0 and world == 1 and not args.no_large:
        large = run_large(args, local)
    if rank == 0 and world == 1 and not args.no_sppm:
        sppm = run_sppm(args, local)
    if rank == 0 and world == 1 and not args.no_batch:
        bctx = api.Context(local, wave_paths=args.batch_wave_paths,
                           hbm_budget_bytes=150 << 30)
        batched = run_batched(bctx, args)
        if not args.no_serve:
            served = run_served(bctx, args, args.serve_capacity * 1e6)
        batched.pop("_capacity")
        bctx.close()
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scene, no dataset)",
            "config": {**config(args), "bvh_width": scene.info()["bvh_width"],
                       "wave_paths": args.wave_paths or (1 << 28),
                       "trace_overlap": os.environ.get("AJG_TRACE_OVERLAP", "1") != "0"},
            "clocks": clk, "e2e": e2e, "roofline": roofline,
            "cpu_baseline": cpu, "gpu_launches": launches_timed,
            "ploc_build_ms": scene.info()["build_ms"],
            "kernel_ms_per_step": {"k_extend": kind_ms.get("closest", 0.0),
                                   "k_extend_packet": kind_ms.get("closest_packets", 0.0),
                                   "k_shadow": kind_ms.get("any", 0.0),
                                   "k_shadow_packet": kind_ms.get("any_packets", 0.0),
                                   "k_shade": kind_ms.get("shade", 0.0),
                                   "step_under_events": prof_ms},
            # bounce 0's packet launches: rays and node visits per ray
            "packet_stats": {k: {"rays": int(sum(r["rays"] for r in v)),
                                 "nodes_per_ray": sum(r["nodes"] for r in v)
                                 / max(1, sum(r["rays"] for r in v))}
                             for k, v in by_kind.items() if k.endswith("_packets")},
            "trace_stats": {
                kind: {"rays_per_step": st[f"{kind}_rays"],
                       "nodes_per_ray": st[f"{kind}_nodes"] / max(1, st[f"{kind}_rays"]),
                       "tris_per_ray": st[f"{kind}_tris"] / max(1, st[f"{kind}_rays"])}
                for kind in ("closest", "any")},
            "step_ms": step_ms, "nonfinite_pixels": nonfinite,
            "mrays_s": value * rays_per_sample,
            # the metric's latency half: p99 of the serving sweep's busiest
            # load point below saturation (its offered load beside it)
            "p99_job_latency_ms": served["p99_ms"] if served else None,
            "p99_at_offered_load": served["latency_at_load"] if served else None,
            # the metric's comparison: batched / served throughput over the
            # plain single-job tracer on the same mixes (films bit-identical)
            "batched_vs_plain": batched["speedup_vs_plain"] if batched else None,
            "small_jobs_batched_vs_plain": (batched["small_jobs"]["speedup_vs_plain"]
                                            if batched else None),
            "served_vs_plain_at_saturation": (served["saturated_vs_plain"]
                                              if served else None),
            "cornell": cornell, "batched": batched, "served": served, "large": large,
            "sppm": sppm, "impl": "ours"}))
    scene.release()
    ctx.close()
    if dist:
        dist.destroy_process_group()


# ------------------------------------------------- batched and served --
BATCH_DEPTH = 12


def _same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def _cam(camera, w, h):
    from ajisai_render_gb300 import scenes as S
    return S.Camera(camera.position, camera.look_at, camera.up, camera.fov, w, h)


def build_mix(ctx, n, seed):
    """Scenes of the batched workload, resident on the GPU."""
    from ajisai_render_gb300 import api
    from ajisai_render_gb300 import scenes as S
    jobs = S.batch_workload(n, seed=seed)
    built, tris = [], 0
    for j in jobs:
        sc = S.mixed_scene(j["scene_seed"], j["tris"], j["res"], j["res"])
        g = api.GpuScene(ctx, sc, api.CreatePLOCAggregate(RADIUS))
        tris += g.flat.n_tris
        built.append((g, sc.camera))
    return jobs, built, tris


def run_batched(ctx, args):
    """The batched workload: the same jobs rendered one by one through
    ajg_render (the plain single-job tracer) and as one ajg_render_batch;
    both with host results.  Films must be identical bit for bit; each
    image's RMSE against an FP64-accumulated render of a central crop."""
    import torch
    from ajisai_render_gb300 import api, autotune
    t0 = time.perf_counter()
    jobs, built, tris = build_mix(ctx, args.batch_jobs, seed=1)
    gen_s = time.perf_counter() - t0
    descs = []
    for j, (g, cam) in zip(jobs, built):
        r = api.PTRenderer(api.PTRendererArgs(spp=j["spp"], min_bounces=MIN_B,
                                              max_bounces=BATCH_DEPTH), seed=7)
        descs.append((g, _cam(cam, j["res"], j["res"]), r))
    samples = sum(j["res"] ** 2 * j["spp"] for j in jobs)
    ctx.configure_serving("fifo", wave_paths=args.batch_wave_paths)
    # warm both paths (arenas, graphs) on a small job
    descs[0][2].Render(descs[0][0], _cam(descs[0][1], 16, 16))
    ctx.render_batch([(descs[0][0], _cam(descs[0][1], 16, 16), descs[0][2])])
    torch.cuda.synchronize()
    # the request loop's wave size for this batch, tuned on 1/8 of its samples
    tuned = None
    if not args.batch_wave_paths:
        tuned = autotune.tune_batch(ctx, descs)
    plain, t_each = [], []
    t = time.perf_counter()
    for g, cam, r in descs:
        t1 = time.perf_counter()
        plain.append(r.Render(g, cam))
        t_each.append(time.perf_counter() - t1)
    t_plain = time.perf_counter() - t
    t = time.perf_counter()
    batched = ctx.render_batch(descs)
    t_batch = time.perf_counter() - t
    identical = all(_same_bits(f.rgbw, p.rgbw) for (f, _), p in zip(batched, plain))
    # the plain arm by job size: where its time goes
    sizes = np.array([j["res"] ** 2 * j["spp"] for j in jobs], np.float64)
    classes = {}
    for name, lo, hi in (("small (< 4 M samples)", 0, 4e6),
                         ("medium (4-64 M samples)", 4e6, 64e6),
                         ("large (>= 64 M samples)", 64e6, np.inf)):
        m = (sizes >= lo) & (sizes < hi)
        if m.any():
            te = float(np.sum(np.array(t_each)[m]))
            classes[name] = {"jobs": int(m.sum()), "samples": int(sizes[m].sum()),
                             "plain_s": te,
                             "plain_msamples_s": float(sizes[m].sum() / te / 1e6)}
    # FP64 references of a central crop (+1 row/column of footprint sources)
    c = args.rmse_crop
    refs = []
    for (g, cam, r), j in zip(descs, jobs):
        res = j["res"]
        x0 = y0 = max(0, (res - c) // 2 - 1)
        rr = api.PTRenderer(api.PTRendererArgs(spp=args.rmse_spp, min_bounces=MIN_B,
                                               max_bounces=BATCH_DEPTH), seed=1234,
                            fp64_film=True)
        refs.append((g, cam, rr, (x0, y0, min(c + 1, res - x0), min(c + 1, res - y0))))
    t = time.perf_counter()
    ref_out = ctx.render_batch(refs)
    t_ref = time.perf_counter() - t
    rmse, trimmed, nonfinite = [], [], []
    for (film, _), (ref, _), (_, _, _, win) in zip(batched, ref_out, refs):
        x0, y0, w, h = win
        cw, ch = min(c, w), min(c, h)
        fa = np.ascontiguousarray(film.rgbw[y0:y0 + ch, x0:x0 + cw])
        fb = np.ascontiguousarray(ref.rgbw[:ch, :cw])
        a = torch.from_numpy(fa).cuda()
        b = torch.from_numpy(fb).cuda()
        e, _ = ctx.image_rmse(a.data_ptr(), b.data_ptr(), cw, ch)
        rmse.append(e)
        # a robust error beside it: the RMSE without the worst 1% of the
        # crop's pixels (a single firefly dominates the plain RMSE)
        ia = fa[..., :3].astype(np.float64) / np.maximum(fa[..., 3:], 1e-30)
        ib = fb[..., :3].astype(np.float64) / np.maximum(fb[..., 3:], 1e-30)
        sq = ((ia - ib) ** 2).mean(-1).ravel()
        sq = np.sort(sq[np.isfinite(sq)])
        keep = sq[:max(1, int(len(sq) * 0.99))]
        trimmed.append(float(np.sqrt(keep.mean())))
        nonfinite.append(int((~np.isfinite(film.rgbw)).any(-1).sum()))
    rmse = np.array(rmse)
    return {
        "workload": f"{len(jobs)} jobs over their own scenes ({tris:,} triangles in all, "
                    "displaced icospheres or random-box clutter, 1k-2M each), "
                    "res {128,256,512,1024}^2, spp log-uniform 16-256, depth 12, Disney",
        "samples": int(samples),
        "batched_msamples_s": samples / t_batch / 1e6,
        "plain_msamples_s": samples / t_plain / 1e6,
        "speedup_vs_plain": t_plain / t_batch,
        "batched_s": t_batch, "plain_s": t_plain,
        "plain_by_job_size": classes,
        # what batching could reach on this mix if every sample ran at the
        # plain rate of the biggest jobs
        "speedup_bound_at_large_job_rate": t_plain / (samples / (1e6 * max(
            c["plain_msamples_s"] for c in classes.values()))) if classes else None,
        "autotuned": tuned,
        "films_bit_identical": bool(identical),
        "rmse_vs_fp64": {"crop": c, "reference_spp": args.rmse_spp,
                         "median": float(np.median(rmse)), "max": float(rmse.max()),
                         "min": float(rmse.min()), "equal_for_both_arms": bool(identical),
                         "trimmed_99pct_median": float(np.median(trimmed)),
                         "trimmed_99pct_max": float(np.max(trimmed)),
                         "per_image": [round(float(x), 6) for x in rmse],
                         "per_image_trimmed_99pct": [round(x, 6) for x in trimmed]},
        "nonfinite_pixels_per_image": nonfinite,
        "results": "host buffers (device-to-host copy of every film inside the timing)",
        "scene_generation_and_build_s": gen_s, "reference_render_s": t_ref,
        "small_jobs": small_mix(ctx, built, jobs),
        "_capacity": samples / t_batch,
    }


def small_mix(ctx, built, jobs):
    """A sub-mix of small jobs over the same scenes (128^2 or 256^2, 16-64
    spp): the jobs whose plain renders leave the GPU underused, rendered one
    by one and as one batch."""
    from ajisai_render_gb300 import api
    rng = np.random.default_rng(11)
    descs, samples = [], 0
    for (g, cam), j in zip(built, jobs):
        res = int(rng.choice([128, 256]))
        spp = int(round(np.exp(rng.uniform(np.log(16), np.log(64)))))
        r = api.PTRenderer(api.PTRendererArgs(spp=spp, min_bounces=MIN_B,
                                              max_bounces=BATCH_DEPTH), seed=13)
        descs.append((g, _cam(cam, res, res), r))
        samples += res * res * spp
    ctx.render_batch(descs[:2])
    t = time.perf_counter()
    plain = [r.Render(g, cam) for g, cam, r in descs]
    t_plain = time.perf_counter() - t
    t = time.perf_counter()
    batched = ctx.render_batch(descs)
    t_batch = time.perf_counter() - t
    return {"workload": f"{len(descs)} jobs over the batched workload's scenes, "
                        "res {128,256}^2, spp log-uniform 16-64, depth 12",
            "samples": int(samples), "plain_msamples_s": samples / t_plain / 1e6,
            "batched_msamples_s": samples / t_batch / 1e6,
            "speedup_vs_plain": t_plain / t_batch,
            "films_bit_identical": all(_same_bits(f.rgbw, p.rgbw)
                                       for (f, _), p in zip(batched, plain))}


def serve_plan(n, seed):
    """n jobs of the serving workload: scene index (of 8), resolution
    {256,512,1024}^2, spp log-uniform 4-1024, camera on a seeded sphere."""
    from ajisai_render_gb300 import scenes as S
    rng = np.random.default_rng(seed)
    plan = []
    for _ in range(n):
        k = int(rng.integers(0, 8))
        res = int(rng.choice([256, 512, 1024]))
        spp = int(round(np.exp(rng.uniform(np.log(4), np.log(1024)))))
        plan.append((k, res, spp, S._orbit_camera(rng, res, res)))
    return plan, rng


def serve_point(ctx, built, plan, rng, rate, capacity_samples_s):
    """Poisson arrivals of the planned jobs at `rate` jobs/s; progressive
    results every 16 spp; returns the load point's statistics."""
    from ajisai_render_gb300 import api
    gaps = rng.exponential(1.0 / rate, len(plan))
    st0 = ctx.serve_stats()
    submitted = []
    t0 = time.perf_counter()
    at = 0.0
    for (k, res, spp, cam), gap in zip(plan, gaps):
        at += gap
        dt = t0 + at - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        r = api.PTRenderer(api.PTRendererArgs(spp=spp, min_bounces=MIN_B,
                                              max_bounces=BATCH_DEPTH),
                           seed=i_seed(k, res, spp))
        submitted.append(ctx.submit(built[k][0], cam, r, progress_spp=16))
    t_arrived = time.perf_counter() - t0
    sts = [j.wait() for j in submitted]
    for j in submitted:
        j.release()
    sub = np.array([s["submit_ms"] for s in sts])
    start = np.array([s["start_ms"] for s in sts])
    done_t = np.array([s["done_ms"] for s in sts])
    lat = done_t - sub
    first = np.array([s["first_result_ms"] for s in sts]) - sub
    size = np.array([r * r * s for _, r, s, _ in plan], np.float64)
    # slowdown: latency over the job's own service time at the measured
    # capacity (a job alone at idle)
    slow = lat / (size / capacity_samples_s * 1e3)
    # jobs in the system (submitted, not done) and waiting for admission,
    # sampled at every submission
    in_sys = [int(((sub <= t) & (done_t > t)).sum()) for t in sub]
    waiting = [int(((sub <= t) & (start > t)).sum()) for t in sub]
    q = len(in_sys) // 4
    span_ms = done_t.max() - sub.min()
    st1 = ctx.serve_stats()
    busy_ms = st1["busy_ms"] - st0["busy_ms"]
    pct = lambda a, p: float(np.percentile(a, p))
    return {
        "jobs": len(plan), "jobs_done": sum(1 for s in sts if s["state_name"] == "done"),
        "rate_jobs_s": rate, "arrivals_s": t_arrived,
        "msamples_s": float(size.sum() / (span_ms / 1e3) / 1e6),
        # the device's side: waves, their summed device time, and the
        # throughput while a wave ran
        "waves": int(st1["waves"] - st0["waves"]),
        "gpu_busy_frac": float(busy_ms / span_ms) if span_ms > 0 else None,
        "msamples_s_while_busy": float(size.sum() / (busy_ms / 1e3) / 1e6)
        if busy_ms > 0 else None,
        "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "mean_ms": float(lat.mean()),
        "first_result_p50_ms": pct(first, 50), "first_result_p99_ms": pct(first, 99),
        "slowdown_p50": pct(slow, 50), "slowdown_p99": pct(slow, 99),
        "admission_wait_p99_ms": pct(start - sub, 99),
        "jobs_in_system_max": int(max(in_sys)),
        "jobs_in_system_by_quarter": [float(np.mean(in_sys[i * q:(i + 1) * q]))
                                      for i in range(4)] if q else [],
        "jobs_waiting_max": int(max(waiting)),
    }


def serve_plain(built, plan):
    """The plain single-job tracer on jobs of the serving workload: each job
    rendered alone through ajg_render (host film), one after another."""
    from ajisai_render_gb300 import api
    samples = 0
    t = time.perf_counter()
    for k, res, spp, cam in plan:
        r = api.PTRenderer(api.PTRendererArgs(spp=spp, min_bounces=MIN_B,
                                              max_bounces=BATCH_DEPTH),
                           seed=i_seed(k, res, spp))
        r.Render(built[k][0], cam)
        samples += res * res * spp
    dt = time.perf_counter() - t
    return {"jobs": len(plan), "samples": int(samples), "s": dt,
            "msamples_s": samples / dt / 1e6}


def run_served(ctx, args, capacity_samples_s=0.0):
    """The serving sweep: Poisson arrivals of render jobs over 8 resident
    scenes at several rates -- fractions of the plain tracer's throughput on
    the same workload (40 jobs of it rendered one by one first), the
    highest past saturation; progressive results every 16 spp, fair
    scheduling; latency from submission to the final result."""
    jobs8, built, tris = build_mix(ctx, 8, seed=2)
    # the same workload through the plain tracer (jobs of another seed): the
    # capacity the load points are fractions of
    plain = serve_plain(built, serve_plan(min(40, args.serve_jobs), seed=4)[0])
    if not capacity_samples_s:
        capacity_samples_s = plain["msamples_s"] * 1e6
    ctx.configure_serving(args.serve_policy, wave_paths=args.batch_wave_paths)
    loads = [float(x) for x in args.serve_loads.split(",") if x]
    points = []
    t0 = time.perf_counter()
    for i, load in enumerate(loads):
        plan, rng = serve_plan(args.serve_jobs, seed=5 + i)
        mean_samples = np.mean([r * r * s for _, r, s, _ in plan])
        rate = load * capacity_samples_s / mean_samples
        pt = serve_point(ctx, built, plan, rng, rate, capacity_samples_s)
        pt["offered_load"] = load
        points.append(pt)
    total = sum(p["jobs"] for p in points)
    below = [p for p in points if p["offered_load"] < 1.0] or points
    head = max(below, key=lambda p: p["offered_load"]) if below else None
    return {
        "workload": f"{args.serve_jobs} jobs per load point ({total} in all; the "
                    "configuration's 10,000-job run is unmeasured), Poisson arrivals at "
                    f"{', '.join(f'{x:.0%}' for x in loads)} of the plain tracer's "
                    f"throughput on this workload ({capacity_samples_s / 1e6:.0f} "
                    "Msamples/s), 8 resident scenes "
                    f"({tris:,} triangles), res {{256,512,1024}}^2, spp log-uniform 4-1024, "
                    "camera on a seeded sphere, depth 12, progressive results every 16 spp, "
                    f"{args.serve_policy} scheduling, HBM budget 150 GB",
        "points": points,
        # the headline latency: the busiest load point below saturation
        "p50_ms": head["p50_ms"] if head else None,
        "p99_ms": head["p99_ms"] if head else None,
        "latency_at_load": head["offered_load"] if head else None,
        "saturated_msamples_s": max((p["msamples_s"] for p in points), default=None),
        "plain": plain,
        "saturated_vs_plain": (max((p["msamples_s"] for p in points), default=0.0) /
                               plain["msamples_s"]),
        "wall_s": time.perf_counter() - t0,
    }


def run_cornell(args, local):
    """The Cornell-style box at its full size (256x256, 64 spp, depth 8,
    roulette after bounce 3): GPU throughput, the oracle's on all host
    threads over the whole film, and both images' RMSE against an
    FP64-accumulated 8192-spp render."""
    import torch
    from ajisai_render_gb300 import api
    from ajisai_render_gb300 import scenes as S
    from oracle import pyoracle as O
    flat = S.flatten(S.cornell_box(256, 256))
    ctx = api.Context(local)
    try:
        scene = api.GpuScene(ctx, flat, api.CreatePLOCAggregate(14))
        p = dict(spp=64, min_bounces=3, max_bounces=8)
        rend = api.PTRenderer(api.PTRendererArgs(**p), seed=1)
        out = torch.empty((256, 256, 4), dtype=torch.float32, device="cuda")
        stream = torch.cuda.current_stream()
        for _ in range(3):
            rend.render_device(scene, flat.camera, out.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        reps = 20
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            rend.render_device(scene, flat.camera, out.data_ptr(), stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / reps
        samples = 256 * 256 * 64
        conv = api.PTRenderer(api.PTRendererArgs(spp=8192, min_bounces=3, max_bounces=8),
                              seed=99, fp64_film=True).Render(scene, flat.camera).rgbw
        d_conv = torch.from_numpy(conv).cuda()
        e_gpu, _ = ctx.image_rmse(out.data_ptr(), d_conv.data_ptr(), 256, 256)
        res = {"workload": "Cornell-style box (34 triangles), 256x256, 64 spp, depth 8, "
                           "roulette after bounce 3, directional 3.0 + environment 0.2",
               "msamples_s": samples / (ms / 1e3) / 1e6, "ms_per_render": ms,
               "rmse_vs_fp64_8192spp": e_gpu}
        if not args.no_cpu:
            threads = os.cpu_count() or 1
            osc = O.OracleScene(flat, 14)
            t = time.perf_counter()
            _, film_o = osc.render(flat.camera, p, seed=1, threads=threads)
            cdt = time.perf_counter() - t
            osc.close()
            d_o = torch.from_numpy(film_o.astype(np.float32)).cuda()
            e_cpu, _ = ctx.image_rmse(d_o.data_ptr(), d_conv.data_ptr(), 256, 256)
            res["cpu_baseline"] = {"value": samples / cdt / 1e6, "unit": "Msamples/s",
                                   "cores": threads, "kind": "port",
                                   "sample": f"the whole film at full size ({cdt:.2f} s)",
                                   "rmse_vs_fp64_8192spp": e_cpu}
        return res
    finally:
        ctx.close()


def run_large(args, local):
    """The large-scene workload: one job over 20 transformed copies of the
    displaced icosphere in one tree, its time and its RMSE against an
    FP64-accumulated render of a 128x128 crop."""
    import torch
    from ajisai_render_gb300 import api
    from ajisai_render_gb300 import scenes as S
    t0 = time.perf_counter()
    spec = S.large_scene(seed=3)
    flat = S.flatten(spec)
    gen_s = time.perf_counter() - t0
    ctx = api.Context(local)
    try:
        scene = api.GpuScene(ctx, flat, api.CreatePLOCAggregate(RADIUS))
        info = scene.info()
        args_r = api.PTRendererArgs(spp=1024, min_bounces=MIN_B, max_bounces=32)
        rend = api.PTRenderer(args_r, seed=21)
        W, H = spec.camera.width, spec.camera.height
        out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        stream = torch.cuda.current_stream()
        warm = api.PTRenderer(api.PTRendererArgs(spp=1, min_bounces=MIN_B, max_bounces=32))
        warm.render_device(scene, flat.camera, out.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        rend.render_device(scene, flat.camera, out.data_ptr(), stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        # the crop: centred on the copy that looks largest on the film
        c = 128
        cam_pos = np.asarray(spec.camera.position)
        px = S.project(spec.camera, spec.copy_centers)
        size = spec.copy_scales / np.linalg.norm(spec.copy_centers - cam_pos, axis=1)
        inside = (px[:, 0] >= c // 2) & (px[:, 0] < W - c // 2 - 1) & \
                 (px[:, 1] >= c // 2) & (px[:, 1] < H - c // 2 - 1)
        k = int(np.argmax(np.where(inside, size, -1.0)))
        x0, y0 = int(px[k, 0]) - c // 2, int(px[k, 1]) - c // 2
        ref_r = api.PTRenderer(api.PTRendererArgs(spp=args.large_ref_spp, min_bounces=MIN_B,
                                                  max_bounces=32), seed=99, fp64_film=True)
        t = time.perf_counter()
        (ref, st), = ctx.render_batch([(scene, flat.camera, ref_r, (x0, y0, c + 1, c + 1))])
        ref_s = time.perf_counter() - t
        crop = out[y0:y0 + c, x0:x0 + c].contiguous()
        refd = torch.from_numpy(np.ascontiguousarray(ref.rgbw[:c, :c])).cuda()
        e, npx = ctx.image_rmse(crop.data_ptr(), refd.data_ptr(), c, c)
        img = out.cpu().numpy()
        samples = W * H * 1024
        return {"workload": f"{flat.n_tris:,} triangles (20 copies of the displaced "
                            "icosphere, random rotation, scale U[0.5,2], in a 100^3 box, "
                            "one tree), 1920x1080, 1024 spp, depth 32, Disney per copy",
                "msamples_s": samples / (ms / 1e3) / 1e6, "render_s": ms / 1e3,
                "ploc_build_ms": info["build_ms"], "bvh_width": info["bvh_width"],
                "device_bytes": info["device_bytes"],
                "rmse_vs_fp64_crop": {"crop": f"{c}x{c} at ({x0},{y0})",
                                      "reference_spp": args.large_ref_spp, "rmse": e,
                                      "pixels": npx, "reference_s": ref_s},
                "nonfinite_pixels": int((~np.isfinite(img)).any(-1).sum()),
                "scene_generation_s": gen_s,
                "cpu_baseline": None if args.no_cpu else large_cpu(flat, args)}
    finally:
        ctx.close()


def large_cpu(flat, args):
    """The oracle on the large scene: its PLOC build (one host thread) and
    the render on all host threads over whole image rows spread over the
    film, as many as fit a few seconds."""
    from oracle import pyoracle as O
    threads = os.cpu_count() or 1
    sc = O.OracleScene(flat, RADIUS)
    W, H = int(flat.camera[34]), int(flat.camera[35])
    params = dict(spp=1024, min_bounces=MIN_B, max_bounces=32)
    t = time.perf_counter()
    sc.render(flat.camera, params, seed=21, pixel_range=((H // 2) * W, (H // 2 + 1) * W),
              threads=threads)
    per_row = time.perf_counter() - t
    nrows = int(max(1, min(H, 0.5 * args.cpu_seconds / max(per_row, 1e-6))))
    rows = np.linspace(0, H - 1, nrows).round().astype(int)
    t = time.perf_counter()
    for y in rows:
        sc.render(flat.camera, params, seed=21, pixel_range=(y * W, (y + 1) * W),
                  threads=threads)
    dt = time.perf_counter() - t
    build_s = sc.build_seconds
    sc.close()
    return {"value": len(rows) * W * 1024 / dt / 1e6, "unit": "Msamples/s",
            "cores": threads, "kind": "port",
            "sample": f"{len(rows)} image rows spread over the film x {W} px x 1024 spp "
                      f"({dt:.1f} s), all host threads",
            "ploc_build_ms": build_s * 1e3,
            "ploc_build_note": "the oracle's PLOCAggregate::Build restatement, one host "
                               f"thread, {flat.n_tris:,} triangles"}


SPPM_RES = 512


def run_sppm(args, local):
    """SPPM on the single-job scene: the photon throughput of ajg_render_sppm
    (camera pass, grid builds, photon wavefronts, updates, the film copy)
    over a render of --sppm-iters x --sppm-photons, and the oracle's SPPM
    timed on a bounded sample of the same scene (one iteration)."""
    from ajisai_render_gb300 import api
    from oracle import pyoracle as O
    flat = workload_scene(SPPM_RES)
    ctx = api.Context(local, wave_paths=args.wave_paths)
    try:
        scene = api.GpuScene(ctx, flat, api.CreatePLOCAggregate(RADIUS))
        sargs = api.SPPMRendererArgs(forward_max_depth=8, init_radius=0.01,
                                     iteration_count=args.sppm_iters,
                                     photons_per_iteration=args.sppm_photons,
                                     photon_min_depth=5, photon_max_depth=10)
        warm = api.SPPMRendererArgs(forward_max_depth=8, init_radius=0.01,
                                    iteration_count=1, photons_per_iteration=100000)
        api.SPPMRenderer(warm, seed=1).Render(scene, flat.camera)
        t = time.perf_counter()
        film = api.SPPMRenderer(sargs, seed=2).Render(scene, flat.camera)
        dt = time.perf_counter() - t
        photons = args.sppm_iters * args.sppm_photons
        img = film.image()
    finally:
        ctx.close()
    out = {"workload": f"SPPM on the single-job scene (1,310,722 triangles), "
                       f"{SPPM_RES}x{SPPM_RES}, {args.sppm_iters} iterations x "
                       f"{args.sppm_photons:,} photons, photon depth 10 (roulette "
                       "after 5), camera depth 8, initial radius 0.01",
           "mphotons_s": photons / dt / 1e6, "render_s": dt,
           "nonfinite_pixels": int((~np.isfinite(img)).any(-1).sum()),
           "mean_radiance": float(np.nanmean(img))}
    if args.no_cpu:
        return out
    # the CPU baseline: the oracle's serial SPPM, one iteration of a photon
    # count sized to the time budget, on a smaller film of the same scene
    small = workload_scene(64)
    sc = O.OracleScene(small, RADIUS)
    params = dict(iterations=1, photons_per_iteration=20000, forward_max_depth=8,
                  init_radius=0.01, photon_min_depth=5, photon_max_depth=10)
    t = time.perf_counter()
    sc.sppm(small.camera, params, seed=1)
    per = time.perf_counter() - t
    n = int(min(50_000_000, max(20000, 20000 * args.cpu_seconds / max(per, 1e-6))))
    params["photons_per_iteration"] = n
    t = time.perf_counter()
    sc.sppm(small.camera, params, seed=1)
    cdt = time.perf_counter() - t
    sc.close()
    out["cpu_baseline"] = {"value": n / cdt / 1e6, "unit": "Mphotons/s", "cores": 1,
                           "kind": "port",
                           "sample": f"oracle SPPM (serial), 64x64 film of the same scene, "
                                     f"1 iteration x {n:,} photons, {cdt:.2f} s"}
    return out


def i_seed(k, res, spp):
    return (k * 1_000_003 + res * 101 + spp) & 0xffffffff


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.only_serve:
        # the serving sweep alone (tuning runs), loads relative to
        # --serve-capacity
        from ajisai_render_gb300 import api
        local = int(os.environ.get("LOCAL_RANK", "0"))
        ctx = api.Context(local, wave_paths=args.batch_wave_paths,
                          hbm_budget_bytes=150 << 30)
        print(json.dumps({"served": run_served(ctx, args, args.serve_capacity * 1e6),
                          "wave_paths": args.batch_wave_paths,
                          "policy": args.serve_policy}))
        ctx.close()
    elif args.only_sppm:
        # the SPPM section alone (profiling runs)
        print(json.dumps({"sppm": run_sppm(args, int(os.environ.get("LOCAL_RANK", "0")))}))
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
