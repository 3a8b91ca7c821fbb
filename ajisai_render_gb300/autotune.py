"""Autotuner for the PT path: picks the traversal tree layout (binary PLOC
tree, 4/8-wide, 4/8-wide with quantised boxes -- each with its own stack
depth) and the wave size (paths in flight) for a scene and render setup by
timing trial renders on the GPU, and caches the choice in a JSON file keyed
by the GPU's name and a signature of the scene and setup; and, for batches
of jobs (the request loop), the wave size of the batch.

Every candidate renders the same samples (the traversal result does not
depend on the tree; waves do not change per-sample results), so the choice
only moves time.  Layouts are timed on a few samples per pixel of the real
film at the default wave; the wave size is then timed for the fastest
layout, each candidate on a trial of at least its own paths (a render's
wave is never larger than the render, so a smaller trial could not tell the
candidates apart), capped at the real render, and compared by time per
sample.  Block shapes and the shared-memory stack depth are compile-time
constants of the kernels, chosen offline with tagged builds
(AJG_BUILD_TAG / AJG_EXTRA_NVCC, e.g. -DAJG_SHADE_THREADS=128 or
-DAJG_SMEM_STACK=8) and loaded through AJG_LIB.

    from ajisai_render_gb300 import api, autotune
    best = autotune.tune(flat_scene, camera, api.PTRendererArgs(spp=256, ...))
    ctx = api.Context(0, wave_paths=best["wave_paths"])
    scene = api.GpuScene(ctx, flat_scene,
                         api.CreatePLOCAggregate(16, bvh_width=best["bvh_width"]))
"""
from __future__ import annotations

import hashlib
import json
import os
import time
from dataclasses import asdict, replace
from pathlib import Path
from typing import Callable, Iterable

import numpy as np

LAYOUTS = (2, 4, 8, 4 | 0x100, 8 | 0x100)
WAVES = (1 << 22, 1 << 24, 1 << 26, 1 << 27, 1 << 28)
DEFAULT_WAVE = 1 << 28
DEFAULT_CACHE = Path(os.environ.get("AJG_TUNE_CACHE",
                                    Path.home() / ".cache" / "ajisai_gpu_tune.json"))


def layout_name(layout: int) -> str:
    w = layout & 0xff
    return f"{w}-wide quantised" if layout & 0x100 else (
        "binary" if w == 2 else f"{w}-wide")


def signature(flat, camera, args, search_radius: int, tri_test: int) -> str:
    """Scene and setup signature: triangle data hash, film, spp and depths."""
    h = hashlib.sha1()
    h.update(np.ascontiguousarray(flat.tris).tobytes())
    h.update(np.ascontiguousarray(flat.materials).tobytes())
    h.update(np.ascontiguousarray(flat.lights).tobytes())
    cam = camera if isinstance(camera, np.ndarray) else camera.pack()
    h.update(np.ascontiguousarray(cam, np.float32).tobytes())
    h.update(json.dumps([asdict(args), search_radius, tri_test]).encode())
    return h.hexdigest()[:20]


def choose(times: dict) -> tuple:
    """The fastest (layout, wave) key of measured trial times; ties go to
    the earlier candidate."""
    best, best_t = None, float("inf")
    for k, t in times.items():
        if t < best_t:
            best, best_t = k, t
    return best


def _gpu_name(device: int) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:  # noqa: BLE001
        return "unknown"


def wave_candidates(waves, paths):
    """The wave sizes worth timing for a render of `paths` paths: those below
    it, and the smallest at or above it (a wave never exceeds the render, so
    the larger ones all run the same single wave)."""
    ws = sorted(set(waves))
    out = [w for w in ws if w < paths]
    above = [w for w in ws if w >= paths]
    if above:
        out.append(above[0])
    return tuple(out)


def wave_trial_spp(wave, npix, args_spp, min_spp):
    """Samples per pixel of a wave candidate's trial: enough paths to fill
    the wave once, at least min_spp, at most the render's own spp."""
    need = -(-wave // max(1, npix))
    return int(max(1, min(args_spp, max(min_spp, need))))


def tune(flat, camera, args, *, device: int = 0, search_radius: int = 16,
         tri_test: int = 0, layouts: Iterable[int] = LAYOUTS,
         waves: Iterable[int] = WAVES, trial_spp: int = 2, repeats: int = 2,
         cache: Path | None = DEFAULT_CACHE, timer: Callable | None = None) -> dict:
    """Time the layouts on `trial_spp` samples per pixel at the default wave,
    then the wave candidates for the fastest layout (each on a trial of at
    least its own paths), and return the fastest pair as
    {"bvh_width", "wave_paths", "ns_per_sample", "candidates"}; cached by GPU
    name and scene signature (cache=None: no cache).  `timer(layout, wave,
    spp)` returns milliseconds and replaces the GPU trial (tests)."""
    layouts, waves = tuple(layouts), tuple(waves)
    cam = camera if isinstance(camera, np.ndarray) else camera.pack()
    npix = int(cam[34]) * int(cam[35])
    paths = npix * int(args.spp)
    wcands = wave_candidates(waves, paths)
    key = None
    if cache is not None:
        key = f"{_gpu_name(device)}|{signature(flat, camera, args, search_radius, tri_test)}"
        try:
            db = json.loads(Path(cache).read_text())
        except (OSError, ValueError):
            db = {}
        hit = db.get(key)
        if hit and hit["bvh_width"] in layouts and hit["wave_paths"] in waves:
            return hit
    close = None
    run = timer
    if run is None:
        run, close = _gpu_trial(flat, camera, args, device, search_radius, tri_test,
                                repeats)
    per_sample = {}
    try:
        w0 = wcands[-1]   # the largest useful wave: the layouts' trial
        s0 = int(max(1, min(args.spp, trial_spp)))
        lt = {}
        for layout in layouts:
            lt[layout] = float(run(layout, w0, s0)) / (npix * s0) * 1e6
            per_sample[(layout, w0)] = lt[layout]
        best_layout = choose({(l, w0): t for l, t in lt.items()})[0]
        for wave in wcands:
            if (best_layout, wave) in per_sample:
                continue
            sp = wave_trial_spp(wave, npix, args.spp, s0)
            per_sample[(best_layout, wave)] = float(run(best_layout, wave, sp)) / \
                (npix * sp) * 1e6
    finally:
        if close:
            close()
    layout, wave = choose({k: v for k, v in per_sample.items() if k[0] == best_layout})
    out = {"bvh_width": layout, "wave_paths": wave,
           "ns_per_sample": per_sample[(layout, wave)],
           "layout": layout_name(layout),
           "candidates": {f"{layout_name(l)} / {w}": t for (l, w), t in per_sample.items()}}
    if cache is not None:
        try:
            db = json.loads(Path(cache).read_text())
        except (OSError, ValueError):
            db = {}
        db[key] = out
        Path(cache).parent.mkdir(parents=True, exist_ok=True)
        Path(cache).write_text(json.dumps(db, indent=1))
    return out


def tune_batch(ctx, jobs, waves=(1 << 24, 1 << 25, 1 << 26, 1 << 27),
               spp_divisor: int = 8, timer: Callable | None = None) -> dict:
    """The request loop's wave size for a batch: times ajg_render_batch of
    the batch's jobs at 1/spp_divisor of their samples per pixel (at least
    one) for each candidate, and configures the context with the fastest
    (FIFO scheduling, as render_batch uses it).  jobs: (scene, camera,
    PTRenderer) tuples.  Returns {"wave_paths", "ns_per_sample",
    "candidates"}.  `timer(wave)` returns (milliseconds, samples) and
    replaces the GPU trial (tests)."""
    from . import api
    per_sample = {}
    for wave in waves:
        if timer is not None:
            ms, samples = timer(wave)
        else:
            ctx.configure_serving("fifo", wave_paths=wave)
            trial = []
            samples = 0
            for scene, cam, r in jobs:
                a = replace(r.args, spp=max(1, r.args.spp // spp_divisor))
                trial.append((scene, cam, api.PTRenderer(a, seed=r.seed)))
                c = cam if isinstance(cam, np.ndarray) else cam.pack()
                samples += int(c[34]) * int(c[35]) * a.spp
            ctx.render_batch(trial[:1])   # graphs and arena for this wave size
            t0 = time.perf_counter()
            ctx.render_batch(trial)
            ms = (time.perf_counter() - t0) * 1e3
        per_sample[wave] = ms / samples * 1e6
    best = min(per_sample, key=lambda w: (per_sample[w], w))
    if timer is None:
        ctx.configure_serving("fifo", wave_paths=best)
    return {"wave_paths": best, "ns_per_sample": per_sample[best],
            "candidates": {str(w): t for w, t in per_sample.items()}}


def _gpu_trial(flat, camera, args, device, search_radius, tri_test, repeats):
    """(timer, close): the timer renders `spp` samples per pixel through the
    C ABI with a given layout and wave size and returns the best wall time
    in ms (the call is synchronous); close releases the trial scenes, then
    their contexts."""
    from . import api

    contexts, scenes = {}, {}

    def run(layout, wave, spp):
        if wave not in contexts:
            contexts[wave] = api.Context(device, wave_paths=wave)
        ctx = contexts[wave]
        if (layout, wave) not in scenes:
            scenes[(layout, wave)] = api.GpuScene(
                ctx, flat, api.CreatePLOCAggregate(search_radius, tri_test,
                                                   bvh_width=layout))
        sc = scenes[(layout, wave)]
        r = api.PTRenderer(replace(args, spp=spp), seed=12345)
        r.Render(sc, camera)  # warm the arena and the caches
        best = float("inf")
        for _ in range(repeats):
            t0 = time.perf_counter()
            r.Render(sc, camera)
            best = min(best, (time.perf_counter() - t0) * 1e3)
        return best

    def close():
        for sc in scenes.values():
            sc.release()
        for ctx in contexts.values():
            ctx.close()

    return run, close
