"""Autotuner for the PT path: picks the traversal tree layout (binary PLOC
tree, 4/8-wide, 4/8-wide with quantised boxes -- each with its own stack
depth) and the wave size (paths in flight) for a scene and render setup by
timing short trial renders on the GPU, and caches the choice in a JSON file
keyed by the GPU's name and a signature of the scene and setup.

Every candidate renders the same samples (the traversal result does not
depend on the tree; waves do not change per-sample results), so the choice
only moves time.  The trial is a few samples per pixel of the real film.

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
WAVES = (1 << 22, 1 << 23, 1 << 24, 1 << 25, 1 << 26, 1 << 27, 1 << 28)
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


def tune(flat, camera, args, *, device: int = 0, search_radius: int = 16,
         tri_test: int = 0, layouts: Iterable[int] = LAYOUTS,
         waves: Iterable[int] = WAVES, trial_spp: int = 2, repeats: int = 2,
         cache: Path | None = DEFAULT_CACHE, timer: Callable | None = None) -> dict:
    """Time every (layout, wave size) candidate on `trial_spp` samples per
    pixel of the film and return the fastest as
    {"bvh_width", "wave_paths", "trial_ms", "candidates"}; cached by GPU
    name and scene signature (cache=None: no cache).  `timer(layout, wave)`
    replaces the GPU trial (tests)."""
    layouts, waves = tuple(layouts), tuple(waves)
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
                                trial_spp, repeats)
    times = {}
    try:
        for layout in layouts:
            for wave in waves:
                times[(layout, wave)] = float(run(layout, wave))
    finally:
        if close:
            close()
    layout, wave = choose(times)
    out = {"bvh_width": layout, "wave_paths": wave, "trial_ms": times[(layout, wave)],
           "layout": layout_name(layout),
           "candidates": {f"{layout_name(l)} / {w}": t for (l, w), t in times.items()}}
    if cache is not None:
        try:
            db = json.loads(Path(cache).read_text())
        except (OSError, ValueError):
            db = {}
        db[key] = out
        Path(cache).parent.mkdir(parents=True, exist_ok=True)
        Path(cache).write_text(json.dumps(db, indent=1))
    return out


def _gpu_trial(flat, camera, args, device, search_radius, tri_test, trial_spp,
               repeats):
    """(timer, close): the timer renders trial_spp samples per pixel through
    the C ABI and returns the best wall time in ms (the call is
    synchronous); close releases the trial scenes, then their contexts."""
    from . import api

    contexts, scenes = {}, {}

    def run(layout, wave):
        if wave not in contexts:
            contexts[wave] = api.Context(device, wave_paths=wave)
        ctx = contexts[wave]
        if (layout, wave) not in scenes:
            scenes[(layout, wave)] = api.GpuScene(
                ctx, flat, api.CreatePLOCAggregate(search_radius, tri_test,
                                                   bvh_width=layout))
        sc = scenes[(layout, wave)]
        r = api.PTRenderer(replace(args, spp=trial_spp), seed=12345)
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
