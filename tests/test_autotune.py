"""Autotuner: selection and cache logic on the CPU with a stand-in timer; a
real tuning run on the GPU whose choice renders the same film."""
import numpy as np
import pytest

from ajisai_render_gb300 import api, autotune
from ajisai_render_gb300 import scenes as S


def test_picks_the_fastest_and_caches(tmp_path):
    flat = S.flatten(S.cornell_box(16, 16))
    args = api.PTRendererArgs(spp=4, min_bounces=3, max_bounces=8)
    calls = []

    def timer(layout, wave):
        calls.append((layout, wave))
        return 10.0 + (layout & 0xff) + (0.5 if layout & 0x100 else 0) + wave / 2 ** 22

    cache = tmp_path / "tune.json"
    best = autotune.tune(flat, flat.camera, args, cache=cache, timer=timer,
                         waves=(1 << 20, 1 << 22))
    assert (best["bvh_width"], best["wave_paths"]) == (2, 1 << 20)
    assert len(calls) == len(autotune.LAYOUTS) * 2
    assert cache.exists()
    again = autotune.tune(flat, flat.camera, args, cache=cache, timer=timer,
                          waves=(1 << 20, 1 << 22))
    assert again == best and len(calls) == len(autotune.LAYOUTS) * 2
    # another setup is another entry
    autotune.tune(flat, flat.camera, api.PTRendererArgs(spp=8), cache=cache, timer=timer,
                  waves=(1 << 20,))
    assert len(calls) == len(autotune.LAYOUTS) * 3


def test_choose_prefers_earlier_on_ties():
    assert autotune.choose({(2, 1): 5.0, (4, 1): 5.0, (8, 1): 6.0}) == (2, 1)


@pytest.mark.gpu
def test_tuned_setup_renders_the_same_film(tmp_path):
    spec = S.icosphere_scene(4, 2, 48, 48)
    flat = S.flatten(spec)
    args = api.PTRendererArgs(spp=4, min_bounces=2, max_bounces=8)
    best = autotune.tune(flat, flat.camera, args, cache=tmp_path / "t.json",
                         waves=(1 << 16, 1 << 20), trial_spp=1, repeats=1)
    assert best["bvh_width"] in autotune.LAYOUTS
    assert len(best["candidates"]) == len(autotune.LAYOUTS) * 2
    ctx = api.Context(0, wave_paths=best["wave_paths"])
    try:
        a = api.PTRenderer(args, seed=1).Render(
            api.GpuScene(ctx, flat, api.CreatePLOCAggregate(16, bvh_width=best["bvh_width"])),
            flat.camera).rgbw
        b = api.PTRenderer(args, seed=1).Render(
            api.GpuScene(ctx, flat, api.CreatePLOCAggregate(16, bvh_width=2)),
            flat.camera).rgbw
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    finally:
        ctx.close()
