"""Autotuner: selection and cache logic on the CPU with a stand-in timer; a
real tuning run on the GPU whose choice renders the same film."""
import numpy as np
import pytest

from ajisai_render_gb300 import api, autotune
from ajisai_render_gb300 import scenes as S


def test_picks_the_fastest_and_caches(tmp_path):
    flat = S.flatten(S.cornell_box(64, 64))     # 4096 pixels
    args = api.PTRendererArgs(spp=256, min_bounces=3, max_bounces=8)
    calls = []

    def timer(layout, wave, spp):
        calls.append((layout, wave, spp))
        # per sample: the 4-wide tree fastest; waves of 2^20 fastest
        per = 10.0 + abs((layout & 0xff) - 4) + (0.5 if layout & 0x100 else 0) + \
            abs(wave.bit_length() - 21) * 0.1
        return per * 4096 * spp / 1e6

    cache = tmp_path / "tune.json"
    waves = (1 << 18, 1 << 20, 1 << 22)
    best = autotune.tune(flat, flat.camera, args, cache=cache, timer=timer, waves=waves)
    assert (best["bvh_width"], best["wave_paths"]) == (4, 1 << 20)
    # layouts at the largest useful wave, then the waves for the best layout
    assert [c[0] for c in calls[:len(autotune.LAYOUTS)]] == list(autotune.LAYOUTS)
    assert len(calls) == len(autotune.LAYOUTS) + 1   # 2^22 exceeds the render
    # every wave candidate's trial holds at least its own paths
    for layout, wave, spp in calls[len(autotune.LAYOUTS):]:
        assert 4096 * spp >= min(wave, 4096 * 256)
    assert cache.exists()
    n = len(calls)
    again = autotune.tune(flat, flat.camera, args, cache=cache, timer=timer, waves=waves)
    assert again == best and len(calls) == n
    # another setup is another entry
    autotune.tune(flat, flat.camera, api.PTRendererArgs(spp=8), cache=cache, timer=timer,
                  waves=(1 << 20,))
    assert len(calls) == n + len(autotune.LAYOUTS)


def test_wave_candidates_stop_at_the_render():
    assert autotune.wave_candidates((1 << 20, 1 << 22, 1 << 24), 3 << 20) == (1 << 20, 1 << 22)
    assert autotune.wave_candidates((1 << 20, 1 << 22), 1 << 30) == (1 << 20, 1 << 22)
    assert autotune.wave_candidates((1 << 20, 1 << 22), 100) == (1 << 20,)
    assert autotune.wave_trial_spp(1 << 22, 1 << 20, 256, 2) == 4
    assert autotune.wave_trial_spp(1 << 28, 1 << 20, 16, 2) == 16
    assert autotune.wave_trial_spp(1 << 10, 1 << 20, 16, 2) == 2


def test_batch_wave_picks_the_fastest():
    got = autotune.tune_batch(None, [], waves=(1 << 24, 1 << 25, 1 << 26),
                              timer=lambda w: ({1 << 24: 30.0, 1 << 25: 20.0,
                                                1 << 26: 25.0}[w], 1_000_000))
    assert got["wave_paths"] == 1 << 25 and len(got["candidates"]) == 3


def test_choose_prefers_earlier_on_ties():
    assert autotune.choose({(2, 1): 5.0, (4, 1): 5.0, (8, 1): 6.0}) == (2, 1)


@pytest.mark.gpu
def test_tuned_setup_renders_the_same_film(tmp_path):
    spec = S.icosphere_scene(4, 2, 48, 48)
    flat = S.flatten(spec)
    args = api.PTRendererArgs(spp=4, min_bounces=2, max_bounces=8)
    best = autotune.tune(flat, flat.camera, args, cache=tmp_path / "t.json",
                         waves=(1 << 12, 1 << 16), trial_spp=1, repeats=1)
    assert best["bvh_width"] in autotune.LAYOUTS
    assert len(best["candidates"]) == len(autotune.LAYOUTS) + 1
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
