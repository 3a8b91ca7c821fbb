"""ajg_render_static, the render entry point that allocates nothing.

Some callers cannot call cudaMalloc: their device memory belongs to another
allocator or a fixed budget, or they must not allocate while they run.  For
them ajg_render_static renders with its scratch in a static device array
instead of the context's arena and a per-call film allocation.  This file
checks, through the C ABI, that it gives the same film as the allocating
ajg_render_device on two calls in a row (the shared array keeps the last
call's contents, so the second call shows that each call clears it); on a
film too large for one wave of the array (many waves, a wave size and
sample split unlike the allocating path's); with a float64 film right after
a float32 one (the doubles occupy the array's first 32 bytes per pixel); on
a non-default stream with the context's trace-stream overlap on and off; and
that films beyond the array's capacity are refused.  It is named so that
pytest collects it last.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_FILM = 1  # AJG_RENDER_FP64_FILM


def _render(lib, fn, scene, cam, prm, w, h, stream):
    import torch
    out = torch.full((h, w, 4), float("nan"), dtype=torch.float32,
                     device=torch.device("cuda", 0))
    torch.cuda.synchronize()  # the fill ran on torch's current stream
    rc = fn(scene.h, C.byref(cam), C.byref(prm), C.c_void_p(out.data_ptr()),
            C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.ajg_last_error(scene.ctx.h)
    stream.synchronize()
    return out.cpu().numpy()


def test_static_render_matches_allocating_render_twice():
    import torch

    from ajisai_render_gb300 import _lib, api
    from ajisai_render_gb300 import scenes as S

    lib = _lib.load()
    ctx = api.Context(0)
    flat = S.flatten(S.icosphere_scene(subdiv=4, seed=2, width=96, height=80))
    scene = api.GpuScene(ctx, flat, api.CreatePLOCAggregate(16))
    rend = api.PTRenderer(api.PTRendererArgs(spp=12, min_bounces=3, max_bounces=10),
                          seed=4)
    cam = api.camera_struct(flat.camera)
    prm = rend.params()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)

    ref_np = _render(lib, lib.ajg_render_device, scene, cam, prm, 96, 80, stream)
    assert np.isfinite(ref_np[..., 3]).all() and ref_np[..., 3].min() > 0

    for _ in range(2):
        out = _render(lib, lib.ajg_render_static, scene, cam, prm, 96, 80, stream)
        # the same samples summed in the same order: equal to float32 rounding
        np.testing.assert_allclose(out, ref_np, rtol=1e-6, atol=1e-6)

    # a film beyond the static array's capacity is refused, not truncated
    big = api.camera_struct(S.Camera((0.0, 0.6, 3.6), (0.0, -0.1, 0.0), (0, 1, 0), 40.0,
                                     1024, 1024).pack())
    sink = torch.empty((1024, 1024, 4), dtype=torch.float32, device=dev)
    rc = lib.ajg_render_static(scene.h, C.byref(big), C.byref(prm),
                               C.c_void_p(sink.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == 1
    assert b"static scratch" in lib.ajg_last_error(ctx.h)
    scene.release()
    ctx.close()


def test_static_render_many_waves_and_float64_film():
    """512x384 at 16 spp: 3.1 M paths, several dozen waves of the array
    (the allocating path renders it in one); then the float64 film right
    after the float32 one, and the float32 one again."""
    import torch

    from ajisai_render_gb300 import _lib, api
    from ajisai_render_gb300 import scenes as S

    lib = _lib.load()
    ctx = api.Context(0)
    W, H = 512, 384
    flat = S.flatten(S.icosphere_scene(subdiv=4, seed=3, width=W, height=H))
    scene = api.GpuScene(ctx, flat, api.CreatePLOCAggregate(16))
    cam = api.camera_struct(flat.camera)
    stream = torch.cuda.current_stream(torch.device("cuda", 0))
    args = api.PTRendererArgs(spp=16, min_bounces=3, max_bounces=10)
    p32 = api.PTRenderer(args, seed=8).params()
    p64 = api.PTRenderer(args, seed=8, fp64_film=True).params()
    assert p64.flags & FP64_FILM
    ref32 = _render(lib, lib.ajg_render_device, scene, cam, p32, W, H, stream)
    ref64 = _render(lib, lib.ajg_render_device, scene, cam, p64, W, H, stream)
    for prm, ref in ((p32, ref32), (p64, ref64), (p32, ref32)):
        out = _render(lib, lib.ajg_render_static, scene, cam, prm, W, H, stream)
        np.testing.assert_allclose(out, ref, rtol=1e-6, atol=1e-6)
    # the two films hold the same samples: their images agree closely
    w = ref32[..., 3:]
    np.testing.assert_allclose(ref64[..., :3] / w, ref32[..., :3] / w, rtol=1e-4,
                               atol=1e-5)
    scene.release()
    ctx.close()


@pytest.mark.parametrize("overlap", ["1", "0"])
def test_static_render_on_a_side_stream(overlap):
    """The static render is ordered on the stream it is given (the trace
    stream's overlapped launches fork from and join back into it): on a
    non-default stream, with the context's overlap on and off, it equals the
    allocating render."""
    import torch

    from ajisai_render_gb300 import _lib, api
    from ajisai_render_gb300 import scenes as S

    lib = _lib.load()
    old = os.environ.get("AJG_TRACE_OVERLAP")
    os.environ["AJG_TRACE_OVERLAP"] = overlap
    try:
        ctx = api.Context(0)
    finally:
        if old is None:
            os.environ.pop("AJG_TRACE_OVERLAP")
        else:
            os.environ["AJG_TRACE_OVERLAP"] = old
    flat = S.flatten(S.icosphere_scene(subdiv=5, seed=4, width=160, height=120))
    scene = api.GpuScene(ctx, flat, api.CreatePLOCAggregate(16))
    cam = api.camera_struct(flat.camera)
    prm = api.PTRenderer(api.PTRendererArgs(spp=8, min_bounces=3, max_bounces=12),
                         seed=5).params()
    side = torch.cuda.Stream(torch.device("cuda", 0))
    ref = _render(lib, lib.ajg_render_device, scene, cam, prm, 160, 120, side)
    for _ in range(2):
        out = _render(lib, lib.ajg_render_static, scene, cam, prm, 160, 120, side)
        np.testing.assert_allclose(out, ref, rtol=1e-6, atol=1e-6)
    scene.release()
    ctx.close()
