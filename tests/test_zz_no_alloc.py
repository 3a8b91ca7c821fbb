"""ajg_render_static, the render entry point that allocates nothing.

Some callers cannot call cudaMalloc: their device memory belongs to another
allocator or a fixed budget, or they must not allocate while they run.  For
them ajg_render_static renders with its scratch in a static device array
instead of the context's arena and a per-call film allocation.  This file
checks, through the C ABI, that it gives the same film as the allocating
ajg_render_device on two calls in a row (the shared array keeps the last
call's contents, so the second call shows that each call clears it), and
that films beyond the array's capacity are refused.  It is named so that
pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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

    ref = torch.full((80, 96, 4), float("nan"), dtype=torch.float32, device=dev)
    rc = lib.ajg_render_device(scene.h, C.byref(cam), C.byref(prm),
                               C.c_void_p(ref.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.ajg_last_error(ctx.h)
    torch.cuda.synchronize(dev)
    ref_np = ref.cpu().numpy()
    assert np.isfinite(ref_np[..., 3]).all() and ref_np[..., 3].min() > 0

    for _ in range(2):
        out = torch.full((80, 96, 4), float("nan"), dtype=torch.float32, device=dev)
        rc = lib.ajg_render_static(scene.h, C.byref(cam), C.byref(prm),
                                   C.c_void_p(out.data_ptr()),
                                   C.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.ajg_last_error(ctx.h)
        torch.cuda.synchronize(dev)
        # the same samples summed in the same order: equal to float32 rounding
        np.testing.assert_allclose(out.cpu().numpy(), ref_np, rtol=1e-6, atol=1e-6)

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
