"""The request loop (ajg_submit / ajg_poll / ajg_wait / ajg_cancel /
ajg_render_batch): every job's film is the same bit for bit as the job
rendered alone through ajg_render, whatever the mix, the scheduling policy,
the admission budget or cancellations around it; progressive results,
windows and the FP64 image error."""
import numpy as np
import pytest

from ajisai_render_gb300 import api
from ajisai_render_gb300 import scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = api.Context(0, wave_paths=1 << 20)
    yield c
    c.close()


def with_lights(scene, lights):
    scene.lights = lights
    return scene


def three_light_box():
    """The Cornell box under two directional lights and an environment."""
    return with_lights(S.cornell_box(64, 64),
                       [S.DirectionalLight((0.3, 1.0, 0.2), 3.0),
                        S.DirectionalLight((-0.5, 1.0, 0.1), 1.5, 5.0),
                        S.EnvLight(0.3)])


@pytest.fixture(scope="module")
def scenes(ctx):
    """Scenes of different sizes, materials, light sets and triangle tests."""
    box = S.cornell_box(64, 64)
    ico = S.icosphere_scene(3, 7, 64, 64)
    clutter = S.mixed_scene(3, 3000, 64, 64)
    if len(clutter.primitives) < 3:  # make sure one scene is clutter
        clutter = S.mixed_scene(4, 3000, 64, 64)
    env_only = with_lights(S.icosphere_scene(2, 11, 64, 64), [S.EnvLight(0.7)])
    area = S.cornell_area(64, 64)
    mats = S.material_box(64, 64)
    three = three_light_box()
    out = {
        "box": (api.GpuScene(ctx, box), box.camera),
        "ico": (api.GpuScene(ctx, ico), ico.camera),
        "clutter": (api.GpuScene(ctx, clutter), clutter.camera),
        "env_only": (api.GpuScene(ctx, env_only), env_only.camera),
        "three": (api.GpuScene(ctx, three), three.camera),
        "ico_wt": (api.GpuScene(ctx, ico, api.CreatePLOCAggregate(14, tri_test=1)),
                   ico.camera),
        "ico_w8": (api.GpuScene(ctx, ico, api.CreatePLOCAggregate(14, bvh_width=8)),
                   ico.camera),
        "clutter_w4": (api.GpuScene(ctx, clutter, api.CreatePLOCAggregate(14, bvh_width=4)),
                       clutter.camera),
        "ico_c8": (api.GpuScene(ctx, ico, api.CreatePLOCAggregate(14, bvh_width=0x108)),
                   ico.camera),
        "box_c4": (api.GpuScene(ctx, box, api.CreatePLOCAggregate(14, bvh_width=0x104)),
                   box.camera),
        # emitters: waves that mix them with emitter-free scenes run the
        # closest-hit MIS BSDF pass for the paths of these only
        "area": (api.GpuScene(ctx, area), area.camera),
        "area_c8": (api.GpuScene(ctx, area, api.CreatePLOCAggregate(14, bvh_width=0x108)),
                    area.camera),
        # mirror, glass, metal, plastic and a null-material emitter
        "mats": (api.GpuScene(ctx, mats), mats.camera),
    }
    return out


def cam_at(camera, w, h):
    c = S.Camera(camera.position, camera.look_at, camera.up, camera.fov, w, h,
                 camera.lens_radius, camera.focal_distance)
    return c


def renderer(spp, min_b=3, max_b=8, mis=True, seed=0, fp64=False, drop=False):
    return api.PTRenderer(api.PTRendererArgs(spp=spp, min_bounces=min_b,
                                             max_bounces=max_b, use_mis=mis),
                          seed=seed, fp64_film=fp64, drop_nonfinite=drop)


def job_list(scenes):
    return [
        ("box", 64, 64, renderer(16)),
        ("ico", 48, 40, renderer(9, min_b=2, max_b=12, seed=5)),
        ("clutter", 32, 32, renderer(33, mis=False)),
        ("env_only", 40, 24, renderer(7, min_b=0, max_b=5, seed=3)),
        ("three", 24, 24, renderer(5, min_b=-1, max_b=6)),
        ("ico_wt", 32, 48, renderer(12, seed=2)),
        ("box", 16, 16, renderer(64, fp64=True)),
        ("ico", 20, 20, renderer(20, drop=True, max_b=16)),
        ("ico_w8", 24, 40, renderer(10, seed=6)),
        ("clutter_w4", 40, 24, renderer(6, seed=8, mis=False)),
        ("ico_c8", 32, 32, renderer(9, seed=11)),
        ("box_c4", 24, 32, renderer(7, seed=12)),
        ("area", 48, 40, renderer(9, seed=13)),
        ("area", 24, 24, renderer(6, mis=False, seed=14)),
        ("area_c8", 32, 24, renderer(5, seed=15, drop=True)),
        ("mats", 40, 40, renderer(8, seed=16)),
        ("mats", 24, 32, renderer(6, mis=False, seed=17)),
    ]


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def alone(scenes, name, w, h, r):
    sc, cam = scenes[name]
    return r.Render(sc, cam_at(cam, w, h)).rgbw


@pytest.mark.parametrize("policy,wave", [("fair", 0), ("fifo", 0), ("fair", 1 << 14)])
def test_batch_equals_alone(ctx, scenes, policy, wave):
    """Many waves of 16 Ki paths or few big ones: the same films."""
    jobs = job_list(scenes)
    ref = [alone(scenes, n, w, h, r) for n, w, h, r in jobs]
    ctx.configure_serving(policy, wave_paths=wave)
    out = ctx.render_batch([(scenes[n][0], cam_at(scenes[n][1], w, h), r)
                            for n, w, h, r in jobs])
    for (film, st), r, j in zip(out, ref, jobs):
        assert st["state_name"] == "done", j[0]
        assert st["spp_done"] == j[3].args.spp
        assert same_bits(film.rgbw, r), j[0]
    ctx.configure_serving("fair")


def test_batch_without_packet_traversal_is_the_same(ctx, scenes):
    """Multi-job waves trace bounce 0's directional-light shadow rays as
    packets (a packet per scene a warp's rays hold; lanes pick the packet
    queue by their own light's type and job); a context with packets off
    renders the same mix to the same films bit for bit."""
    import os
    old = {k: os.environ.get(k) for k in ("AJG_PACKET_SHADOW",)}
    try:
        os.environ.update({"AJG_PACKET_SHADOW": "0"})
        plain = api.Context(0, wave_paths=1 << 20)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k)
            else:
                os.environ[k] = v
    ico = S.icosphere_scene(3, 7, 64, 64)
    own = {"box": api.GpuScene(plain, S.cornell_box(64, 64)),
           "ico": api.GpuScene(plain, ico),
           "three": api.GpuScene(plain, three_light_box()),
           "ico_wt": api.GpuScene(plain, ico, api.CreatePLOCAggregate(14, tri_test=1)),
           "env_only": api.GpuScene(plain, with_lights(S.icosphere_scene(2, 11, 64, 64),
                                                       [S.EnvLight(0.7)]))}
    jobs = [(n, 40, 32, renderer(20, seed=i, max_b=10))
            for i, n in enumerate(["box", "ico", "three", "ico_wt", "env_only", "ico"])]
    ctx.configure_serving("fair")
    out = ctx.render_batch([(scenes[n][0], cam_at(scenes[n][1], w, h), r)
                            for n, w, h, r in jobs])
    ref = plain.render_batch([(own[n], cam_at(scenes[n][1], w, h), r)
                              for n, w, h, r in jobs])
    for (film, st), (rfilm, rst), j in zip(out, ref, jobs):
        assert st["state_name"] == rst["state_name"] == "done", j[0]
        assert same_bits(film.rgbw, rfilm.rgbw), j[0]
    for sc in own.values():
        sc.release()
    plain.close()


def test_serve_stats_count_wave_device_time(ctx, scenes):
    """The request loop sums each retired wave's device time."""
    before = ctx.serve_stats()
    sc, cam, r = scenes["box"][0], scenes["box"][1], api.PTRenderer(
        api.PTRendererArgs(spp=4, min_bounces=2, max_bounces=6), seed=2)
    ctx.render_batch([(sc, cam, r)])
    after = ctx.serve_stats()
    assert after["waves"] > before["waves"]
    assert after["busy_ms"] > before["busy_ms"]


def test_batch_of_many_small_jobs_shares_waves(ctx, scenes):
    """Forty jobs small enough to share waves."""
    rng = np.random.default_rng(1)
    names = list(scenes)
    jobs = []
    for i in range(40):
        n = names[i % len(names)]
        w = int(rng.integers(8, 40))
        h = int(rng.integers(8, 40))
        jobs.append((n, w, h, renderer(int(rng.integers(1, 24)), seed=i,
                                       max_b=int(rng.integers(1, 10)))))
    ctx.configure_serving("fair")
    before = ctx.serve_stats()
    out = ctx.render_batch([(scenes[n][0], cam_at(scenes[n][1], w, h), r)
                            for n, w, h, r in jobs])
    after = ctx.serve_stats()
    for (film, st), (n, w, h, r) in zip(out, jobs):
        assert st["state_name"] == "done"
        assert same_bits(film.rgbw, alone(scenes, n, w, h, r))
    # far fewer waves than jobs: the jobs shared them
    assert after["waves"] - before["waves"] < len(jobs) // 2


def test_progressive_results(ctx, scenes):
    sc, cam = scenes["ico"]
    r = renderer(24, seed=9)
    job = ctx.submit(sc, cam_at(cam, 64, 64), r, progress_spp=8)
    st = job.wait()
    assert st["state_name"] == "done"
    assert st["updates"] >= 1 and st["spp_done"] == 24
    assert st["submit_ms"] <= st["start_ms"] <= st["first_result_ms"] <= st["done_ms"]
    assert same_bits(job.film.rgbw, alone(scenes, "ico", 64, 64, r))
    job.release()


def test_progressive_steps_equal_shorter_renders(ctx, scenes):
    """Each delivered result at k spp is the render with spp = k (same
    sampler keys, same film order): read results while the job runs."""
    sc, cam = scenes["ico"]
    r = renderer(64, seed=4)
    job = ctx.submit(sc, cam_at(cam, 256, 256), r, progress_spp=8)
    seen = {}
    while True:
        img, st = job.read()
        if st["updates"] and st["spp_done"] not in seen:
            seen[st["spp_done"]] = img
        if st["state_name"] != "running" and st["state_name"] != "queued":
            break
    assert st["state_name"] == "done" and seen
    assert st["updates"] == 8
    for k, img in seen.items():
        assert k % 8 == 0
        assert same_bits(img, alone(scenes, "ico", 256, 256, renderer(k, seed=4))), k
    job.release()


def test_device_result_buffer(ctx, scenes):
    torch = pytest.importorskip("torch")
    sc, cam = scenes["box"]
    r = renderer(40, seed=4)
    dev = torch.zeros((64, 64, 4), dtype=torch.float32, device="cuda")
    job = ctx.submit(sc, cam_at(cam, 64, 64), r, progress_spp=8, host=False,
                     d_out_ptr=dev.data_ptr())
    st = job.wait()
    assert st["state_name"] == "done" and st["spp_done"] == 40
    assert same_bits(dev.cpu().numpy(), alone(scenes, "box", 64, 64, r))
    job.release()


def test_window_matches_full_render(ctx, scenes):
    sc, cam = scenes["ico"]
    r = renderer(8, seed=1)
    full = alone(scenes, "ico", 64, 48, r)
    for (x0, y0, w, h) in [(0, 0, 20, 16), (10, 7, 30, 20), (40, 30, 24, 18)]:
        job = ctx.submit(sc, cam_at(cam, 64, 48), r, window=(x0, y0, w, h))
        assert job.wait()["state_name"] == "done"
        win = job.film.rgbw
        # targets whose 2x2 sources lie in the window
        wx = w if x0 + w == 64 else w - 1
        wy = h if y0 + h == 48 else h - 1
        assert same_bits(win[:wy, :wx], full[y0:y0 + wy, x0:x0 + wx])
        job.release()


def test_cancel_leaves_other_jobs_intact(ctx, scenes):
    big_sc, big_cam = scenes["ico"]
    big = ctx.submit(big_sc, cam_at(big_cam, 512, 512), renderer(256))
    sc, cam = scenes["box"]
    r = renderer(16, seed=2)
    small = ctx.submit(sc, cam_at(cam, 32, 32), r)
    big.cancel()
    st = big.wait()
    assert st["state_name"] == "cancelled"
    assert small.wait()["state_name"] == "done"
    assert same_bits(small.film.rgbw, alone(scenes, "box", 32, 32, r))
    big.release()
    small.release()


def test_scene_in_use_cannot_be_released(ctx, scenes):
    tmp = S.cornell_box(64, 64)
    sc = api.GpuScene(ctx, tmp)
    job = ctx.submit(sc, cam_at(tmp.camera, 256, 256), renderer(256))
    with pytest.raises(api._lib.AjgError):
        ctx.check(ctx.lib.ajg_scene_release(sc.h))
    job.cancel()
    job.wait()
    job.release()
    sc.release()


def overlap(sts):
    """Most jobs whose [start, done] intervals overlap at one time."""
    ev = sorted([(s["start_ms"], 1) for s in sts] + [(s["done_ms"], -1) for s in sts],
                key=lambda e: (e[0], e[1]))
    cur = best = 0
    for _, d in ev:
        cur += d
        best = max(best, cur)
    return best


def test_one_active_job_runs_jobs_one_after_another(scenes):
    c = api.Context(0, wave_paths=1 << 18)
    try:
        box = S.cornell_box(32, 32)
        sc = api.GpuScene(c, box)
        c.configure_serving("fifo", max_active_jobs=1)
        rs = [renderer(8, seed=i) for i in range(5)]
        jobs = [c.submit(sc, cam_at(box.camera, 32, 32), r) for r in rs]
        sts = [j.wait() for j in jobs]
        for a, b in zip(sts, sts[1:]):
            assert b["start_ms"] >= a["done_ms"]
        for j, r in zip(jobs, rs):
            ref = r.Render(sc, cam_at(box.camera, 32, 32)).rgbw
            assert same_bits(j.film.rgbw, ref)
            j.release()
        sc.release()
    finally:
        c.close()


def test_hbm_budget_admits_and_refuses(scenes):
    """A budget for two films at a time: jobs queue until films free up; a
    job that can never fit fails with AJG_ERR_OOM."""
    box = S.cornell_box(32, 32)
    probe = api.Context(0)
    sc0 = api.GpuScene(probe, box)
    scene_bytes = sc0.info()["device_bytes"]
    sc0.release()
    probe.close()
    film = 512 * 512 * 48                       # film + result buffer
    arena = 2 << 20                             # above a 4 Ki-path arena
    c = api.Context(0, wave_paths=1 << 12,
                    hbm_budget_bytes=scene_bytes + arena + int(2.5 * film))
    try:
        sc = api.GpuScene(c, box)
        rs = [renderer(2, seed=i, max_b=3) for i in range(5)]
        jobs = [c.submit(sc, cam_at(box.camera, 512, 512), r) for r in rs]
        huge = c.submit(sc, cam_at(box.camera, 2048, 2048), renderer(1))
        sts = [j.wait() for j in jobs]
        assert all(s["state_name"] == "done" for s in sts)
        assert overlap(sts) <= 2
        st = huge.wait()
        assert st["state_name"] == "failed" and st["error"] == 3
        for j, r in zip(jobs, rs):
            assert same_bits(j.film.rgbw, r.Render(sc, cam_at(box.camera, 512, 512)).rgbw)
            j.release()
        huge.release()
        sc.release()
    finally:
        c.close()


def test_image_rmse_fp64(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    a = rng.uniform(0, 2, (37, 53, 4)).astype(np.float32)
    b = rng.uniform(0, 2, (37, 53, 4)).astype(np.float32)
    a[..., 3] = rng.integers(0, 3, (37, 53))
    b[..., 3] = rng.integers(1, 3, (37, 53))
    a[3, 4, 1] = np.nan
    b[9, 9, 0] = np.inf
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    r, n = ctx.image_rmse(ta.data_ptr(), tb.data_ptr(), 53, 37)
    m = (a[..., 3] > 0) & (b[..., 3] > 0) & np.isfinite(a[..., :3]).all(-1) & \
        np.isfinite(b[..., :3]).all(-1)
    ia = a[..., :3].astype(np.float64) / np.where(m, a[..., 3], 1)[..., None]
    ib = b[..., :3].astype(np.float64) / np.where(m, b[..., 3], 1)[..., None]
    ref = np.sqrt(((ia - ib)[m] ** 2).mean())
    assert n == m.sum()
    assert abs(r - ref) <= 1e-12 * max(1.0, ref)
    # a sub-rectangle through strides
    r2, n2 = ctx.image_rmse(ta.data_ptr() + 16 * (53 * 5 + 7), tb.data_ptr() + 16 * (53 * 5 + 7),
                            20, 10, 53, 53)
    m2 = m[5:15, 7:27]
    ref2 = np.sqrt(((ia - ib)[5:15, 7:27][m2] ** 2).mean())
    assert n2 == m2.sum() and abs(r2 - ref2) <= 1e-12 * max(1.0, ref2)
