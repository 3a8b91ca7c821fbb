"""Host-side mirror of the reference's interface for the PT path.

The names follow the reference's factory functions and interfaces:

  Context                     one CUDA device, stream and wavefront arena
  CreatePLOCAggregate(r)      aggregate options (core/aggregate/aggregate.h:45)
  CreateDefaultScene(...)     GpuScene: PLOC BVH built on the GPU
                              (core/scene/scene.h:64)
  GpuScene.Intersect/Occlude  batched Aggregate::Intersect / Occlude
  CreatePTRenderer(args)      PTRenderer with Render(scene, camera, film)
                              (core/renderer/renderer.h:37-80)
  Film                        per-pixel (sum of radiance, sum of weights)

Everything runs in libajisai_gpu.so; this module only packs arguments.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass

import numpy as np

from . import _lib
from .scenes import FlatScene, Scene, flatten

F32 = np.float32


def _ptr(a):
    return a.ctypes.data if a is not None else None


class Context:
    def __init__(self, device: int = 0, wave_paths: int = 0, hbm_budget_bytes: int = 0):
        self.lib = _lib.load()
        cfg = _lib.Config(device, wave_paths, hbm_budget_bytes)
        h = C.c_void_p()
        _lib.check(self.lib.ajg_create_context(C.byref(cfg), C.byref(h)))
        self.h = h
        self._scenes = weakref.WeakSet()

    def close(self):
        """Destroy the context; its scenes still alive are released first."""
        if self.h:
            for sc in list(self._scenes):
                sc.release()
            self.lib.ajg_destroy_context(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc):
        _lib.check(rc, self.h)

    def set_profiling(self, enable: bool):
        self.check(self.lib.ajg_set_profiling(self.h, int(enable)))

    def stats(self, reset: bool = False) -> dict:
        s = _lib.Stats()
        self.check(self.lib.ajg_get_stats(self.h, C.byref(s), int(reset)))
        return {n: getattr(s, n) for n, _ in s._fields_}

    KINDS = ("closest", "any", "shade", "any_packets", "closest_packets")

    def launch_log(self, reset: bool = True) -> list:
        """The launches timed since the last reset (profiling on): per
        launch its kind, device ms, and the rays, node visits and triangle
        tests of that launch alone."""
        n = C.c_uint32()
        self.check(self.lib.ajg_get_launch_log(self.h, None, 0, C.byref(n), 0))
        recs = (_lib.LaunchRecord * max(1, n.value))()
        self.check(self.lib.ajg_get_launch_log(self.h, recs, n.value, C.byref(n),
                                               int(reset)))
        return [{"kind": self.KINDS[r.kind], "ms": r.ms, "rays": r.rays,
                 "nodes": r.nodes, "tris": r.tris} for r in recs[:n.value]]

    def bsdf_query(self, materials, ng, ns, wo, wi, sam, op):
        """BSDF::EvalAll+PdfAll (op 0) or SampleAll (op 1) after
        Material::Shade, one query per row; returns [n, 8]."""
        mats = np.ascontiguousarray(materials, F32).reshape(-1, 16)
        n = mats.shape[0]
        recs = (_lib.Material * n)()
        C.memmove(recs, mats.ctypes.data, mats.nbytes)
        for i in range(n):
            recs[i].type = int(mats[i, 0])
        arrs = [np.ascontiguousarray(x, F32).reshape(n, 3) for x in (ng, ns, wo, wi, sam)]
        opa = np.ascontiguousarray(op, np.int32).reshape(n)
        out = np.zeros((n, 8), F32)
        self.check(self.lib.ajg_bsdf_query(self.h, C.cast(recs, C.c_void_p),
                                           *[_ptr(a) for a in arrs], _ptr(opa),
                                           n, _ptr(out)))
        return out

    # ---- request loop (ajg_submit / ajg_poll / ajg_wait / ajg_cancel) ----
    def configure_serving(self, policy: str = "fair", max_active_jobs: int = 0,
                          inflight_waves: int = 0, wave_paths: int = 0):
        pol = {"fair": _lib.SCHED_FAIR, "fifo": _lib.SCHED_FIFO}[policy]
        o = _lib.ServeOpts(pol, max_active_jobs, inflight_waves, wave_paths)
        self.check(self.lib.ajg_serve_configure(self.h, C.byref(o)))

    def submit(self, scene: "GpuScene", camera, renderer: "PTRenderer",
               window=None, progress_spp: int = 0, host: bool = True,
               d_out_ptr: int = 0) -> "RenderJob":
        """Queue a render job; its result (window-sized Film) fills in as the
        request loop delivers progressive and final results."""
        desc, film = _job_desc(scene, camera, renderer, window, progress_spp, host,
                               d_out_ptr)
        jid = C.c_uint64()
        self.check(self.lib.ajg_submit(self.h, C.byref(desc), C.byref(jid)))
        return RenderJob(self, jid.value, film)

    def render_batch(self, jobs) -> list:
        """Blocking batch of (scene, camera, renderer[, window]) tuples; returns
        [(Film, status dict)] in order."""
        descs = (_lib.JobDesc * len(jobs))()
        films = []
        for i, j in enumerate(jobs):
            scene, camera, renderer = j[:3]
            window = j[3] if len(j) > 3 else None
            d, film = _job_desc(scene, camera, renderer, window, 0, True, 0)
            descs[i] = d
            films.append(film)
        st = (_lib.JobStatus * len(jobs))()
        self.check(self.lib.ajg_render_batch(self.h, descs, len(jobs), st))
        return [(films[i], _status(st[i])) for i in range(len(jobs))]

    def serve_stats(self) -> dict:
        s = _lib.ServeStats()
        self.check(self.lib.ajg_serve_get_stats(self.h, C.byref(s)))
        return {n: getattr(s, n) for n, _ in s._fields_}

    def image_rmse(self, d_a: int, d_b: int, width: int, height: int,
                   stride_a: int | None = None, stride_b: int | None = None):
        """FP64 RMSE of rgb / w between two device rgbw images (pointers);
        returns (rmse, pixels compared)."""
        r = C.c_double()
        n = C.c_uint64()
        self.check(self.lib.ajg_image_rmse(
            self.h, C.c_void_p(d_a), stride_a or width, C.c_void_p(d_b),
            stride_b or width, width, height, C.byref(r), C.byref(n)))
        return r.value, n.value

    def camera_rays(self, camera36, raster):
        cam = camera_struct(camera36)
        r = np.ascontiguousarray(raster, F32).reshape(-1, 4)
        out = np.zeros((r.shape[0], 6), F32)
        self.check(self.lib.ajg_camera_rays(self.h, C.byref(cam), _ptr(r),
                                            r.shape[0], _ptr(out)))
        return out


@dataclass
class AggregateOptions:
    search_radius: int = 14
    tri_test: int = 0          # 0 Moller-Trumbore (as the reference), 1 watertight
    radix_compat: bool = False  # reproduce the reference's Morton sort exactly
    bvh_width: int = 0         # 2 binary PLOC tree, 4/8 collapsed; 0 default


def CreatePLOCAggregate(search_radius: int = 14, tri_test: int = 0,
                        radix_compat: bool = False, bvh_width: int = 0) -> AggregateOptions:
    return AggregateOptions(search_radius, tri_test, radix_compat, bvh_width)


def camera_struct(camera36) -> _lib.Camera:
    c = np.ascontiguousarray(camera36, F32)
    cam = _lib.Camera()
    C.memmove(cam.raster2camera, c[0:16].ctypes.data, 64)
    C.memmove(cam.camera2world, c[16:32].ctypes.data, 64)
    cam.lens_radius = float(c[32])
    cam.focal_distance = float(c[33])
    cam.width = int(c[34])
    cam.height = int(c[35])
    return cam


def _materials(arr):
    arr = np.ascontiguousarray(arr, F32).reshape(-1, 16)
    recs = (_lib.Material * arr.shape[0])()
    C.memmove(recs, arr.ctypes.data, arr.nbytes)
    for i in range(arr.shape[0]):
        recs[i].type = int(arr[i, 0])
    return recs


def _lights(arr):
    arr = np.ascontiguousarray(arr, F32).reshape(-1, 12)
    recs = (_lib.Light * max(1, arr.shape[0]))()
    if arr.shape[0]:
        C.memmove(recs, arr.ctypes.data, arr.nbytes)
    for i in range(arr.shape[0]):
        recs[i].type = int(arr[i, 0])
    return recs


def _emitters(flat):
    """ajg_emitter records of the flat scene's emissive primitives (radiance,
    and first triangle, count, geometry, two-sided)."""
    rad = np.asarray(getattr(flat, "emit_rad", np.zeros((0, 3))), F32).reshape(-1, 3)
    info = np.asarray(getattr(flat, "emit_info", np.zeros((0, 4))), np.int64).reshape(-1, 4)
    recs = (_lib.Emitter * max(1, rad.shape[0]))()
    for i in range(rad.shape[0]):
        recs[i].radiance[:] = [float(x) for x in rad[i]]
        recs[i].first_triangle = int(info[i, 0])
        recs[i].num_triangles = int(info[i, 1])
        recs[i].geometry = int(info[i, 2])
        recs[i].two_sided = int(info[i, 3])
    return recs, rad.shape[0]


class GpuScene:
    """A scene resident on the GPU: triangles, materials, lights and the PLOC
    tree built by the GPU (PLOCAggregate::Build + DefaultScene)."""

    def __init__(self, ctx: Context, scene, aggregate: AggregateOptions | None = None):
        self.ctx = ctx
        agg = aggregate or AggregateOptions()
        flat = scene if isinstance(scene, FlatScene) else flatten(scene)
        self.flat = flat
        opts = _lib.SceneOpts(agg.search_radius, agg.tri_test, int(agg.radix_compat),
                              agg.bvh_width)
        mats = _materials(flat.materials)
        lights = _lights(flat.lights)
        tris = np.ascontiguousarray(flat.tris, F32)
        cn = np.ascontiguousarray(flat.corner_n, F32)
        tm = np.ascontiguousarray(flat.tri_mat, np.int32)
        tf = np.ascontiguousarray(flat.tri_flags, np.int32)
        world = np.ascontiguousarray(flat.world, F32)
        emitters, n_emit = _emitters(flat)
        h = C.c_void_p()
        ctx.check(ctx.lib.ajg_scene_create_flat_ex(
            ctx.h, _ptr(tris), _ptr(cn), _ptr(tm), _ptr(tf), tris.shape[0],
            _ptr(world), mats, flat.materials.shape[0], lights,
            flat.lights.shape[0], emitters, n_emit, C.byref(opts), C.byref(h)))
        self.h = h
        ctx._scenes.add(self)

    def release(self):
        if self.h and self.ctx.h:
            self.ctx.lib.ajg_scene_release(self.h)
        self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    def info(self) -> dict:
        i = _lib.SceneInfo()
        self.ctx.check(self.ctx.lib.ajg_scene_get_info(self.h, C.byref(i)))
        return {n: getattr(i, n) for n, _ in i._fields_}

    def download_bvh(self):
        n = self.flat.n_tris
        nb = np.zeros((2 * n - 1, 6), F32)
        ncf = np.zeros((2 * n - 1, 2), np.int64)
        perm = np.zeros(n, np.int64)
        self.ctx.check(self.ctx.lib.ajg_scene_download_bvh(self.h, _ptr(nb), _ptr(ncf),
                                                           _ptr(perm)))
        return nb, ncf, perm

    def Intersect(self, rays):
        """Closest hits of rays [n, 8] (o, d, t_min, t_max): returns
        (t, prim, u, v); prim -1 on a miss."""
        r = np.ascontiguousarray(rays, F32).reshape(-1, 8)
        out = np.zeros((r.shape[0], 4), F32)
        self.ctx.check(self.ctx.lib.ajg_trace_closest(self.h, _ptr(r), r.shape[0],
                                                      _ptr(out)))
        prim = out[:, 3].view(np.int32).copy()
        return out[:, 0].copy(), prim, out[:, 1].copy(), out[:, 2].copy()

    def Occlude(self, rays):
        r = np.ascontiguousarray(rays, F32).reshape(-1, 8)
        out = np.zeros(r.shape[0], np.uint8)
        self.ctx.check(self.ctx.lib.ajg_trace_any(self.h, _ptr(r), r.shape[0], _ptr(out)))
        return out.astype(bool)


def CreateDefaultScene(ctx: Context, scene: Scene | FlatScene,
                       aggregate: AggregateOptions | None = None) -> GpuScene:
    return GpuScene(ctx, scene, aggregate)


@dataclass
class PTRendererArgs:
    """PTRendererArgs (core/renderer/renderer.h:37-45) with the defaults of
    the YAML creator (factory/creator/renderer_creators.cpp:33-39)."""
    spp: int
    tile_size: int = 16
    min_bounces: int = 5
    max_bounces: int = 10
    cont_prob: float = 0.9
    use_mis: bool = True
    specular_depth: int = 20


class Film:
    """The film of a render: rgbw [h, w, 4] = (sum of radiance, sum of
    weights) per pixel in the reference's box-footprint convention."""

    def __init__(self, width: int, height: int, rgbw: np.ndarray | None = None):
        """rgbw: an optional caller-owned float32 [height, width, 4] buffer
        (e.g. pinned host memory, which the device-to-host copy of the
        result reads faster); zeros are allocated otherwise."""
        self.width, self.height = width, height
        if rgbw is None:
            rgbw = np.zeros((height, width, 4), F32)
        elif (rgbw.dtype != F32 or rgbw.shape != (height, width, 4)
              or not rgbw.flags.c_contiguous):
            raise ValueError("rgbw must be a contiguous float32 [height, width, 4] array")
        self.rgbw = rgbw

    def image(self) -> np.ndarray:
        w = self.rgbw[..., 3:4]
        return np.where(w != 0, self.rgbw[..., :3] / np.where(w != 0, w, 1), 0).astype(F32)

    def write_pfm(self, path):
        """Little-endian float32 PFM of image() (bottom row first)."""
        img = self.image()
        with open(path, "wb") as f:
            f.write(b"PF\n%d %d\n-1.0\n" % (self.width, self.height))
            f.write(np.ascontiguousarray(img[::-1], "<f4").tobytes())


class PTRenderer:
    """Renderer::Render for the PT path, on the GPU."""

    def __init__(self, args: PTRendererArgs, seed: int = 0, fp64_film: bool = False,
                 drop_nonfinite: bool = False):
        self.args = args
        self.seed = seed
        self.fp64_film = fp64_film
        self.drop_nonfinite = drop_nonfinite

    def params(self) -> _lib.RenderParams:
        a = self.args
        flags = (1 if self.fp64_film else 0) | (2 if self.drop_nonfinite else 0)
        return _lib.RenderParams(a.spp, a.min_bounces, a.max_bounces, a.cont_prob,
                                 int(a.use_mis), flags, self.seed)

    def render_device(self, scene: GpuScene, camera, out_ptr: int, stream_ptr: int = 0):
        """Render into device memory (float [h][w][4] at out_ptr), ordered on
        the given CUDA stream (a cudaStream_t as an integer)."""
        cam36 = camera if isinstance(camera, np.ndarray) else camera.pack()
        cam = camera_struct(cam36)
        p = self.params()
        scene.ctx.check(scene.ctx.lib.ajg_render_device(
            scene.h, C.byref(cam), C.byref(p), C.c_void_p(out_ptr),
            C.c_void_p(stream_ptr) if stream_ptr else None))

    def Render(self, scene: GpuScene, camera, film: Film | None = None) -> Film:
        cam36 = camera if isinstance(camera, np.ndarray) else camera.pack()
        cam = camera_struct(cam36)
        film = film or Film(cam.width, cam.height)
        p = self.params()
        scene.ctx.check(scene.ctx.lib.ajg_render(scene.h, C.byref(cam), C.byref(p),
                                                 _ptr(film.rgbw)))
        return film

    def RenderSamples(self, scene: GpuScene, camera, pixel_begin=0, pixel_end=None):
        """Per-sample radiance [pixels, spp, 3] (parity checks)."""
        cam36 = camera if isinstance(camera, np.ndarray) else camera.pack()
        cam = camera_struct(cam36)
        pe = pixel_end if pixel_end is not None else cam.width * cam.height
        out = np.zeros((pe - pixel_begin, self.args.spp, 3), F32)
        p = self.params()
        scene.ctx.check(scene.ctx.lib.ajg_render_samples(
            scene.h, C.byref(cam), C.byref(p), pixel_begin, pe, _ptr(out)))
        return out


@dataclass
class SPPMRendererArgs:
    """SPPMRendererArgs (core/renderer/renderer.h:82-96) with the defaults of
    the YAML creator (factory/creator/renderer_creators.cpp:57-76)."""
    forward_max_depth: int = 8
    init_radius: float = 0.1
    iteration_count: int = 100
    photons_per_iteration: int = 100000
    photon_min_depth: int = 5
    photon_max_depth: int = 10
    photon_cont_prob: float = 0.9
    update_alpha: float = 2.0 / 3


class SPPMRenderer:
    """SPPMRenderer::Render (core/renderer/sppm.cpp:180-296), on the GPU."""

    def __init__(self, args: SPPMRendererArgs, seed: int = 0):
        self.args = args
        self.seed = seed

    def params(self) -> _lib.SppmParams:
        a = self.args
        return _lib.SppmParams(a.iteration_count, a.photons_per_iteration,
                               a.forward_max_depth, a.photon_min_depth,
                               a.photon_max_depth, a.photon_cont_prob,
                               a.init_radius, a.update_alpha, self.seed)

    def _run(self, scene: GpuScene, camera, film, radiance):
        cam36 = camera if isinstance(camera, np.ndarray) else camera.pack()
        cam = camera_struct(cam36)
        p = self.params()
        scene.ctx.check(scene.ctx.lib.ajg_render_sppm(
            scene.h, C.byref(cam), C.byref(p),
            _ptr(film.rgbw) if film is not None else None,
            _ptr(radiance) if radiance is not None else None))
        return cam

    def Render(self, scene: GpuScene, camera, film: Film | None = None) -> Film:
        cam36 = camera if isinstance(camera, np.ndarray) else camera.pack()
        cam = camera_struct(cam36)
        film = film or Film(cam.width, cam.height)
        self._run(scene, cam36, film, None)
        return film

    def RenderRadiance(self, scene: GpuScene, camera) -> np.ndarray:
        """ComputePixelRadiance per pixel [h, w, 3] (parity checks)."""
        cam36 = camera if isinstance(camera, np.ndarray) else camera.pack()
        cam = camera_struct(cam36)
        out = np.zeros((cam.height, cam.width, 3), F32)
        self._run(scene, cam36, None, out)
        return out


def CreateSPPMRenderer(args: SPPMRendererArgs, seed: int = 0) -> SPPMRenderer:
    return SPPMRenderer(args, seed)


def CreatePTRenderer(args: PTRendererArgs, seed: int = 0) -> PTRenderer:
    return PTRenderer(args, seed)


def _status(st: _lib.JobStatus) -> dict:
    d = {n: getattr(st, n) for n, _ in st._fields_}
    d["state_name"] = _lib.JOB_STATES.get(st.state, str(st.state))
    return d


def _job_desc(scene: GpuScene, camera, renderer: PTRenderer, window, progress_spp,
              host, d_out_ptr):
    cam36 = camera if isinstance(camera, np.ndarray) else camera.pack()
    cam = camera_struct(cam36)
    x0, y0, w, h = window if window else (0, 0, cam.width, cam.height)
    d = _lib.JobDesc()
    d.scene = scene.h.value if isinstance(scene.h, C.c_void_p) else scene.h
    d.camera = cam
    d.params = renderer.params()
    d.window[:] = [x0, y0, w, h]
    d.progress_spp = progress_spp
    film = Film(w, h) if host else None
    d.out_rgbw = film.rgbw.ctypes.data if film is not None else None
    d.d_out_rgbw = d_out_ptr or None
    return d, film


class RenderJob:
    """A job of the context's request loop.  `film` (host results) is
    rewritten in place with every delivered result."""

    def __init__(self, ctx: Context, job_id: int, film: Film | None):
        self.ctx, self.id, self.film = ctx, job_id, film

    def poll(self) -> dict:
        st = _lib.JobStatus()
        self.ctx.check(self.ctx.lib.ajg_poll(self.ctx.h, self.id, C.byref(st)))
        return _status(st)

    def wait(self, timeout_ms: int = -1) -> dict:
        """Block until the job ends; returns its status (state_name 'done',
        'cancelled' or 'failed'), or the running status on a timeout."""
        st = _lib.JobStatus()
        rc = self.ctx.lib.ajg_wait(self.ctx.h, self.id, timeout_ms, C.byref(st))
        if rc not in (_lib.AJG_OK, _lib.AJG_ERR_CANCELLED, _lib.AJG_ERR_TIMEOUT) and \
                st.state != 4:
            self.ctx.check(rc)
        return _status(st)

    def read(self):
        """(rgbw copy of the latest delivered result, status): consistent
        with each other even while the job runs."""
        st = _lib.JobStatus()
        out = np.zeros_like(self.film.rgbw)
        self.ctx.check(self.ctx.lib.ajg_job_read(self.ctx.h, self.id, _ptr(out),
                                                 C.byref(st)))
        return out, _status(st)

    def cancel(self):
        self.ctx.check(self.ctx.lib.ajg_cancel(self.ctx.h, self.id))

    def release(self):
        self.ctx.check(self.ctx.lib.ajg_job_release(self.ctx.h, self.id))


# ---------------------------------------------------------- scene files --
@dataclass
class SceneFile:
    """An Ajisai YAML scene file as the GPU path reads it (see
    include/ajisai_host.h): the flat scene, the camera record, the
    renderer's arguments and seed, the PLOC options and the files its
    save_to_img post processors name."""
    flat: FlatScene
    camera: np.ndarray
    args: "PTRendererArgs | SPPMRendererArgs"
    seed: int
    aggregate: AggregateOptions
    outputs: list


def load_scene_file(path) -> SceneFile:
    """Read a scene file (the reference's YAML format) with the host
    library: main.cpp's scene, camera and renderer nodes."""
    lib = _lib.load_host()
    h = C.c_void_p()
    err = C.create_string_buffer(1024)
    if lib.ajh_load_scene(str(path).encode(), C.byref(h), err, len(err)) != 0:
        raise ValueError(err.value.decode())
    try:
        v = _lib.HostSceneView()
        lib.ajh_scene_view_get(h, C.byref(v))
        n = v.num_triangles

        def arr(ptr, count, dtype, shape):
            if count == 0:
                return np.zeros(shape, dtype)
            buf = (C.c_char * (count * np.dtype(dtype).itemsize)).from_address(ptr)
            return np.frombuffer(buf, dtype).copy().reshape(shape)

        mats = arr(v.materials, v.num_materials * 16, F32, (v.num_materials, 16))
        mats[:, 0] = arr(v.materials, v.num_materials * 16, np.uint32,
                         (v.num_materials, 16))[:, 0]
        lights = arr(v.lights, v.num_lights * 12, F32, (v.num_lights, 12))
        if v.num_lights:
            lights[:, 0] = arr(v.lights, v.num_lights * 12, np.uint32,
                               (v.num_lights, 12))[:, 0]
        cam = np.zeros(36, F32)
        cam[0:16] = np.array(v.camera.raster2camera, F32)
        cam[16:32] = np.array(v.camera.camera2world, F32)
        cam[32], cam[33] = v.camera.lens_radius, v.camera.focal_distance
        cam[34], cam[35] = v.camera.width, v.camera.height
        ne = v.num_emitters
        emit_rad = np.array([list(v.emitters[i].radiance) for i in range(ne)],
                            F32).reshape(-1, 3)
        emit_info = np.array([[v.emitters[i].first_triangle, v.emitters[i].num_triangles,
                               v.emitters[i].geometry, v.emitters[i].two_sided]
                              for i in range(ne)], np.int32).reshape(-1, 4)
        flat = FlatScene(
            tris=arr(v.tris, n * 9, F32, (n, 9)),
            corner_n=arr(v.corner_normals, n * 9, F32, (n, 9)),
            tri_mat=arr(v.tri_material, n, np.int32, (n,)),
            tri_flags=arr(v.tri_flags, n, np.int32, (n,)),
            world=np.array(v.world, F32), materials=mats, lights=lights, camera=cam,
            emit_rad=emit_rad, emit_info=emit_info)
        p = v.params
        if v.renderer == 1:  # sppm
            q = v.sppm
            args = SPPMRendererArgs(q.forward_max_depth, q.init_radius, q.iterations,
                                    q.photons_per_iteration, q.photon_min_depth,
                                    q.photon_max_depth, q.photon_cont_prob,
                                    q.update_alpha)
            p.seed = q.seed
        else:
            args = PTRendererArgs(spp=p.spp, min_bounces=p.min_bounces,
                                  max_bounces=p.max_bounces, cont_prob=p.cont_prob,
                                  use_mis=bool(p.use_mis))
        agg = AggregateOptions(v.opts.search_radius, v.opts.tri_test,
                               bool(v.opts.radix_compat), v.opts.bvh_width)
        outs = [v.outputs[i].decode() for i in range(v.num_outputs)]
        return SceneFile(flat, cam, args, int(p.seed), agg, outs)
    finally:
        lib.ajh_scene_free(h)


def write_image(path, rgbw: np.ndarray):
    """Write a film (rgbw [h, w, 4]) as .pfm (float) or .png (8-bit, the
    reference's ImageWriter conversion)."""
    lib = _lib.load_host()
    a = np.ascontiguousarray(rgbw, F32)
    err = C.create_string_buffer(1024)
    if lib.ajh_write_image(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0],
                           err, len(err)) != 0:
        raise ValueError(err.value.decode())
