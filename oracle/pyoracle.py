"""ctypes wrappers of the oracle and of the reference harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker; never by the product.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")

_lib = None
_ref = None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def lib():
    global _lib
    if _lib is None:
        from oracle import build as b
        so = b.build_oracle()
        L = C.CDLL(str(so))
        L.orc_ploc_build.argtypes = [_f32p, C.c_int64, _f32p, C.c_int64,
                                     C.c_int, _f32p, _i64p, _i64p]
        L.orc_morton.argtypes = [_f32p, C.c_int64, _f32p, _u32p]
        L.orc_trace.argtypes = [_f32p, C.c_int64, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_int, _f32p, C.c_int64, C.c_int,
                                C.c_int, _f32p, _i32p, _f32p, _f32p, C.c_int]
        L.orc_bsdf.argtypes = [_f32p] * 6 + [C.c_int, _f32p]
        L.orc_camera_rays.argtypes = [_f32p, _f32p, C.c_int64, _f32p]
        L.orc_rng.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_rng.restype = C.c_float
        L.orc_render.argtypes = [_f32p, _f32p, _i32p, _i32p, C.c_int64,
                                 _f32p, C.c_int32, _f32p, C.c_int32, _f32p,
                                 _f32p, _f64p, C.c_uint64, C.c_int64,
                                 C.c_int64, C.c_void_p, C.c_void_p, C.c_int,
                                 _f32p, _i32p, C.c_int32]
        L.orc_scene_create.restype = C.c_void_p
        L.orc_scene_create.argtypes = [_f32p, _f32p, _i32p, _i32p, C.c_int64, _f32p,
                                       C.c_int32, _f32p, C.c_int32, _f32p,
                                       C.c_int64, C.c_int, C.c_int, _f32p, _i32p,
                                       C.c_int32]
        L.orc_scene_render.argtypes = [C.c_void_p, _f32p, _f64p, C.c_uint64,
                                       C.c_int64, C.c_int64, C.c_void_p,
                                       C.c_void_p, C.c_int]
        L.orc_scene_sppm.argtypes = [C.c_void_p, _f32p, _f64p, C.c_uint64,
                                     C.c_void_p, C.c_void_p]
        L.orc_scene_sppm.restype = C.c_int
        L.orc_scene_build_seconds.argtypes = [C.c_void_p]
        L.orc_scene_build_seconds.restype = C.c_double
        L.orc_scene_destroy.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _emitters(flat):
    """(radiance [k][3] float32, info [k][4] int32) of the flat scene's
    emissive primitives."""
    er = getattr(flat, "emit_rad", None)
    ei = getattr(flat, "emit_info", None)
    if er is None or len(er) == 0:
        return np.zeros((1, 3), np.float32)[:0], np.zeros((1, 4), np.int32)[:0]
    return _c(er, np.float32).reshape(-1, 3), _c(ei, np.int32).reshape(-1, 4)


def _emitter_args(flat):
    er, ei = _emitters(flat)
    return er, ei, er.shape[0]


class OracleScene:
    """Oracle scene built once (PLOC on the CPU) and rendered many times."""

    def __init__(self, flat, search_radius=14, radix_compat=False, tri_test=0):
        er, ei = _emitters(flat)
        self._keep = [_c(flat.tris, np.float32), _c(flat.corner_n, np.float32),
                      _c(flat.tri_mat, np.int32), _c(flat.tri_flags, np.int32),
                      _c(flat.materials, np.float32), _c(flat.lights, np.float32),
                      _c(flat.world, np.float32), er, ei]
        k = self._keep
        self.h = lib().orc_scene_create(k[0], k[1], k[2], k[3], flat.n_tris, k[4],
                                        k[4].shape[0], k[5], k[5].shape[0], k[6],
                                        search_radius, int(radix_compat), tri_test,
                                        er, ei, er.shape[0])
        if not self.h:
            raise RuntimeError("orc_scene_create failed")
        self.build_seconds = lib().orc_scene_build_seconds(self.h)

    def sppm(self, camera, params, seed=0):
        """SPPMRenderer::Render restated: (radiance [H, W, 3], film
        [H, W, 4] float64)."""
        cam = _c(camera, np.float32)
        W, H = int(cam[34]), int(cam[35])
        rad = np.zeros((H, W, 3), np.float32)
        film = np.zeros((H, W, 4), np.float64)
        rc = lib().orc_scene_sppm(self.h, cam, sppm_param_array(params), seed,
                                  rad.ctypes.data, film.ctypes.data)
        assert rc == 0
        return rad, film

    def render(self, camera, params, seed=0, pixel_range=None, per_sample=False,
               threads=None):
        cam = _c(camera, np.float32)
        W, H = int(cam[34]), int(cam[35])
        spp = int(params["spp"])
        p = np.array([spp, params.get("min_bounces", 5), params.get("max_bounces", 10),
                      params.get("cont_prob", 0.9), params.get("use_mis", 1), 0, 0, 0],
                     np.float64)
        b, e = pixel_range if pixel_range else (0, W * H)
        li = np.zeros((e - b, spp, 3), np.float32) if per_sample else None
        film = np.zeros((H, W, 4), np.float64)
        rc = lib().orc_scene_render(self.h, cam, p, seed, b, e,
                                    li.ctypes.data if li is not None else None,
                                    film.ctypes.data, threads or threads_default())
        assert rc == 0
        return li, film

    def render_window(self, camera, params, seed, x0, y0, w, h, threads=None):
        """Per-sample radiance [h, w, spp, 3] of a window of the film (one
        pixel range per row), each pixel keyed as in the full render."""
        W = int(_c(camera, np.float32)[34])
        rows = [self.render(camera, params, seed,
                            pixel_range=((y0 + r) * W + x0, (y0 + r) * W + x0 + w),
                            per_sample=True, threads=threads)[0] for r in range(h)]
        return np.stack(rows)

    def close(self):
        if self.h:
            lib().orc_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def threads_default():
    return max(1, min(os.cpu_count() or 1, 64))


def ploc_build(tris, world, radius=14, radix_compat=False):
    tris = _c(tris, np.float32).reshape(-1, 9)
    n = tris.shape[0]
    nb = np.zeros((2 * n - 1, 6), np.float32)
    ncf = np.zeros((2 * n - 1, 2), np.int64)
    perm = np.zeros(n, np.int64)
    rc = lib().orc_ploc_build(tris, n, _c(world, np.float32), radius,
                              int(radix_compat), nb, ncf, perm)
    if rc != 0:
        raise RuntimeError("orc_ploc_build failed: %d" % rc)
    return nb, ncf, perm


def morton(tris, world):
    tris = _c(tris, np.float32).reshape(-1, 9)
    out = np.zeros(tris.shape[0], np.uint32)
    lib().orc_morton(tris, tris.shape[0], _c(world, np.float32), out)
    return out


def trace(tris, rays, any_hit=False, tri_test=0, bvh=None, threads=None):
    """bvh: None (brute force) or (node_bounds, node_count_first, perm)."""
    tris = _c(tris, np.float32).reshape(-1, 9)
    rays = _c(rays, np.float32).reshape(-1, 8)
    n = rays.shape[0]
    t = np.zeros(n, np.float32)
    p = np.zeros(n, np.int32)
    u = np.zeros(n, np.float32)
    v = np.zeros(n, np.float32)
    keep = []
    if bvh is not None:
        nb, ncf, perm = (_c(bvh[0], np.float32), _c(bvh[1], np.int64),
                         _c(bvh[2], np.int64))
        keep = [nb, ncf, perm]
        ptrs = [x.ctypes.data for x in keep]
    else:
        ptrs = [None, None, None]
    lib().orc_trace(tris, tris.shape[0], *ptrs, 1 if bvh is not None else 0,
                    rays, n, int(any_hit), int(tri_test), t, p, u, v,
                    threads or threads_default())
    del keep
    return t, p, u, v


def bsdf(material, ng, ns, wo, wi, sam, op):
    out = np.zeros(8, np.float32)
    lib().orc_bsdf(*(_c(x, np.float32) for x in (material, ng, ns, wo, wi, sam)),
                   int(op), out)
    return out


def camera_rays(camera, raster):
    raster = _c(raster, np.float32).reshape(-1, 4)
    out = np.zeros((raster.shape[0], 6), np.float32)
    lib().orc_camera_rays(_c(camera, np.float32), raster, raster.shape[0], out)
    return out


def rng(seed, pixel, sample, dim):
    return lib().orc_rng(seed, pixel, sample, dim)


def render(flat, params, seed=0, pixel_range=None, per_sample=True,
           threads=None):
    """flat: scenes.FlatScene with camera; params: dict with spp,
    min_bounces, max_bounces, cont_prob, use_mis, tri_test, search_radius."""
    cam = _c(flat.camera, np.float32)
    W, H = int(cam[34]), int(cam[35])
    spp = int(params["spp"])
    p = np.array([spp, params.get("min_bounces", 5), params.get("max_bounces", 10),
                  params.get("cont_prob", 0.9), params.get("use_mis", 1),
                  params.get("tri_test", 0), params.get("search_radius", 14),
                  params.get("radix_compat", 0)],
                 np.float64)
    b, e = pixel_range if pixel_range else (0, W * H)
    li = np.zeros((e - b, spp, 3), np.float32) if per_sample else None
    film = np.zeros((H, W, 4), np.float64)
    rc = lib().orc_render(_c(flat.tris, np.float32), _c(flat.corner_n, np.float32),
                          _c(flat.tri_mat, np.int32), _c(flat.tri_flags, np.int32),
                          flat.n_tris, _c(flat.materials, np.float32),
                          flat.materials.shape[0], _c(flat.lights, np.float32),
                          flat.lights.shape[0], _c(flat.world, np.float32), cam,
                          p, seed, b, e,
                          li.ctypes.data if li is not None else None,
                          film.ctypes.data, threads or threads_default(),
                          *_emitter_args(flat))
    assert rc == 0
    return li, film


# ----------------------------------------------------- reference harness --
def ref():
    """The reference's own sources compiled with the harness, or None when
    the reference is not present (only in the development container)."""
    global _ref
    if _ref is None:
        from oracle import build as b
        so = b.build_ref()
        if so is None:
            return None
        L = C.CDLL(str(so))
        L.ref_scene_create.restype = C.c_void_p
        L.ref_scene_create.argtypes = [_i32p, _f32p, C.c_int32, _f32p, _f32p,
                                       _u32p, _f32p, C.c_int32, _f32p,
                                       C.c_int32, C.c_void_p, C.c_int32,
                                       C.c_int32, C.c_int64, _f32p]
        L.ref_scene_destroy.argtypes = [C.c_void_p]
        L.ref_scene_num_tris.argtypes = [C.c_void_p]
        L.ref_scene_num_tris.restype = C.c_int64
        L.ref_scene_dump.argtypes = [C.c_void_p, _f32p, _f32p, _i32p, _i32p,
                                     _f32p, C.c_void_p, C.c_void_p, _i32p]
        L.ref_scene_ploc.argtypes = [C.c_void_p, _f32p, _i64p, _i64p]
        L.ref_scene_trace.argtypes = [C.c_void_p, _f32p, C.c_int64, C.c_int,
                                      _f32p, _i32p, _f32p, _f32p]
        L.ref_bsdf.argtypes = [_f32p] * 6 + [C.c_int, _f32p]
        L.ref_scene_render.argtypes = [C.c_void_p, _f64p, C.c_uint64, _f32p,
                                       _f32p]
        L.ref_scene_render.restype = C.c_int
        L.ref_scene_render_window.argtypes = [C.c_void_p, _f64p, C.c_uint64, C.c_int,
                                              C.c_int, C.c_int, C.c_int, _f32p]
        L.ref_scene_render_window.restype = C.c_int
        L.ref_camera_rays.argtypes = [C.c_void_p, _f32p, C.c_int64, _f32p]
        L.ref_has_diffuse.argtypes = [_f32p]
        L.ref_has_diffuse.restype = C.c_int
        L.ref_sppm_render.argtypes = [C.c_void_p, _f64p, C.c_uint64, _f32p, _f32p]
        L.ref_sppm_render.restype = C.c_int
        _ref = L
    return _ref


class RefScene:
    """A scene built by the reference's Create* functions (scenes.Scene
    spec), with its PLOC aggregate built."""

    def __init__(self, scene, search_radius=14):
        L = ref()
        # The reference's radix sort writes past its arrays on some inputs
        # (the stale digit-0 offset, ploc_aggregate.cpp:97-130); refuse such
        # scenes instead of running undefined behaviour.
        from ajisai_render_gb300.scenes import flatten
        fl = flatten(scene)
        ploc_build(fl.tris, fl.world, search_radius, radix_compat=True)
        prims, pf = [], []
        pos, nrm, idx = [], [], []
        voff = ioff = 0
        for p in scene.primitives:
            rec = np.zeros(8, np.int32)
            f = np.zeros(16, np.float32)
            rec[0], rec[1], rec[2] = p.kind, int(p.two_sided), p.material
            if p.kind == 0:
                f[:12] = np.concatenate([p.a, p.b, p.c, p.d])
            elif p.kind == 1:
                f[:] = np.asarray(p.transform, np.float32)
            else:
                P = np.asarray(p.positions, np.float32).reshape(-1, 3)
                I = np.asarray(p.indices, np.uint32).reshape(-1, 3)
                rec[3], rec[4], rec[5], rec[6] = voff, P.shape[0], ioff, I.shape[0]
                rec[7] = 1 if p.normals is not None else 0
                pos.append(P)
                nrm.append(np.asarray(p.normals, np.float32).reshape(-1, 3)
                           if p.normals is not None else np.zeros_like(P))
                idx.append(I)
                voff += P.shape[0]
                ioff += I.shape[0]
            prims.append(rec)
            pf.append(f)
        self.mat_of_prim = np.array([p.material for p in scene.primitives], np.int32)
        def emis(p):
            e = getattr(p, "emission", None)
            return np.broadcast_to(np.asarray(0.0 if e is None else e, np.float32), 3)
        self.emission = np.array([emis(p) for p in scene.primitives],
                                 np.float32).reshape(-1, 3)
        self.flat_emitters = (fl.emit_rad, fl.emit_info)
        self._keep = dict(
            prims=np.stack(prims), pf=np.stack(pf),
            pos=np.concatenate(pos) if pos else np.zeros((1, 3), np.float32),
            nrm=np.concatenate(nrm) if nrm else np.zeros((1, 3), np.float32),
            idx=np.concatenate(idx) if idx else np.zeros((1, 3), np.uint32),
            mats=np.stack([m.pack() for m in scene.materials]).astype(np.float32),
            lights=(np.stack([l.harness_pack() for l in scene.lights]).astype(np.float32)
                    if scene.lights else np.zeros((1, 12), np.float32)))
        cam = scene.camera
        self.cam_in = cam.harness_pack() if cam is not None else None
        k = self._keep
        self.h = L.ref_scene_create(
            k["prims"], k["pf"], len(prims), _c(k["pos"], np.float32),
            _c(k["nrm"], np.float32), _c(k["idx"], np.uint32), k["mats"],
            len(scene.materials), k["lights"], len(scene.lights),
            self.cam_in.ctypes.data if cam is not None else None,
            cam.width if cam else 0, cam.height if cam else 0, search_radius,
            self.emission)
        self.n = L.ref_scene_num_tris(self.h)
        self.n_lights = len(scene.lights)
        self.scene = scene

    def close(self):
        if self.h:
            ref().ref_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dump(self):
        """FlatScene exactly as the reference gathered it."""
        from ajisai_render_gb300.scenes import FlatScene
        n = self.n
        tris = np.zeros((n, 9), np.float32)
        cn = np.zeros((n, 9), np.float32)
        tm = np.zeros(n, np.int32)
        tf = np.zeros(n, np.int32)
        world = np.zeros(6, np.float32)
        cam = np.zeros(36, np.float32)
        lights = np.zeros((max(1, self.n_lights), 12), np.float32)
        ref().ref_scene_dump(self.h, tris, cn, tm, tf, world, cam.ctypes.data,
                             lights.ctypes.data, self.mat_of_prim)
        mats = self._keep["mats"]
        return FlatScene(tris, cn, tm, tf, world, mats.copy(),
                         lights[:self.n_lights].copy(),
                         cam if self.cam_in is not None else None,
                         emit_rad=self.flat_emitters[0].copy(),
                         emit_info=self.flat_emitters[1].copy())

    def ploc(self):
        n = self.n
        nb = np.zeros((2 * n - 1, 6), np.float32)
        ncf = np.zeros((2 * n - 1, 2), np.int64)
        perm = np.zeros(n, np.int64)
        ref().ref_scene_ploc(self.h, nb, ncf, perm)
        return nb, ncf, perm

    def trace(self, rays, any_hit=False):
        rays = _c(rays, np.float32).reshape(-1, 8)
        m = rays.shape[0]
        t = np.zeros(m, np.float32)
        p = np.zeros(m, np.int32)
        u = np.zeros(m, np.float32)
        v = np.zeros(m, np.float32)
        ref().ref_scene_trace(self.h, rays, m, int(any_hit), t, p, u, v)
        return t, p, u, v

    def render(self, params, seed=0):
        cam = self.scene.camera
        W, H, spp = cam.width, cam.height, int(params["spp"])
        p = np.array([spp, params.get("min_bounces", 5),
                      params.get("max_bounces", 10), params.get("cont_prob", 0.9),
                      params.get("use_mis", 1), 0, 0, 0], np.float64)
        li = np.zeros((H * W, spp, 3), np.float32)
        film = np.zeros((H, W, 4), np.float32)
        rc = ref().ref_scene_render(self.h, p, seed, li, film)
        assert rc == 0
        return li, film

    def render_window(self, params, seed, x0, y0, w, h):
        """Per-sample radiance [h, w, spp, 3] of a window of the film, each
        pixel keyed as in the full render."""
        spp = int(params["spp"])
        p = np.array([spp, params.get("min_bounces", 5),
                      params.get("max_bounces", 10), params.get("cont_prob", 0.9),
                      params.get("use_mis", 1), 0, 0, 0], np.float64)
        li = np.zeros((h, w, spp, 3), np.float32)
        rc = ref().ref_scene_render_window(self.h, p, seed, x0, y0, w, h, li)
        assert rc == 0, rc
        return li

    def sppm(self, params, seed=0):
        """SPPMRenderer::Render over the reference's own SPPM functions (see
        ref_sppm_render): (radiance [H, W, 3], film [H, W, 4])."""
        cam = self.scene.camera
        W, H = cam.width, cam.height
        p = sppm_param_array(params)
        rad = np.zeros((H, W, 3), np.float32)
        film = np.zeros((H, W, 4), np.float32)
        rc = ref().ref_sppm_render(self.h, p, seed, rad, film)
        assert rc == 0
        return rad, film

    def camera_rays(self, raster):
        raster = _c(raster, np.float32).reshape(-1, 4)
        out = np.zeros((raster.shape[0], 6), np.float32)
        ref().ref_camera_rays(self.h, raster, raster.shape[0], out)
        return out


def ref_bsdf(material, ng, ns, wo, wi, sam, op):
    out = np.zeros(8, np.float32)
    ref().ref_bsdf(*(_c(x, np.float32) for x in (material, ng, ns, wo, wi, sam)),
                   int(op), out)
    return out


SPPM_DEFAULTS = dict(iterations=100, photons_per_iteration=100000,
                     forward_max_depth=8, photon_min_depth=5, photon_max_depth=10,
                     photon_cont_prob=0.9, init_radius=0.1, update_alpha=2.0 / 3)


def sppm_param_array(params):
    """SPPMRendererArgs (core/renderer/renderer.h:82-96) as [8] float64, the
    YAML creator's defaults (renderer_creators.cpp:57-76) filling gaps."""
    q = dict(SPPM_DEFAULTS, **params)
    return np.array([q["iterations"], q["photons_per_iteration"],
                     q["forward_max_depth"], q["photon_min_depth"],
                     q["photon_max_depth"], q["photon_cont_prob"],
                     q["init_radius"], q["update_alpha"]], np.float64)


def ref_has_diffuse(material):
    return bool(ref().ref_has_diffuse(_c(material, np.float32)))
