"""Generate the golden fixtures from the reference's own sources.

Run in the development container, where the reference is present:

    python tests/golden/gen_golden.py

It compiles the reference's PT-MIS / PLOC translation units (unmodified,
from where they lie) with oracle/ref_harness/harness.cpp via
oracle/build.py, builds the scenes below through the reference's Create*
functions, and stores what the reference computes:

  ploc_*.npz     PLOCAggregate's tree (nodes_, primitive_indices_)
  trace_*.npz    Scene::Intersect / Occlude hits of seeded ray sets
  bsdf.npz       Material::Shade + BSDF::SampleAll/EvalAll/PdfAll values
  bsdf_more.npz  the same for mirror, glass, metal, plastic and null
  render_*.npz   per-sample radiance of PathTracing::TraceMIS driven by the
                 counter sampler, and the merged film
  camera.npz     ThinLensCamera::GenerateRay rays
  sppm_*.npz     SPPMRenderer's radiance and film (ref_sppm_render)

Every input is seeded; the fixtures are small enough to commit.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from ajisai_render_gb300 import scenes as S  # noqa: E402
from oracle import pyoracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent


def save(name, **arrays):
    np.savez_compressed(OUT / name, **arrays)
    print("wrote", name, sum(a.nbytes for a in arrays.values()) // 1024, "KiB raw")


def mesh_scene(flat_tris, material=0):
    """A scene of one harness mesh holding the given triangles (so hits name
    their triangle)."""
    P = np.asarray(flat_tris, np.float32).reshape(-1, 3)
    I = np.arange(P.shape[0], dtype=np.int32).reshape(-1, 3)
    return S.Scene([S.Mesh(P, I, None, material)], [S.Diffuse((0.5, 0.5, 0.5))], [], None)


def random_soup(rng, n):
    """Random triangles of mixed sizes, with some degenerate ones: repeated
    vertices (point and line boxes) and exact duplicates."""
    c = rng.uniform(-1, 1, (n, 1, 3))
    s = np.exp(rng.uniform(np.log(1e-3), np.log(0.3), (n, 1, 1)))
    t = (c + s * rng.normal(size=(n, 3, 3))).astype(np.float32)
    k = n // 50
    t[:k, 1] = t[:k, 0]
    t[:k, 2] = t[:k, 0]            # point triangles
    t[k:2 * k, 2] = t[k:2 * k, 1]  # line triangles
    t[2 * k:3 * k] = t[3 * k:4 * k]  # duplicates
    return t.reshape(n, 9)


def rays_for(rng, n, lo=-2.0, hi=2.0, tmax_frac=0.25):
    o = rng.uniform(lo, hi, (n, 3))
    tgt = rng.uniform(-1, 1, (n, 3))
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmin = np.full((n, 1), 1e-4)
    tmax = np.full((n, 1), np.inf)
    m = rng.uniform(size=n) < tmax_frac
    tmax[m, 0] = rng.uniform(0.5, 3.0, m.sum())
    return np.concatenate([o, d, tmin, tmax], 1).astype(np.float32)


def gen_ploc():
    rng = np.random.default_rng(11)
    cases = {
        "ploc_cornell.npz": (S.cornell_box(8, 8), 14),
        "ploc_ico4.npz": (S.icosphere_scene(subdiv=4, seed=3, width=8, height=8), 16),
        "ploc_soup.npz": (mesh_scene(random_soup(rng, 3000)), 14),
        # a planar grid: one flat axis, so the Morton grid coordinate is NaN
        "ploc_flat.npz": (mesh_scene(flat_grid(24)), 8),
    }
    for name, (sc, r) in cases.items():
        rs = O.RefScene(sc, search_radius=r)
        fl = rs.dump()
        nb, ncf, perm = rs.ploc()
        save(name, tris=fl.tris, world=fl.world, radius=np.int64(r),
             node_bounds=nb, node_count_first=ncf, perm=perm)


def flat_grid(k):
    xs = np.linspace(-1, 1, k + 1, dtype=np.float32)
    tris = []
    for i in range(k):
        for j in range(k):
            a = (xs[i], 0.25, xs[j]); b = (xs[i + 1], 0.25, xs[j])
            c = (xs[i + 1], 0.25, xs[j + 1]); d = (xs[i], 0.25, xs[j + 1])
            tris += [a + b + c, a + c + d]
    return np.array(tris, np.float32)


def gen_trace():
    rng = np.random.default_rng(12)
    ico = S.icosphere_scene(subdiv=4, seed=3, width=8, height=8)
    fl = S.flatten(ico)
    for name, tris, n in (("trace_ico4.npz", fl.tris, 6000),
                          ("trace_soup.npz", random_soup(rng, 1500), 4000)):
        sc = mesh_scene(tris)
        rs = O.RefScene(sc, search_radius=14)
        d = rs.dump()
        rays = rays_for(rng, n)
        t, p, u, v = rs.trace(rays)
        _, occ, _, _ = rs.trace(rays, any_hit=True)
        save(name, tris=d.tris, world=d.world, radius=np.int64(14), rays=rays,
             t=t, prim=p, u=u, v=v, occluded=occ)


def gen_bsdf():
    rng = np.random.default_rng(13)
    n = 1500
    mats, ngs, nss, wos, wis, sams, ops, outs = [], [], [], [], [], [], [], []

    def unit(v):
        return v / np.linalg.norm(v)

    for i in range(n):
        if i % 3 == 0:
            m = S.Diffuse(rng.uniform(0, 1, 3)).pack()
        else:
            m = S.disney_params(rng).pack()
            if i % 4 == 0:
                m[4] = rng.uniform(0, 1)      # subsurface
            if i % 5 == 0:
                m[10] = rng.uniform(0, 1)     # sheen
            m[7] = rng.uniform(0, 1) if i % 2 else 0.0   # specular_tint
            m[11] = rng.uniform(0, 1)                    # sheen_tint
            if i % 11 == 0:
                m[5] = 1.0                    # metallic 1
        ng = unit(rng.normal(size=3)).astype(np.float32)
        ns = unit(ng + 0.35 * rng.normal(size=3)).astype(np.float32)
        if i % 7 == 0:
            ns = (ns * 1.07).astype(np.float32)   # unnormalised (MeshGeo)
        wo = unit(rng.normal(size=3)).astype(np.float32)
        if i % 4:
            wo = (np.sign(wo @ ng) * wo).astype(np.float32)
        wi = unit(rng.normal(size=3)).astype(np.float32)
        sam = rng.uniform(0, 1, 3).astype(np.float32)
        for op in (0, 1):
            mats.append(m); ngs.append(ng); nss.append(ns); wos.append(wo)
            wis.append(wi); sams.append(sam); ops.append(op)
            outs.append(O.ref_bsdf(m, ng, ns, wo, wi, sam, op))
    save("bsdf.npz", material=np.stack(mats), ng=np.stack(ngs), ns=np.stack(nss),
         wo=np.stack(wos), wi=np.stack(wis), sam=np.stack(sams),
         op=np.array(ops, np.int32), out=np.stack(outs))


def material_queries(rng, n):
    """Seeded queries over mirror, glass, metal, plastic and null materials:
    (material, ng, ns, wo, wi, sam) tuples.  Every plastic has ior 1.5: the
    reference fixes its diffuse-Fresnel term once per process, from the
    first plastic it shades."""
    def unit(v):
        return v / np.linalg.norm(v)

    kinds = ("mirror", "glass", "metal", "plastic", "null")
    out = []
    for i in range(n):
        kind = kinds[i % len(kinds)]
        if kind == "mirror":
            m = S.Mirror(rng.uniform(0, 1, 3)).pack()
        elif kind == "glass":
            m = S.Glass(float(rng.uniform(1.1, 2.5)), rng.uniform(0, 1, 3),
                        rng.uniform(0, 1, 3)).pack()
        elif kind == "metal":
            m = S.Metal(rng.uniform(0, 1, 3), rng.uniform(0, 5, 3),
                        rng.uniform(0.1, 3, 3), float(rng.uniform(0.05, 1)),
                        float(rng.uniform(0.05, 1))).pack()
        elif kind == "plastic":
            m = S.Plastic(rng.uniform(0, 1, 3), 1.5, float(rng.uniform(0, 2)),
                          float(rng.uniform(0, 1)) if i % 2 else 0.0).pack()
        else:
            m = S.Null().pack()
        ng = unit(rng.normal(size=3)).astype(np.float32)
        ns = unit(ng + 0.35 * rng.normal(size=3)).astype(np.float32)
        if i % 7 == 0:
            ns = (ns * 1.07).astype(np.float32)   # unnormalised (MeshGeo)
        wo = unit(rng.normal(size=3)).astype(np.float32)
        if i % 4:
            wo = (np.sign(wo @ ng) * wo).astype(np.float32)
        wi = unit(rng.normal(size=3)).astype(np.float32)
        if i % 9 == 0:   # exactly the mirror direction about ns
            nn = unit(ns.astype(np.float64))
            wi = (2 * (wo @ nn) * nn - wo).astype(np.float32)
        sam = rng.uniform(0, 1, 3).astype(np.float32)
        out.append((m, ng, ns, wo, wi, sam))
    return out


def gen_bsdf_more():
    rng = np.random.default_rng(17)
    mats, ngs, nss, wos, wis, sams, ops, outs = [], [], [], [], [], [], [], []
    for m, ng, ns, wo, wi, sam in material_queries(rng, 2000):
        for op in (0, 1):
            mats.append(m); ngs.append(ng); nss.append(ns); wos.append(wo)
            wis.append(wi); sams.append(sam); ops.append(op)
            outs.append(O.ref_bsdf(m, ng, ns, wo, wi, sam, op))
    save("bsdf_more.npz", material=np.stack(mats), ng=np.stack(ngs), ns=np.stack(nss),
         wo=np.stack(wos), wi=np.stack(wis), sam=np.stack(sams),
         op=np.array(ops, np.int32), out=np.stack(outs))


def gen_render():
    cases = [
        ("render_cornell.npz", S.cornell_box(32, 32),
         dict(spp=8, min_bounces=3, max_bounces=8, cont_prob=0.9, use_mis=1)),
        ("render_ico.npz", S.icosphere_scene(subdiv=3, seed=5, width=24, height=24),
         dict(spp=4, min_bounces=5, max_bounces=16, cont_prob=0.9, use_mis=1)),
        ("render_cornell_nomis.npz", S.cornell_box(16, 16),
         dict(spp=4, min_bounces=3, max_bounces=8, cont_prob=0.9, use_mis=0)),
        # every emitter kind: one-sided and two-sided quads, a mesh, a cube
        ("render_area.npz", S.cornell_area(24, 24),
         dict(spp=4, min_bounces=3, max_bounces=8, cont_prob=0.9, use_mis=1)),
        ("render_area_nomis.npz", S.cornell_area(16, 16),
         dict(spp=4, min_bounces=3, max_bounces=8, cont_prob=0.9, use_mis=0)),
        # plastic, mirror, metal, glass and a null-material emitter
        ("render_materials.npz", S.material_box(24, 24),
         dict(spp=4, min_bounces=3, max_bounces=8, cont_prob=0.9, use_mis=1)),
        ("render_materials_nomis.npz", S.material_box(16, 16),
         dict(spp=4, min_bounces=3, max_bounces=8, cont_prob=0.9, use_mis=0)),
    ]
    for name, sc, params in cases:
        rs = O.RefScene(sc, search_radius=14)
        fl = rs.dump()
        li, film = rs.render(params, seed=7)
        save(name, tris=fl.tris, corner_n=fl.corner_n, tri_mat=fl.tri_mat,
             tri_flags=fl.tri_flags, world=fl.world, materials=fl.materials,
             lights=fl.lights, camera=fl.camera, seed=np.uint64(7),
             emit_rad=fl.emit_rad, emit_info=fl.emit_info,
             params=np.array([params["spp"], params["min_bounces"],
                              params["max_bounces"], params["cont_prob"],
                              params["use_mis"]], np.float64),
             li=li, film=film)


SPPM_PARAMS = dict(iterations=4, photons_per_iteration=20000, forward_max_depth=6,
                   photon_min_depth=3, photon_max_depth=8, photon_cont_prob=0.9,
                   init_radius=0.03, update_alpha=2.0 / 3)


def sppm_scenes():
    """The SPPM fixtures' scenes: the Cornell box; the emitter box without its
    emissive mesh (whose straddling sampler windows make NaN samples); the
    material box with a Disney box in place of the metal one (the
    reference's SPPM faults on metal: AggregateBSDF::HasDiffuseComponent
    runs off its end, aggregate_bsdf.cpp:37-41)."""
    area = S.cornell_area(64, 64)
    area.primitives[9].emission = None
    mats = S.material_box(64, 64)
    mats.materials[5] = S.Disney((0.9, 0.7, 0.4), metallic=0.6, roughness=0.3)
    return [("sppm_cornell.npz", S.cornell_box(64, 64)), ("sppm_area.npz", area),
            ("sppm_materials.npz", mats)]


def gen_sppm():
    """SPPMRenderer's result (per-pixel radiance and film) from the
    reference's own TracerVP / TracerPhoton / VisiblePointSearcher /
    UpdatePixel / ComputePixelRadiance, driven by ref_sppm_render."""
    for name, sc in sppm_scenes():
        rs = O.RefScene(sc, search_radius=14)
        fl = rs.dump()
        rad, film = rs.sppm(SPPM_PARAMS, seed=5)
        save(name, tris=fl.tris, corner_n=fl.corner_n, tri_mat=fl.tri_mat,
             tri_flags=fl.tri_flags, world=fl.world, materials=fl.materials,
             lights=fl.lights, camera=fl.camera, seed=np.uint64(5),
             emit_rad=fl.emit_rad, emit_info=fl.emit_info,
             params=O.sppm_param_array(SPPM_PARAMS), rad=rad, film=film)


def gen_camera():
    rng = np.random.default_rng(14)
    out = {}
    for tag, cam in (("pinhole", S.Camera((0.2, 0.3, 2.5), (0, 0, 0), (0, 1, 0), 35.0, 64, 48)),
                     ("lens", S.Camera((1.0, 0.5, 3.0), (0, 0.1, 0), (0, 1, 0), 50.0, 40, 30,
                                       lens_radius=0.08, focal_distance=3.1))):
        sc = S.cornell_box(8, 8)
        sc.camera = cam
        rs = O.RefScene(sc)
        fl = rs.dump()
        raster = np.concatenate([rng.uniform(0, cam.width, (500, 1)),
                                 rng.uniform(0, cam.height, (500, 1)),
                                 rng.uniform(0, 1, (500, 2))], 1).astype(np.float32)
        out[tag + "_camera"] = fl.camera
        out[tag + "_raster"] = raster
        out[tag + "_rays"] = rs.camera_rays(raster)
    save("camera.npz", **out)


if __name__ == "__main__":
    if O.ref() is None:
        sys.exit("the reference sources are not available here")
    gen_ploc()
    gen_trace()
    gen_bsdf()
    gen_bsdf_more()
    gen_render()
    gen_sppm()
    gen_camera()
