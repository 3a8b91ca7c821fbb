/*
 * Oracle for the PT-MIS / PLOC path: a plain C++ restatement of the
 * reference's CPU algorithm.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: it may be loaded by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and by
 * nothing else.  The product (ajisai_render_gb300 + libajisai_gpu.so) never
 * links, imports or calls it.
 *
 * Parity pin: the functions below are checked against golden vectors dumped
 * by the reference's own sources compiled in this container
 * (oracle/ref_harness, tests/golden/gen_golden.py): PLOC trees, ray hits,
 * BSDF sample/eval/pdf values and per-sample radiance of full renders.
 *
 * Flat scene layout shared with the GPU library (all float32 unless noted):
 *   tris        [n][9]   a,b,c of each triangle in the order the reference's
 *                        PLOCAggregate gathers them (ploc_aggregate.cpp:259-285)
 *   corner_n    [n][9]   per-corner shading normals (only read when the
 *                        triangle's flags have ORC_TRI_HAS_NORMALS)
 *   tri_mat     [n]      int32 material index
 *   tri_flags   [n]      int32 ORC_TRI_* bits
 *   materials   [m][16]  type, base rgb, subsurface, metallic, specular,
 *                        specular_tint, roughness, anisotropic, sheen,
 *                        sheen_tint, clearcoat, clearcoat_gloss, pad, pad
 *   lights      [l][12]  type, rgb, dir xyz (toward the light), cos(angle),
 *                        scaler, rot_deg, pad, pad
 *   world       [6]      lo xyz, hi xyz: Join of the primitives' AABBs
 *                        (default_scene.cpp:32-39), also the Morton box
 *   camera      [36]     raster2camera[16], camera2world[16] (column-major,
 *                        as ajisai/math matrices), lens_radius, focal_distance,
 *                        width, height
 *   emit_rad    [k][3]   emissive primitives (area lights, in primitive
 *   emit_info   [k][4]   order): radiance; int32 first triangle, triangle
 *                        count, ORC_GEOM_* kind, two_sided.  The scene's
 *                        light list is the area lights, then `lights`
 *                        (default_scene.cpp:31-48).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_TRI_TWO_SIDED = 1,   /* TwoSided wrapper (two_sided.cpp:44-53) */
  ORC_TRI_NG_REVERSED = 2, /* Cube's tuple-order normal (cube.cpp:96-108) */
  ORC_TRI_HAS_NORMALS = 4  /* MeshGeo interpolated normals (mesh.cpp:183-204) */
};
/* Material records ([16] floats: type, base colour, ten parameters, two
 * reserved).  Mirror: base = kr.  Glass: base = color_reflection, p0..2 =
 * color_refraction (before its square root), p3 = ior.  Metal: base =
 * color, p0..2 = k, p3..5 = eta, p6/p7 = u/v roughness.  Plastic: base =
 * albedo, p0 = ior, p1 = thickness, p2 = sigma_a.  Null: nothing. */
enum {
  ORC_MAT_DIFFUSE = 0,
  ORC_MAT_DISNEY = 1,
  ORC_MAT_MIRROR = 2,
  ORC_MAT_GLASS = 3,
  ORC_MAT_METAL = 4,
  ORC_MAT_PLASTIC = 5,
  ORC_MAT_NULL = 6
};
enum { ORC_LIGHT_DIRECTIONAL = 0, ORC_LIGHT_ENV = 1, ORC_LIGHT_AREA = 2 };
enum { ORC_GEOM_QUAD = 0, ORC_GEOM_CUBE = 1, ORC_GEOM_MESH = 2 };
/* ORC_TEST_REF_ORDER: Moller-Trumbore inside the reference's own traversal
 * (its slab test, left child first, a strictly closer hit replacing the
 * best), so that of two triangles at one t the first visited wins, as in
 * PLOCAggregate::Intersect (ploc_aggregate.cpp:329-391) -- the mode that
 * pins the oracle to the reference bit for bit on rays that hit an edge.
 * The other two modes give ties to the lowest primitive index. */
enum { ORC_TEST_MT = 0, ORC_TEST_WATERTIGHT = 1, ORC_TEST_REF_ORDER = 2 };

/* SPPMRenderer::Render restated (sppm.cpp:180-296) over a scene of
 * orc_scene_create; see ajg_oracle.cpp for the sampler streams.
 * params[8]: iterations, photons per iteration, forward_max_depth,
 * photon_min_depth, photon_max_depth, photon_cont_prob, init_radius,
 * update_alpha.  out_rad [H][W][3] (may be NULL), out_film [H][W][4]. */
int orc_scene_sppm(void* scene, const float* camera, const double* params,
                   uint64_t seed, float* out_rad, double* out_film);

/* Fresnel::computeDiffuseFresnel(ior, n) (bsdf/helper.h:58-73): the
 * hemispherical integral PlasticBsdf divides the albedo by. */
float orc_diffuse_fresnel(float ior, int n);

/* PLOCAggregate::Build restated (ploc_aggregate.cpp:252-327).  Writes
 * 2n-1 nodes: bounds [6] (lo, hi), count_first [2] (primitive_count,
 * first_child_or_primitive), and the Morton permutation perm[n].
 * radix_compat != 0 reproduces the reference's radix sort including its
 * stale digit-0 offset (ploc_aggregate.cpp:97-130); 0 sorts stably and
 * correctly.  Returns -2 when the compatible sort would write out of bounds. */
int orc_ploc_build(const float* tris, int64_t n, const float* world,
                   int64_t search_radius, int radix_compat, float* node_bounds,
                   int64_t* node_count_first, int64_t* perm);

/* Morton codes of the triangle centroids (ploc_aggregate.cpp:56-82,
 * 513-541). */
void orc_morton(const float* tris, int64_t n, const float* world,
                uint32_t* codes);

/* Ray queries.  rays [n][8]: o xyz, d xyz, t_min, t_max.  bvh == 0 tests
 * every triangle (brute force), otherwise the PLOC tree from
 * orc_ploc_build is traversed with the same conservative slab test as the
 * GPU.  any_hit != 0 answers the occlusion query.  Ties in t go to the
 * lowest primitive index.  Outputs: t, prim (-1 on a miss), u, v. */
int orc_trace(const float* tris, int64_t n_tris, const float* node_bounds,
              const int64_t* node_count_first, const int64_t* perm,
              int use_bvh, const float* rays, int64_t n_rays, int any_hit,
              int tri_test, float* out_t, int32_t* out_prim, float* out_u,
              float* out_v, int threads);

/* One BSDF query for golden-vector parity.  op 0: eval+pdf of (wi, wo);
 * op 1: sample(wo, sam).  ng, ns, wi, wo, sam are float[3].
 * out[8]: f rgb, pdf, wi xyz (sample only), valid. */
void orc_bsdf(const float* material, const float* ng, const float* ns,
              const float* wo, const float* wi, const float* sam, int op,
              float* out);

/* ThinLensCamera::GenerateRay (thin_lens.cpp:62-83) after the Ray
 * constructor: raster [n][4] (x, y, lens u, lens v) -> rays [n][6] (o, d). */
void orc_camera_rays(const float* camera, const float* raster, int64_t n,
                     float* rays);

/* Counter RNG used by both sides for parity renders. */
float orc_rng(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t dim);

/* The path tracer: TiledIntegrator::Render + PathTracing::TraceMIS/Trace
 * (pt.cpp:40-73, 98-311) with the counter sampler.  params[8]: spp,
 * min_bounces, max_bounces, cont_prob, use_mis, tri_test, search_radius,
 * radix_compat.  Writes per-sample radiance out_li[pixel][spp][3] when out_li is
 * non-null, and the per-pixel FP64 film sums out_film[pixel][4] (radiance
 * rgb, weight) in the reference's 2x2 box-footprint convention
 * (film.cpp:27-63, film.h:119-129). */
int orc_render(const float* tris, const float* corner_n,
               const int32_t* tri_mat, const int32_t* tri_flags, int64_t n_tris,
               const float* materials, int32_t n_materials,
               const float* lights, int32_t n_lights, const float* world,
               const float* camera, const double* params, uint64_t seed,
               int64_t pixel_begin, int64_t pixel_end, float* out_li,
               double* out_film, int threads, const float* emit_rad,
               const int32_t* emit_info, int32_t n_emit);

/* The same split in two: build once (PLOC tree), render many times.  The
 * arrays passed to orc_scene_create must outlive the handle. */
void* orc_scene_create(const float* tris, const float* corner_n,
                       const int32_t* tri_mat, const int32_t* tri_flags,
                       int64_t n_tris, const float* materials,
                       int32_t n_materials, const float* lights,
                       int32_t n_lights, const float* world,
                       int64_t search_radius, int radix_compat, int tri_test,
                       const float* emit_rad, const int32_t* emit_info,
                       int32_t n_emit);
int orc_scene_render(void* scene, const float* camera, const double* params,
                     uint64_t seed, int64_t pixel_begin, int64_t pixel_end,
                     float* out_li, double* out_film, int threads);
double orc_scene_build_seconds(void* scene);
void orc_scene_destroy(void* scene);

#ifdef __cplusplus
}
#endif
