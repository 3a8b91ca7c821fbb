/*
 * ajisai_gpu: GB300 (sm_103a) wavefront path tracer for Ajisai's PT-MIS
 * path over a PLOC BVH.  Plain C ABI: plain pointers and sizes, int status
 * returns, no exceptions and no CUDA or torch types across the boundary.
 *
 * What each entry point replaces in the reference (siyuanpan/ajisai_render):
 *
 *   ajg_scene_create*    PLOCAggregate::Build      core/aggregate/ploc_aggregate.cpp:252-327
 *                        + DefaultScene ctor       core/scene/default_scene.cpp:31-61
 *   ajg_trace_closest    Aggregate::Intersect      core/aggregate/aggregate.h:36-37
 *                        (PLOCAggregate::Intersect ploc_aggregate.cpp:329-335,367-391)
 *   ajg_trace_any        Aggregate::Occlude        core/aggregate/aggregate.h:39
 *                        (PLOCAggregate::Occlude   ploc_aggregate.cpp:337-365)
 *   ajg_camera_rays      Camera::GenerateRay       core/camera/camera.h:38-39
 *                        (ThinLensCamera           core/camera/thin_lens.cpp:62-83)
 *   ajg_bsdf_query       BSDF::SampleAll/EvalAll/PdfAll after Material::Shade
 *                                                  core/bsdf/bsdf.h:80-96, core/material/material.h:32-38
 *   ajg_render*          Renderer::Render          core/renderer/renderer.h:53-59
 *                        (TiledIntegrator::Render  core/renderer/pt.cpp:40-73 with
 *                         PathTracing::TraceMIS/Trace pt.cpp:98-311)
 *   ajg_render_sppm      SPPMRenderer::Render      core/renderer/sppm.cpp:180-296
 *   ajg_submit/poll/...  (no counterpart: the request loop that keeps scenes
 *                         resident and batches jobs on one GPU)
 *
 * Ownership: the caller owns every host array it passes and may free it when
 * the call returns; the library owns its device copies.  A scene is
 * immutable after creation and may be traced and rendered concurrently from
 * several host threads of one context (calls on one context serialise on an
 * internal mutex).  Errors: every call returns AJG_OK or an AJG_ERR_* code
 * and leaves a message for ajg_last_error().
 */
#ifndef AJISAI_GPU_H
#define AJISAI_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AJG_API __attribute__((visibility("default")))
#define AJG_ABI_VERSION 1

enum ajg_status {
  AJG_OK = 0,
  AJG_ERR_INVALID = 1,     /* bad argument or scene description */
  AJG_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  AJG_ERR_OOM = 3,         /* device allocation or HBM budget exceeded */
  AJG_ERR_UNSUPPORTED = 4, /* valid input the library does not implement */
  AJG_ERR_DEVICE = 5,      /* a kernel's own guard tripped (stack depth,
                              queue capacity, iteration bound); the context
                              stays usable */
  AJG_ERR_NOT_FOUND = 6,   /* unknown job id */
  AJG_ERR_CANCELLED = 7,
  AJG_ERR_TIMEOUT = 8      /* ajg_wait: the job is still running */
};

/* Per-triangle PostIntersect rules, one set per mesh. */
enum {
  AJG_MESH_TWO_SIDED = 1,   /* TwoSided (core/geometry/two_sided.cpp:44-53) */
  AJG_MESH_NG_REVERSED = 2, /* Cube: normal from (c,b,a) (core/geometry/cube.cpp:96-108) */
  AJG_MESH_HAS_NORMALS = 4  /* MeshGeo shading normals (core/geometry/mesh.cpp:183-204) */
};
enum {
  AJG_MAT_DIFFUSE = 0, /* Diffuse (diffuse.cpp) */
  AJG_MAT_DISNEY = 1,  /* Disney (disney.cpp) */
  AJG_MAT_MIRROR = 2,  /* Mirror (mirror.cpp) */
  AJG_MAT_GLASS = 3,   /* Glass (glass.cpp) */
  AJG_MAT_METAL = 4,   /* Metal (metal.cpp) */
  AJG_MAT_PLASTIC = 5, /* Plastic (plastic.cpp, bsdf/plastic_bsdf.cpp) */
  AJG_MAT_NULL = 6     /* Null (null.cpp): rays pass straight through */
};
enum { AJG_LIGHT_DIRECTIONAL = 0, AJG_LIGHT_ENV = 1 };
enum { AJG_TRI_MOLLER_TRUMBORE = 0, AJG_TRI_WATERTIGHT = 1 };
#define AJG_BVH_COMPRESSED 0x100 /* ajg_scene_opts.bvh_width flag */

typedef struct ajg_ctx ajg_ctx;
typedef struct ajg_scene ajg_scene;

typedef struct ajg_config {
  int32_t device;            /* CUDA device ordinal */
  uint32_t wave_paths;       /* paths in flight per wave, at most 2^28
                                (0: default 256 Mi; a render takes no more
                                than its own paths, at most 96 GB of wave
                                state, and fewer than 2^31 / (lights + 1);
                                the request loop's default is at most 32 Mi) */
  uint64_t hbm_budget_bytes; /* admission budget for resident scenes and
                                films (0: no limit) */
} ajg_config;

/* One triangle mesh as the reference's PLOC aggregate gathers it: the
 * triangles of every mesh in order, each in MeshView index order
 * (ploc_aggregate.cpp:259-285).  Global primitive index = position in that
 * concatenation. */
typedef struct ajg_mesh_desc {
  const float* positions;  /* [num_vertices][3] */
  const float* normals;    /* [num_vertices][3], read with HAS_NORMALS */
  const uint32_t* indices; /* [num_triangles][3] */
  uint32_t num_vertices;
  uint32_t num_triangles;
  uint32_t material;       /* index into the material array */
  uint32_t flags;          /* AJG_MESH_* */
} ajg_mesh_desc;

/* Constant-texture material (Diffuse: base_color is the albedo). */
/* Constant-texture material.  base_color: the diffuse albedo, Disney's
 * base colour, the mirror's kr, the glass's color_reflection, the metal's
 * color, the plastic's albedo.  The ten floats after it are Disney's named
 * parameters, or as `params`:
 *   glass:   color_refraction[3] (as given; shading takes its square root,
 *            glass.cpp:131-138), ior
 *   metal:   k[3], eta[3], uroughness, vroughness
 *   plastic: ior, thickness, sigma_a
 * pad: 0 (the library keeps plastic's precomputed terms there). */
typedef struct ajg_material {
  uint32_t type; /* AJG_MAT_* */
  float base_color[3];
  union {
    struct {
      float subsurface, metallic, specular, specular_tint, roughness,
          anisotropic, sheen, sheen_tint, clearcoat, clearcoat_gloss;
    };
    float params[10];
  };
  float pad[2];
} ajg_material; /* 64 bytes, the [16]-float record of the flat layout */

/* Lights in scene order (YAML order; default_scene.cpp:41-48). */
typedef struct ajg_light {
  uint32_t type;       /* AJG_LIGHT_* */
  float rgb[3];        /* directional radiance, or the env texel */
  float direction[3];  /* directional: toward the light (YAML `direction`) */
  float cos_angle;     /* directional: cos of the cone half-angle */
  float scaler;        /* env: radiance scale */
  float rot_deg;       /* env: rotation about y */
  float pad[2];
} ajg_light; /* 48 bytes */

/* An emissive primitive (GeometricPrimitive with a non-black `emission`,
 * core/primitive/geometric.cpp:33-45): its AreaLight samples the
 * primitive's geometry (core/light/area_light.cpp:36-79).  The triangles
 * [first_triangle, first_triangle + num_triangles) of the scene's order are
 * the primitive's, as its MeshView lays them out: a quad's two (a,b,c),
 * (a,c,d); a cube's twelve as the cube mesh gives them; a mesh's in index
 * order.  Area lights precede the scene's other lights, in emitter order
 * (default_scene.cpp:41-48). */
enum { AJG_GEOM_QUAD = 0, AJG_GEOM_CUBE = 1, AJG_GEOM_MESH = 2 };
typedef struct ajg_emitter {
  float radiance[3];       /* emission; a black one adds no light */
  uint32_t first_triangle;
  uint32_t num_triangles;  /* quad 2, cube 12, mesh >= 1 */
  uint32_t geometry;       /* AJG_GEOM_*: the sampler of its surface */
  uint32_t two_sided;      /* TwoSided wrapper (two_sided.cpp:65-114); its
                              triangles carry AJG_MESH_TWO_SIDED alike */
  uint32_t reserved;       /* 0 */
} ajg_emitter; /* 32 bytes */

typedef struct ajg_scene_opts {
  uint32_t search_radius; /* PLOC neighbour radius (reference default 14) */
  uint32_t tri_test;      /* AJG_TRI_*; Moller-Trumbore matches the reference */
  uint32_t radix_compat;  /* 1: reproduce the reference's Morton radix sort,
                             including its stale digit-0 offset
                             (ploc_aggregate.cpp:97-130), so the tree is the
                             reference's own; 0: correct stable sort */
  uint32_t bvh_width;     /* traversal tree: 2 the binary PLOC tree, 4 or 8
                             the tree collapsed into 4/8-wide nodes, either
                             | AJG_BVH_COMPRESSED for nodes with 8-bit
                             quantised child boxes (same hits: the traversal
                             result does not depend on the tree and the
                             quantised boxes enclose the exact ones); 0: the
                             library's default, 4.  With the plain 4-wide
                             tree the binary layout is kept beside it and
                             closest-hit rays walk that one (the faster
                             closest-hit tree; any-hit and photon rays keep
                             the 4-wide one) */
} ajg_scene_opts;

/* Thin-lens camera: the two matrices ThinLensCamera keeps
 * (thin_lens.cpp:40-54), column-major, plus lens and film size. */
typedef struct ajg_camera {
  float raster2camera[16];
  float camera2world[16];
  float lens_radius;
  float focal_distance;
  uint32_t width;
  uint32_t height;
} ajg_camera;

/* PTRendererArgs (renderer.h:37-45) plus the counter-sampler seed. */
typedef struct ajg_render_params {
  uint32_t spp;
  int32_t min_bounces;
  int32_t max_bounces;
  float cont_prob;
  uint32_t use_mis;
  uint32_t flags;  /* AJG_RENDER_* */
  uint64_t seed;
} ajg_render_params;

enum {
  AJG_RENDER_FP64_FILM = 1,      /* accumulate the film in FP64 (oracle
                                    renders and error references) */
  AJG_RENDER_DROP_NONFINITE = 2  /* leave samples whose radiance is NaN or
                                    inf out of the film (radiance and
                                    weight).  Off by default: the reference
                                    keeps them -- its Disney pdf is 0 for a
                                    half vector with no positive component
                                    (disney.cpp:190-191) while the path
                                    continues on pdf == 0 (pt.cpp:217) */
};

typedef struct ajg_ray {
  float o[3], d[3];
  float t_min, t_max;
} ajg_ray; /* the Ray's fields after its constructor (ray.h:28-45) */

typedef struct ajg_hit {
  float t, u, v; /* u, v: Moller-Trumbore barycentrics of b and c */
  int32_t prim;  /* global primitive index, -1 on a miss */
} ajg_hit;

typedef struct ajg_scene_info {
  uint64_t num_triangles;
  uint64_t num_nodes;      /* 2n-1 PLOC nodes */
  uint64_t device_bytes;   /* resident bytes of the scene */
  uint32_t ploc_iterations;
  float build_ms;          /* GPU time of the last PLOC build */
  uint32_t bvh_width;      /* node width of the traversal tree */
  uint32_t bvh_node_bytes; /* bytes per traversal node */
  uint64_t bvh_nodes;      /* traversal nodes */
  uint32_t closest_node_bytes; /* bytes per node of the tree the closest-hit
                                  traversal walks: the binary layout (64)
                                  beside a plain 4-wide tree, else as above */
  uint32_t reserved;
} ajg_scene_info;

typedef struct ajg_stats {
  uint64_t closest_rays, any_rays;
  uint64_t nodes_visited, tris_tested; /* summed over both ray kinds */
  uint64_t closest_nodes, closest_tris, any_nodes, any_tris;
  uint64_t paths;
  uint64_t kernel_launches;  /* kernels the library launched */
  /* with ajg_set_profiling(ctx, 1): launches and summed device time
   * (CUDA events on the launching stream) per kernel kind */
  uint64_t closest_launches, any_launches, shade_launches;
  double closest_ms, any_ms, shade_ms;
} ajg_stats;

/* ---- context --------------------------------------------------------- */
AJG_API int ajg_abi_version(void);
AJG_API int ajg_create_context(const ajg_config* cfg, ajg_ctx** out);
AJG_API int ajg_destroy_context(ajg_ctx* ctx);
AJG_API const char* ajg_last_error(ajg_ctx* ctx);
AJG_API int ajg_get_stats(ajg_ctx* ctx, ajg_stats* out, int reset);
/* Time every traversal and shading launch with CUDA events (for roofline
 * measurements; adds two event records per launch). */
AJG_API int ajg_set_profiling(ajg_ctx* ctx, int enable);

/* One launch timed while profiling is on: its kind (0 closest-hit
 * traversal, 1 any-hit traversal, 2 shading, 3 any-hit traversal of coherent
 * shadow rays as packets, 4 closest-hit traversal of camera rays as
 * packets), device time, and the rays, node visits and triangle tests of
 * that launch alone (0 for shading).  The statistics count kinds 3 and 4
 * with 1 and 0.  No counterpart in the reference. */
typedef struct ajg_launch_record {
  uint32_t kind;
  float ms;
  uint64_t rays, nodes, tris;
} ajg_launch_record; /* 32 bytes */
/* The launches timed since the last reset, in launch order: up to
 * `capacity` records into `out` (NULL: none), their number in `*count`;
 * `reset` clears the log.  The log holds the last 65,536 launches of a
 * profiling run.  Blocking (waits for the context's work). */
AJG_API int ajg_get_launch_log(ajg_ctx* ctx, ajg_launch_record* out,
                               uint32_t capacity, uint32_t* count, int reset);

/* ---- scenes (PLOCAggregate::Build + DefaultScene) --------------------- */
AJG_API int ajg_scene_create(ajg_ctx* ctx, const ajg_mesh_desc* meshes,
                             uint32_t num_meshes,
                             const ajg_material* materials,
                             uint32_t num_materials, const ajg_light* lights,
                             uint32_t num_lights, const ajg_scene_opts* opts,
                             ajg_scene** out);
/* The same from the flat per-triangle layout: tris [n][9] (a,b,c),
 * corner_normals [n][9] (read where flags has HAS_NORMALS, may be NULL),
 * tri_material [n], tri_flags [n], world [6] = Join of the primitives'
 * AABBs (lo, hi). */
AJG_API int ajg_scene_create_flat(ajg_ctx* ctx, const float* tris,
                                  const float* corner_normals,
                                  const int32_t* tri_material,
                                  const int32_t* tri_flags, uint64_t n,
                                  const float* world,
                                  const ajg_material* materials,
                                  uint32_t num_materials,
                                  const ajg_light* lights, uint32_t num_lights,
                                  const ajg_scene_opts* opts, ajg_scene** out);
/* The same with emissive primitives (area lights).  At most 15 lights in
 * all: the non-black emitters plus `lights`. */
AJG_API int ajg_scene_create_ex(ajg_ctx* ctx, const ajg_mesh_desc* meshes,
                                uint32_t num_meshes,
                                const ajg_material* materials,
                                uint32_t num_materials,
                                const ajg_light* lights, uint32_t num_lights,
                                const ajg_emitter* emitters,
                                uint32_t num_emitters,
                                const ajg_scene_opts* opts, ajg_scene** out);
AJG_API int ajg_scene_create_flat_ex(
    ajg_ctx* ctx, const float* tris, const float* corner_normals,
    const int32_t* tri_material, const int32_t* tri_flags, uint64_t n,
    const float* world, const ajg_material* materials, uint32_t num_materials,
    const ajg_light* lights, uint32_t num_lights, const ajg_emitter* emitters,
    uint32_t num_emitters, const ajg_scene_opts* opts, ajg_scene** out);
AJG_API int ajg_scene_release(ajg_scene* scene);
AJG_API int ajg_scene_get_info(ajg_scene* scene, ajg_scene_info* out);
/* The built tree in the reference's layout (ploc_aggregate.cpp:146-152):
 * node_bounds [2n-1][6], node_count_first [2n-1][2], perm [n]. */
AJG_API int ajg_scene_download_bvh(ajg_scene* scene, float* node_bounds,
                                   int64_t* node_count_first, int64_t* perm);

/* ---- ray queries (Aggregate::Intersect / Occlude) ---------------------- */
/* Host arrays.  Closest hit: ties in t go to the lowest primitive index. */
AJG_API int ajg_trace_closest(ajg_scene* scene, const ajg_ray* rays,
                              uint64_t n, ajg_hit* hits);
AJG_API int ajg_trace_any(ajg_scene* scene, const ajg_ray* rays, uint64_t n,
                          uint8_t* occluded);
/* Device arrays, asynchronous on `stream` (a cudaStream_t; NULL is the legacy
 * default stream). */
AJG_API int ajg_trace_closest_device(ajg_scene* scene, const ajg_ray* d_rays,
                                     uint64_t n, ajg_hit* d_hits,
                                     void* stream);
AJG_API int ajg_trace_any_device(ajg_scene* scene, const ajg_ray* d_rays,
                                 uint64_t n, uint8_t* d_occluded, void* stream);

/* ---- shading and camera queries (golden-vector entry points) ---------- */
/* n queries; op[i] 0: eval+pdf of (wi, wo), 1: sample(wo, sam).
 * ng, ns, wo, wi, sam: [n][3]; out [n][8]: f rgb, pdf, wi xyz, and the
 * sample's flag: valid (1) + delta (2). */
AJG_API int ajg_bsdf_query(ajg_ctx* ctx, const ajg_material* materials,
                           const float* ng, const float* ns, const float* wo,
                           const float* wi, const float* sam,
                           const int32_t* op, uint64_t n, float* out);
/* raster [n][4] (x, y, lens u, lens v) -> rays [n][6] (o, d) after the Ray
 * constructor. */
AJG_API int ajg_camera_rays(ajg_ctx* ctx, const ajg_camera* cam,
                            const float* raster, uint64_t n, float* rays);

/* ---- rendering (Renderer::Render) -------------------------------------- */
/* Blocking.  out_rgbw: host [height][width][4] = (sum of radiance, sum of
 * weights) per pixel in the reference's film convention: each sample lands
 * on the 2x2 box footprint (x-1..x, y-1..y) with row/column -1 folded into 0
 * (film.cpp:27-63, film.h:119-129, image.h:38-42).  image = rgb / w. */
AJG_API int ajg_render(ajg_scene* scene, const ajg_camera* cam,
                       const ajg_render_params* params, float* out_rgbw);
/* ---- stochastic progressive photon mapping (SPPMRenderer) ------------ */
/* SPPMRendererArgs (core/renderer/renderer.h:82-96) and the sampler seed. */
typedef struct ajg_sppm_params {
  uint32_t iterations;            /* iteration_count (100) */
  uint32_t photons_per_iteration; /* 100000 */
  int32_t forward_max_depth;      /* camera pass depth (8) */
  int32_t photon_min_depth;       /* roulette after this depth (5) */
  int32_t photon_max_depth;       /* 10 */
  float photon_cont_prob;         /* 0.9 */
  float init_radius;              /* 0.1; < 0: the world diagonal / 1000 */
  float update_alpha;             /* 2/3 */
  uint64_t seed;
} ajg_sppm_params; /* 40 bytes */

/* SPPMRenderer::Render (sppm.cpp:180-296), blocking.  out_rgbw as
 * ajg_render's (each pixel's radiance is one sample of weight 1);
 * out_radiance [h][w][3] ComputePixelRadiance per pixel; either may be
 * NULL.  The camera pass draws sample 0 of each pixel's counter stream every
 * iteration (the reference reseeds each pixel every iteration); photon i of
 * iteration k draws from its own stream. */
AJG_API int ajg_render_sppm(ajg_scene* scene, const ajg_camera* cam,
                            const ajg_sppm_params* params, float* out_rgbw,
                            float* out_radiance);

/* Same into device memory (float [h][w][4]), asynchronous on `stream`. */
AJG_API int ajg_render_device(ajg_scene* scene, const ajg_camera* cam,
                              const ajg_render_params* params,
                              float* d_out_rgbw, void* stream);
/* Rendering that allocates nothing, for callers that cannot call cudaMalloc
 * (device memory owned by another allocator or a fixed budget, or code that
 * must not allocate while it runs).  No counterpart in the reference.
 * Same result as ajg_render_device, asynchronous on `stream`, but the film
 * accumulators and the wave state live in a 32 MiB static device array that
 * every GPU loading this library keeps until exit: a film needs 32 bytes per
 * pixel of it next to a wave of at least 1,024 paths, so films above about
 * 1,000,000 pixels (1024x1024 does not fit; 512x512 does) are rejected with
 * AJG_ERR_INVALID.  The first call on a device looks the array's address up
 * and should come before any stream capture.  All calls on a device share
 * the array: each clears what it needs, and calls whose GPU work overlaps
 * (other streams, other contexts) race on it.  Unlike ajg_render_device,
 * whose work runs on the context's stream joined to `stream`, every launch
 * is ordered on `stream` itself (NULL: the legacy default stream); the
 * closest-hit launches the context overlaps on its trace stream fork from
 * `stream` and join back into it by events, so the film in d_out_rgbw is
 * complete when `stream` reaches the call's end. */
AJG_API int ajg_render_static(ajg_scene* scene, const ajg_camera* cam,
                              const ajg_render_params* params,
                              float* d_out_rgbw, void* stream);
/* ---- batched rendering and serving ------------------------------------
 * No counterpart in the reference, whose renderer runs one job per process
 * (main.cpp:84-112).  Jobs -- each a scene, camera, film window, spp and
 * parameters -- go to a per-context request loop that keeps scenes and
 * films resident, admits jobs as the HBM budget (ajg_config) allows, and
 * fills every wave of paths from many jobs at once: a wave carries chunks
 * (pixel range x sample range) of up to 1,024 jobs over their own scenes,
 * and its bounce loop is one CUDA graph launch.  Each pixel receives its
 * samples in sample order, so a job's film is bit-identical to the same job
 * rendered alone (ajg_render) or in any mix.  Progressive results: every
 * `progress_spp` samples per pixel the job's window is resolved and
 * delivered (host buffer and/or device buffer). */
enum {
  AJG_JOB_QUEUED = 0,    /* waiting for admission (HBM budget, job slots) */
  AJG_JOB_RUNNING = 1,
  AJG_JOB_DONE = 2,
  AJG_JOB_CANCELLED = 3,
  AJG_JOB_FAILED = 4
};
enum {
  AJG_SCHED_FAIR = 0,  /* every wave splits its paths evenly between the
                          running jobs (processor sharing) */
  AJG_SCHED_FIFO = 1   /* every wave takes the oldest jobs' work first */
};

typedef struct ajg_job_desc {
  ajg_scene* scene;
  ajg_camera camera;
  ajg_render_params params;
  uint32_t window[4];     /* x0, y0, w, h of the rendered part of the film;
                             w == 0 or h == 0: the whole film.  Results cover
                             the window; a target pixel equals the whole
                             render's where its 2x2 footprint sources lie in
                             the window (all but a last row/column that does
                             not end at the film's edge) */
  uint32_t progress_spp;  /* deliver a result every this many samples per
                             pixel (0: the final result only) */
  uint32_t reserved;
  float* out_rgbw;        /* host [h][w][4] (window), or NULL */
  float* d_out_rgbw;      /* device [h][w][4] (window), or NULL; written in
                             the request loop's stream order before the
                             result is reported */
} ajg_job_desc;

typedef struct ajg_job_status {
  uint32_t state;      /* AJG_JOB_* */
  uint32_t spp_done;   /* samples per pixel of the last delivered result */
  uint32_t spp_total;
  uint32_t updates;    /* results delivered so far */
  int32_t error;       /* AJG_OK, or the failure's status code */
  uint32_t reserved;
  /* host clock, milliseconds since the context was created */
  double submit_ms, start_ms, first_result_ms, done_ms;
} ajg_job_status;

typedef struct ajg_serve_opts {
  uint32_t policy;          /* AJG_SCHED_* */
  uint32_t max_active_jobs; /* jobs holding films at once (<= 1024; 0: 256) */
  uint32_t inflight_waves;  /* waves queued on the GPU ahead of the host
                               (0: 2) */
  uint32_t wave_paths;      /* paths per wave of the request loop (0: the
                               context's, at most 32 Mi); smaller waves
                               deliver results sooner, bigger ones run
                               faster */
} ajg_serve_opts;

typedef struct ajg_serve_stats {
  uint64_t jobs_submitted, jobs_done, jobs_cancelled, jobs_failed;
  uint64_t waves, paths, results_delivered, graph_builds;
  uint64_t kernel_launches;
  uint64_t active_bytes;  /* films and result buffers held now */
  double busy_ms;         /* summed device time of the retired waves (CUDA
                             events around each wave's work on the loop's
                             stream, its result copies included) */
} ajg_serve_stats;

/* Scheduling options; takes effect for the waves planned after the call. */
AJG_API int ajg_serve_configure(ajg_ctx* ctx, const ajg_serve_opts* opts);
/* Queue a job; returns at once.  The job keeps `scene` in use until it ends
 * (ajg_scene_release refuses a scene with unfinished jobs). */
AJG_API int ajg_submit(ajg_ctx* ctx, const ajg_job_desc* job,
                       uint64_t* job_id);
AJG_API int ajg_poll(ajg_ctx* ctx, uint64_t job_id, ajg_job_status* out);
/* Block until the job ends (AJG_OK when done, AJG_ERR_CANCELLED, the
 * failure's code) or `timeout_ms` passes (AJG_ERR_TIMEOUT; < 0: forever). */
AJG_API int ajg_wait(ajg_ctx* ctx, uint64_t job_id, int32_t timeout_ms,
                     ajg_job_status* out);
/* The job's latest delivered result (a copy of its host result buffer,
 * taken while no result is being written into it; out_rgbw may be NULL)
 * together with the matching status. */
AJG_API int ajg_job_read(ajg_ctx* ctx, uint64_t job_id, float* out_rgbw,
                         ajg_job_status* out);
/* Stop a job: no further waves take its work; state CANCELLED once the
 * waves already on the GPU retire. */
AJG_API int ajg_cancel(ajg_ctx* ctx, uint64_t job_id);
/* Forget an ended job's record. */
AJG_API int ajg_job_release(ajg_ctx* ctx, uint64_t job_id);
/* Blocking batch: submits every job, waits for all; status[i] per job (may
 * be NULL).  Returns the first failing job's code. */
AJG_API int ajg_render_batch(ajg_ctx* ctx, const ajg_job_desc* jobs,
                             uint32_t n, ajg_job_status* status);
AJG_API int ajg_serve_get_stats(ajg_ctx* ctx, ajg_serve_stats* out);

/* Image error in FP64 on the device: RMSE of rgb / w, all three channels,
 * between two device images [h][stride][4] (strides in pixels), over the
 * pixels where both weights are positive and both sums finite (`pixels`
 * returns how many; a pixel holding a NaN sample is left out).  Blocking. */
AJG_API int ajg_image_rmse(ajg_ctx* ctx, const float* d_a, uint32_t stride_a,
                           const float* d_b, uint32_t stride_b,
                           uint32_t width, uint32_t height, double* rmse,
                           uint64_t* pixels);

/* Per-sample radiance of pixels [pixel_begin, pixel_end): host
 * out_li [count][spp][3], for parity checks on small renders. */
AJG_API int ajg_render_samples(ajg_scene* scene, const ajg_camera* cam,
                               const ajg_render_params* params,
                               uint64_t pixel_begin, uint64_t pixel_end,
                               float* out_li);

#ifdef __cplusplus
}
#endif
#endif /* AJISAI_GPU_H */
