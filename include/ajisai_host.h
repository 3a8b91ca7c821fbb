/*
 * ajisai_host: the host side of the drop-in around libajisai_gpu -- Ajisai
 * YAML scene files (the reference's factory, app/main.cpp:84-112 and
 * factory/creator/*.cpp, for the nodes the PT/PLOC path renders) read into
 * the flat description ajg_scene_create_flat_ex takes, and the film written as
 * PFM (float) or PNG (8-bit, as the reference's ImageWriter).  Plain C ABI;
 * no CUDA.  Errors: status 1 with a message in `err`.
 */
#ifndef AJISAI_HOST_H
#define AJISAI_HOST_H

#include <stddef.h>
#include <stdint.h>

#include "ajisai_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define AJH_API __attribute__((visibility("default")))

typedef struct ajh_scene ajh_scene;

/* Borrowed views into a loaded scene, valid until ajh_scene_free. */
typedef struct ajh_scene_view {
  uint64_t num_triangles;
  const float* tris;            /* [n][9] */
  const float* corner_normals;  /* [n][9] */
  const int32_t* tri_material;  /* [n] */
  const int32_t* tri_flags;     /* [n] */
  float world[6];
  uint32_t num_materials;
  uint32_t num_lights;
  const ajg_material* materials;
  const ajg_light* lights;
  ajg_scene_opts opts;
  ajg_camera camera;
  ajg_render_params params;
  uint32_t num_outputs;  /* save_to_img files: filename + "." + ext */
  uint32_t num_emitters; /* emissive primitives (area lights) */
  const char* const* outputs;
  const ajg_emitter* emitters;
  uint32_t renderer; /* AJH_RENDERER_* */
  uint32_t reserved;
  ajg_sppm_params sppm; /* AJH_RENDERER_SPPM: the renderer node */
} ajh_scene_view;

enum { AJH_RENDERER_PT = 0, AJH_RENDERER_SPPM = 1 };

AJH_API int ajh_load_scene(const char* path, ajh_scene** out, char* err,
                           size_t err_len);
AJH_API int ajh_scene_view_get(const ajh_scene* s, ajh_scene_view* out);
AJH_API void ajh_scene_free(ajh_scene* s);
/* rgbw [h][w][4] as the renderer returns it; .pfm or .png by extension. */
AJH_API int ajh_write_image(const char* path, const float* rgbw,
                            uint32_t width, uint32_t height, char* err,
                            size_t err_len);

#ifdef __cplusplus
}
#endif
#endif /* AJISAI_HOST_H */
