// The C ABI of include/ajisai_host.h over the scene-file reader and the
// image writer.
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "../../include/ajisai_host.h"
#include "image_out.h"
#include "scene_file.h"

struct ajh_scene {
  ajh::SceneFile f;
  std::vector<const char*> out_ptrs;
};

namespace {
void set_err(char* err, size_t n, const char* what) {
  if (!err || !n) return;
  std::strncpy(err, what, n - 1);
  err[n - 1] = '\0';
}
}  // namespace

extern "C" {

int ajh_load_scene(const char* path, ajh_scene** out, char* err,
                   size_t err_len) {
  if (!path || !out) {
    set_err(err, err_len, "NULL argument");
    return 1;
  }
  *out = nullptr;
  try {
    auto* s = new ajh_scene();
    s->f = ajh::LoadSceneFile(path);
    for (const std::string& o : s->f.outputs) s->out_ptrs.push_back(o.c_str());
    *out = s;
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

int ajh_scene_view_get(const ajh_scene* s, ajh_scene_view* v) {
  if (!s || !v) return 1;
  std::memset(v, 0, sizeof(*v));
  const ajh::SceneFile& f = s->f;
  v->num_triangles = f.tri_material.size();
  v->tris = f.tris.data();
  v->corner_normals = f.corner_normals.data();
  v->tri_material = f.tri_material.data();
  v->tri_flags = f.tri_flags.data();
  std::memcpy(v->world, f.world, sizeof(v->world));
  v->num_materials = (uint32_t)f.materials.size();
  v->num_lights = (uint32_t)f.lights.size();
  v->materials = f.materials.data();
  v->lights = f.lights.data();
  v->opts = f.opts;
  v->camera = f.camera;
  v->params = f.params;
  v->num_outputs = (uint32_t)s->out_ptrs.size();
  v->outputs = s->out_ptrs.data();
  v->num_emitters = (uint32_t)f.emitters.size();
  v->emitters = f.emitters.data();
  v->renderer = f.is_sppm ? AJH_RENDERER_SPPM : AJH_RENDERER_PT;
  v->sppm = f.sppm;
  return 0;
}

void ajh_scene_free(ajh_scene* s) { delete s; }

int ajh_write_image(const char* path, const float* rgbw, uint32_t width,
                    uint32_t height, char* err, size_t err_len) {
  if (!path || !rgbw) {
    set_err(err, err_len, "NULL argument");
    return 1;
  }
  try {
    ajh::WriteImage(path, rgbw, width, height);
    return 0;
  } catch (const std::exception& e) {
    set_err(err, err_len, e.what());
    return 1;
  }
}

}  // extern "C"
