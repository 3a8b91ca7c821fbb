// Test-side entry points into the reference-side adapters
// (ajisai_render_gb300/adapters), called through ctypes by
// tests/test_adapters_cpu.py.  Built only where the reference's sources are
// present, against its headers and the harness library that holds its
// compiled translation units (oracle/_ref/libajref.so).
#include <ajisai/core/film.h>
#include <ajisai/core/primitive/primitive.h>

#include <cstring>
#include <vector>

#include "../ajisai_render_gb300/adapters/gpu_adapters.h"

extern "C" const void* ref_scene_primitives(void* h);

namespace {
const std::vector<aj::Rc<aj::Primitive>>& prims_of(void* harness_scene) {
  return *static_cast<const std::vector<aj::Rc<aj::Primitive>>*>(
      ref_scene_primitives(harness_scene));
}
}  // namespace

extern "C" {

// The triangles the adapters hand the library for a harness scene, in
// PLOCAggregate's gathering order: n, or -1 when out_tris is too small.
int64_t adapter_gather(void* harness_scene, float* out_tris, int64_t cap_tris,
                       float* world, int64_t* ids) {
  std::vector<float> tris;
  std::vector<const aj::Primitive*> prim;
  std::vector<uint32_t> id;
  ajg_adapters::GatherMeshViewTriangles(prims_of(harness_scene), &tris, &prim,
                                        &id, world);
  const int64_t n = (int64_t)id.size();
  if (n > cap_tris) return -1;
  std::memcpy(out_tris, tris.data(), tris.size() * sizeof(float));
  for (int64_t i = 0; i < n; ++i) ids[i] = id[i];
  return n;
}

// Builds the "ploc_gpu" aggregate over a harness scene's primitives.
void adapter_build_aggregate(void* harness_scene, int64_t radius) {
  auto agg = ajg_adapters::CreateGpuPLOCAggregate((size_t)radius);
  agg->Build(prims_of(harness_scene));
}

// Renders the scene file with "pt_gpu" into a reference Film of w x h.
void adapter_render(const char* scene_file, int w, int h, int spp) {
  aj::PTRendererArgs a{spp, 16, 5, 10, 0.9f, true, 20};
  auto r = ajg_adapters::CreateGpuPTRenderer(a, scene_file);
  aj::Film film(aj::Vector2i{w, h}, nullptr);
  r->Render(nullptr, nullptr, &film, nullptr);
}

}  // extern "C"
